// Shared definitions for libdaggergb300: status codes, launch helpers and
// small device utilities.  Everything here is internal; the public C ABI is
// include/dagger_gb300.h.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "../../include/dagger_gb300.h"

// A failed runtime call is recorded (dg_last_error) and, when the error does
// not persist in the context (an allocation or an argument refused), cleared
// from the runtime's per-thread error state, so that the next CUDA call of the
// process, in this library or another, does not report it as its own.
#define DG_CUDA_TRY(expr)                                                       \
  do {                                                                          \
    cudaError_t _e = (expr);                                                    \
    if (_e != cudaSuccess) {                                                    \
      dg_set_last_error(__FILE__, __LINE__, cudaGetErrorString(_e));            \
      cudaGetLastError();                                                       \
      return _e == cudaErrorMemoryAllocation ? DG_ERR_NOMEM : DG_ERR_CUDA;      \
    }                                                                           \
  } while (0)

#define DG_CHECK_ARG(cond, idx)                                                 \
  do {                                                                          \
    if (!(cond)) {                                                              \
      dg_set_last_error(__FILE__, __LINE__, "invalid argument " #idx ": " #cond); \
      return -(idx);                                                            \
    }                                                                           \
  } while (0)

#define DG_TRY(expr)          \
  do {                        \
    int _rc = (expr);         \
    if (_rc) return _rc;      \
  } while (0)

void dg_set_last_error(const char *file, int line, const char *msg);

// Number of SMs of the current device (cached per device).
int dg_num_sms();

namespace dg {
// Stream-ordered device allocation from the library's own memory pool on the
// current device.  The pool keeps freed memory mapped for reuse (no release
// threshold), so calls that allocate the same workspaces again (a factor per
// request, a solve per factor) do not map and unmap gigabytes each time;
// dg_finalize trims it.  Free with cudaFreeAsync.
cudaError_t pool_malloc_async(void **p, size_t bytes, cudaStream_t s);
void pool_trim_all();
}  // namespace dg

// Kernels of one factorization skip their work when either of two device
// "abort" words is non-zero on entry (a failed pivot or a failed step).
__device__ __forceinline__ bool aborted(const int *a, const int *b) {
  return (a && *(volatile const int *)a) || (b && *(volatile const int *)b);
}

// ---------------------------------------------------------------------------
// Internal host entry points shared between translation units.
// ---------------------------------------------------------------------------
namespace dg {

enum Tri { TRI_NONE = 0, TRI_UPPER = 1, TRI_LOWER = 2 };

// C = alpha * op(A) * op(B) + beta * C, column-major.  tri restricts the
// update (and the stores) to the upper or lower triangle of C (SYRK).
int gemm_f64(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
             const double *B, int ldb, double beta, double *C, int ldc, Tri tri,
             const int *abort_flag, cudaStream_t s, const int *abort2 = nullptr);
int gemm_f32(char ta, char tb, int m, int n, int k, float alpha, const float *A, long long lda,
             const float *B, long long ldb, float beta, float *C, long long ldc, Tri tri,
             const int *abort_flag, cudaStream_t s, const int *abort2 = nullptr);

// C = alpha * A * X + beta * C with A the n x n tile grid of a DArray
// (Blocks(nb, nb)) given as a DEVICE array of tile pointers, tile (i, j) =
// tiles_dev[i + j*mt], column-major with ld = its row count.
int gemm_tiles_f64(int n, int nb, int nrhs, double alpha, const double *const *tiles_dev,
                   const double *X, long long ldx, double beta, double *C, long long ldc,
                   const int *abort_flag, cudaStream_t s);
int gemm_tiles_f32(int n, int nb, int nrhs, float alpha, const float *const *tiles_dev,
                   const float *X, long long ldx, float beta, float *C, long long ldc,
                   const int *abort_flag, cudaStream_t s);

int trsm_f64(char side, char uplo, char transa, char diag, int m, int n, double alpha,
             const double *A, int lda, double *B, int ldb, const int *abort_flag,
             cudaStream_t s, const int *abort2 = nullptr);
int trsm_f32(char side, char uplo, char transa, char diag, int m, int n, float alpha,
             const float *A, long long lda, float *B, long long ldb, const int *abort_flag,
             cudaStream_t s, const int *abort2 = nullptr);

// The same with the off-diagonal updates of the recursion emulated on the
// tensor cores, slices in `scratch` (FP64 engine 2).  status (TRSM) and
// info_out (POTRF) are the factorization's info word: kernels skip when it
// is set, and a timeout records DG_ERR_TIMEOUT there.
int trsm_f64_oz(char side, char uplo, char transa, char diag, int m, int n, double alpha,
                const double *A, int lda, double *B, int ldb, void *scratch, size_t bytes,
                int *status, cudaStream_t s);
int potrf_f64_oz(char uplo, int n, double *A, int lda, int *info_out, int info_offset,
                 void *scratch, size_t bytes, cudaStream_t s);

// C = alpha op(A) op(B) + beta C: emulated (scratch of `bytes`, see
// oz_gemm_general) when the scratch allows, else on the FP64 tile kernels.
// Kernels skip when *status is non-zero; a timeout records DG_ERR_TIMEOUT.
int gemm_update_f64(char ta, char tb, int m, int n, int k, double alpha, const double *A,
                    long long lda, const double *B, long long ldb, double beta, double *C,
                    long long ldc, void *scratch, size_t bytes, int *status, cudaStream_t s);

// Tiled LU pieces (lu.cu).  lu_panel_f64 factors the mrows x wcols panel P
// (ld) in place: with pivoting like LAPACK getrf (lpiv[p] = panel row of
// column p's pivot; ipiv_out[p] = info_offset + lpiv[p] + 1; lists = the
// rows the interchanges move, see lu_laswp_tiles), without it like
// generic_lufact!(NoPivot); lists may be null (ipiv only, any width).
// info: atomicMin with info_offset + the 1-based
// column of an exactly zero pivot.  oz (bytes): scratch of the emulated
// updates, or null for the FP64 kernels.  leaf_scratch: lu_leaf_scratch_bytes().
constexpr int kMaxTileRows = 256;  // tile rows of one block column a kernel addresses
size_t lu_leaf_scratch_bytes();
// Sets the LU kernels' shared-memory attributes (once; call before a capture).
void lu_prepare();
int lu_panel_f64(double *P, long long ld, int mrows, int wcols, bool pivot, int *lpiv, int *info,
                 int info_offset, void *leaf_scratch, int *status, void *oz, size_t oz_bytes,
                 long long *ipiv_out, int *lists, int list_cap, cudaStream_t s);
// The (destination, source) row list of one panel applied to a block column
// of ntiles tiles (rows in total, nb per tile, ld = the tile's rows).
int lu_laswp_tiles(double *const *tiles, int ntiles, int nb, int rows, int ncols, const int *lists,
                   int list_cap, cudaStream_t s);
// perm = the composite of npiv interchanges (ipiv, 1-based) on n rows;
// lu_rows_tiles permutes a tiled block column by it through X (n x ncols).
int lu_perm(const long long *ipiv, int npiv, int n, int *perm, cudaStream_t s);
int lu_rows_tiles(double *const *tiles, int ntiles, int nb, int n, int ncols, const int *perm,
                  double *X, cudaStream_t s);
int lu_iota(long long *ipiv, int n, cudaStream_t s);

// W (n x n, ldw) = U^-T for uplo 'U', L^-T for 'L', of the triangular factor
// A (lda), by column-parallel forward substitution on the unit vectors
// (n <= 4096).  Kernels skip when *abort_flag is set.
int trinv_t_f64(char uplo, int n, const double *A, int lda, double *W, int ldw,
                const int *abort_flag, cudaStream_t s);

// W (n x n, ldw) = L^-1 of the unit lower triangle of A (lda; the diagonal
// taken as 1), by column-parallel forward substitution on the unit vectors.
int trinv_unit_lower_f64(int n, const double *A, int lda, double *W, int ldw,
                         const int *abort_flag, cudaStream_t s);

// Tile upload (upload.cu): the rows x cols block at host (row-major, row
// stride ldh, page-locked host or device memory) into a column-major tile
// (ld = rows).  device_readable: whether a kernel may read p.
int upload_tile(const double *host, long long ldh, int rows, int cols, double *tile,
                cudaStream_t s);
bool device_readable(const void *p);

// Tile copies of copytri! (tiles.cu): dst (cols x rows, ldd) = src (rows x
// cols, lds)'; the upper triangle of the n x n tile A mirrored into the lower.
int tile_transpose(const double *src, long long lds, int rows, int cols, double *dst,
                   long long ldd, cudaStream_t s);
int tile_mirror_upper(double *A, long long lda, int n, cudaStream_t s);

// Cholesky of one tile.  info_out receives offset + local pivot index of
// the first failure (written once); kernels skip when info_out, abort_flag
// or abort2 is already non-zero.  The plain FP64 path passes its info word
// as both info_out and abort word.
int potrf_f64(char uplo, int n, double *A, int lda, int *info_out, int info_offset,
              cudaStream_t s, const int *abort_flag = nullptr, const int *abort2 = nullptr);
int potrf_f32(char uplo, int n, float *A, long long lda, int *info_out, int info_offset,
              cudaStream_t s, const int *abort_flag = nullptr, const int *abort2 = nullptr);

// FP32 factor U (A = U'U, upper, in place) of one n x n block (n <= 1024) and
// V = U^-1 (upper, zero below), one cooperative launch (mixed_diag.cu).
// mode 0 factors and inverts (info: atomicCAS of info_off + column + 1 on a
// failed pivot); mode 1 only inverts an already factored block, and runs only
// when *run_if != 0.  scratch: diag_chol_inv_scratch_bytes(), not shared by
// launches that may overlap.
size_t diag_chol_inv_scratch_bytes();
int diag_chol_inv_f32(float *D, long long ld, int n, float *V, long long ldv, void *scratch,
                      int *info, int info_off, int *status, const int *run_if, int mode,
                      cudaStream_t s);

// W (n x n, ldw) = I.
int eye_f64(int n, double *W, int ldw, const int *abort_flag, cudaStream_t s);
int scale_f64(int m, int n, double alpha, double *B, int ldb, const int *abort_flag,
              cudaStream_t s, const int *abort2 = nullptr);
int scale_f32(int m, int n, float alpha, float *B, long long ldb, const int *abort_flag,
              cudaStream_t s, const int *abort2 = nullptr);

// FP64 GEMM emulated on the BF16 tensor cores (oz_gemm.cu).  oz_split cuts
// ncols FP64 vectors of length K (element k of vector c at
// src[c*cstride + k*kstride]) into 7 BF16 slices (slice s of vector c at
// slices + s*sstride + c*ldk) and one 8-byte scale word per vector; oz_gemm
// computes C(m x n) = alpha * sum_p A(p, i) B(p, j) + beta * C from the
// slices of the m A-vectors and n B-vectors (K <= 131072, ldk a multiple of 8);
// tri 1 / 2 stores only the upper / lower triangle.  Kernels skip when
// *status or *abort2 is non-zero; a timed-out wait records DG_ERR_TIMEOUT in
// *status.
constexpr int kOzSlices = 7;
// diag_out (square operands): element c of vector c is written to diag_out[c]
// and left out of the slices and the scale.  dscale: when set, the beta of
// output row i (dmode 1) or column j (dmode 2) is dscale[i] / dscale[j]
// (C = alpha A'B + diag(d) C, or C d), instead of the scalar beta.
// blocks_per_cta > 1: each CTA computes that many 128 x 64 output blocks in
// turn, forming one block's outputs while the next one's products run (for
// launches that share the GPU with others); 0: ceil(blocks / SMs), one wave.
int oz_split(const double *src, long long cstride, long long kstride, int K, int ncols,
             void *slices, long long ldk, long long sstride, unsigned long long *scales,
             const int *abort_flag, cudaStream_t s, const int *abort2 = nullptr,
             double *diag_out = nullptr);
int oz_gemm(int m, int n, int k, double alpha, const void *a_slices, long long lda_k,
            long long a_sstride, const unsigned long long *a_scales, const void *b_slices,
            long long ldb_k, long long b_sstride, const unsigned long long *b_scales, double beta,
            double *C, long long ldc, int tri, int *status, cudaStream_t s,
            const int *abort2 = nullptr, const double *dscale = nullptr, int dmode = 0,
            int blocks_per_cta = 1);
// The rows of the n x n matrix held as an nb x nb tile grid (tile (i, j) at
// tiles_dev[i + j*mt], column-major, ld = its row count): vector c = row c,
// K = n, into slices + s*ldk*n + c*ldk (n <= 131072).
int oz_split_tile_rows(const double *const *tiles_dev, int n, int nb, void *slices, long long ldk,
                       unsigned long long *scales, const int *abort_flag, cudaStream_t s);

// C = alpha op(A) op(B) + beta C (BLAS gemm / syrk arguments; tri as above)
// through split + oz_gemm with the slices in caller scratch of `bytes`
// (oz_scratch_bytes).  Returns 1 without work when k > 131072 or the scratch
// is too small, so the caller can use the FP64 kernels instead.
size_t oz_scratch_bytes(int m, int n, int k, bool same_operand);
int oz_gemm_general(char ta, char tb, int m, int n, int k, double alpha, const double *A,
                    long long lda, const double *B, long long ldb, double beta, double *C,
                    long long ldc, int tri, void *scratch, size_t bytes, int *status,
                    const int *abort2, cudaStream_t s);

// Kernel launch accounting: every kernel launch site adds to a process-wide
// counter (graph captures move their launches into the graph's count, which
// is added back each time the graph is launched).
void count_launches(long long n);
long long launches();

// Selects the FP64 inner product engine: 0 = DFMA register tiles, 1 = DMMA
// (mma.sync m8n8k4 f64), 2 = DFMA tiles plus, for the trailing SYRK/GEMM
// tasks of the tiled Cholesky region, the emulated FP64 GEMM on the tensor
// cores.  DFMA measures faster than DMMA on GB300 (1.25 vs 1.10 TFLOP/s on a
// 4096^3 GEMM).
void set_f64_engine(int engine);
int get_f64_engine();

}  // namespace dg
