/*
 * libdaggergb300 — C ABI of the GB300-native tiled Cholesky factor-and-solve.
 *
 * This is the boundary a Dagger.jl backend binds with `ccall`.  Every entry
 * point replaces one call the reference makes on its CUDA path, or hands the
 * whole datadeps region of one such call to the library.  Conventions:
 *   - matrices are column-major FP64 (or the stated type) with an explicit
 *     leading dimension, exactly the LAPACK/BLAS argument conventions;
 *   - pointers are device pointers unless the name says host;
 *   - `stream` is a cudaStream_t passed as void* (NULL = the legacy default
 *     stream), so the header needs no CUDA include;
 *   - the return value is a status: 0 = success, > 0 = LAPACK info (the
 *     1-based order of the first leading minor that is not positive definite),
 *     -i = argument i is invalid, <= -1000 = one of the DG_ERR_* codes below.
 *     dg_last_error() returns a message for the last failure on this thread.
 * Entry points may be called from several host threads at once (the
 * reference runs each task on its own Julia task, ext/CUDAExt.jl:309-327).
 * Calls on different streams run concurrently: each stream handle gets its
 * own workspace for the emulated FP64 engine and the LU, grown in stream
 * order, and results do not depend on what runs beside them.  Calls on the
 * same stream handle from different threads take turns (the later call's
 * work is ordered after the earlier one's); the noalloc entry point, which
 * has one static scratch, takes turns across all streams.
 *
 * Reference paths are within JuliaParallel/Dagger.jl v0.22.0.
 */
#ifndef DAGGER_GB300_H
#define DAGGER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DG_OK 0
#define DG_ERR_CUDA (-1000)        /* a CUDA runtime call failed              */
#define DG_ERR_TIMEOUT (-1001)     /* a bounded device wait gave up           */
#define DG_ERR_NOMEM (-1002)       /* allocation refused / budget exceeded    */
#define DG_ERR_UNSUPPORTED (-1003) /* option not supported by this build      */
#define DG_ERR_NOCONVERGE (-1004)  /* iterative refinement did not converge   */
#define DG_ERR_STATE (-1005)       /* handle used in the wrong state          */

/* ---------------------------------------------------------------------------
 * Library state
 * ------------------------------------------------------------------------- */

/* Version string of this build. */
const char *dg_version(void);

/* Message describing the last failure on the calling thread ("" if none). */
const char *dg_last_error(void);

/* Number of kernels this process has launched through the library so far
 * (a graph launch counts every kernel node it contains). */
long long dg_kernel_launches(void);

/* Frees library-owned workspaces and cached graphs of the current device.
 * Caller memory is never freed by the library. */
int dg_finalize(void);
/* Returns to the device the memory that the library keeps for reuse on the
 * current device: the per-stream workspaces that no call is using (after the
 * work queued with them has finished) and the free blocks of the library's
 * stream-ordered pool.  Blocks in use are not touched; later calls allocate
 * again as needed. */
int dg_release_memory(void);

/* Device memory and streams for hosts that do not link a CUDA binding (the
 * reference reaches the GPU through CUDA.jl; a backend on this library
 * allocates its tiles here instead: CuArray allocation and copies in
 * ext/CUDAExt.jl:120-154 are what these replace).  kind: 0 host->device,
 * 1 device->host, 2 device->device. */
int dg_set_device(int device);
int dg_device_alloc(size_t bytes, void **out);
int dg_device_free(void *p);
/* Page-locked host memory the device can read directly (the source of
 * dg_cholesky_tiled_host). */
int dg_host_alloc(size_t bytes, void **out);
int dg_host_free(void *p);
int dg_copy(void *dst, const void *src, size_t bytes, int kind, void *stream);
int dg_stream_create(void **out);
int dg_stream_destroy(void *stream);
int dg_stream_synchronize(void *stream);

/* ---------------------------------------------------------------------------
 * Tile operations: the BLAS/LAPACK calls the reference substitutes with
 * CUBLAS/CUSOLVER through Dagger.move(::CPUProc, ::CuArrayDeviceProc,
 * ::typeof(fn)) (ext/CUDAExt.jl:329-348).  Same arguments, same meaning.
 * ------------------------------------------------------------------------- */

/* LAPACK.potrf!(uplo, A) -> (A, info): Cholesky of one tile, in place.
 * Replaces the call in potrf_checked! (src/array/cholesky.jl:3).  When
 * info_host is non-NULL the call synchronises `stream` and stores info there
 * (the reference's potrf! returns info to the host); the return value is then
 * that info.  When NULL the call is asynchronous and info is not reported;
 * use dg_potrf_async with a device word of the caller's to read it later. */
int dg_potrf(char uplo, int n, double *A, int lda, int *info_host, void *stream);

/* Asynchronous form: info (0 or the failing pivot) is written to the device
 * int info_dev, which must be zero on entry. */
int dg_potrf_async(char uplo, int n, double *A, int lda, int *info_dev, void *stream);

/* BLAS.trsm!(side, uplo, transa, diag, alpha, A, B): B <- alpha op(A)^-1 B
 * ('L') or alpha B op(A)^-1 ('R').  Replaces src/array/cholesky.jl:41,86 and
 * src/array/trsm.jl:95-183. */
int dg_trsm(char side, char uplo, char transa, char diag, int m, int n, double alpha,
            const double *A, int lda, double *B, int ldb, void *stream);

/* BLAS.syrk!(uplo, trans, alpha, A, beta, C): C <- alpha A'A + beta C
 * (trans 'T') or alpha AA' + beta C ('N'), one triangle of C.  Replaces
 * src/array/cholesky.jl:47,92. */
int dg_syrk(char uplo, char trans, int n, int k, double alpha, const double *A, int lda,
            double beta, double *C, int ldc, void *stream);

/* BLAS.gemm!(tA, tB, alpha, A, B, beta, C): C <- alpha op(A) op(B) + beta C.
 * Replaces src/array/cholesky.jl:50,95 and src/array/trsm.jl:99-183. */
int dg_gemm(char transa, char transb, int m, int n, int k, double alpha, const double *A,
            int lda, const double *B, int ldb, double beta, double *C, int ldc, void *stream);

/* BLAS.trsv!(uplo, trans, diag, A, x) and BLAS.gemv!(trans, alpha, A, x,
 * beta, y): the vector-RHS tile calls of src/array/trsm.jl:21-49. */
int dg_trsv(char uplo, char trans, char diag, int n, const double *A, int lda, double *x,
            void *stream);
int dg_gemv(char trans, int m, int n, double alpha, const double *A, int lda,
            const double *x, double beta, double *y, void *stream);

/* ---------------------------------------------------------------------------
 * Datadeps regions: the library-side form of Dagger.spawn_datadeps
 * (src/datadeps/queue.jl:64-106).  Tasks are recorded in submission order with
 * the BLAS arguments above; each matrix argument carries its access mode
 * (In / Out / InOut, src/datadeps/aliasing.jl:165-181) and the library derives
 * the dependencies with the datadeps rules (a writer waits for the last
 * writer and the readers since; a reader waits for the last writer; overlap
 * is decided on the strided byte footprint of each argument).  dg_region_run
 * issues the DAG onto a pool of CUDA streams joined by events, captured into
 * a CUDA graph that is cached and replayed when the same region (same tasks,
 * same pointers) runs again.
 * ------------------------------------------------------------------------- */

typedef struct dg_region dg_region;

#define DG_IN 1
#define DG_OUT 2
#define DG_INOUT 3

enum dg_op {
  DG_OP_POTRF = 1, /* a = tile (InOut)                                     */
  DG_OP_TRSM = 2,  /* a = triangle (In), c = B (InOut)                      */
  DG_OP_SYRK = 3,  /* a (In), c (InOut)                                     */
  DG_OP_GEMM = 4,  /* a, b (In), c (InOut)                                  */
  DG_OP_COPY = 5   /* a (In) copied to c (Out), same shape                  */
};

typedef struct dg_task {
  int op;                     /* enum dg_op                                */
  char side, uplo, transa, transb, diag, trans;
  int m, n, k;                /* BLAS sizes of the op                      */
  double alpha, beta;
  const double *a; int lda;
  const double *b; int ldb;
  double *c; int ldc;
  int mode_a, mode_b, mode_c; /* DG_IN / DG_OUT / DG_INOUT (0 = default)   */
  int info_offset;            /* POTRF: global row offset of the tile      */
} dg_task;

dg_region *dg_region_create(void);
int dg_region_add(dg_region *r, const dg_task *t);
/* Number of tasks recorded and of dependency edges derived. */
int dg_region_stats(const dg_region *r, int *ntasks, int *nedges);
/* Fills preds (size >= nedges) with (task, predecessor) pairs, in order. */
int dg_region_edges(const dg_region *r, int *pairs, int cap);
/* Runs the region on `stream` (the graph is launched there, or the streams
 * are forked from and joined back to it).  use_graph = 0 issues the same
 * streams and events without capture; serial = 1 issues every task on
 * `stream` in submission order (for differential tests).  Returns the LAPACK
 * info of the first failed POTRF (synchronising), or 0. */
int dg_region_run(dg_region *r, int use_graph, int serial, void *stream);
void dg_region_destroy(dg_region *r);

/* ---------------------------------------------------------------------------
 * Whole-call entry points: the datadeps region of one reference call, built
 * natively with the reference's task loop and run as one cached graph.
 * `tiles` is the mt x mt column-major grid of tile pointers of a DArray with
 * Blocks(nb, nb) (DArray.chunks), tile (i, j) = tiles[i + j*mt], each tile
 * column-major with leading dimension = its row count (min(nb, n - i*nb)).
 * ------------------------------------------------------------------------- */

/* LinearAlgebra._chol!(A::DArray, UpperTriangular|LowerTriangular)
 * (src/array/cholesky.jl:19-108).  Returns info (0 on success). */
int dg_cholesky_tiled(char uplo, int n, int nb, double *const *tiles, void *stream);

/* ldiv!(C::Cholesky{T,<:DMatrix}, B) (src/array/linalg.jl:352-405) with the
 * factor's tiles and B (n x nrhs) blocked Blocks(nb, nb): btiles is the
 * bmt x bnt column-major grid, bmt = mt, bnt = ceil(nrhs / nb). */
int dg_cholesky_solve_tiled(char uplo, int n, int nb, double *const *tiles, int nrhs,
                            double *const *btiles, void *stream);

/* Extension of the two calls above for the emulated FP64 engine (engine 2,
 * nb <= 1024; DG_ERR_UNSUPPORTED otherwise, without work): the factorization
 * forms W_k = U_kk^-T (uplo 'U') or L_kk^-T ('L') of every diagonal factor
 * tile for its panel products anyway; dg_cholesky_tiled_winv keeps all mt of
 * them in winv (device, mt * nb * nb doubles: W_k at winv + k*nb*nb,
 * column-major, ld = the tile's row count), and dg_cholesky_solve_tiled_winv
 * then applies each diagonal block's solve as one emulated product with W_k
 * (or W_k') instead of a substitution on the FP64 pipe.  winv belongs to the
 * factor it was made with: the solve reads both.  Results satisfy the same
 * bounds as dg_cholesky_tiled / dg_cholesky_solve_tiled. */
int dg_cholesky_tiled_winv(char uplo, int n, int nb, double *const *tiles, double *winv,
                           void *stream);
/* cholesky(distribute(A, Blocks(nb, nb))) with A on the host: the factor's
 * graph also moves the tiles to the device, one upload task per tile
 * (element (r, c) of A at host[r*ldh + c], row-major, so a C-contiguous or
 * symmetric array; page-locked host memory or device memory, argument 4
 * otherwise), so each tile's first task waits only for its own transfer and
 * the transfers overlap the first steps' updates (Dagger moves CPU chunks to
 * the GPU processor when the first task needs them, ext/CUDAExt.jl:329-348).
 * tiles receive the whole matrix as dg_cholesky_tiled expects it, then the
 * factor; winv (engine 2 only, else DG_ERR_UNSUPPORTED; may be NULL) as in
 * dg_cholesky_tiled_winv.  Returns info. */
int dg_cholesky_tiled_host(char uplo, int n, int nb, const double *host, long long ldh,
                           double *const *tiles, double *winv, void *stream);
int dg_cholesky_solve_tiled_winv(char uplo, int n, int nb, double *const *tiles,
                                 const double *winv, int nrhs, double *const *btiles,
                                 void *stream);

/* LinearAlgebra.mul! on DArrays (src/array/mul.jl): the datadeps regions of
 * gemm_dagger! (mul.jl:133-215) and syrk_dagger! + copytri! (mul.jl:230-425)
 * as one cached graph each.  Square Blocks(nb, nb) tile grids (column-major
 * grids of column-major tiles, ld = a tile's row count, ragged last
 * row/column), the layout of dg_cholesky_tiled.
 * dg_gemm_tiled: C (m x n) = alpha op(A) op(B) + beta C, op(A) m x k, op(B)
 * k x n; transa/transb 'N' or 'T' ('C' reads as 'T' for real data).
 * dg_syrk_tiled: C (n x n) = alpha op(A) op(A)' + beta C, op(A) n x k
 * ('N': A is n x k, 'T': A is k x n): the upper tiles are computed (syrk! on
 * the diagonal, gemm! above it) and copied to the lower ones, so C is the
 * full symmetric result, as syrk_dagger! leaves it.
 * With dg_set_f64_engine(2) and nb <= 1024 every tile product is the emulated
 * FP64 GEMM (each tile's vectors cut into slices once per contraction step). */
int dg_gemm_tiled(char transa, char transb, int m, int n, int k, int nb, double alpha,
                  double *const *atiles, double *const *btiles, double beta,
                  double *const *ctiles, void *stream);
int dg_syrk_tiled(char trans, int n, int k, int nb, double alpha, double *const *atiles,
                  double beta, double *const *ctiles, void *stream);

/* ishermitian(::DArray) (src/array/linalg.jl:90-124; pair test
 * is_cross_hermitian, linalg.jl:43-48) over the same tile grid.  Returns 1
 * (Hermitian), 0 (not), or a negative status.  Synchronises `stream`. */
int dg_ishermitian_tiled(int n, int nb, double *const *tiles, void *stream);

/* LAPACK.chkfinite(::DArray) (src/array/linalg.jl:138-148): 1 when every
 * element is finite, 0 otherwise.  Synchronises `stream`. */
int dg_chkfinite_tiled(int n, int nb, double *const *tiles, void *stream);
/* The same over an m x n tile grid with Blocks(mb, nb) (lu!'s chkfinite of a
 * rectangular DArray, src/array/lu.jl:306-309 -> linalg.jl:138-148). */
int dg_chkfinite_tiled_mn(int m, int n, int mb, int nb, double *const *tiles, void *stream);

/* copyto!(buffer, A) between two tilings of one m x n matrix: the copy of
 * maybe_copy_buffered / copy_buffered (src/array/copy.jl:3-37), which
 * _chol! (cholesky.jl:34), ldiv! (linalg.jl:362-404) and mul!
 * (mul.jl:11-41) use to move an argument to the Blocks they need and back.
 * src_tiles / dst_tiles: host arrays of device tile pointers for Blocks(src_mb,
 * src_nb) and Blocks(dst_mb, dst_nb); a vector is n = 1 with nb = 1.
 * Stream-ordered (the pointer grids are staged before the call returns). */
int dg_copy_reblock(int m, int n, int src_mb, int src_nb, double *const *src_tiles, int dst_mb,
                    int dst_nb, double *const *dst_tiles, void *stream);

/* Selects the FP64 tile engine: 0 = DFMA register tiles, 1 = DMMA
 * (mma.sync.m8n8k4.f64), 2 = DFMA for POTRF/TRSM plus, inside
 * dg_cholesky_tiled with nb <= 1024, the trailing SYRK/GEMM tile updates
 * emulated on the BF16 tensor cores with FP64 accuracy (7 slices of 8 bits
 * per operand vector, exact products, FP64 sum; see
 * dg_gemm_f64_emulated_tn).  Returns the previous setting.  The setting is
 * process-wide. */
int dg_set_f64_engine(int engine);
/* The current setting of dg_set_f64_engine. */
int dg_get_f64_engine(void);

/* ---------------------------------------------------------------------------
 * Mixed-precision form (no counterpart in the reference: a faster path beside
 * the FP64 drop-in, reached from the same DArray tiles).  The factor of the
 * diagonally scaled matrix is computed with 16-bit tensor-core trailing
 * updates (tcgen05, FP32 accumulation), FP32 diagonal blocks with an FP64
 * retry on a failed pivot, and FP32 panel solves; solutions are refined in
 * FP64 (iterative refinement, GMRES-IR when it stalls) to a normwise backward
 * error tolerance.  The caller's FP64 tiles must stay valid while the handle
 * is used (they give the FP64 residuals).
 * ------------------------------------------------------------------------- */

#define DG_PREC_BF16 1    /* BF16 operands                                   */
#define DG_PREC_BF16X3 3  /* BF16 hi/lo split, three products               */
#define DG_PREC_FP16 11   /* FP16 operands, per-panel power-of-two scaling   */
#define DG_PREC_FP16X3 13 /* FP16 hi/lo split with per-panel scaling        */
#define DG_PREC_FP32 32   /* FP32 CUDA-core trailing updates                */
#define DG_PREC_BF16X6 6  /* BF16 hi/mid/lo split, six products: FP32-accurate
                             tensor-core trailing updates                    */
#define DG_PREC_FP8 8     /* FP8 E4M3 operands with a power-of-two scale per
                             vector, one kind::f8f6f4 product (4 significant
                             bits: for well-conditioned matrices)            */

typedef struct dg_mixed dg_mixed;

typedef struct dg_mixed_stats {
  int n, nb, precision;
  int info;              /* 0, or the order of the first non-positive pivot */
  int retries;           /* diagonal blocks refactored in FP64              */
  float factor_ms;       /* device time of the factorization                */
  double norm_inf;       /* ||A||_inf                                       */
  long long device_bytes;
  double shift;          /* diagonal shift the factor was computed with     */
} dg_mixed_stats;

typedef struct dg_ir_opts {
  double tol;            /* normwise backward error target (default 1e-12)  */
  int max_iter;          /* outer refinement steps (default 30)             */
  int gmres;             /* 0 = switch when refinement stalls, 1 = always,
                            2 = never                                       */
  int restart;           /* GMRES cycle length (default 30)                 */
  double gmres_inner_tol;/* relative residual of each GMRES cycle (1e-4)    */
} dg_ir_opts;

typedef struct dg_ir_report {
  int iterations, gmres_iterations, used_gmres, converged;
  double backward_error; /* worst column                                    */
  float solve_ms;
} dg_ir_report;

/* Factors the n x n FP64 tile grid (same layout as dg_cholesky_tiled; nb a
 * multiple of 64).  Returns 0, the info of a failed pivot (> 0, the handle is
 * still returned for inspection), or a negative status. */
int dg_mixed_factor(dg_mixed **out, int n, int nb, double *const *tiles, int precision,
                    void *stream);

/* As dg_mixed_factor, factoring S A S + shift I instead (S = diag(a_ii)^-1/2,
 * so the scaled matrix has a unit diagonal).  A small shift keeps the
 * low-precision factorization of a very ill-conditioned matrix from breaking
 * down; the factor then serves as a preconditioner and refinement (GMRES-IR)
 * still converges to the solution of A x = b. */
int dg_mixed_factor_ex(dg_mixed **out, int n, int nb, double *const *tiles, int precision,
                       double shift, void *stream);

/* X = A^-1 B (FP64, device, column-major) by refinement with the factor. */
int dg_mixed_solve(const dg_mixed *f, int nrhs, const double *B, int ldb, double *X, int ldx,
                   const dg_ir_opts *opts, dg_ir_report *report, void *stream);
int dg_mixed_info(const dg_mixed *f, dg_mixed_stats *stats);
/* Frees the handle's device memory, stream-ordered on the stream the factor
 * was created on (work on other streams that uses the handle must be complete). */
void dg_mixed_destroy(dg_mixed *f);

/* The tensor-core building block: C = alpha A'B + beta C with 16-bit K-major
 * operands (A k x m and B k x n column-major, BF16 or FP16 when fp16 = 1),
 * terms = 1 or 3 (hi/lo split), FP32 C.  k, lda, ldb multiples of 8. */
int dg_gemm_tc_tn(int m, int n, int k, int terms, int fp16, const void *a_hi, const void *a_lo,
                  int lda, const void *b_hi, const void *b_lo, int ldb, float alpha, float beta,
                  float *C, int ldc, int bn, int *status, void *stream);

/* FP32-accurate GEMM on the BF16 tensor cores (the mixed factor's panel
 * solve and its bf16x6 updates; no counterpart in the reference): C = alpha
 * A'B + beta C with A k x m, B k x n and C m x n column-major FP32 on the
 * device; each operand is cut into three BF16 slices and the six slice
 * products whose orders sum to at most 4 accumulate in FP32 (about 24
 * significant bits).  k, lda, ldb multiples of 8.  Allocates stream-ordered
 * scratch for the slices. */
int dg_gemm_f32_tc_tn(int m, int n, int k, float alpha, const float *A, int lda, const float *B,
                      int ldb, float beta, float *C, int ldc, void *stream);

/* The FP8 form of the same product: C = alpha A'B + beta C with FP32 K-major
 * operands (A k x m, B k x n, column-major) cut to E4M3 with a power-of-two
 * scale per vector (each vector's largest magnitude in [128, 256) before
 * rounding) and multiplied by one tcgen05.mma kind::f8f6f4 per K step of 32;
 * the scales are applied to the FP32 accumulators.  Each operand value keeps
 * 4 significant bits.  Allocates stream-ordered scratch. */
int dg_gemm_f8_tc_tn(int m, int n, int k, float alpha, const float *A, int lda, const float *B,
                     int ldb, float beta, float *C, int ldc, void *stream);

/* The diagonal-block kernel of the mixed factor (no counterpart in the
 * reference): the FP32 Cholesky factor U (A = U'U, upper, in place) of one
 * n x n block, n <= 1024, and V = U^-1 (upper, zero below), both column-major
 * on the device, in one cooperative launch.  Returns (and stores in
 * *info_host) the 1-based column of the first pivot that is not positive, or
 * 0.  Synchronises `stream`. */
int dg_potrf_inv_f32(int n, float *A, int lda, float *V, int ldv, int *info_host, void *stream);

/* FP64 GEMM emulated on the BF16 tensor cores: C = alpha A'B + beta C with
 * A k x m, B k x n and C m x n column-major FP64 on the device, k <= 131072.
 * The building block of engine 2's trailing updates (BLAS.gemm!('T', 'N')
 * of src/array/cholesky.jl:50); its error is that of an FP64 GEMM relative
 * to max|A(:, i)| max|B(:, j)| k.  Allocates stream-ordered scratch. */
int dg_gemm_f64_emulated_tn(int m, int n, int k, double alpha, const double *A, int lda,
                            const double *B, int ldb, double beta, double *C, int ldc,
                            void *stream);

/* Its two stages, for operands reused across products.  dg_f64_slices cuts
 * ncols FP64 vectors of length k <= 131072 (element p of vector c at
 * src[c*cstride + p*kstride]) into 7 BF16 slices, slice s of vector c at
 * slices + 2*(s*ldk*ncols + c*ldk) bytes (ldk >= k, a multiple of 8; the
 * buffer 16-byte aligned, 14*ldk*ncols bytes), and one 8-byte scale word per
 * vector in `scales` (8-byte aligned, 8*ncols bytes).  dg_gemm_f64_slices
 * computes C = alpha A'B + beta C from the slices of the m columns of A and
 * the n columns of B (lda_k, ldb_k: their ldk).  status: optional device
 * word; the kernel skips when it is non-zero and records DG_ERR_TIMEOUT
 * there if a wait times out. */
int dg_f64_slices(int k, int ncols, const double *src, long long cstride, long long kstride,
                  void *slices, int ldk, void *scales, void *stream);
int dg_gemm_f64_slices(int m, int n, int k, double alpha, const void *a_slices, int lda_k,
                       const void *a_scales, const void *b_slices, int ldb_k,
                       const void *b_scales, double beta, double *C, int ldc, int *status,
                       void *stream);

/* ---------------------------------------------------------------------------
 * Batched persistent launch (no counterpart in the reference, which would
 * spawn one datadeps region per system): `count` independent SPD systems of
 * order n[i] <= 1024 with nrhs[i] <= 8 right-hand sides, all factored and
 * solved in ONE launch.  A[i] (n x n, column-major, ld n) is overwritten by
 * its lower Cholesky factor in mode 0 (FP64) and left intact in mode 1 (FP32
 * factor + FP64 iterative refinement to normwise backward error `tol`, at
 * most max_iter steps).  B[i], X[i]: n x nrhs, ld n.  bucket_w (5 entries,
 * for n <= 64, 128, 256, 512, 1024) gives each size bucket's panel width (16
 * or 32; NULL = 32), ctas_per_sm the persistent grid per SM.  info (2*count
 * ints, may be NULL) receives each system's pivot info and refinement steps,
 * berr (count doubles, may be NULL) its backward error (mode 1).  Returns 0,
 * or 1 + the index of the first system whose factorization failed.
 * ------------------------------------------------------------------------- */
int dg_batched_potrs(int count, const int *n, const int *nrhs, double *const *A,
                     const double *const *B, double *const *X, int mode, double tol, int max_iter,
                     const int *bucket_w, int ctas_per_sm, int *info, double *berr,
                     float *elapsed_ms, void *stream);

/* Allocation-free form of dg_batched_potrs (no counterpart in the reference).
 * For callers that must not allocate device memory while they run: a server
 * that reserved its whole device budget at start-up and admits work against
 * it, a host whose pool allocator must not be bypassed, or a real-time loop
 * that forbids allocation after initialisation.  dg_batched_potrs allocates
 * descriptors and FP32 workspaces per call; this entry point takes them from
 * one library-owned static device array of 64 MiB instead (held by every GPU
 * that loads the library until exit) and calls no allocator.  Limits: at most
 * 4096 systems, and in mode 1 the FP32 workspaces (4 n^2 bytes per system,
 * 256-byte aligned) plus the descriptors must fit the 64 MiB; a larger batch
 * returns DG_ERR_NOMEM without launching.  Each call looks up the array's
 * device address on the current device (cudaGetSymbolAddress, no
 * allocation).  The call is synchronous: it stages descriptors from host
 * memory and synchronises `stream` before it returns, so it cannot be called
 * while `stream` is being captured into a graph.  Every call uses the same
 * array: calls from several host threads take turns on a library lock held
 * until the call's work has finished.  Arguments and results as
 * dg_batched_potrs, without the timing output. */
int dg_batched_potrs_noalloc(int count, const int *n, const int *nrhs, double *const *A,
                             const double *const *B, double *const *X, int mode, double tol,
                             int max_iter, const int *bucket_w, int ctas_per_sm, int *info,
                             double *berr, void *stream);

/* ---------------------------------------------------------------------------
 * LU factorization (src/array/lu.jl) and the solve with it (linalg.jl:264-308)
 * ------------------------------------------------------------------------- */

/* LAPACK.getrf!(A) -> (A, ipiv, info) on one column-major m x n matrix in
 * device memory: the pivoted LU in place, L unit lower below the diagonal and
 * U on and above it; ipiv (device, min(m, n) int64) the 1-based rows
 * interchanged with each row, as LAPACK.  Replaces the panel task of
 * lu!(A, RowMaximum()) (factor_panel_lapack!, src/array/lu.jl:263-304, whose
 * GPU form is the per-column search_and_update_ipiv! / swaprows_panel! /
 * update_panel_diag! / update_panel_offdiag! tasks, lu.jl:24-127).  Same
 * pivots as LAPACK: the first row of largest magnitude; an exactly zero
 * pivot sets info to its 1-based column and the factorization continues.
 * Synchronises `stream`; *info_host = info, and the return value is info
 * (>= 0) or a negative error.  m <= 73728 (DG_ERR_UNSUPPORTED above). */
int dg_getrf(int m, int n, double *A, int lda, long long *ipiv, int *info_host, void *stream);

/* lu!(A, RowMaximum()) (pivot = 1, lu.jl:306-410) or lu!(A, NoPivot())
 * (pivot = 0, lu.jl:5-54) of the m x n DArray with Blocks(nb, nb) held as
 * the mt x nt column-major tile grid `tiles` (tile (i, j) = tiles[i + j*mt],
 * column-major, ld = its rows; ragged last row and column), in place, as one
 * cached graph of the reference's task loop: per step the block column's
 * panel factorization (dg_getrf's algorithm on the gathered panel, or the
 * diagonal tile without pivoting), its row interchanges applied to every
 * other block column (swaprows_trail!), TRSM('L','L','N','U') of the row
 * panel (and, without pivoting, TRSM('R','U','N','N') of the column panel)
 * and GEMM('N','N',-1) of the trailing tiles, with the FP64 engine chosen by
 * dg_set_f64_engine (engine 2: emulated trailing updates).  ipiv (device,
 * min(m, n) int64) receives the 1-based global pivots (1..min(m, n) without
 * pivoting, as the reference's DVector).  Synchronises `stream`.  Returns 0,
 * info > 0 (the first exactly zero pivot, 1-based, for
 * LinearAlgebra._check_lu_success / SingularException), or a negative error.
 * nb <= 1024, mt <= 256, m <= 73728; library-owned workspace (one per device, shared with
 * the other tiled calls: calls that overlap on the GPU must not share it). */
int dg_lu_tiled(int m, int n, int nb, double *const *tiles, int pivot, long long *ipiv,
                void *stream);

/* ldiv!(F::LU, B) (linalg.jl:264-308) for the n x n factors of dg_lu_tiled
 * (tiles, ipiv) and the n x nrhs right-hand sides held as the tile grid
 * btiles (Blocks(nb, nb), tile (i, j) = btiles[i + j*mt]), overwritten with
 * the solution: B's rows permuted by ipiv (_apply_ipiv_rows!, one
 * permutation per block column of B), then the unit-lower forward and the
 * upper backward block solves (Dagger.trsm!).  Synchronises `stream`. */
int dg_lu_solve_tiled(int n, int nb, double *const *tiles, const long long *ipiv, int nrhs,
                      double *const *btiles, void *stream);

/* Measures the device's FP64 fused-multiply-add throughput (TFLOP/s) with
 * independent FMA chains on every SM; the benchmark's FP64 roofline.  No
 * counterpart in the reference (measurement utility). */
int dg_probe_fp64_fma_tflops(int iters, double *tflops, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* DAGGER_GB300_H */
