// Shared definitions for libdaggergb300: status codes, launch helpers and
// small device utilities.  Everything here is internal; the public C ABI is
// include/dagger_gb300.h.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/dagger_gb300.h"

#define DG_CUDA_TRY(expr)                                                       \
  do {                                                                          \
    cudaError_t _e = (expr);                                                    \
    if (_e != cudaSuccess) {                                                    \
      dg_set_last_error(__FILE__, __LINE__, cudaGetErrorString(_e));            \
      return DG_ERR_CUDA;                                                       \
    }                                                                           \
  } while (0)

#define DG_CHECK_ARG(cond, idx)                                                 \
  do {                                                                          \
    if (!(cond)) {                                                              \
      dg_set_last_error(__FILE__, __LINE__, "invalid argument " #idx ": " #cond); \
      return -(idx);                                                            \
    }                                                                           \
  } while (0)

void dg_set_last_error(const char *file, int line, const char *msg);

// Number of SMs of the current device (cached per device).
int dg_num_sms();

// ---------------------------------------------------------------------------
// Internal host entry points shared between translation units.  They take a
// device "abort" word: when non-null and non-zero when a kernel starts, the
// kernel returns immediately.  The factorization sets it to the LAPACK info
// of the first failing pivot, so later tile tasks of the same factorization
// stop instead of computing on a matrix that is not positive definite.
// ---------------------------------------------------------------------------
namespace dg {

enum Tri { TRI_NONE = 0, TRI_UPPER = 1, TRI_LOWER = 2 };

// C = alpha * op(A) * op(B) + beta * C, FP64, column-major.  tri restricts the
// update (and the stores) to the upper or lower triangle of C (SYRK).
int gemm_f64(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
             const double *B, int ldb, double beta, double *C, int ldc, Tri tri,
             const int *abort_flag, cudaStream_t s);

int trsm_f64(char side, char uplo, char transa, char diag, int m, int n, double alpha,
             const double *A, int lda, double *B, int ldb, const int *abort_flag,
             cudaStream_t s);

// info_dev: device int receiving the LAPACK info (offset + local pivot index,
// written once, by the first failure).  It doubles as the abort word.
int potrf_f64(char uplo, int n, double *A, int lda, int *info_dev, int info_offset,
              cudaStream_t s);

int scale_f64(int m, int n, double alpha, double *B, int ldb, const int *abort_flag,
              cudaStream_t s);

// Kernel launch accounting: every kernel launch site adds to a process-wide
// counter (graph captures move their launches into the graph's count, which
// is added back each time the graph is launched).
void count_launches(long long n);
long long launches();

// Selects the FP64 inner product engine: 0 = DFMA register tiles, 1 = DMMA
// (mma.sync m8n8k4 f64).  Default DFMA: on GB300 it measures faster (1.25 vs
// 1.10 TFLOP/s on a 4096^3 GEMM).
void set_f64_engine(int engine);
int get_f64_engine();

}  // namespace dg
