// FP64 triangular solve (TRSM) and Cholesky (POTRF) of one tile.
//
// These replace LAPACK.potrf! in potrf_checked! (src/array/cholesky.jl:3 of
// Dagger.jl) and BLAS.trsm! in the panel step (cholesky.jl:41,86) and in the
// block solves (src/array/trsm.jl:95-183).
//
// Both are recursive: the triangle is halved until a 64 x 64 diagonal block
// remains, and the off-diagonal work of each level is a GEMM / SYRK on the
// tile GEMM kernel (gemm_f64.cu), so nearly all flops run in the GEMM.  The
// 64 x 64 base cases are shared-memory kernels:
//   trsm_base: the 64 x 64 triangle and a 64 x 8 slab of the right-hand side
//              are staged in shared memory; each warp solves one column by
//              forward/backward substitution with the column held in two
//              registers per lane and the solved entry broadcast by shuffle.
//   potrf_base: one CTA factors the 64 x 64 block in shared memory
//              (right-looking, column by column).  A pivot that is not
//              positive (or NaN) records the LAPACK info in a device word and
//              stops; the word is also the abort flag every later kernel of
//              the same factorization checks on entry.
// Every access is bounds-checked against the block length, so ragged last
// tiles (n not a multiple of the block size) need no padding.
#include "dg_common.cuh"

namespace dg {

namespace {

constexpr int TB = 64;      // base block size
constexpr int TRSM_W = 8;   // right-hand-side columns per CTA (one per warp)

struct TriView {
  const double *T;
  int ld;
  bool trans;  // M(i, j) = T(j, i)
  bool lower;  // M is lower triangular
  bool unit;   // unit diagonal
};

__device__ __forceinline__ bool aborted(const int *f) {
  return f && *(volatile const int *)f;
}

// Solve M[r0:r0+len, r0:r0+len] X = X in place for the columns handled by
// this CTA.  X(i, c) lives at X[i * rs + c * cs].
__global__ void __launch_bounds__(256) trsm_base_kernel(TriView tv, int r0, int len, double *X,
                                                        long long rs, long long cs, int nn,
                                                        const int *abort_flag) {
  if (aborted(abort_flag)) return;
  __shared__ double Ms[TB][TB + 1];
  __shared__ double dinv[TB];
  __shared__ double Xs[TB][TRSM_W + 1];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int c0 = blockIdx.x * TRSM_W;
  const int wcols = min(TRSM_W, nn - c0);
  // stage the triangle (coalesced along whichever index is contiguous)
  for (int e = tid; e < len * len; e += nt) {
    int i, j;
    if (!tv.trans) { i = e % len; j = e / len; } else { j = e % len; i = e / len; }
    if (tv.lower ? (j <= i) : (j >= i)) {
      size_t off = tv.trans ? (size_t)(r0 + j) + (size_t)(r0 + i) * tv.ld
                            : (size_t)(r0 + i) + (size_t)(r0 + j) * tv.ld;
      Ms[i][j] = tv.T[off];
    }
  }
  // stage the right-hand side slab
  for (int e = tid; e < len * wcols; e += nt) {
    int i, c;
    if (rs == 1) { i = e % len; c = e / len; } else { c = e % wcols; i = e / wcols; }
    Xs[i][c] = X[(size_t)(r0 + i) * rs + (size_t)(c0 + c) * cs];
  }
  __syncthreads();
  if (tid < len) dinv[tid] = tv.unit ? 1.0 : 1.0 / Ms[tid][tid];
  __syncthreads();
  const int lane = tid & 31, warp = tid >> 5;
  if (warp < wcols) {
    const int c = warp;
    double x0 = lane < len ? Xs[lane][c] : 0.0;
    double x1 = lane + 32 < len ? Xs[lane + 32][c] : 0.0;
    if (tv.lower) {
      for (int i = 0; i < len; i++) {
        double xi = __shfl_sync(0xffffffffu, i < 32 ? x0 : x1, i & 31) * dinv[i];
        if (i < 32) { if (lane == i) x0 = xi; } else { if (lane == i - 32) x1 = xi; }
        if (lane > i && lane < len) x0 = fma(-Ms[lane][i], xi, x0);
        if (lane + 32 > i && lane + 32 < len) x1 = fma(-Ms[lane + 32][i], xi, x1);
      }
    } else {
      for (int i = len - 1; i >= 0; i--) {
        double xi = __shfl_sync(0xffffffffu, i < 32 ? x0 : x1, i & 31) * dinv[i];
        if (i < 32) { if (lane == i) x0 = xi; } else { if (lane == i - 32) x1 = xi; }
        if (lane < i) x0 = fma(-Ms[lane][i], xi, x0);
        if (lane + 32 < i) x1 = fma(-Ms[lane + 32][i], xi, x1);
      }
    }
    if (lane < len) Xs[lane][c] = x0;
    if (lane + 32 < len) Xs[lane + 32][c] = x1;
  }
  __syncthreads();
  for (int e = tid; e < len * wcols; e += nt) {
    int i, c;
    if (rs == 1) { i = e % len; c = e / len; } else { c = e % wcols; i = e / wcols; }
    X[(size_t)(r0 + i) * rs + (size_t)(c0 + c) * cs] = Xs[i][c];
  }
}

// Cholesky of one block of length len <= 64 at A (leading dimension lda).
// Works on the lower triangle L; for uplo 'U' the block is staged transposed
// (U' = L) and written back transposed, so only the uplo triangle is touched.
__global__ void __launch_bounds__(256) potrf_base_kernel(int upper, int len, double *A, int lda,
                                                         int *info, int info_offset) {
  if (aborted(info)) return;
  __shared__ double Ms[TB][TB + 1];
  __shared__ int fail_at;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < len * len; e += nt) {
    int i, j;
    if (!upper) { i = e % len; j = e / len; } else { j = e % len; i = e / len; }
    if (j <= i) Ms[i][j] = upper ? A[(size_t)j + (size_t)i * lda] : A[(size_t)i + (size_t)j * lda];
  }
  if (tid == 0) fail_at = -1;
  __syncthreads();
  for (int j = 0; j < len; j++) {
    double d = Ms[j][j];
    if (!(d > 0.0)) {  // not positive, or NaN: LAPACK's test in dpotrf2/dpotf2
      if (tid == 0) fail_at = j;
      break;           // d is the same for every thread: uniform exit
    }
    d = sqrt(d);
    const double r = 1.0 / d;
    __syncthreads();   // every thread has read Ms[j][j]
    for (int i = j + 1 + tid; i < len; i += nt) Ms[i][j] *= r;
    if (tid == 0) Ms[j][j] = d;
    __syncthreads();
    const int w = len - j - 1;
    for (int e = tid; e < w * w; e += nt) {
      int i = j + 1 + e % w, k = j + 1 + e / w;
      if (k <= i) Ms[i][k] = fma(-Ms[i][j], Ms[k][j], Ms[i][k]);
    }
    __syncthreads();
  }
  __syncthreads();
  if (fail_at >= 0 && tid == 0) atomicCAS(info, 0, info_offset + fail_at + 1);
  for (int e = tid; e < len * len; e += nt) {
    int i, j;
    if (!upper) { i = e % len; j = e / len; } else { j = e % len; i = e / len; }
    if (j <= i) {
      if (upper) A[(size_t)j + (size_t)i * lda] = Ms[i][j];
      else A[(size_t)i + (size_t)j * lda] = Ms[i][j];
    }
  }
}

inline int split_point(int len) {
  int h = ((len / 2) + TB - 1) / TB * TB;
  return h >= len ? len - TB : h;
}

struct TrsmPlan {
  TriView tv;
  bool side_right;
  double *B;
  int ldb;
  int nn;  // right-hand-side columns of the canonical (left) problem
  const int *abort_flag;
  cudaStream_t s;
};

int trsm_rec(const TrsmPlan &p, int r0, int len) {
  if (len <= 0) return 0;
  if (len <= TB) {
    long long rs = p.side_right ? p.ldb : 1, cs = p.side_right ? 1 : p.ldb;
    int grid = (p.nn + TRSM_W - 1) / TRSM_W;
    trsm_base_kernel<<<grid, 32 * TRSM_W, 0, p.s>>>(p.tv, r0, len, p.B, rs, cs, p.nn, p.abort_flag);
    DG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return 0;
  }
  const int h = split_point(len);
  // first solved half and the half it updates
  int a0, alen, b0, blen;
  if (p.tv.lower) { a0 = r0; alen = h; b0 = r0 + h; blen = len - h; }
  else { a0 = r0 + h; alen = len - h; b0 = r0; blen = h; }
  int rc = trsm_rec(p, a0, alen);
  if (rc) return rc;
  // X[b] -= M[b, a] X[a]
  const double *Msub;
  char opM;
  if (!p.tv.trans) { Msub = p.tv.T + (size_t)b0 + (size_t)a0 * p.tv.ld; opM = 'N'; }
  else { Msub = p.tv.T + (size_t)a0 + (size_t)b0 * p.tv.ld; opM = 'T'; }
  if (!p.side_right) {
    rc = gemm_f64(opM, 'N', blen, p.nn, alen, -1.0, Msub, p.tv.ld, p.B + a0, p.ldb, 1.0,
                  p.B + b0, p.ldb, TRI_NONE, p.abort_flag, p.s);
  } else {
    // rows of X' are columns of B: B[:, b] -= B[:, a] * M[b, a]'
    rc = gemm_f64('N', opM == 'N' ? 'T' : 'N', p.nn, blen, alen, -1.0,
                  p.B + (size_t)a0 * p.ldb, p.ldb, Msub, p.tv.ld, 1.0,
                  p.B + (size_t)b0 * p.ldb, p.ldb, TRI_NONE, p.abort_flag, p.s);
  }
  if (rc) return rc;
  return trsm_rec(p, b0, blen);
}

}  // namespace

int trsm_f64(char side, char uplo, char transa, char diag, int m, int n, double alpha,
             const double *A, int lda, double *B, int ldb, const int *abort_flag,
             cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  const bool right = (side == 'R' || side == 'r');
  const bool tr = !(transa == 'N' || transa == 'n');
  TrsmPlan p;
  p.side_right = right;
  p.tv.T = A;
  p.tv.ld = lda;
  p.tv.trans = tr != right;
  p.tv.lower = (uplo == 'L' || uplo == 'l') != p.tv.trans;
  p.tv.unit = (diag == 'U' || diag == 'u');
  p.B = B;
  p.ldb = ldb;
  p.nn = right ? m : n;
  p.abort_flag = abort_flag;
  p.s = s;
  if (alpha != 1.0) {
    int rc = scale_f64(m, n, alpha, B, ldb, abort_flag, s);
    if (rc) return rc;
    if (alpha == 0.0) return 0;
  }
  return trsm_rec(p, 0, right ? n : m);
}

static int potrf_rec(bool upper, int n, double *A, int lda, int *info, int off, cudaStream_t s) {
  if (n <= 0) return 0;
  if (n <= TB) {
    potrf_base_kernel<<<1, 256, 0, s>>>(upper ? 1 : 0, n, A, lda, info, off);
    DG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return 0;
  }
  const int n1 = split_point(n), n2 = n - n1;
  int rc = potrf_rec(upper, n1, A, lda, info, off, s);
  if (rc) return rc;
  double *A22 = A + (size_t)n1 + (size_t)n1 * lda;
  if (upper) {
    double *A12 = A + (size_t)n1 * lda;
    rc = trsm_f64('L', 'U', 'T', 'N', n1, n2, 1.0, A, lda, A12, lda, info, s);
    if (!rc) rc = gemm_f64('T', 'N', n2, n2, n1, -1.0, A12, lda, A12, lda, 1.0, A22, lda,
                           TRI_UPPER, info, s);
  } else {
    double *A21 = A + n1;
    rc = trsm_f64('R', 'L', 'T', 'N', n2, n1, 1.0, A, lda, A21, lda, info, s);
    if (!rc) rc = gemm_f64('N', 'T', n2, n2, n1, -1.0, A21, lda, A21, lda, 1.0, A22, lda,
                           TRI_LOWER, info, s);
  }
  if (rc) return rc;
  return potrf_rec(upper, n2, A22, lda, info, off + n1, s);
}

int potrf_f64(char uplo, int n, double *A, int lda, int *info_dev, int info_offset,
              cudaStream_t s) {
  return potrf_rec(uplo == 'U' || uplo == 'u', n, A, lda, info_dev, info_offset, s);
}

}  // namespace dg
