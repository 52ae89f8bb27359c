// Triangular solve (TRSM) and Cholesky (POTRF) of one tile, FP64 and FP32.
//
// FP64 replaces LAPACK.potrf! in potrf_checked! (src/array/cholesky.jl:3 of
// Dagger.jl) and BLAS.trsm! in the panel step (cholesky.jl:41,86) and in the
// block solves (src/array/trsm.jl:95-183).  FP32 is the diagonal-block
// factorization, panel solve and triangular solves of the mixed-precision
// form.
//
// Both are recursive: the triangle is halved until a 64 x 64 diagonal block
// remains, and the off-diagonal work of each level is a GEMM / SYRK on the
// tile GEMM kernels (gemm_tile.cu), so nearly all flops run in the GEMM.  The
// 64 x 64 base cases are shared-memory kernels:
//   trsm_base: the 64 x 64 triangle and a 64 x 8 slab of the right-hand side
//              are staged in shared memory; each warp solves one column by
//              forward/backward substitution with the column held in two
//              registers per lane and the solved entry broadcast by shuffle
//              (the reciprocal of each pivot is formed once, as OpenBLAS's
//              trsm kernels do).
//   potrf_base: one CTA factors the 64 x 64 block in shared memory
//              (right-looking, column by column).  A pivot that is not
//              positive (or NaN) records the LAPACK info in a device word and
//              stops; every later kernel of the same factorization checks the
//              word on entry and returns at once.
// Every access is bounds-checked against the block length, so ragged last
// tiles (n not a multiple of the block size) need no padding.
// With the emulated FP64 engine the caller passes scratch for BF16 slices,
// and the off-diagonal GEMM / SYRK of every level runs on the tensor cores
// (oz_gemm_general) with FP64 accuracy; the base cases stay FP64.
#include "dg_common.cuh"

namespace dg {

namespace {

constexpr int TB = 64;     // base block size
constexpr int TRSM_W = 8;  // right-hand-side columns per CTA (one per warp)

template <typename T>
struct TriView {
  const T *T_;
  long long ld;
  bool trans;  // M(i, j) = T(j, i)
  bool lower;  // M is lower triangular
  bool unit;   // unit diagonal
};

// Solve M[r0:r0+len, r0:r0+len] X = X in place for the columns handled by
// this CTA.  X(i, c) lives at X[i * rs + c * cs].
template <typename T>
__global__ void __launch_bounds__(256) trsm_base_kernel(TriView<T> tv, int r0, int len, T *X,
                                                        long long rs, long long cs, int nn,
                                                        const int *a1, const int *a2) {
  if (aborted(a1, a2)) return;
  __shared__ T Ms[TB][TB + 1];
  __shared__ T dinv[TB];
  __shared__ T Xs[TB][TRSM_W + 1];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int c0 = blockIdx.x * TRSM_W;
  const int wcols = min(TRSM_W, nn - c0);
  for (int e = tid; e < len * len; e += nt) {
    int i, j;
    if (!tv.trans) { i = e % len; j = e / len; } else { j = e % len; i = e / len; }
    if (tv.lower ? (j <= i) : (j >= i)) {
      size_t off = tv.trans ? (size_t)(r0 + j) + (size_t)(r0 + i) * tv.ld
                            : (size_t)(r0 + i) + (size_t)(r0 + j) * tv.ld;
      Ms[i][j] = tv.T_[off];
    }
  }
  for (int e = tid; e < len * wcols; e += nt) {
    int i, c;
    if (rs == 1) { i = e % len; c = e / len; } else { c = e % wcols; i = e / wcols; }
    Xs[i][c] = X[(size_t)(r0 + i) * rs + (size_t)(c0 + c) * cs];
  }
  __syncthreads();
  if (tid < len) dinv[tid] = tv.unit ? T(1) : T(1) / Ms[tid][tid];
  __syncthreads();
  const int lane = tid & 31, warp = tid >> 5;
  if (warp < wcols) {
    const int c = warp;
    T x0 = lane < len ? Xs[lane][c] : T(0);
    T x1 = lane + 32 < len ? Xs[lane + 32][c] : T(0);
    if (tv.lower) {
      for (int i = 0; i < len; i++) {
        T xi = __shfl_sync(0xffffffffu, i < 32 ? x0 : x1, i & 31) * dinv[i];
        if (i < 32) { if (lane == i) x0 = xi; } else { if (lane == i - 32) x1 = xi; }
        if (lane > i && lane < len) x0 = fma(-Ms[lane][i], xi, x0);
        if (lane + 32 > i && lane + 32 < len) x1 = fma(-Ms[lane + 32][i], xi, x1);
      }
    } else {
      for (int i = len - 1; i >= 0; i--) {
        T xi = __shfl_sync(0xffffffffu, i < 32 ? x0 : x1, i & 31) * dinv[i];
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

// Solve M X = X of a few right-hand-side columns (one CTA per column; for a
// right-side solve the columns are B's rows) for the whole triangle: the
// column lives in shared memory, blocks
// of 64 rows are finished in order; each block first subtracts the solved
// part (all 256 threads, reading M coalesced in either orientation), then
// warp 0 substitutes through the 64 x 64 diagonal block staged in shared
// memory.  Used for skinny right-hand sides (the solves of ldiv!), where the
// recursive form has too little parallelism in its updates.
constexpr int TC_MAX_LEN = 4096;
constexpr int TC_MAX_RHS = 128;
// Inside POTRF the TRSM of each level is on the critical path: one
// column-parallel launch replaces the recursion up to this width.
constexpr int kPotrfColsMax = 512;

// eye (forward solves only): column c starts as e_c instead of being read, so
// its first c entries stay zero and the blocks above c are skipped (the
// columns of a triangular inverse).
template <typename T>
__global__ void __launch_bounds__(256) trsm_cols_kernel(TriView<T> tv, int len, T *X,
                                                        long long rs, long long cs, int eye,
                                                        const int *a1, const int *a2) {
  if (aborted(a1, a2)) return;
  extern __shared__ unsigned char tc_smem[];
  T (*D)[TB + 1] = (T (*)[TB + 1])tc_smem;              // diagonal block
  T *x = (T *)(tc_smem + sizeof(T) * TB * (TB + 1));    // the column
  __shared__ T part[4][TB];
  const int tid = threadIdx.x;
  const int col = blockIdx.x;
  T *xc = X + (size_t)col * cs;  // element i of this column at xc[i * rs]
  for (int i = tid; i < len; i += 256) x[i] = eye ? T(i == col ? 1 : 0) : xc[(size_t)i * rs];
  __syncthreads();
  const int nblk = (len + TB - 1) / TB;
  const int b_first = (eye && tv.lower) ? col / TB : 0;
  for (int bi = b_first; bi < nblk; bi++) {
    const int b = tv.lower ? bi : nblk - 1 - bi;
    const int r0 = b * TB, rl = min(TB, len - r0);
    const int p0 = tv.lower ? b_first * TB : r0 + rl, p1 = tv.lower ? r0 : len;  // solved rows
    // x[r0 + i] -= sum_{p0 <= p < p1} M(r0 + i, p) x[p]
    if (!tv.trans) {  // M(i, p) = T_[i + p ld]: threads along i, 4 groups over p
      const int i = tid & (TB - 1), g = tid >> 6;
      T acc = T(0);
      if (i < rl)
        for (int p = p0 + g; p < p1; p += 4)
          acc = fma(tv.T_[(size_t)(r0 + i) + (size_t)p * tv.ld], x[p], acc);
      part[g][i] = acc;
      __syncthreads();
      if (tid < rl) x[r0 + tid] -= (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]);
    } else {          // M(i, p) = T_[p + i ld]: a warp per row, lanes along p
      const int w = tid >> 5, lane = tid & 31;
      for (int i = w; i < rl; i += 8) {
        T acc = T(0);
        for (int p = p0 + lane; p < p1; p += 32)
          acc = fma(tv.T_[(size_t)p + (size_t)(r0 + i) * tv.ld], x[p], acc);
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) x[r0 + i] -= acc;
      }
    }
    // the diagonal block's triangle
    for (int e = tid; e < rl * rl; e += 256) {
      int i, j;
      if (!tv.trans) { i = e % rl; j = e / rl; } else { j = e % rl; i = e / rl; }
      if (tv.lower ? (j <= i) : (j >= i))
        D[i][j] = tv.trans ? tv.T_[(size_t)(r0 + j) + (size_t)(r0 + i) * tv.ld]
                           : tv.T_[(size_t)(r0 + i) + (size_t)(r0 + j) * tv.ld];
    }
    __syncthreads();
    if (tid < 32) {
      const int lane = tid;
      const T d0 = tv.unit ? T(1) : (lane < rl ? T(1) / D[lane][lane] : T(1));
      const T d1 = tv.unit ? T(1) : (lane + 32 < rl ? T(1) / D[lane + 32][lane + 32] : T(1));
      T x0 = lane < rl ? x[r0 + lane] : T(0);
      T x1 = lane + 32 < rl ? x[r0 + lane + 32] : T(0);
      if (tv.lower) {
        for (int i = 0; i < rl; i++) {
          const T di = __shfl_sync(0xffffffffu, i < 32 ? d0 : d1, i & 31);
          const T xi = __shfl_sync(0xffffffffu, i < 32 ? x0 : x1, i & 31) * di;
          if (i < 32) { if (lane == i) x0 = xi; } else { if (lane == i - 32) x1 = xi; }
          if (lane > i && lane < rl) x0 = fma(-D[lane][i], xi, x0);
          if (lane + 32 > i && lane + 32 < rl) x1 = fma(-D[lane + 32][i], xi, x1);
        }
      } else {
        for (int i = rl - 1; i >= 0; i--) {
          const T di = __shfl_sync(0xffffffffu, i < 32 ? d0 : d1, i & 31);
          const T xi = __shfl_sync(0xffffffffu, i < 32 ? x0 : x1, i & 31) * di;
          if (i < 32) { if (lane == i) x0 = xi; } else { if (lane == i - 32) x1 = xi; }
          if (lane < i) x0 = fma(-D[lane][i], xi, x0);
          if (lane + 32 < i) x1 = fma(-D[lane + 32][i], xi, x1);
        }
      }
      if (lane < rl) x[r0 + lane] = x0;
      if (lane + 32 < rl) x[r0 + lane + 32] = x1;
    }
    __syncthreads();
  }
  for (int i = tid; i < len; i += 256) xc[(size_t)i * rs] = x[i];
}

template <typename T>
int trsm_cols(const TriView<T> &tv, int len, T *X, long long rs, long long cs, int nn,
              const int *a1, const int *a2, cudaStream_t s, int eye = 0) {
  const size_t smem = sizeof(T) * (TB * (TB + 1) + (size_t)len);
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr[dev & 63]) {
    DG_CUDA_TRY(cudaFuncSetAttribute(trsm_cols_kernel<T>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(sizeof(T) * (TB * (TB + 1) + TC_MAX_LEN))));
    attr[dev & 63] = true;
  }
  trsm_cols_kernel<T><<<nn, 256, smem, s>>>(tv, len, X, rs, cs, eye, a1, a2);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

// Cholesky of one block of length len <= 64 at A (leading dimension lda).
// Works on the lower triangle L; for uplo 'U' the block is staged transposed
// (U' = L) and written back transposed, so only the uplo triangle is touched.
// Right-looking with the column scaling deferred: step j subtracts
// M(i, j) M(k, j) / d_j (d_j the pivot) from the trailing triangle, and each
// column is scaled by 1 / sqrt(d_j) once at the end (square roots and
// divisions for all columns at once, off the sequential path).  Each step
// stages M(i, j) / d_j once, then warps 0-6 update the trailing triangle,
// its elements handed out densely from a table (on GB300 a warp's FP64
// instruction costs the same with idle lanes, so a rectangular thread grid
// over the shrinking triangle wasted most of them), while warp 7 updates
// element (j+1, j+1) first and forms 1 / d_{j+1}
// by Newton's iteration for the reciprocal (x <- x + x (1 - d x), quadratic
// convergence from the hardware's approximate reciprocal, two steps to FP64
// precision), so the sequential path per column is a few FMAs.  A pivot that
// is not positive (or NaN) stops the factorization at that column,
// info = column + 1 (LAPACK's dpotf2 test); the columns before it are
// factored.
template <typename T>
__device__ __forceinline__ T recip_newton(T d);
template <>
__device__ __forceinline__ double recip_newton<double>(double d) {
  double x;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(x) : "d"(d));
  x = fma(x, fma(-d, x, 1.0), x);
  return fma(x, fma(-d, x, 1.0), x);
}
template <>
__device__ __forceinline__ float recip_newton<float>(float d) {
  float x;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(x) : "f"(d));
  return fmaf(x, fmaf(-d, x, 1.0f), x);
}

template <typename T>
__global__ void __launch_bounds__(256) potrf_base_kernel(int upper, int len, T *A, long long lda,
                                                         int *info, int info_offset,
                                                         const int *a1, const int *a2) {
  if (aborted(info, a1) || aborted(a2, nullptr)) return;
  __shared__ T Ms[TB][TB + 1];
  __shared__ T dinv[TB];  // 1 / d_j
  __shared__ T S[TB];     // M(i, j) / d_j of the current column
  // the lower triangle's elements (i << 8 | k), columns in decreasing order:
  // the elements of columns > j, step j's update, are its first
  // (len-1-j)(len-j)/2 entries, handed out densely to the threads
  __shared__ uint32_t tri[TB * (TB + 1) / 2];
  __shared__ int fail_at;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < len * len; e += nt) {
    int i, j;
    if (!upper) { i = e % len; j = e / len; } else { j = e % len; i = e / len; }
    if (j <= i) Ms[i][j] = upper ? A[(size_t)j + (size_t)i * lda] : A[(size_t)i + (size_t)j * lda];
  }
  for (int k = tid; k < len; k += nt) {
    const int off = (len - 1 - k) * (len - k) / 2;
    for (int i = k; i < len; i++) tri[off + i - k] = ((uint32_t)i << 8) | (uint32_t)k;
  }
  __syncthreads();
  // the approximate reciprocal flushes subnormals: extreme pivots divide
  const T lo = sizeof(T) == 8 ? T(1e-300) : T(1e-36), hi = sizeof(T) == 8 ? T(1e300) : T(1e36);
  auto pivot = [&](int j, T d) {
    if (!(d > T(0)))  // not positive, or NaN
      fail_at = j;
    else
      dinv[j] = (d > lo && d < hi) ? recip_newton<T>(d) : T(1) / d;
  };
  if (tid == 0) {
    fail_at = -1;
    pivot(0, Ms[0][0]);
  }
  __syncthreads();
  int done = 0;  // columns factored
  for (int j = 0; j < len; j++) {
    if (fail_at >= 0 && fail_at <= j) break;  // the same value for every thread
    done = j + 1;
    const T r2 = dinv[j];
    for (int i = j + 1 + tid; i < len; i += nt) S[i] = Ms[i][j] * r2;
    __syncthreads();
    if (tid == 7 * 32) {
      if (j + 1 < len) {
        const T d = fma(-S[j + 1], Ms[j + 1][j], Ms[j + 1][j + 1]);
        Ms[j + 1][j + 1] = d;
        pivot(j + 1, d);
      }
    } else if (tid < 7 * 32) {  // warps 0-6: every other element of columns > j
      const int P = (len - 1 - j) * (len - j) / 2;
      const int skip = (len - 2 - j) * (len - 1 - j) / 2;  // (j+1, j+1), warp 7's
      for (int e = tid; e < P; e += 7 * 32) {
        if (e == skip) continue;
        const uint32_t ik = tri[e];
        const int i = (int)(ik >> 8), k = (int)(ik & 255u);
        Ms[i][k] = fma(-S[i], Ms[k][j], Ms[i][k]);
      }
    }
    __syncthreads();
  }
  // scale the factored columns: L(j, j) = sqrt(d_j), L(i, j) = M(i, j) / sqrt(d_j)
  __shared__ T sq[TB], rs[TB];
  for (int j = tid; j < done; j += nt) {
    sq[j] = sqrt(Ms[j][j]);
    rs[j] = T(1) / sq[j];
  }
  __syncthreads();
  for (int e = tid; e < len * len; e += nt) {
    const int i = e % len, j = e / len;
    if (j < done && i >= j) Ms[i][j] = (i == j) ? sq[j] : Ms[i][j] * rs[j];
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

template <typename T>
int gemm_t(char ta, char tb, int m, int n, int k, T alpha, const T *A, long long lda, const T *B,
           long long ldb, T beta, T *C, long long ldc, Tri tri, const int *a1, cudaStream_t s,
           const int *a2);

template <>
int gemm_t<double>(char ta, char tb, int m, int n, int k, double alpha, const double *A,
                   long long lda, const double *B, long long ldb, double beta, double *C,
                   long long ldc, Tri tri, const int *a1, cudaStream_t s, const int *a2) {
  return gemm_f64(ta, tb, m, n, k, alpha, A, (int)lda, B, (int)ldb, beta, C, (int)ldc, tri, a1, s,
                  a2);
}

template <>
int gemm_t<float>(char ta, char tb, int m, int n, int k, float alpha, const float *A,
                  long long lda, const float *B, long long ldb, float beta, float *C,
                  long long ldc, Tri tri, const int *a1, cudaStream_t s, const int *a2) {
  return gemm_f32(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, a1, s, a2);
}

// Slice scratch of the emulated FP64 engine (none: p == nullptr); status is
// the writable word that records a timeout.
struct OzScratch {
  void *p = nullptr;
  size_t bytes = 0;
  int *status = nullptr;
};

// The off-diagonal update of one recursion level: emulated when the scratch
// allows it (FP64 only), else the tile GEMM kernels.
template <typename T>
int update_t(char ta, char tb, int m, int n, int k, T alpha, const T *A, long long lda, const T *B,
             long long ldb, T beta, T *C, long long ldc, Tri tri, const int *a1, cudaStream_t s,
             const int *a2, const OzScratch &oz) {
  if (sizeof(T) == 8 && oz.p) {
    // a1 and a2 are both abort words; the status word is a1 itself when given
    const int *other = (oz.status == a1) ? a2 : (a2 ? a2 : a1);
    int rc = oz_gemm_general(ta, tb, m, n, k, (double)alpha, (const double *)A, lda,
                             (const double *)B, ldb, (double)beta, (double *)C, ldc, (int)tri,
                             oz.p, oz.bytes, oz.status, other, s);
    if (rc <= 0) return rc;
  }
  return gemm_t<T>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, a1, s, a2);
}

template <typename T>
struct TrsmPlan {
  TriView<T> tv;
  bool side_right;
  T *B;
  long long ldb;
  int nn;  // right-hand-side columns of the canonical (left) problem
  const int *a1, *a2;
  cudaStream_t s;
  OzScratch oz;
};

template <typename T>
int trsm_rec(const TrsmPlan<T> &p, int r0, int len) {
  if (len <= 0) return 0;
  if (len <= TB) {
    long long rs = p.side_right ? p.ldb : 1, cs = p.side_right ? 1 : p.ldb;
    int grid = (p.nn + TRSM_W - 1) / TRSM_W;
    trsm_base_kernel<T><<<grid, 32 * TRSM_W, 0, p.s>>>(p.tv, r0, len, p.B, rs, cs, p.nn, p.a1,
                                                       p.a2);
    DG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return 0;
  }
  const int h = split_point(len);
  int a0, alen, b0, blen;
  if (p.tv.lower) { a0 = r0; alen = h; b0 = r0 + h; blen = len - h; }
  else { a0 = r0 + h; alen = len - h; b0 = r0; blen = h; }
  DG_TRY(trsm_rec(p, a0, alen));
  // X[b] -= M[b, a] X[a]
  const T *Msub;
  char opM;
  if (!p.tv.trans) { Msub = p.tv.T_ + (size_t)b0 + (size_t)a0 * p.tv.ld; opM = 'N'; }
  else { Msub = p.tv.T_ + (size_t)a0 + (size_t)b0 * p.tv.ld; opM = 'T'; }
  if (!p.side_right) {
    DG_TRY(update_t<T>(opM, 'N', blen, p.nn, alen, T(-1), Msub, p.tv.ld, p.B + a0, p.ldb, T(1),
                       p.B + b0, p.ldb, TRI_NONE, p.a1, p.s, p.a2, p.oz));
  } else {
    // rows of X' are columns of B: B[:, b] -= B[:, a] * M[b, a]'
    DG_TRY(update_t<T>('N', opM == 'N' ? 'T' : 'N', p.nn, blen, alen, T(-1),
                       p.B + (size_t)a0 * p.ldb, p.ldb, Msub, p.tv.ld, T(1),
                       p.B + (size_t)b0 * p.ldb, p.ldb, TRI_NONE, p.a1, p.s, p.a2, p.oz));
  }
  return trsm_rec(p, b0, blen);
}

// cols_max: widest right-hand side solved by the column-parallel kernel
// (latency-bound callers raise it).
template <typename T>
int trsm_t(char side, char uplo, char transa, char diag, int m, int n, T alpha, const T *A,
           long long lda, T *B, long long ldb, const int *a1, cudaStream_t s, const int *a2,
           const OzScratch &oz = OzScratch(), int cols_max = TC_MAX_RHS) {
  if (m <= 0 || n <= 0) return 0;
  const bool right = (side == 'R' || side == 'r');
  const bool tr = !(transa == 'N' || transa == 'n');
  TrsmPlan<T> p;
  p.side_right = right;
  p.tv.T_ = A;
  p.tv.ld = lda;
  p.tv.trans = tr != right;
  p.tv.lower = (uplo == 'L' || uplo == 'l') != p.tv.trans;
  p.tv.unit = (diag == 'U' || diag == 'u');
  p.B = B;
  p.ldb = ldb;
  p.nn = right ? m : n;
  p.a1 = a1;
  p.a2 = a2;
  p.s = s;
  p.oz = oz;
  if (alpha != T(1)) {
    if (sizeof(T) == 8)
      DG_TRY(scale_f64(m, n, (double)alpha, (double *)B, (int)ldb, a1, s, a2));
    else
      DG_TRY(scale_f32(m, n, (float)alpha, (float *)B, ldb, a1, s, a2));
    if (alpha == T(0)) return 0;
  }
  const int len = right ? n : m;
  if (p.nn <= cols_max && len > 2 * TB && len <= TC_MAX_LEN)
    return trsm_cols<T>(p.tv, len, B, right ? ldb : 1, right ? 1 : ldb, p.nn, a1, a2, s);
  return trsm_rec(p, 0, len);
}

template <typename T>
int potrf_rec(bool upper, int n, T *A, long long lda, int *info, int off, cudaStream_t s,
              const int *a1, const int *a2, const OzScratch &oz = OzScratch()) {
  if (n <= 0) return 0;
  if (n <= TB) {
    potrf_base_kernel<T><<<1, 256, 0, s>>>(upper ? 1 : 0, n, A, lda, info, off, a1, a2);
    DG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return 0;
  }
  const int n1 = split_point(n), n2 = n - n1;
  DG_TRY(potrf_rec<T>(upper, n1, A, lda, info, off, s, a1, a2, oz));
  // the remaining kernels stop when this factorization's info is set, or on
  // either caller abort word (two words per kernel: info + the first caller
  // word; the base kernel checks all three)
  const int *k1 = info, *k2 = a1 ? a1 : a2;
  T *A22 = A + (size_t)n1 + (size_t)n1 * lda;
  OzScratch oz1 = oz;
  if (oz1.p) oz1.status = info;  // this factorization's word records a timeout
  if (upper) {
    T *A12 = A + (size_t)n1 * lda;
    DG_TRY(trsm_t<T>('L', 'U', 'T', 'N', n1, n2, T(1), A, lda, A12, lda, k1, s, k2, oz1,
                     kPotrfColsMax));
    DG_TRY(update_t<T>('T', 'N', n2, n2, n1, T(-1), A12, lda, A12, lda, T(1), A22, lda, TRI_UPPER,
                       k1, s, k2, oz1));
  } else {
    T *A21 = A + n1;
    DG_TRY(trsm_t<T>('R', 'L', 'T', 'N', n2, n1, T(1), A, lda, A21, lda, k1, s, k2, oz1,
                     kPotrfColsMax));
    DG_TRY(update_t<T>('N', 'T', n2, n2, n1, T(-1), A21, lda, A21, lda, T(1), A22, lda, TRI_LOWER,
                       k1, s, k2, oz1));
  }
  return potrf_rec<T>(upper, n2, A22, lda, info, off + n1, s, a1, a2, oz);
}

}  // namespace

int trsm_f64(char side, char uplo, char transa, char diag, int m, int n, double alpha,
             const double *A, int lda, double *B, int ldb, const int *abort_flag,
             cudaStream_t s, const int *abort2) {
  return trsm_t<double>(side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, abort_flag, s,
                        abort2);
}

int trsm_f64_oz(char side, char uplo, char transa, char diag, int m, int n, double alpha,
                const double *A, int lda, double *B, int ldb, void *scratch, size_t bytes,
                int *status, cudaStream_t s) {
  OzScratch oz;
  oz.p = scratch;
  oz.bytes = bytes;
  oz.status = status;
  return trsm_t<double>(side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, status, s, nullptr,
                        oz);
}

int potrf_f64_oz(char uplo, int n, double *A, int lda, int *info_out, int info_offset,
                 void *scratch, size_t bytes, cudaStream_t s) {
  OzScratch oz;
  oz.p = scratch;
  oz.bytes = bytes;
  oz.status = info_out;
  return potrf_rec<double>(uplo == 'U' || uplo == 'u', n, A, lda, info_out, info_offset, s,
                           nullptr, nullptr, oz);
}

int gemm_update_f64(char ta, char tb, int m, int n, int k, double alpha, const double *A,
                    long long lda, const double *B, long long ldb, double beta, double *C,
                    long long ldc, void *scratch, size_t bytes, int *status, cudaStream_t s) {
  OzScratch oz;
  oz.p = scratch;
  oz.bytes = bytes;
  oz.status = status;
  return update_t<double>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, TRI_NONE, status,
                          s, nullptr, oz);
}

int trinv_t_f64(char uplo, int n, const double *A, int lda, double *W, int ldw,
                const int *abort_flag, cudaStream_t s) {
  if (n <= 0) return 0;
  if (n > TC_MAX_LEN) return DG_ERR_UNSUPPORTED;
  // W = U^-T: U' W = I, left side; W = L^-T: W L' = I, right side.  Both are
  // forward substitutions whose right-hand sides are the unit vectors.
  const bool up = (uplo == 'U' || uplo == 'u');
  TriView<double> tv;
  tv.T_ = A;
  tv.ld = lda;
  tv.trans = up;   // left, 'T' -> M = U'; right, 'T' -> M = L (canonical forward)
  tv.lower = true;
  tv.unit = false;
  return trsm_cols<double>(tv, n, W, up ? 1 : ldw, up ? ldw : 1, n, abort_flag, nullptr, s, 1);
}

int trinv_unit_lower_f64(int n, const double *A, int lda, double *W, int ldw,
                         const int *abort_flag, cudaStream_t s) {
  if (n <= 0) return 0;
  if (n > TC_MAX_LEN) return DG_ERR_UNSUPPORTED;
  // L W = I, left side: column c of W is the solve with the unit vector e_c
  TriView<double> tv;
  tv.T_ = A;
  tv.ld = lda;
  tv.trans = false;
  tv.lower = true;
  tv.unit = true;
  return trsm_cols<double>(tv, n, W, 1, ldw, n, abort_flag, nullptr, s, 1);
}

int trsm_f32(char side, char uplo, char transa, char diag, int m, int n, float alpha,
             const float *A, long long lda, float *B, long long ldb, const int *abort_flag,
             cudaStream_t s, const int *abort2) {
  return trsm_t<float>(side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, abort_flag, s,
                       abort2);
}

int potrf_f64(char uplo, int n, double *A, int lda, int *info_out, int info_offset, cudaStream_t s,
              const int *abort_flag, const int *abort2) {
  return potrf_rec<double>(uplo == 'U' || uplo == 'u', n, A, lda, info_out, info_offset, s,
                           abort_flag, abort2);
}

int potrf_f32(char uplo, int n, float *A, long long lda, int *info_out, int info_offset,
              cudaStream_t s, const int *abort_flag, const int *abort2) {
  return potrf_rec<float>(uplo == 'U' || uplo == 'u', n, A, lda, info_out, info_offset, s,
                          abort_flag, abort2);
}

}  // namespace dg
