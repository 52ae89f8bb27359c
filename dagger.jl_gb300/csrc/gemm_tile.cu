// CUDA-core tile GEMM / SYRK in FP64 and FP32.
//
// FP64: the trailing-update kernels of the plain tiled Cholesky (BLAS.gemm! at
// src/array/cholesky.jl:50,95 and BLAS.syrk! at :47,92 of Dagger.jl) and the
// update step of the block triangular solves; also the FP64 residual
// b - A x of iterative refinement, reading A straight from its tile layout.
// FP32: the panel TRSM / POTRF updates and triangular solves of the
// mixed-precision form.
//
// C <- alpha * op(A) * op(B) + beta * C, column-major, any transposes.  One
// CTA owns a BM x BN tile of C and walks K in steps of BK, staging the A and
// B slabs in shared memory (register-prefetched double buffer: the next slab
// is fetched from global memory while the current one is multiplied).  Each
// thread accumulates a TM x TN register tile (rows tx + (BM/TM) r, columns
// ty + (BN/TN) c, so shared-memory reads are conflict-free and global stores
// are coalesced along rows).  GB300 executes FP64 at a small fraction of its
// FP32 rate, so the FP64 kernel is bounded by the FP64 pipe, not by memory.
// A DMMA variant (mma.sync.m8n8k4.f64) is kept for the engine switch.
//
// SYRK uses the same kernels with a triangle mask: CTA tiles wholly outside
// the requested triangle exit at once and stores are limited to the triangle.
#include <atomic>

#include "dg_common.cuh"

namespace dg {

namespace {

struct GemmArgs {
  int m, n, k;
  double alpha, beta;
  const void *A;
  long long lda;
  const void *B;
  long long ldb;
  void *C;
  long long ldc;
  int ta, tb, tri;
  const int *abort_flag, *abort2;
  // tiled A (op 'N' only): A is the tile grid of a DArray given as a device
  // array of tile pointers, tile (i, j) = tptr[i + j*tmt], column-major with
  // leading dimension equal to its row count min(tnb, tn - i*tnb)
  int tnb, tmt;
  long long tn;
  const void *const *tptr;
};

std::atomic<int> g_engine{0};  // process-wide setting, read by every call

template <typename T>
__device__ __forceinline__ T load_a(const GemmArgs &g, int gi, int gp) {
  const T *A = (const T *)g.A;
  if (g.tnb) {
    const int ti = gi / g.tnb, tp = gp / g.tnb;
    const long long rows = min((long long)g.tnb, g.tn - (long long)ti * g.tnb);
    const T *t = (const T *)g.tptr[ti + (size_t)tp * g.tmt];
    return t[(gi - ti * g.tnb) + (size_t)(gp - tp * g.tnb) * rows];
  }
  return g.ta == 0 ? A[(size_t)gi + (size_t)gp * g.lda] : A[(size_t)gp + (size_t)gi * g.lda];
}

template <typename T, int BM, int BN, int BK, int NT>
struct SlabLoader {
  static constexpr int PA = (BM * BK) / NT, PB = (BN * BK) / NT;
  static constexpr int LDS_A = BM + 4, LDS_B = BN + 4;
  T ra[PA], rb[PB];

  __device__ __forceinline__ void fetch(const GemmArgs &g, int row0, int col0, int k0, int tid) {
    const T *B = (const T *)g.B;
#pragma unroll
    for (int q = 0; q < PA; q++) {
      int e = tid + q * NT, i, p;
      if (g.ta == 0) { i = e % BM; p = e / BM; } else { p = e % BK; i = e / BK; }
      int gi = row0 + i, gp = k0 + p;
      ra[q] = (gi < g.m && gp < g.k) ? load_a<T>(g, gi, gp) : T(0);
    }
#pragma unroll
    for (int q = 0; q < PB; q++) {
      int e = tid + q * NT, j, p;
      if (g.tb == 0) { p = e % BK; j = e / BK; } else { j = e % BN; p = e / BN; }
      int gj = col0 + j, gp = k0 + p;
      T w = T(0);
      if (gj < g.n && gp < g.k)
        w = g.tb == 0 ? B[(size_t)gp + (size_t)gj * g.ldb] : B[(size_t)gj + (size_t)gp * g.ldb];
      rb[q] = w;
    }
  }

  __device__ __forceinline__ void store(const GemmArgs &g, T *As, T *Bs, int tid) {
#pragma unroll
    for (int q = 0; q < PA; q++) {
      int e = tid + q * NT, i, p;
      if (g.ta == 0) { i = e % BM; p = e / BM; } else { p = e % BK; i = e / BK; }
      As[p * LDS_A + i] = ra[q];
    }
#pragma unroll
    for (int q = 0; q < PB; q++) {
      int e = tid + q * NT, j, p;
      if (g.tb == 0) { p = e % BK; j = e / BK; } else { j = e % BN; p = e / BN; }
      Bs[p * LDS_B + j] = rb[q];
    }
  }
};

template <int BM, int BN>
__device__ __forceinline__ bool tile_outside_triangle(int tri, int row0, int col0) {
  if (tri == TRI_UPPER) return row0 > col0 + BN - 1;
  if (tri == TRI_LOWER) return col0 > row0 + BM - 1;
  return false;
}

template <typename T>
__device__ __forceinline__ void store_c(const GemmArgs &g, int i, int j, T acc) {
  if (i >= g.m || j >= g.n) return;
  if (g.tri == TRI_UPPER && i > j) return;
  if (g.tri == TRI_LOWER && i < j) return;
  T *c = (T *)g.C + (size_t)i + (size_t)j * g.ldc;
  T v = T(g.alpha) * acc;
  if (g.beta != 0.0) v = fma(T(g.beta), *c, v);
  *c = v;
}

// CUDA-core engine: (BM/TM) x (BN/TN) threads, TM x TN register tile each.
template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN)) gemm_fma(GemmArgs g) {
  constexpr int NX = BM / TM, NY = BN / TN, NT = NX * NY;
  using LD = SlabLoader<T, BM, BN, BK, NT>;
  if (aborted(g.abort_flag, g.abort2)) return;
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
  if (tile_outside_triangle<BM, BN>(g.tri, row0, col0)) return;
  __shared__ T As[2][BK * LD::LDS_A];
  __shared__ T Bs[2][BK * LD::LDS_B];
  const int tid = threadIdx.x, tx = tid % NX, ty = tid / NX;
  T acc[TM][TN];
#pragma unroll
  for (int r = 0; r < TM; r++)
#pragma unroll
    for (int c = 0; c < TN; c++) acc[r][c] = T(0);
  LD ld;
  const int nk = (g.k + BK - 1) / BK;
  if (nk > 0) {
    ld.fetch(g, row0, col0, 0, tid);
    ld.store(g, As[0], Bs[0], tid);
  }
  __syncthreads();
  for (int kt = 0; kt < nk; kt++) {
    const int cur = kt & 1;
    if (kt + 1 < nk) ld.fetch(g, row0, col0, (kt + 1) * BK, tid);
#pragma unroll
    for (int p = 0; p < BK; p++) {
      T a[TM], b[TN];
#pragma unroll
      for (int r = 0; r < TM; r++) a[r] = As[cur][p * LD::LDS_A + tx + NX * r];
#pragma unroll
      for (int c = 0; c < TN; c++) b[c] = Bs[cur][p * LD::LDS_B + ty + NY * c];
#pragma unroll
      for (int r = 0; r < TM; r++)
#pragma unroll
        for (int c = 0; c < TN; c++) acc[r][c] = fma(a[r], b[c], acc[r][c]);
    }
    if (kt + 1 < nk) ld.store(g, As[cur ^ 1], Bs[cur ^ 1], tid);
    __syncthreads();
  }
  // epilogue: all reads of C are issued before any write, so the TM x TN
  // read-modify-writes overlap instead of serialising on possible aliasing
  T old[TM][TN];
#pragma unroll
  for (int r = 0; r < TM; r++)
#pragma unroll
    for (int c = 0; c < TN; c++) {
      const int i = row0 + tx + NX * r, j = col0 + ty + NY * c;
      old[r][c] = (g.beta != 0.0 && i < g.m && j < g.n)
                      ? ((const T *)g.C)[(size_t)i + (size_t)j * g.ldc] : T(0);
    }
#pragma unroll
  for (int r = 0; r < TM; r++)
#pragma unroll
    for (int c = 0; c < TN; c++) {
      const int i = row0 + tx + NX * r, j = col0 + ty + NY * c;
      if (i >= g.m || j >= g.n) continue;
      if (g.tri == TRI_UPPER && i > j) continue;
      if (g.tri == TRI_LOWER && i < j) continue;
      T v = T(g.alpha) * acc[r][c];
      if (g.beta != 0.0) v = fma(T(g.beta), old[r][c], v);
      ((T *)g.C)[(size_t)i + (size_t)j * g.ldc] = v;
    }
}

// DMMA engine (FP64 only): 4 warps in a 2 x 2 grid, warp tile 32 x 32 =
// 4 x 4 fragments of m8n8.  Fragment layouts (PTX ISA, mma.m8n8k4 f64):
//   A 8x4 row: lane holds A[lane/4][lane%4]; B 4x8 col: lane holds
//   B[lane%4][lane/4]; C 8x8: lane holds C[lane/4][2*(lane%4) + {0,1}].
__device__ __forceinline__ void dmma_m8n8k4(double &d0, double &d1, double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
      : "+d"(d0), "+d"(d1)
      : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(128) gemm_dmma(GemmArgs g) {
  constexpr int BM = 64, BN = 64, BK = 16;
  using LD = SlabLoader<double, BM, BN, BK, 128>;
  if (aborted(g.abort_flag, g.abort2)) return;
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
  if (tile_outside_triangle<BM, BN>(g.tri, row0, col0)) return;
  __shared__ double As[2][BK * LD::LDS_A];
  __shared__ double Bs[2][BK * LD::LDS_B];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
  const int qr = lane >> 2, qc = lane & 3;
  double acc[4][4][2];
#pragma unroll
  for (int mi = 0; mi < 4; mi++)
#pragma unroll
    for (int ni = 0; ni < 4; ni++) acc[mi][ni][0] = acc[mi][ni][1] = 0.0;
  LD ld;
  const int nk = (g.k + BK - 1) / BK;
  if (nk > 0) {
    ld.fetch(g, row0, col0, 0, tid);
    ld.store(g, As[0], Bs[0], tid);
  }
  __syncthreads();
  for (int kt = 0; kt < nk; kt++) {
    const int cur = kt & 1;
    if (kt + 1 < nk) ld.fetch(g, row0, col0, (kt + 1) * BK, tid);
#pragma unroll
    for (int k4 = 0; k4 < BK; k4 += 4) {
      double a[4], b[4];
#pragma unroll
      for (int mi = 0; mi < 4; mi++) a[mi] = As[cur][(k4 + qc) * LD::LDS_A + wm + mi * 8 + qr];
#pragma unroll
      for (int ni = 0; ni < 4; ni++) b[ni] = Bs[cur][(k4 + qc) * LD::LDS_B + wn + ni * 8 + qr];
#pragma unroll
      for (int mi = 0; mi < 4; mi++)
#pragma unroll
        for (int ni = 0; ni < 4; ni++) dmma_m8n8k4(acc[mi][ni][0], acc[mi][ni][1], a[mi], b[ni]);
    }
    if (kt + 1 < nk) ld.store(g, As[cur ^ 1], Bs[cur ^ 1], tid);
    __syncthreads();
  }
#pragma unroll
  for (int mi = 0; mi < 4; mi++)
#pragma unroll
    for (int ni = 0; ni < 4; ni++)
#pragma unroll
      for (int h = 0; h < 2; h++)
        store_c<double>(g, row0 + wm + mi * 8 + qr, col0 + wn + ni * 8 + 2 * qc + h, acc[mi][ni][h]);
}

template <typename T>
__global__ void scale_kernel(int m, int n, double alpha, T *B, long long ldb,
                             const int *abort_flag, const int *abort2) {
  if (aborted(abort_flag, abort2)) return;
  size_t total = (size_t)m * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(e % m), j = (int)(e / m);
    T *p = B + (size_t)i + (size_t)j * ldb;
    *p = alpha == 0.0 ? T(0) : T(alpha) * *p;
  }
}

__global__ void eye_kernel(int n, double *W, long long ldw, const int *abort_flag) {
  if (aborted(abort_flag, nullptr)) return;
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    W[(size_t)i + (size_t)j * ldw] = (i == j) ? 1.0 : 0.0;
}

GemmArgs make_args(char ta, char tb, int m, int n, int k, double alpha, const void *A,
                   long long lda, const void *B, long long ldb, double beta, void *C, long long ldc,
                   Tri tri, const int *abort_flag, const int *abort2) {
  GemmArgs g;
  memset(&g, 0, sizeof g);
  g.abort2 = abort2;
  g.m = m; g.n = n; g.k = (alpha == 0.0) ? 0 : k;
  g.alpha = alpha; g.beta = beta;
  g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.C = C; g.ldc = ldc;
  g.ta = (ta == 'N' || ta == 'n') ? 0 : 1;
  g.tb = (tb == 'N' || tb == 'n') ? 0 : 1;
  g.tri = tri;
  g.abort_flag = abort_flag;
  return g;
}

template <typename T>
int launch(const GemmArgs &g, cudaStream_t s) {
  if (g.m <= 0 || g.n <= 0) return 0;
  if (sizeof(T) == 8) {
    dim3 grid((g.m + 63) / 64, (g.n + 63) / 64);
    if (grid.y > 65535) return DG_ERR_UNSUPPORTED;
    if (g_engine == 1 && !g.tnb)
      gemm_dmma<<<grid, 128, 0, s>>>(g);
    else
      gemm_fma<double, 64, 64, 16, 4, 4><<<grid, 256, 0, s>>>(g);
  } else if (g.n <= 64 && !g.tnb && (long long)g.m >= 128LL * dg_num_sms()) {
    // tall and narrow (the refinement's triangular solves with up to 64
    // right-hand sides): 128 x 64 tiles, 8 x 4 registers per thread
    dim3 grid((g.m + 127) / 128, (g.n + 63) / 64);
    if (grid.y > 65535) return DG_ERR_UNSUPPORTED;
    gemm_fma<float, 128, 64, 16, 8, 4><<<grid, 256, 0, s>>>(g);
  } else if (g.n <= 64 || (long long)g.m * g.n < 128LL * 128 * 2 * dg_num_sms()) {
    // narrow or small outputs (the triangular solves' few right-hand sides):
    // 32 x 64 tiles give enough CTAs to fill the GPU
    dim3 grid((g.m + 31) / 32, (g.n + 63) / 64);
    if (grid.y > 65535) return DG_ERR_UNSUPPORTED;
    gemm_fma<float, 32, 64, 16, 2, 4><<<grid, 256, 0, s>>>(g);
  } else {
    dim3 grid((g.m + 127) / 128, (g.n + 127) / 128);
    if (grid.y > 65535) return DG_ERR_UNSUPPORTED;
    gemm_fma<float, 128, 128, 16, 8, 8><<<grid, 256, 0, s>>>(g);
  }
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

}  // namespace

void set_f64_engine(int engine) { g_engine = (engine >= 0 && engine <= 2) ? engine : 0; }
int get_f64_engine() { return g_engine; }

int gemm_f64(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
             const double *B, int ldb, double beta, double *C, int ldc, Tri tri,
             const int *abort_flag, cudaStream_t s, const int *abort2) {
  return launch<double>(make_args(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri,
                                  abort_flag, abort2), s);
}

int gemm_f32(char ta, char tb, int m, int n, int k, float alpha, const float *A, long long lda,
             const float *B, long long ldb, float beta, float *C, long long ldc, Tri tri,
             const int *abort_flag, cudaStream_t s, const int *abort2) {
  return launch<float>(make_args(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri,
                                 abort_flag, abort2), s);
}

int gemm_tiles_f64(int n, int nb, int nrhs, double alpha, const double *const *tiles_dev,
                   const double *X, long long ldx, double beta, double *C, long long ldc,
                   const int *abort_flag, cudaStream_t s) {
  GemmArgs g = make_args('N', 'N', n, nrhs, n, alpha, nullptr, n, X, ldx, beta, C, ldc, TRI_NONE,
                         abort_flag, nullptr);
  g.tnb = nb;
  g.tmt = (n + nb - 1) / nb;
  g.tn = n;
  g.tptr = (const void *const *)tiles_dev;
  return launch<double>(g, s);
}

int gemm_tiles_f32(int n, int nb, int nrhs, float alpha, const float *const *tiles_dev,
                   const float *X, long long ldx, float beta, float *C, long long ldc,
                   const int *abort_flag, cudaStream_t s) {
  GemmArgs g = make_args('N', 'N', n, nrhs, n, alpha, nullptr, n, X, ldx, beta, C, ldc, TRI_NONE,
                         abort_flag, nullptr);
  g.tnb = nb;
  g.tmt = (n + nb - 1) / nb;
  g.tn = n;
  g.tptr = (const void *const *)tiles_dev;
  return launch<float>(g, s);
}

int scale_f64(int m, int n, double alpha, double *B, int ldb, const int *abort_flag,
              cudaStream_t s, const int *abort2) {
  if (m <= 0 || n <= 0 || alpha == 1.0) return 0;
  size_t total = (size_t)m * n;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4 * dg_num_sms()) blocks = 4 * dg_num_sms();
  scale_kernel<double><<<blocks, 256, 0, s>>>(m, n, alpha, B, ldb, abort_flag, abort2);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

int eye_f64(int n, double *W, int ldw, const int *abort_flag, cudaStream_t s) {
  if (n <= 0) return 0;
  eye_kernel<<<n, 256, 0, s>>>(n, W, ldw, abort_flag);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

int scale_f32(int m, int n, float alpha, float *B, long long ldb, const int *abort_flag,
              cudaStream_t s, const int *abort2) {
  if (m <= 0 || n <= 0 || alpha == 1.0f) return 0;
  size_t total = (size_t)m * n;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4 * dg_num_sms()) blocks = 4 * dg_num_sms();
  scale_kernel<float><<<blocks, 256, 0, s>>>(m, n, alpha, B, ldb, abort_flag, abort2);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

}  // namespace dg
