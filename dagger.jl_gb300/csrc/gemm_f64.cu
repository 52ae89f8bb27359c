// FP64 tile GEMM / SYRK: the trailing-update kernels of the tiled Cholesky
// (BLAS.gemm! at src/array/cholesky.jl:50,95 and BLAS.syrk! at :47,92 of
// Dagger.jl), and the update step of the block triangular solves.
//
// C <- alpha * op(A) * op(B) + beta * C, column-major, any transposes.  One
// CTA owns a 64 x 64 tile of C and walks K in steps of 16, staging the A and
// B slabs in shared memory (register-prefetched double buffer: the next slab
// is fetched from global memory while the current one is multiplied).  The
// inner product runs on one of two FP64 engines:
//   DMMA  mma.sync.aligned.m8n8k4.row.col.f64 (4 warps, 32 x 32 per warp)
//   DFMA  scalar fused multiply-add, 4 x 4 register tile per thread
// GB300 executes FP64 at a small fraction of its FP32 rate, so both engines
// are bounded by the FP64 pipe, not by memory; which one is faster is decided
// by measurement (dg_set_f64_engine).
//
// SYRK uses the same kernel with a triangle mask: CTA tiles wholly outside
// the requested triangle exit at once and stores are limited to the triangle.
#include "dg_common.cuh"

namespace dg {

namespace {

constexpr int BM = 64, BN = 64, BK = 16, PAD = 4;
constexpr int LDS_A = BM + PAD, LDS_B = BN + PAD;

struct GemmArgs {
  int m, n, k;
  double alpha, beta;
  const double *A;
  int lda;
  const double *B;
  int ldb;
  double *C;
  int ldc;
  int ta, tb, tri;
  const int *abort_flag;
};

int g_engine = 0;

// Fetch one BM x BK slab of op(A) and one BK x BN slab of op(B) into
// registers.  Each of the NT threads fetches (BM*BK)/NT elements of each.
template <int NT>
struct SlabLoader {
  static constexpr int PER = (BM * BK) / NT;
  double ra[PER], rb[PER];

  __device__ __forceinline__ void fetch(const GemmArgs &g, int row0, int col0, int k0, int tid) {
#pragma unroll
    for (int q = 0; q < PER; q++) {
      int e = tid + q * NT;
      int i, p;
      if (g.ta == 0) { i = e % BM; p = e / BM; } else { p = e % BK; i = e / BK; }
      int gi = row0 + i, gp = k0 + p;
      double v = 0.0;
      if (gi < g.m && gp < g.k)
        v = g.ta == 0 ? g.A[(size_t)gi + (size_t)gp * g.lda] : g.A[(size_t)gp + (size_t)gi * g.lda];
      ra[q] = v;
      int j;
      if (g.tb == 0) { p = e % BK; j = e / BK; } else { j = e % BN; p = e / BN; }
      int gj = col0 + j;
      gp = k0 + p;
      double w = 0.0;
      if (gj < g.n && gp < g.k)
        w = g.tb == 0 ? g.B[(size_t)gp + (size_t)gj * g.ldb] : g.B[(size_t)gj + (size_t)gp * g.ldb];
      rb[q] = w;
    }
  }

  __device__ __forceinline__ void store(const GemmArgs &g, double *As, double *Bs, int tid) {
#pragma unroll
    for (int q = 0; q < PER; q++) {
      int e = tid + q * NT;
      int i, p;
      if (g.ta == 0) { i = e % BM; p = e / BM; } else { p = e % BK; i = e / BK; }
      As[p * LDS_A + i] = ra[q];
      int j;
      if (g.tb == 0) { p = e % BK; j = e / BK; } else { j = e % BN; p = e / BN; }
      Bs[p * LDS_B + j] = rb[q];
    }
  }
};

__device__ __forceinline__ bool tile_outside_triangle(int tri, int row0, int col0) {
  if (tri == TRI_UPPER) return row0 > col0 + BN - 1;
  if (tri == TRI_LOWER) return col0 > row0 + BM - 1;
  return false;
}

__device__ __forceinline__ void store_c(const GemmArgs &g, int i, int j, double acc) {
  if (i >= g.m || j >= g.n) return;
  if (g.tri == TRI_UPPER && i > j) return;
  if (g.tri == TRI_LOWER && i < j) return;
  double *c = g.C + (size_t)i + (size_t)j * g.ldc;
  double v = g.alpha * acc;
  if (g.beta != 0.0) v = fma(g.beta, *c, v);
  *c = v;
}

// ---- DFMA engine: 256 threads, thread (tx, ty) owns rows tx + 16 r and
// ---- columns ty + 16 c, r, c in [0, 4).
__global__ void __launch_bounds__(256) gemm_f64_dfma(GemmArgs g) {
  if (g.abort_flag && *(volatile const int *)g.abort_flag) return;
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
  if (tile_outside_triangle(g.tri, row0, col0)) return;
  __shared__ double As[2][BK * LDS_A];
  __shared__ double Bs[2][BK * LDS_B];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < 4; c++) acc[r][c] = 0.0;

  SlabLoader<256> ld;
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
      double a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; r++) a[r] = As[cur][p * LDS_A + tx + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; c++) b[c] = Bs[cur][p * LDS_B + ty + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[r][c] = fma(a[r], b[c], acc[r][c]);
    }
    if (kt + 1 < nk) ld.store(g, As[cur ^ 1], Bs[cur ^ 1], tid);
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < 4; c++) store_c(g, row0 + tx + 16 * r, col0 + ty + 16 * c, acc[r][c]);
}

// ---- DMMA engine: 128 threads = 4 warps in a 2 x 2 grid, warp tile 32 x 32
// ---- = 4 x 4 fragments of m8n8.  Fragment layouts (PTX ISA, mma.m8n8k4 f64):
// ----   A 8x4 row:  lane holds A[lane/4][lane%4]
// ----   B 4x8 col:  lane holds B[lane%4][lane/4]
// ----   C 8x8:      lane holds C[lane/4][2*(lane%4) + {0,1}]
__device__ __forceinline__ void dmma_m8n8k4(double &d0, double &d1, double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
      : "+d"(d0), "+d"(d1)
      : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(128) gemm_f64_dmma(GemmArgs g) {
  if (g.abort_flag && *(volatile const int *)g.abort_flag) return;
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
  if (tile_outside_triangle(g.tri, row0, col0)) return;
  __shared__ double As[2][BK * LDS_A];
  __shared__ double Bs[2][BK * LDS_B];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
  const int qr = lane >> 2, qc = lane & 3;
  double acc[4][4][2];
#pragma unroll
  for (int mi = 0; mi < 4; mi++)
#pragma unroll
    for (int ni = 0; ni < 4; ni++) acc[mi][ni][0] = acc[mi][ni][1] = 0.0;

  SlabLoader<128> ld;
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
      for (int mi = 0; mi < 4; mi++) a[mi] = As[cur][(k4 + qc) * LDS_A + wm + mi * 8 + qr];
#pragma unroll
      for (int ni = 0; ni < 4; ni++) b[ni] = Bs[cur][(k4 + qc) * LDS_B + wn + ni * 8 + qr];
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
        store_c(g, row0 + wm + mi * 8 + qr, col0 + wn + ni * 8 + 2 * qc + h, acc[mi][ni][h]);
}

__global__ void scale_f64_kernel(int m, int n, double alpha, double *B, int ldb,
                                 const int *abort_flag) {
  if (abort_flag && *(volatile const int *)abort_flag) return;
  size_t total = (size_t)m * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(e % m), j = (int)(e / m);
    double *p = B + (size_t)i + (size_t)j * ldb;
    *p = alpha == 0.0 ? 0.0 : alpha * *p;
  }
}

}  // namespace

void set_f64_engine(int engine) { g_engine = engine ? 1 : 0; }
int get_f64_engine() { return g_engine; }

int gemm_f64(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
             const double *B, int ldb, double beta, double *C, int ldc, Tri tri,
             const int *abort_flag, cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  GemmArgs g;
  g.m = m; g.n = n; g.k = (alpha == 0.0) ? 0 : k;
  g.alpha = alpha; g.beta = beta;
  g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.C = C; g.ldc = ldc;
  g.ta = (ta == 'N' || ta == 'n') ? 0 : 1;
  g.tb = (tb == 'N' || tb == 'n') ? 0 : 1;
  g.tri = tri;
  g.abort_flag = abort_flag;
  dim3 grid((m + BM - 1) / BM, (n + BN - 1) / BN);
  if (grid.y > 65535) return DG_ERR_UNSUPPORTED;
  if (g_engine)
    gemm_f64_dmma<<<grid, 128, 0, s>>>(g);
  else
    gemm_f64_dfma<<<grid, 256, 0, s>>>(g);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

int scale_f64(int m, int n, double alpha, double *B, int ldb, const int *abort_flag,
              cudaStream_t s) {
  if (m <= 0 || n <= 0 || alpha == 1.0) return 0;
  size_t total = (size_t)m * n;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4 * dg_num_sms()) blocks = 4 * dg_num_sms();
  scale_f64_kernel<<<blocks, 256, 0, s>>>(m, n, alpha, B, ldb, abort_flag);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

}  // namespace dg
