// Batched factor-and-solve of many independent SPD systems of uneven size in
// ONE persistent launch.
//
// Systems are grouped into size buckets (n <= 64, 128, 256, 512, 1024, more)
// and each bucket is a queue of system indices sorted by decreasing n.  The
// grid is sized to the SM count; every CTA repeatedly takes the next system
// from the queue of the largest non-empty bucket (an atomic ticket per
// bucket), so big systems start first and small ones fill the tail (longest
// processing time first).  Each bucket carries its own panel width, chosen by
// the autotuner (dagger_gb300/autotune.py) and stored per (n-range, dtype).
//
// One CTA owns one system at a time and runs, in global memory (the matrix
// stays L2-resident while the CTA works on it):
//   factor   left-looking blocked Cholesky, lower form: for each panel of W
//            columns, the panel is updated with the already factored columns
//            (a shared-memory staged GEMM), its W x W diagonal block is
//            factored in shared memory, and the rows below are solved
//            against it (one thread per row);
//   solve    forward and backward substitution with the right-hand sides
//            held in shared memory (up to 8 columns).
// FP64 variant: factor and solve in FP64, in place.
// FP32+IR variant: the system is rounded into an FP32 copy which is
// factored; the solution is refined in FP64 (residual b - A x with the
// original FP64 matrix, correction from the FP32 factor) until the normwise
// backward error of every column is at most tol, inside the same CTA.
// A pivot that is not positive records info for that system and the CTA
// moves on; no wait in this kernel depends on another CTA.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "dg_common.cuh"
#include "runtime.h"

namespace dg {
namespace {

constexpr int NT = 256;      // threads per CTA
constexpr int WMAX = 32;     // largest panel width
constexpr int RB = 64;       // rows per block of the panel update
constexpr int RMAX = 8;      // right-hand sides per system
constexpr int NSMEM_X = 1024 * RMAX;  // solution vector capacity (elements)

struct BatchSys {
  int n, nrhs;
  double *A;        // n x n, column-major, lda = n (factor written in place for FP64)
  const double *B;  // n x nrhs, ldb = n
  double *X;        // n x nrhs, ldx = n
  float *W32;       // FP32 workspace n x n (FP32+IR), else null
  int *info;        // per-system info / iteration count output (2 ints)
  double *berr;     // per-system worst backward error
};

struct BucketCfg {
  int start, count;  // range in the order array
  int w;             // panel width (16 or 32)
};

struct BatchParams {
  const BatchSys *sys;
  const int *order;
  int *tickets;      // one per bucket
  BucketCfg bucket[8];
  int nbuckets;
  int mode;          // 0 = FP64, 1 = FP32 + IR
  double tol;
  int max_iter;
  int *status;
};

template <typename T>
struct Shared {
  T As[RB][WMAX + 1];
  T Bs[WMAX][WMAX + 1];
  T Ld[WMAX][WMAX + 1];
  int flag;
  int ticket;
};

// Left-looking blocked Cholesky (lower) of the n x n matrix L (ld n) in place.
// Returns 0 or the 1-based index of the failing pivot (uniform across the CTA).
template <typename T, int W>
__device__ int factor_lower(T *L, int n, Shared<T> &sh) {
  const int tid = threadIdx.x;
  const int tx = tid % W, ty = tid / W;  // W columns x (NT/W) row groups
  constexpr int RG = NT / W;
  constexpr int RPT = RB / RG;           // rows per thread per row block
  for (int j0 = 0; j0 < n; j0 += W) {
    const int w = min(W, n - j0);
    // 1. panel update A[j0:, j0:j0+w] -= L[j0:, :j0] L[j0:j0+w, :j0]'
    if (j0 > 0) {
      for (int r0 = j0; r0 < n; r0 += RB) {
        T acc[RPT];
#pragma unroll
        for (int q = 0; q < RPT; q++) acc[q] = T(0);
        for (int k0 = 0; k0 < j0; k0 += W) {
          const int kw = min(W, j0 - k0);
          __syncthreads();
          for (int e = tid; e < RB * W; e += NT) {
            const int i = e % RB, k = e / RB;
            sh.As[i][k] = (r0 + i < n && k < kw) ? L[(r0 + i) + (size_t)(k0 + k) * n] : T(0);
          }
          for (int e = tid; e < W * W; e += NT) {
            const int c = e % W, k = e / W;
            sh.Bs[c][k] = (c < w && k < kw) ? L[(j0 + c) + (size_t)(k0 + k) * n] : T(0);
          }
          __syncthreads();
#pragma unroll 4
          for (int k = 0; k < W; k++) {
            const T b = sh.Bs[tx][k];
#pragma unroll
            for (int q = 0; q < RPT; q++) acc[q] = fma(sh.As[ty + RG * q][k], b, acc[q]);
          }
        }
        if (tx < w)
#pragma unroll
          for (int q = 0; q < RPT; q++) {
            const int i = r0 + ty + RG * q;
            if (i < n && i >= j0 + tx) L[i + (size_t)(j0 + tx) * n] -= acc[q];
          }
      }
      __syncthreads();
    }
    // 2. factor the diagonal block in shared memory
    for (int e = tid; e < w * w; e += NT) {
      const int i = e % w, c = e / w;
      if (i >= c) sh.Ld[i][c] = L[(j0 + i) + (size_t)(j0 + c) * n];
    }
    if (tid == 0) sh.flag = 0;
    __syncthreads();
    if (tid < 32) {
      // one warp: right-looking on the w x w block, lane = row
      const int lane = tid;
      for (int c = 0; c < w; c++) {
        T d = sh.Ld[c][c];
        if (!(d > T(0))) {
          if (lane == 0) sh.flag = j0 + c + 1;
          break;
        }
        d = sqrt(d);
        __syncwarp();
        if (lane > c && lane < w) sh.Ld[lane][c] /= d;
        if (lane == c) sh.Ld[c][c] = d;
        __syncwarp();
        for (int k = c + 1; k < w; k++)
          if (lane >= k && lane < w) sh.Ld[lane][k] = fma(-sh.Ld[lane][c], sh.Ld[k][c], sh.Ld[lane][k]);
        __syncwarp();
      }
    }
    __syncthreads();
    if (sh.flag) return sh.flag;
    for (int e = tid; e < w * w; e += NT) {
      const int i = e % w, c = e / w;
      if (i >= c) L[(j0 + i) + (size_t)(j0 + c) * n] = sh.Ld[i][c];
    }
    // 3. rows below: L[i, j0:j0+w] = A[i, j0:j0+w] Ld^-T (one thread per row)
    for (int i = j0 + w + tid; i < n; i += NT) {
      T x[W];
#pragma unroll
      for (int c = 0; c < W; c++) x[c] = c < w ? L[i + (size_t)(j0 + c) * n] : T(0);
#pragma unroll
      for (int c = 0; c < W; c++) {
        if (c < w) {
          T v = x[c];
          for (int k = 0; k < c; k++) v = fma(-x[k], sh.Ld[c][k], v);
          x[c] = v / sh.Ld[c][c];
        }
      }
#pragma unroll
      for (int c = 0; c < W; c++)
        if (c < w) L[i + (size_t)(j0 + c) * n] = x[c];
    }
    __syncthreads();
  }
  return 0;
}

// X (n x r in shared memory, column stride n) <- L^-T L^-1 X.
template <typename T, typename TX>
__device__ void solve_lower(const T *L, int n, int r, TX *X) {
  const int tid = threadIdx.x;
  // forward: L y = x
  for (int j0 = 0; j0 < n; j0 += WMAX) {
    const int w = min(WMAX, n - j0);
    // x[j0:j0+w] -= L[j0:j0+w, :j0] x[:j0]  (thread per (row, column))
    for (int e = tid; e < w * r; e += NT) {
      const int i = j0 + e % w, c = e / w;
      TX acc = 0;
      for (int k = 0; k < j0; k++) acc += (TX)L[i + (size_t)k * n] * X[k + c * n];
      X[i + c * n] -= acc;
    }
    __syncthreads();
    if (tid < r) {
      const int c = tid;
      for (int i = j0; i < j0 + w; i++) {
        TX v = X[i + c * n];
        for (int k = j0; k < i; k++) v -= (TX)L[i + (size_t)k * n] * X[k + c * n];
        X[i + c * n] = v / (TX)L[i + (size_t)i * n];
      }
    }
    __syncthreads();
  }
  // backward: L' x = y
  for (int j1 = n; j1 > 0; j1 -= WMAX) {
    const int j0 = max(0, j1 - WMAX), w = j1 - j0;
    for (int e = tid; e < w * r; e += NT) {
      const int i = j0 + e % w, c = e / w;
      TX acc = 0;
      for (int k = j1; k < n; k++) acc += (TX)L[k + (size_t)i * n] * X[k + c * n];
      X[i + c * n] -= acc;
    }
    __syncthreads();
    if (tid < r) {
      const int c = tid;
      for (int i = j1 - 1; i >= j0; i--) {
        TX v = X[i + c * n];
        for (int k = i + 1; k < j1; k++) v -= (TX)L[k + (size_t)i * n] * X[k + c * n];
        X[i + c * n] = v / (TX)L[i + (size_t)i * n];
      }
    }
    __syncthreads();
  }
}

__device__ double block_max(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double m = 0.0;
  for (int i = 0; i < NT / 32; i++) m = fmax(m, red[i]);
  return m;
}

template <int W>
__device__ void run_fp64(const BatchSys &S, Shared<double> &sh, double *X) {
  const int n = S.n, r = S.nrhs;
  const int info = factor_lower<double, W>(S.A, n, sh);
  if (threadIdx.x == 0) {
    S.info[0] = info;
    S.info[1] = 0;
  }
  if (info) return;
  for (int e = threadIdx.x; e < n * r; e += NT) X[e] = S.B[e];
  __syncthreads();
  solve_lower<double, double>(S.A, n, r, X);
  for (int e = threadIdx.x; e < n * r; e += NT) S.X[e] = X[e];
  __syncthreads();
}

template <int W>
__device__ void run_fp32_ir(const BatchSys &S, Shared<float> &sh, double *X, double *Rv, float *Z,
                            const BatchParams &p) {
  const int n = S.n, r = S.nrhs;
  __shared__ double red[NT / 32];
  float *L = S.W32;
  for (size_t e = threadIdx.x; e < (size_t)n * n; e += NT) L[e] = (float)S.A[e];
  __syncthreads();
  const int info = factor_lower<float, W>(L, n, sh);
  if (threadIdx.x == 0) S.info[0] = info;
  if (info) return;
  // ||A||_inf (A symmetric: max column sum)
  double na = 0.0;
  for (int c = threadIdx.x; c < n; c += NT) {
    double acc = 0.0;
    for (int i = 0; i < n; i++) acc += fabs(S.A[i + (size_t)c * n]);
    na = fmax(na, acc);
  }
  na = block_max(na, red);
  double bmax[RMAX];
  for (int c = 0; c < r; c++) {
    double m = 0.0;
    for (int i = threadIdx.x; i < n; i += NT) m = fmax(m, fabs(S.B[i + (size_t)c * n]));
    bmax[c] = block_max(m, red);
  }
  for (int e = threadIdx.x; e < n * r; e += NT) {
    X[e] = 0.0;
    Rv[e] = S.B[e];
  }
  __syncthreads();
  int it = 0;
  double worst = 0.0;
  for (it = 0; it < p.max_iter; it++) {
    // correction z = L^-T L^-1 r (FP32), x += z
    for (int e = threadIdx.x; e < n * r; e += NT) Z[e] = (float)Rv[e];
    __syncthreads();
    solve_lower<float, float>(L, n, r, Z);
    for (int e = threadIdx.x; e < n * r; e += NT) X[e] += (double)Z[e];
    __syncthreads();
    // r = b - A x (FP64)
    for (int e = threadIdx.x; e < n * r; e += NT) {
      const int i = e % n, c = e / n;
      double acc = S.B[e];
      for (int k = 0; k < n; k++) acc = fma(-S.A[i + (size_t)k * n], X[k + c * n], acc);
      Rv[e] = acc;
    }
    __syncthreads();
    worst = 0.0;
    for (int c = 0; c < r; c++) {
      double rm = 0.0, xm = 0.0;
      for (int i = threadIdx.x; i < n; i += NT) {
        rm = fmax(rm, fabs(Rv[i + c * n]));
        xm = fmax(xm, fabs(X[i + c * n]));
      }
      rm = block_max(rm, red);
      xm = block_max(xm, red);
      const double den = na * xm + bmax[c];
      worst = fmax(worst, den > 0 ? rm / den : 0.0);
    }
    if (worst <= p.tol) {
      it++;
      break;
    }
  }
  if (threadIdx.x == 0) {
    S.info[1] = it;
    *S.berr = worst;
  }
  for (int e = threadIdx.x; e < n * r; e += NT) S.X[e] = X[e];
  __syncthreads();
}

// Shared-memory budget: the staging tiles plus the solution (and, for FP32+IR,
// the residual) vectors.
__global__ void __launch_bounds__(NT) batched_kernel(BatchParams p) {
  extern __shared__ double dyn[];
  __shared__ Shared<double> sh64;
  Shared<float> &sh32 = *reinterpret_cast<Shared<float> *>(&sh64);
  double *X = dyn, *Rv = dyn + NSMEM_X;
  float *Z = (float *)(dyn + 2 * NSMEM_X);
  for (;;) {
    if (threadIdx.x == 0) {
      int t = -1;
      for (int b = 0; b < p.nbuckets && t < 0; b++) {
        if (p.bucket[b].count == 0) continue;
        const int k = atomicAdd(&p.tickets[b], 1);
        if (k < p.bucket[b].count) t = (b << 24) | k;
      }
      sh64.ticket = t;
    }
    __syncthreads();
    const int t = sh64.ticket;
    __syncthreads();
    if (t < 0) break;
    const int b = t >> 24, k = t & 0xFFFFFF;
    const BatchSys S = p.sys[p.order[p.bucket[b].start + k]];
    const int w = p.bucket[b].w;
    if (p.mode == 0) {
      if (w == 16) run_fp64<16>(S, sh64, X); else run_fp64<32>(S, sh64, X);
    } else {
      if (w == 16) run_fp32_ir<16>(S, sh32, X, Rv, Z, p); else run_fp32_ir<32>(S, sh32, X, Rv, Z, p);
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace dg

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// The kernel's dynamic shared memory (solution, residual and correction
// vectors) exceeds the 48 KiB default; the limit is raised once per device.
static int set_batched_smem() {
  static std::atomic<bool> done[64];  // zero-initialised: false
  int dev = 0;
  DG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && done[dev]) return 0;
  DG_CUDA_TRY(cudaFuncSetAttribute(dg::batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)((sizeof(double) * 2 + sizeof(float)) * dg::NSMEM_X)));
  if (dev >= 0 && dev < 64) done[dev] = true;
  return 0;
}

extern "C" int dg_batched_potrs(int count, const int *n, const int *nrhs, double *const *A,
                                const double *const *B, double *const *X, int mode, double tol,
                                int max_iter, const int *bucket_w, int ctas_per_sm, int *info,
                                double *berr, float *elapsed_ms, void *stream) {
  DG_CHECK_ARG(count >= 0, 1);
  DG_CHECK_ARG(mode == 0 || mode == 1, 7);
  if (count == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  const int edges[] = {64, 128, 256, 512, 1024};
  const int NB = 5;
  std::vector<int> idx(count);
  for (int i = 0; i < count; i++) {
    DG_CHECK_ARG(n[i] > 0 && n[i] <= 1024, 2);
    DG_CHECK_ARG(nrhs[i] > 0 && nrhs[i] <= dg::RMAX, 3);
    idx[i] = i;
  }
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return n[a] > n[b]; });
  dg::BatchParams p;
  memset(&p, 0, sizeof p);
  // buckets from the largest sizes down
  int pos = 0;
  for (int bb = NB - 1; bb >= 0; bb--) {
    const int lo = bb ? edges[bb - 1] : 0, hi = edges[bb];
    dg::BucketCfg &c = p.bucket[p.nbuckets];
    c.start = pos;
    while (pos < count && n[idx[pos]] > lo && n[idx[pos]] <= hi) pos++;
    c.count = pos - c.start;
    c.w = bucket_w ? bucket_w[bb] : 32;
    if (c.w != 16) c.w = 32;
    p.nbuckets++;
  }
  // device copies of the descriptors and workspaces
  size_t ws = 0;
  for (int i = 0; i < count; i++) ws += mode ? (size_t)n[i] * n[i] : 0;
  dg::BatchSys *dsys = nullptr;
  int *dorder = nullptr, *dtick = nullptr, *dinfo = nullptr;
  double *dberr = nullptr;
  float *dws = nullptr;
  DG_CUDA_TRY(cudaMallocAsync((void **)&dsys, sizeof(dg::BatchSys) * count, s));
  DG_CUDA_TRY(cudaMallocAsync((void **)&dorder, sizeof(int) * count + 64, s));
  DG_CUDA_TRY(cudaMallocAsync((void **)&dinfo, sizeof(int) * 2 * count, s));
  DG_CUDA_TRY(cudaMallocAsync((void **)&dberr, sizeof(double) * count, s));
  if (ws) DG_CUDA_TRY(cudaMallocAsync((void **)&dws, sizeof(float) * ws, s));
  dtick = dorder + count + (count & 1);
  std::vector<dg::BatchSys> hs(count);
  size_t off = 0;
  for (int i = 0; i < count; i++) {
    hs[i].n = n[i];
    hs[i].nrhs = nrhs[i];
    hs[i].A = A[i];
    hs[i].B = B[i];
    hs[i].X = X[i];
    hs[i].W32 = mode ? dws + off : nullptr;
    off += mode ? (size_t)n[i] * n[i] : 0;
    hs[i].info = dinfo + 2 * i;
    hs[i].berr = dberr + i;
  }
  DG_CUDA_TRY(cudaMemcpyAsync(dsys, hs.data(), sizeof(dg::BatchSys) * count, cudaMemcpyHostToDevice, s));
  DG_CUDA_TRY(cudaMemcpyAsync(dorder, idx.data(), sizeof(int) * count, cudaMemcpyHostToDevice, s));
  DG_CUDA_TRY(cudaMemsetAsync(dtick, 0, sizeof(int) * 8, s));
  DG_CUDA_TRY(cudaMemsetAsync(dberr, 0, sizeof(double) * count, s));
  p.sys = dsys;
  p.order = dorder;
  p.tickets = dtick;
  p.mode = mode;
  p.tol = tol > 0 ? tol : 1e-12;
  p.max_iter = max_iter > 0 ? max_iter : 30;
  const size_t dyn = mode ? (sizeof(double) * 2 + sizeof(float)) * dg::NSMEM_X
                          : sizeof(double) * dg::NSMEM_X;
  DG_TRY(set_batched_smem());
  if (ctas_per_sm < 1) ctas_per_sm = 1;
  const int grid = std::min(count, dg_num_sms() * ctas_per_sm);
  cudaEvent_t e0, e1;
  DG_CUDA_TRY(cudaEventCreate(&e0));
  DG_CUDA_TRY(cudaEventCreate(&e1));
  cudaEventRecord(e0, s);
  dg::batched_kernel<<<grid, dg::NT, dyn, s>>>(p);
  cudaEventRecord(e1, s);
  cudaError_t le = cudaGetLastError();
  dg::count_launches(1);
  std::vector<int> hinfo(2 * count);
  cudaMemcpyAsync(hinfo.data(), dinfo, sizeof(int) * 2 * count, cudaMemcpyDeviceToHost, s);
  if (berr) cudaMemcpyAsync(berr, dberr, sizeof(double) * count, cudaMemcpyDeviceToHost, s);
  cudaError_t se = cudaStreamSynchronize(s);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  if (elapsed_ms) *elapsed_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(dsys, s);
  cudaFreeAsync(dorder, s);
  cudaFreeAsync(dinfo, s);
  cudaFreeAsync(dberr, s);
  if (dws) cudaFreeAsync(dws, s);
  DG_CUDA_TRY(le);
  DG_CUDA_TRY(se);
  int first_bad = 0;
  for (int i = 0; i < count; i++) {
    if (info) {
      info[2 * i] = hinfo[2 * i];
      info[2 * i + 1] = hinfo[2 * i + 1];
    }
    if (hinfo[2 * i] && !first_bad) first_bad = i + 1;
  }
  return first_bad;  // 0, or 1 + index of the first system whose factorization failed
}

// ---------------------------------------------------------------------------
// Allocation-free entry point
// ---------------------------------------------------------------------------
// Some callers cannot allocate device memory while they run: a host that
// reserved all of its device memory up front (a serving process that admits
// work against a fixed memory budget), a pool-based allocator that must not
// be bypassed, or a real-time loop that forbids allocation after start-up.
// dg_batched_potrs allocates its descriptors and FP32 workspaces per call;
// this variant takes them from one file-scope device array instead.
//
// The array lives in every GPU that loads the library until the process
// exits.  In host code the symbol is only a host-side stand-in, so every call
// looks up its device address for the current device (cudaGetSymbolAddress,
// which allocates nothing); no address is cached, so a context that was reset
// and reloaded the module gets the new address.  The call is synchronous: it
// stages its descriptors from host memory and waits for the launch, so it
// cannot be made while its stream is being captured.  Every call shares the
// array and it keeps the previous call's contents, so the ticket counters and
// error words are cleared on each call, and calls take turns on a lock that
// each holds until its launch has finished (host threads on different
// streams would otherwise overlap on the array).
namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;  // 64 MiB
constexpr int kNoAllocMaxSystems = 4096;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

thread_local dg::BatchSys t_sys[kNoAllocMaxSystems];
thread_local int t_idx[kNoAllocMaxSystems];
thread_local int t_info[2 * kNoAllocMaxSystems];

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

std::mutex g_noalloc_mu;  // one call at a time owns the array

// The array's device address on the current device, looked up on each call.
int noalloc_scratch(void **out) {
  void *p = nullptr;
  DG_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  *out = p;
  return 0;
}

}  // namespace

extern "C" int dg_batched_potrs_noalloc(int count, const int *n, const int *nrhs,
                                        double *const *A, const double *const *B,
                                        double *const *X, int mode, double tol, int max_iter,
                                        const int *bucket_w, int ctas_per_sm, int *info,
                                        double *berr, void *stream) {
  DG_CHECK_ARG(count >= 0 && count <= kNoAllocMaxSystems, 1);
  DG_CHECK_ARG(mode == 0 || mode == 1, 7);
  if (count == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  for (int i = 0; i < count; i++) {
    DG_CHECK_ARG(n[i] > 0 && n[i] <= 1024, 2);
    DG_CHECK_ARG(nrhs[i] > 0 && nrhs[i] <= dg::RMAX, 3);
  }
  // layout of the scratch: descriptors | order | tickets | info | berr | FP32 workspaces
  const size_t o_sys = 0;
  const size_t o_order = align256(o_sys + sizeof(dg::BatchSys) * count);
  const size_t o_tick = align256(o_order + sizeof(int) * count);
  const size_t o_info = align256(o_tick + sizeof(int) * 8);
  const size_t o_berr = align256(o_info + sizeof(int) * 2 * count);
  const size_t o_ws = align256(o_berr + sizeof(double) * count);
  size_t ws = 0;
  for (int i = 0; i < count; i++) ws += mode ? align256(sizeof(float) * (size_t)n[i] * n[i]) : 0;
  if (o_ws + ws > kNoAllocScratchBytes) {
    dg_set_last_error(__FILE__, __LINE__,
                      "batch exceeds the 64 MiB scratch of dg_batched_potrs_noalloc");
    return DG_ERR_NOMEM;
  }
  std::lock_guard<std::mutex> turn(g_noalloc_mu);
  void *base = nullptr;
  DG_TRY(noalloc_scratch(&base));
  unsigned char *sc = (unsigned char *)base;
  for (int i = 0; i < count; i++) t_idx[i] = i;
  std::stable_sort(t_idx, t_idx + count, [&](int a, int b) { return n[a] > n[b]; });
  dg::BatchParams p;
  memset(&p, 0, sizeof p);
  const int edges[] = {64, 128, 256, 512, 1024};
  int pos = 0;
  for (int bb = 4; bb >= 0; bb--) {
    const int lo = bb ? edges[bb - 1] : 0, hi = edges[bb];
    dg::BucketCfg &c = p.bucket[p.nbuckets];
    c.start = pos;
    while (pos < count && n[t_idx[pos]] > lo && n[t_idx[pos]] <= hi) pos++;
    c.count = pos - c.start;
    c.w = (bucket_w && bucket_w[bb] == 16) ? 16 : 32;
    p.nbuckets++;
  }
  size_t off = o_ws;
  for (int i = 0; i < count; i++) {
    dg::BatchSys &d = t_sys[i];
    d.n = n[i];
    d.nrhs = nrhs[i];
    d.A = A[i];
    d.B = B[i];
    d.X = X[i];
    d.W32 = mode ? (float *)(sc + off) : nullptr;
    off += mode ? align256(sizeof(float) * (size_t)n[i] * n[i]) : 0;
    d.info = (int *)(sc + o_info) + 2 * i;
    d.berr = (double *)(sc + o_berr) + i;
  }
  DG_CUDA_TRY(cudaMemcpyAsync(sc + o_sys, t_sys, sizeof(dg::BatchSys) * count,
                              cudaMemcpyHostToDevice, s));
  DG_CUDA_TRY(cudaMemcpyAsync(sc + o_order, t_idx, sizeof(int) * count, cudaMemcpyHostToDevice, s));
  // the array keeps the last call's contents: clear what must start at zero
  DG_CUDA_TRY(cudaMemsetAsync(sc + o_tick, 0, sizeof(int) * 8, s));
  DG_CUDA_TRY(cudaMemsetAsync(sc + o_info, 0, sizeof(int) * 2 * count, s));
  DG_CUDA_TRY(cudaMemsetAsync(sc + o_berr, 0, sizeof(double) * count, s));
  p.sys = (const dg::BatchSys *)(sc + o_sys);
  p.order = (const int *)(sc + o_order);
  p.tickets = (int *)(sc + o_tick);
  p.mode = mode;
  p.tol = tol > 0 ? tol : 1e-12;
  p.max_iter = max_iter > 0 ? max_iter : 30;
  DG_TRY(set_batched_smem());
  const size_t dyn = mode ? (sizeof(double) * 2 + sizeof(float)) * dg::NSMEM_X
                          : sizeof(double) * dg::NSMEM_X;
  if (ctas_per_sm < 1) ctas_per_sm = 1;
  const int grid = std::min(count, dg_num_sms() * ctas_per_sm);
  dg::batched_kernel<<<grid, dg::NT, dyn, s>>>(p);
  DG_CUDA_TRY(cudaGetLastError());
  dg::count_launches(1);
  DG_CUDA_TRY(cudaMemcpyAsync(t_info, sc + o_info, sizeof(int) * 2 * count,
                              cudaMemcpyDeviceToHost, s));
  if (berr)
    DG_CUDA_TRY(cudaMemcpyAsync(berr, sc + o_berr, sizeof(double) * count,
                                cudaMemcpyDeviceToHost, s));
  DG_CUDA_TRY(cudaStreamSynchronize(s));
  int first_bad = 0;
  for (int i = 0; i < count; i++) {
    if (info) {
      info[2 * i] = t_info[2 * i];
      info[2 * i + 1] = t_info[2 * i + 1];
    }
    if (t_info[2 * i] && !first_bad) first_bad = i + 1;
  }
  return first_bad;
}
