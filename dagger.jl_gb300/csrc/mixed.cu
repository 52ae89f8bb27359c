// Mixed-precision Cholesky factor-and-solve with iterative refinement.
//
// The plain FP64 path (runtime.cu) is the drop-in for Dagger.jl's DArray
// Cholesky; this file is the faster form beside it.  Given the caller's FP64
// tiles of A it computes, on the GPU:
//
//   1. Scaling: s_i = 1/sqrt(a_ii), A~ = S A S (unit diagonal, so every entry
//      of its Cholesky factor has magnitude <= 1), rounded to FP32 and packed
//      into upper row panels: panel r holds rows r*nb .. r*nb+nb-1, columns
//      r*nb .. n-1, column-major with leading dimension nb (about n^2/2 floats).
//   2. A right-looking blocked factorization over the panels.  Step k:
//        POTRF of the nb x nb diagonal block in FP32; if a pivot fails, the
//        block (kept from before the attempt) is widened to FP64 and factored
//        again by a one-CTA FP64 kernel, which only runs on failure;
//        TRSM of the rest of panel k in FP32;
//        conversion of that panel to 16-bit operands: BF16 or FP16, one term
//        or hi/lo split (x = hi + lo), FP16 with a per-panel power-of-two
//        scale chosen from the panel's largest entry (FP16's range is narrow);
//        the trailing update A~[k+1:, k+1:] -= P' P of the upper triangle in
//        one tcgen05 launch (tc_gemm.cu), FP32 accumulation in TMEM, or on
//        the FP32 CUDA-core GEMM for the FP32 precision setting.
//   3. Refinement in FP64: r = b - A x with the caller's FP64 tiles, the
//      correction from the low-precision factor (FP32 triangular solves on the
//      packed panels), x += S z.  The normwise backward error of each column,
//      ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf), decides convergence.
//      When plain refinement stalls, GMRES-IR takes over: restarted GMRES on
//      the correction equation, left-preconditioned by the low-precision
//      factor, with FP64 Krylov vectors and FP64 matrix-vector products.
// Only the residual, the solution update, the POTRF retry and GMRES's
// vectors run in FP64.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "dg_common.cuh"
#include "runtime.h"
#include "tc_gemm.h"

struct dg_mixed {
  int n = 0, nb = 0, mt = 0, precision = 0;
  int dev = 0;
  float *W = nullptr;            // packed upper panels of the scaled factor
  double *s = nullptr;           // diagonal scaling
  double **tiles_dev = nullptr;  // caller's FP64 tiles (device array of pointers)
  void *P_hi = nullptr, *P_lo = nullptr;  // FP16 (scaled) panel operands (T x nb, K-major)
  uint8_t *P8 = nullptr;         // FP8 form: E4M3 panel operands, two buffers (T x nb)
  float *s8 = nullptr;           // FP8 form: their per-vector scales, two buffers (T)
  float *diag_backup = nullptr;  // diagonal block before its FP32 factorization
  double *d64 = nullptr;         // FP64 scratch of the retry
  float *panel_max = nullptr;    // per-step |panel| maximum (FP16 scaling)
  float *alpha_dev = nullptr;    // per-step -1/scale^2 of the trailing update
  float *Vinv = nullptr;         // inverses of the diagonal blocks (mt x nb x nb)
  void *diag_scratch = nullptr;  // the diagonal-block kernel's barrier words and scratch
  void *S3r = nullptr;           // 3 BF16 slices of panel k's rest before its solve
  // FP32-accurate BF16 slices (hi | mid | lo) of the finished factor: the
  // operands of the trailing updates (hi, mid = the hi/lo split of bf16x3)
  // and of the refinement's triangular solves on the tensor cores
  __nv_bfloat16 *R3 = nullptr;   // every panel's rest, at the offsets of W
  long long r3_stride = 0;       // elements per slice of R3
  __nv_bfloat16 *V3 = nullptr;   // every Vinv_k (k nb^2 offsets)
  __nv_bfloat16 *VT3 = nullptr;  // every Vinv_k'
  __nv_bfloat16 *L3 = nullptr;   // block columns of U transposed (lp_base offsets)
  long long v3_stride = 0, l3_stride = 0;
  // slices of A's rows for the emulated FP64 residual, cut on `aux2` while
  // the factorization runs (ev_oz marks their completion)
  void *ozA = nullptr;
  unsigned long long *ozAs = nullptr;
  long long oz_ldk = 0;
  cudaStream_t aux2 = nullptr;
  cudaEvent_t ev_oz = nullptr;
  int *words = nullptr;          // [0] status, [1] retries, [2] first bad diagonal,
                                 // [3..3+mt) info_k, [3+mt..3+2mt) retried_k
  double normA = 0.0;            // ||A||_inf
  size_t bytes = 0;
  int info = 0, retries = 0;
  float factor_ms = 0.f;
  cudaStream_t stream = nullptr;  // allocations are stream-ordered on this stream
  double shift = 0.0;             // added to the unit diagonal of S A S before factoring
  cudaStream_t aux = nullptr;     // lookahead stream (the next panel's step)
  cudaEvent_t ev_next = nullptr, ev_panel = nullptr;
  // BF16 forms: the trailing updates by block row, on streams by priority
  // (near_s[d]: the row d+2 steps ahead of the panel; far_s: the others in
  // kFar launches of consecutive rows); ev_row[r] marks block row r's latest
  // update, which the next one waits for
  static constexpr int kNear = 3, kFar = 4;
  cudaStream_t near_s[kNear] = {}, far_s[kFar] = {};
  std::vector<cudaEvent_t> ev_row;
  // recorded by the BF16 schedule at mid-factorization: the slicing of A for
  // the residual (memory-bound) starts there, behind the heaviest bulk updates
  cudaEvent_t ev_gate = nullptr;
};

namespace dg {
namespace {

__device__ __forceinline__ const double *tile_ptr(const double *const *tiles, int mt, int i, int j) {
  return tiles[i + (size_t)j * mt];
}

// s_i = 1 / sqrt(a_ii); the first non-positive diagonal is recorded (atomicMin).
__global__ void diag_scale_kernel(const double *const *tiles, int n, int nb, int mt, double *s,
                                  int *bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int t = i / nb, p = i - t * nb;
    const int rows = min(nb, n - t * nb);
    const double a = tile_ptr(tiles, mt, t, t)[p + (size_t)p * rows];
    if (!(a > 0.0)) {
      atomicMin(bad, i + 1);
      s[i] = 1.0;
    } else {
      s[i] = 1.0 / sqrt(a);
    }
  }
}

// Row sums of |A| over the tile grid (for ||A||_inf): CTA (x, y) sums the
// rows x*256.. over tile column y (each thread one row, reading down the
// tile's columns: consecutive threads read consecutive addresses) and adds its
// partial sums into out (zeroed before the launch).
__global__ void row_abs_sum_kernel(const double *const *tiles, int n, int nb, int mt, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, tj = blockIdx.y;
  if (i >= n) return;
  const int t = i / nb, p = i - t * nb;
  const int rows = min(nb, n - t * nb), cols = min(nb, n - tj * nb);
  const double *a = tile_ptr(tiles, mt, t, tj) + p;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int c = 0;
  for (; c + 4 <= cols; c += 4) {
    s0 += fabs(a[(size_t)c * rows]);
    s1 += fabs(a[(size_t)(c + 1) * rows]);
    s2 += fabs(a[(size_t)(c + 2) * rows]);
    s3 += fabs(a[(size_t)(c + 3) * rows]);
  }
  for (; c < cols; c++) s0 += fabs(a[(size_t)c * rows]);
  atomicAdd(out + i, (s0 + s1) + (s2 + s3));
}

__host__ __device__ inline long long panel_base(long long r, long long n, long long nb) {
  return nb * (r * n - nb * r * (r - 1) / 2);
}

// Block column k of the factor (rows 0 .. (k+1) nb - 1), transposed: an
// nb x (k+1) nb matrix with leading dimension nb at Lp + lp_base(k).
__host__ __device__ inline long long lp_base(long long k, long long nb) {
  return nb * nb * (k * (k + 1) / 2);
}

// One block of a transposing three-slice split: dst(c, r) = slices of
// src(r, c) for a rows x cols block (src column-major lds, dst column-major
// ldd); every slice array is `stride` elements after the previous one.
struct TJob {
  long long src, dst;
  int rows, cols;
};

// 32 x 32 tiles through shared memory; blockIdx.z enumerates the jobs.
__global__ void tsplit3_kernel(const float *src, long long lds, __nv_bfloat16 *dst,
                               long long ldd, long long stride, const TJob *jobs) {
  __shared__ float t[32][33];
  const TJob jb = jobs[blockIdx.z];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  if (r0 >= jb.rows || c0 >= jb.cols) return;
  const float *S = src + jb.src;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int c = c0 + y, r = r0 + threadIdx.x;
    t[y][threadIdx.x] = (c < jb.cols && r < jb.rows) ? S[r + (long long)c * lds] : 0.f;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int r = r0 + y, c = c0 + threadIdx.x;  // dst(c, r)
    if (r >= jb.rows || c >= jb.cols) continue;
    const float x = t[threadIdx.x][y];
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    const __nv_bfloat16 m = __float2bfloat16_rn(r1);
    __nv_bfloat16 *D = dst + jb.dst + c + (long long)r * ldd;
    D[0] = h;
    D[stride] = m;
    D[2 * stride] = __float2bfloat16_rn(r1 - __bfloat162float(m));
  }
}

// W = float(S A S) on the upper row panels; the strict lower part of each
// diagonal block and the padding rows of a ragged last panel are zero.
__global__ void pack_kernel(const double *const *tiles, int n, int nb, int mt, const double *s,
                            float *W, double shift) {
  const int r = blockIdx.y;
  const long long w = n - (long long)r * nb;
  const long long total = (long long)nb * w;
  float *P = W + panel_base(r, n, nb);
  const int rows_r = min(nb, n - r * nb);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int p = (int)(e % nb);
    const long long c = e / nb;
    const long long i = (long long)r * nb + p, j = (long long)r * nb + c;
    float v = 0.f;
    if (p < rows_r && i <= j) {
      const int tj = (int)(j / nb), cj = (int)(j - (long long)tj * nb);
      const double a = tile_ptr(tiles, mt, r, tj)[p + (size_t)cj * rows_r];
      v = (float)(s[i] * a * s[j] + (i == j ? shift : 0.0));
    }
    P[e] = v;
  }
}

// FP64 retry of a failed FP32 diagonal-block factorization: one CTA, only
// when info_k is set.  The block from before the FP32 attempt is widened,
// factored right-looking in FP64 (lower form, L = U'), narrowed back.
__global__ void __launch_bounds__(1024) retry_potrf_kernel(int nbk, int ld, const float *backup,
                                                           double *L, float *diag, int *info_k,
                                                           int *status, int *retries, int offset,
                                                           int *retried_k) {
  if (*(volatile int *)info_k == 0 || *(volatile int *)status != 0) return;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < nbk * nbk; e += nt) {
    const int j = e % nbk, i = e / nbk;  // read backup(j, i) coalesced along j
    if (j <= i) L[i + (size_t)j * ld] = (double)backup[j + (size_t)i * ld];
  }
  __shared__ int fail;
  if (tid == 0) fail = -1;
  __syncthreads();
  for (int j = 0; j < nbk; j++) {
    double d = L[j + (size_t)j * ld];
    if (!(d > 0.0)) {
      if (tid == 0) fail = j;
      break;
    }
    d = sqrt(d);
    const double rcp = 1.0 / d;
    __syncthreads();
    for (int i = j + 1 + tid; i < nbk; i += nt) L[i + (size_t)j * ld] *= rcp;
    if (tid == 0) L[j + (size_t)j * ld] = d;
    __syncthreads();
    const int w = nbk - j - 1;
    for (long long e = tid; e < (long long)w * w; e += nt) {
      const int i = j + 1 + (int)(e % w), k = j + 1 + (int)(e / w);
      if (k <= i)
        L[i + (size_t)k * ld] = fma(-L[i + (size_t)j * ld], L[k + (size_t)j * ld], L[i + (size_t)k * ld]);
    }
    __syncthreads();
  }
  __syncthreads();
  if (fail >= 0) {
    if (tid == 0) atomicCAS(status, 0, offset + fail + 1);
    return;
  }
  for (int e = tid; e < nbk * nbk; e += nt) {
    const int j = e % nbk, i = e / nbk;
    if (j <= i) diag[j + (size_t)i * ld] = (float)L[i + (size_t)j * ld];
  }
  __syncthreads();
  if (tid == 0) {
    *info_k = 0;
    *retried_k = 1;
    atomicAdd(retries, 1);
  }
}

__global__ void absmax_kernel(const float *x, long long n, float *out, const int *a1, const int *a2) {
  if (aborted(a1, a2)) return;
  float m = 0.f;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[e]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax((int *)out, __float_as_int(m));  // m >= 0: int order
}

// Panel -> 16-bit operands.  FP16 panels are scaled by a power of two so the
// largest entry lands near 2^12; the trailing update's alpha is -1/scale^2.
template <bool FP16>
__global__ void convert_kernel(const float *src, long long n, int terms, void *hi_, void *lo_,
                               const float *pmax, float *alpha_out, const int *a1, const int *a2) {
  if (aborted(a1, a2)) return;
  float scale = 1.f;
  if (FP16) {
    const float m = *pmax;
    int e = 0;
    if (m > 0.f) frexpf(m, &e);  // m in [2^(e-1), 2^e)
    scale = ldexpf(1.f, 12 - e);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *alpha_out = -1.f / (scale * scale);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float x = src[i] * scale;
    if (FP16) {
      const __half h = __float2half_rn(x);
      ((__half *)hi_)[i] = h;
      if (terms == 3) ((__half *)lo_)[i] = __float2half_rn(x - __half2float(h));
    } else {
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      ((__nv_bfloat16 *)hi_)[i] = h;
      if (terms == 3) ((__nv_bfloat16 *)lo_)[i] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
  }
}

// x -> three BF16 slices (x = hi + mid + lo up to the rounding of lo): the
// operands of the FP32-accurate tensor-core product (tc_gemm terms 6).
// With rows > 0, `rows` of every `ld` source elements are converted (n in
// all) to the same positions with leading dimension ldd (default ld).
__global__ void split3_kernel(const float *src, long long n, __nv_bfloat16 *hi, __nv_bfloat16 *mid,
                              __nv_bfloat16 *lo, const int *a1, const int *a2, int rows = 0,
                              long long ld = 0, long long ldd = 0) {
  if (aborted(a1, a2)) return;
  if (ldd == 0) ldd = ld;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = rows ? (e % rows) + (e / rows) * ld : e;
    const long long o = rows ? (e % rows) + (e / rows) * ldd : e;
    const float x = src[i];
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    const __nv_bfloat16 m = __float2bfloat16_rn(r1);
    hi[o] = h;
    mid[o] = m;
    lo[o] = __float2bfloat16_rn(r1 - __bfloat162float(m));
  }
}

// Z = float(s .* R) and X += s .* double(Z), column by column.
__global__ void scale_to_f32_kernel(const double *R, long long ldr, const double *s, float *Z,
                                    long long ldz, int n, int r) {
  const long long total = (long long)n * r;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    Z[i + j * ldz] = (float)(s[i] * R[i + j * ldr]);
  }
}

__global__ void update_x_kernel(double *X, long long ldx, const double *s, const float *Z,
                                long long ldz, int n, int r) {
  const long long total = (long long)n * r;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    X[i + j * ldx] += s[i] * (double)Z[i + j * ldz];
  }
}

// out[j] = max_i |M(i, j)| (one CTA per column).
__global__ void colmax_kernel(const double *M, long long ld, int n, double *out) {
  const int j = blockIdx.x;
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(M[i + j * ld]));
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) out[j] = m;
  }
}

int grid_for(long long n) {
  long long b = (n + 255) / 256;
  long long cap = 8LL * dg_num_sms();
  return (int)std::max(1LL, std::min(b, cap));
}

}  // namespace

// ---------------------------------------------------------------------------
// factorization
// ---------------------------------------------------------------------------

// Step k's panel: the FP32 factor of the diagonal block and its inverse in
// one cooperative launch (mixed_diag.cu; an FP64 retry on a failed pivot,
// then the inverse of the retried factor), the inverse cut into three BF16
// slices (kept for the refinement's solves), the solve of the rest of the
// panel as the product Vinv_k' A(k, k+1:) on the tensor cores with
// FP32-accurate operands (3 BF16 slices, 6 products), and the result cut
// into the three slices the trailing updates and the solves read (FP16
// forms: also the scaled conversion into P buffer k % 2).
static int panel_step(dg_mixed *f, int k, cudaStream_t s) {
  const int n = f->n, nb = f->nb, mt = f->mt;
  int *status = f->words, *retries = f->words + 1, *ik = f->words + 3 + k;
  int *retried = f->words + 3 + mt + k;
  float *Pk = f->W + panel_base(k, n, nb);
  float *Vk = f->Vinv + (size_t)k * nb * nb;
  const int nbk = std::min(nb, n - k * nb);
  const long long T = (long long)n - (long long)(k + 1) * nb;
  DG_CUDA_TRY(cudaMemcpyAsync(f->diag_backup, Pk, sizeof(float) * (size_t)nb * nbk,
                              cudaMemcpyDeviceToDevice, s));
  DG_TRY(diag_chol_inv_f32(Pk, nb, nbk, Vk, nb, f->diag_scratch, ik, k * nb, status, nullptr, 0,
                           s));
  retry_potrf_kernel<<<1, 1024, 0, s>>>(nbk, nb, f->diag_backup, f->d64, Pk, ik, status, retries,
                                        k * nb, retried);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  DG_TRY(diag_chol_inv_f32(Pk, nb, nbk, Vk, nb, f->diag_scratch, ik, k * nb, status, retried, 1,
                           s));
  const size_t vn = (size_t)nb * nb;
  __nv_bfloat16 *v3 = f->V3 + (size_t)k * vn;
  split3_kernel<<<grid_for((long long)vn), 256, 0, s>>>(Vk, (long long)vn, v3, v3 + f->v3_stride,
                                                        v3 + 2 * f->v3_stride, ik, status);
  count_launches(1);
  if (T <= 0) return 0;
  float *Rk = Pk + (size_t)nb * nb;  // the rest of panel k: nb x T
  const size_t rn = (size_t)nb * T;
  {
    // Rk = Vk' Rk: both operands cut into three BF16 slices
    __nv_bfloat16 *r3 = (__nv_bfloat16 *)f->S3r;
    const size_t rcap = (size_t)nb * std::max(0, n - nb);
    split3_kernel<<<grid_for((long long)rn), 256, 0, s>>>(Rk, (long long)rn, r3, r3 + rcap,
                                                          r3 + 2 * rcap, ik, status);
    count_launches(1);
    DG_CUDA_TRY(cudaGetLastError());
    TcGemmArgs g;
    memset(&g, 0, sizeof g);
    g.m = nbk; g.n = (int)T; g.k = nbk; g.terms = 6;
    g.a_hi = v3; g.a_mid = v3 + f->v3_stride; g.a_lo = v3 + 2 * f->v3_stride;
    g.lda = nb; g.a_rows = nbk; g.a_row0 = 0;
    g.b_hi = r3; g.b_mid = r3 + rcap; g.b_lo = r3 + 2 * rcap;
    g.ldb = nb; g.b_rows = (int)T; g.b_row0 = 0;
    g.alpha = 1.f; g.beta = 0.f;
    g.c = Rk; g.ldc = nb; g.layout = 0; g.upper = 0;
    g.bn = 128; g.status = status;
    DG_TRY(tc_gemm_bf16(g, s));
  }
  {
    __nv_bfloat16 *o3 = f->R3 + (Rk - f->W);
    split3_kernel<<<grid_for((long long)rn), 256, 0, s>>>(Rk, (long long)rn, o3, o3 + f->r3_stride,
                                                          o3 + 2 * f->r3_stride, ik, status);
    count_launches(1);
  }
  if (f->precision == DG_PREC_FP8) {
    // E4M3 with a power-of-two scale per vector (column of the panel)
    const size_t tmax = (size_t)std::max(0, n - nb);
    DG_TRY(split_e4m3(Rk, nb, nbk, (int)T, f->P8 + (size_t)(k & 1) * tmax * nb, nb,
                      f->s8 + (size_t)(k & 1) * tmax, ik, status, s));
  }
  const bool fp16 = (f->precision == DG_PREC_FP16 || f->precision == DG_PREC_FP16X3);
  if (fp16) {
    const int terms = f->precision == DG_PREC_FP16X3 ? 3 : 1;
    const size_t half = (size_t)std::max(0LL, (long long)n - nb) * nb;  // elements per P buffer
    void *hi = (char *)f->P_hi + (size_t)(k & 1) * half * 2;
    void *lo = (char *)f->P_lo + (size_t)(k & 1) * half * 2;
    float *pmax = f->panel_max + k;
    float *alpha = f->alpha_dev + k;
    const long long elems = (long long)nb * T;
    DG_CUDA_TRY(cudaMemsetAsync(pmax, 0, sizeof(float), s));
    absmax_kernel<<<grid_for(elems), 256, 0, s>>>(Rk, elems, pmax, ik, status);
    convert_kernel<true><<<grid_for(elems), 256, 0, s>>>(Rk, elems, terms, hi, lo, pmax, alpha, ik,
                                                         status);
    count_launches(2);
  }
  DG_CUDA_TRY(cudaGetLastError());
  return 0;
}

// Step k's trailing update on the tensor cores of block rows r0 .. r1-1
// (r0 > k; their columns from r0 nb on: the upper part).  BF16 forms read
// the factor's slices of panel k (hi; hi + mid as the hi/lo pair of bf16x3;
// all three for bf16x6), FP16 forms the scaled P buffer, the FP8 form the
// E4M3 buffer and its per-vector scales.
static int trailing_rows(dg_mixed *f, int k, int r0, int r1, cudaStream_t s) {
  const int n = f->n, nb = f->nb;
  const long long T = (long long)n - (long long)(k + 1) * nb;
  const long long row0 = (long long)r0 * nb, row1 = std::min<long long>((long long)r1 * nb, n);
  if (T <= 0 || row1 <= row0) return 0;
  const bool fp16 = (f->precision == DG_PREC_FP16 || f->precision == DG_PREC_FP16X3);
  const int terms = f->precision == DG_PREC_BF16X6 ? 6
                  : (f->precision == DG_PREC_BF16X3 || f->precision == DG_PREC_FP16X3) ? 3 : 1;
  TcGemmArgs g;
  memset(&g, 0, sizeof g);
  g.m = (int)(row1 - row0); g.n = (int)(n - row0);
  g.a_row0 = g.b_row0 = (int)(row0 - (long long)(k + 1) * nb);
  g.off = row0;
  g.k = nb; g.terms = terms; g.fp16 = fp16;
  if (f->precision == DG_PREC_FP8) {
    const size_t tmax = (size_t)std::max(0, n - nb);
    g.fp8 = 1;
    g.a_hi = f->P8 + (size_t)(k & 1) * tmax * nb;
    g.a_scale = f->s8 + (size_t)(k & 1) * tmax;
    g.b_scale = g.a_scale;
  } else if (fp16) {
    const size_t half = (size_t)std::max(0LL, (long long)n - nb) * nb;
    g.a_hi = (char *)f->P_hi + (size_t)(k & 1) * half * 2;
    g.a_lo = (char *)f->P_lo + (size_t)(k & 1) * half * 2;
    g.alpha_dev = f->alpha_dev + k;
  } else {
    const __nv_bfloat16 *r3 = f->R3 + (panel_base(k, n, nb) + (long long)nb * nb);
    g.a_hi = r3;
    g.a_mid = r3 + f->r3_stride;
    g.a_lo = terms == 3 ? r3 + f->r3_stride : r3 + 2 * f->r3_stride;  // bf16x3: lo = mid slice
  }
  g.b_hi = g.a_hi; g.b_lo = g.a_lo; g.b_mid = g.a_mid;
  g.lda = nb; g.ldb = nb; g.a_rows = (int)T; g.b_rows = (int)T;
  g.alpha = -1.f; g.beta = 1.f;
  g.c = f->W; g.layout = 1; g.upper = 1;
  g.nb = nb; g.ntot = n;
  g.bn = 256; g.status = f->words;
  // CTAs of the bulk update finish every few tiles, so the critical chain's
  // launches on the high-priority stream get SMs without waiting for it
  g.tiles_per_cta = 8;
  return tc_gemm_bf16(g, s);
}

static int trailing_tc(dg_mixed *f, int k, bool next, cudaStream_t s) {
  return next ? trailing_rows(f, k, k + 1, k + 2, s) : trailing_rows(f, k, k + 2, f->mt, s);
}

// Step k's trailing update on the FP32 CUDA-core GEMM, one call per row panel.
static int trailing_f32(dg_mixed *f, int k, cudaStream_t s) {
  const int n = f->n, nb = f->nb, mt = f->mt;
  float *Pk = f->W + panel_base(k, n, nb);
  const int nbk = std::min(nb, n - k * nb);
  const float *Rk = Pk + (size_t)nb * nb;
  for (int r = k + 1; r < mt; r++) {
    float *Pr = f->W + panel_base(r, n, nb);
    const int nbr = std::min(nb, n - r * nb);
    const long long wr = (long long)n - (long long)r * nb;
    const float *Ar = Rk + (size_t)(r - k - 1) * nb * nb;  // columns r*nb.. of panel k
    DG_TRY(gemm_f32('T', 'N', nbr, (int)wr, nbk, -1.f, Ar, nb, Ar, nb, 1.f, Pr, nb, TRI_UPPER,
                    f->words + 3 + k, s, f->words));
  }
  return 0;
}

// The status words, the diagonal scaling and the packed FP32 copy S A S.
int mixed_prepare(dg_mixed *f, cudaStream_t s) {
  const int n = f->n, nb = f->nb, mt = f->mt;
  int *bad = f->words + 2;
  DG_CUDA_TRY(cudaMemsetAsync(f->words, 0, sizeof(int) * (3 + 2 * mt), s));
  DG_CUDA_TRY(cudaMemsetAsync(bad, 0x7f, sizeof(int), s));
  diag_scale_kernel<<<grid_for(n), 256, 0, s>>>(f->tiles_dev, n, nb, mt, f->s, bad);
  pack_kernel<<<dim3(std::max(1, std::min(1024, (int)((long long)nb * n / 256 + 1))), mt), 256, 0,
                s>>>(f->tiles_dev, n, nb, mt, f->s, f->W, f->shift);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(2);
  return 0;
}

// The BF16 forms' schedule, whose trailing operands are the per-panel slices
// (no buffer is reused across steps).  Step k's update of block rows k+2,
// k+3 and k+4 are launches of their own, on streams whose priority follows
// how soon the chain needs the row (just below the chain's); the rows past
// them are kFar launches of consecutive rows at the least priority.  Each
// launch waits for panel k and for the previous update of its rows (an event
// per block row), so a near row never waits for the bulk of its own step and
// the bulk of step k overlaps that of step k-1.  The critical chain on
// `aux` (greatest priority) waits only for block row k+1's last update,
// updates it by panel k and factors panel k+1; through the near rows it
// depends on the bulk launch of three steps earlier.  (One launch per row
// and step, about 30 per step at N = 32768, kept the chain's own launches
// waiting about 1.3 ms per step behind the launches released by the same
// panel; one launch for all rows made the chain wait for the whole bulk, and
// one launch for all far rows serialised the bulk updates of successive steps:
// 8 % slower at N = 65536 with six products.)
static int factor_by_rows(dg_mixed *f, cudaStream_t s) {
  const int mt = f->mt;
  if (!f->far_s[0]) {
    int least = 0, greatest = 0;
    DG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    for (int d = 0; d < dg_mixed::kNear; d++)
      DG_CUDA_TRY(cudaStreamCreateWithPriority(&f->near_s[d], cudaStreamNonBlocking,
                                               std::min(least, greatest + 1 + d)));
    for (int q = 0; q < dg_mixed::kFar; q++)
      DG_CUDA_TRY(cudaStreamCreateWithPriority(&f->far_s[q], cudaStreamNonBlocking, least));
  }
  while ((int)f->ev_row.size() < mt) {
    cudaEvent_t e = nullptr;
    DG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    f->ev_row.push_back(e);
  }
  std::vector<char> recorded(mt, 0);
  for (int k = 0; k + 1 < mt; k++) {
    // ev_panel marks panel k here (panel 0: after the packed copy on s)
    const int far0 = k + 2 + dg_mixed::kNear;
    for (int r = k + 2; r < std::min(far0, mt); r++) {
      cudaStream_t rs = f->near_s[r - k - 2];
      DG_CUDA_TRY(cudaStreamWaitEvent(rs, f->ev_panel, 0));
      if (recorded[r]) DG_CUDA_TRY(cudaStreamWaitEvent(rs, f->ev_row[r], 0));
      DG_TRY(trailing_rows(f, k, r, r + 1, rs));
      DG_CUDA_TRY(cudaEventRecord(f->ev_row[r], rs));
      recorded[r] = 1;
    }
    const int nfar = mt - far0;
    for (int q = 0; q < dg_mixed::kFar && nfar > 0; q++) {
      const int r0 = far0 + (int)((long long)nfar * q / dg_mixed::kFar);
      const int r1 = far0 + (int)((long long)nfar * (q + 1) / dg_mixed::kFar);
      if (r1 <= r0) continue;
      cudaStream_t rs = f->far_s[q];
      DG_CUDA_TRY(cudaStreamWaitEvent(rs, f->ev_panel, 0));
      for (int r = r0; r < r1; r++)
        if (recorded[r]) DG_CUDA_TRY(cudaStreamWaitEvent(rs, f->ev_row[r], 0));
      DG_TRY(trailing_rows(f, k, r0, r1, rs));
      for (int r = r0; r < r1; r++) {
        DG_CUDA_TRY(cudaEventRecord(f->ev_row[r], rs));
        recorded[r] = 1;
      }
    }
    if (recorded[k + 1]) DG_CUDA_TRY(cudaStreamWaitEvent(f->aux, f->ev_row[k + 1], 0));
    DG_TRY(trailing_rows(f, k, k + 1, k + 2, f->aux));
    DG_TRY(panel_step(f, k + 1, f->aux));
    DG_CUDA_TRY(cudaEventRecord(f->ev_panel, f->aux));
    if (f->ev_gate && k + 1 == mt / 2) DG_CUDA_TRY(cudaEventRecord(f->ev_gate, f->aux));
  }
  // the caller's stream resumes after every row's last update and the chain
  for (int r = 2; r < mt; r++)
    if (recorded[r]) DG_CUDA_TRY(cudaStreamWaitEvent(s, f->ev_row[r], 0));
  DG_CUDA_TRY(cudaStreamWaitEvent(s, f->ev_panel, 0));
  return 0;
}

// The blocked factorization of the packed copy (after mixed_prepare).
int mixed_factor_run(dg_mixed *f, cudaStream_t s) {
  const bool tensor = f->precision != DG_PREC_FP32;
  DG_TRY(panel_step(f, 0, s));
  if (!tensor) {
    for (int k = 0; k + 1 < f->mt; k++) {
      DG_TRY(trailing_f32(f, k, s));
      DG_TRY(panel_step(f, k + 1, s));
    }
    return 0;
  }
  // One-step lookahead.  The critical chain runs on the auxiliary stream at
  // the device's greatest priority: the update of block row k+1 by panel k
  // (`next`, which waits for the previous step's bulk update of the rows
  // below it), then panel k+1.  The bulk update of the rows below (`rest`)
  // runs on `s` beside it and waits only for panel k.  Block rows written by
  // two launches are always ordered: row k+1 by rest(k-1) before next(k).
  if (!f->aux) {
    int least = 0, greatest = 0;
    DG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    DG_CUDA_TRY(cudaStreamCreateWithPriority(&f->aux, cudaStreamNonBlocking, greatest));
  }
  if (!f->ev_next) DG_CUDA_TRY(cudaEventCreateWithFlags(&f->ev_next, cudaEventDisableTiming));
  if (!f->ev_panel) DG_CUDA_TRY(cudaEventCreateWithFlags(&f->ev_panel, cudaEventDisableTiming));
  DG_CUDA_TRY(cudaEventRecord(f->ev_panel, s));  // panel 0
  DG_CUDA_TRY(cudaStreamWaitEvent(f->aux, f->ev_panel, 0));
  const bool slices = f->precision == DG_PREC_BF16 || f->precision == DG_PREC_BF16X3 ||
                      f->precision == DG_PREC_BF16X6;
  if (slices) return factor_by_rows(f, s);
  for (int k = 0; k + 1 < f->mt; k++) {
    if (k > 0) DG_CUDA_TRY(cudaStreamWaitEvent(f->aux, f->ev_next, 0));  // rest(k-1)
    DG_TRY(trailing_tc(f, k, /*next=*/true, f->aux));
    DG_TRY(panel_step(f, k + 1, f->aux));
    DG_CUDA_TRY(cudaEventRecord(f->ev_panel, f->aux));
    DG_TRY(trailing_tc(f, k, /*next=*/false, s));
    DG_CUDA_TRY(cudaEventRecord(f->ev_next, s));
    DG_CUDA_TRY(cudaStreamWaitEvent(s, f->ev_panel, 0));  // panel k+1 before rest(k+1)
  }
  return 0;
}


// One FP32-accurate product on the tensor cores for the triangular solves:
// C (m x r, ldc) = alpha A' Zb + beta C with A given by its three slices
// (K-major, lda, stride apart) and Zb the k x r FP32 block at Zsrc (ldz), cut
// into slices in zs (3 k x r, ld nb) first.
static int tc6(const dg_mixed *f, int m, int r, int k, const __nv_bfloat16 *a3, long long astride,
               int lda, const float *Zsrc, long long ldz, __nv_bfloat16 *zs, float alpha,
               float beta, float *C, long long ldc, cudaStream_t s) {
  const int nb = f->nb;
  const size_t zn = (size_t)nb * r;
  const long long e = (long long)k * r;
  split3_kernel<<<grid_for(e), 256, 0, s>>>(Zsrc, e, zs, zs + zn, zs + 2 * zn, nullptr, nullptr,
                                            k, ldz, nb);
  count_launches(1);
  TcGemmArgs g;
  memset(&g, 0, sizeof g);
  g.m = m; g.n = r; g.k = k; g.terms = 6;
  g.a_hi = a3; g.a_mid = a3 + astride; g.a_lo = a3 + 2 * astride;
  g.lda = lda; g.a_rows = m; g.a_row0 = 0;
  g.b_hi = zs; g.b_mid = zs + zn; g.b_lo = zs + 2 * zn;
  g.ldb = nb; g.b_rows = r; g.b_row0 = 0;
  g.alpha = alpha; g.beta = beta;
  g.c = C; g.ldc = ldc; g.layout = 0; g.upper = 0;
  g.bn = 128; g.status = nullptr;
  return tc_gemm_bf16(g, s);
}

// Solves U~' U~ Z = Z (FP32, n x r, column-major ldz) with the factor's
// slices on the tensor cores (FP32-accurate products), Z2 (same shape) the
// second buffer: forward Z2_k = Vinv_k' Z_k and Z_(k+1:) -= U~_(k,k+1:)' Z2_k;
// backward, right-looking, Z_k = Vinv_k Z2_k and Z2_(0:k) -= U~_(0:k, k) Z_k
// as one tall product with the transposed block column.  zs: 3 nb r BF16
// (the right-hand block's slices).  The result is in Z.
static int tri_solve_passes(const dg_mixed *f, float *Z, float *Z2, long long ldz, int r,
                            __nv_bfloat16 *zs, cudaStream_t s) {
  const int n = f->n, nb = f->nb, mt = f->mt;
  for (int k = 0; k < mt; k++) {
    const int nbk = std::min(nb, n - k * nb);
    const long long T = (long long)n - (long long)(k + 1) * nb;
    DG_TRY(tc6(f, nbk, r, nbk, f->V3 + (size_t)k * nb * nb, f->v3_stride, nb,
               Z + (size_t)k * nb, ldz, zs, 1.f, 0.f, Z2 + (size_t)k * nb, ldz, s));
    if (T > 0)
      DG_TRY(tc6(f, (int)T, r, nbk, f->R3 + (panel_base(k, n, nb) + (long long)nb * nb),
                 f->r3_stride, nb, Z2 + (size_t)k * nb, ldz, zs, -1.f, 1.f,
                 Z + (size_t)(k + 1) * nb, ldz, s));
  }
  for (int k = mt - 1; k >= 0; k--) {
    const int nbk = std::min(nb, n - k * nb);
    DG_TRY(tc6(f, nbk, r, nbk, f->VT3 + (size_t)k * nb * nb, f->v3_stride, nb,
               Z2 + (size_t)k * nb, ldz, zs, 1.f, 0.f, Z + (size_t)k * nb, ldz, s));
    if (k > 0)
      DG_TRY(tc6(f, k * nb, r, nbk, f->L3 + lp_base(k, nb), f->l3_stride, nb,
                 Z + (size_t)k * nb, ldz, zs, -1.f, 1.f, Z2, ldz, s));
  }
  return 0;
}

int mixed_tri_solve(const dg_mixed *f, float *Z, float *Z2, long long ldz, int r, cudaStream_t s) {
  __nv_bfloat16 *zs = nullptr;
  DG_CUDA_TRY(dg::pool_malloc_async((void **)&zs, sizeof(__nv_bfloat16) * 3 * (size_t)f->nb * r, s));
  const int rc = tri_solve_passes(f, Z, Z2, ldz, r, zs, s);
  cudaFreeAsync(zs, s);
  return rc;
}

// After the factorization: the slices of every Vinv_k' (VT3) and of the
// factor's block columns transposed (L3, the blocks (j, k), j < k), in one
// transposing split launch over a job table.
int mixed_transpose_columns(dg_mixed *f, cudaStream_t s) {
  const int mt = f->mt, nb = f->nb, n = f->n;
  std::vector<TJob> jv, jl;
  for (int k = 0; k < mt; k++) {
    const int nbk = std::min(nb, n - k * nb);
    jv.push_back({(long long)k * nb * nb, (long long)k * nb * nb, nbk, nbk});
    for (int j = 0; j < k; j++)  // U(j, k): nb x nbk at W (ld nb) -> Lp_k block j (nbk x nb)
      jl.push_back({panel_base(j, n, nb) + (long long)(k - j) * nb * nb,
                    lp_base(k, nb) + (long long)j * nb * nb, nb, nbk});
  }
  TJob *dj = nullptr;
  const size_t nj = jv.size() + jl.size();
  DG_CUDA_TRY(dg::pool_malloc_async((void **)&dj, sizeof(TJob) * nj, s));
  DG_CUDA_TRY(cudaMemcpyAsync(dj, jv.data(), sizeof(TJob) * jv.size(), cudaMemcpyHostToDevice, s));
  if (!jl.empty())
    DG_CUDA_TRY(cudaMemcpyAsync(dj + jv.size(), jl.data(), sizeof(TJob) * jl.size(),
                                cudaMemcpyHostToDevice, s));
  const dim3 blk(32, 8), g1((nb + 31) / 32, (nb + 31) / 32, (unsigned)jv.size());
  tsplit3_kernel<<<g1, blk, 0, s>>>(f->Vinv, nb, f->VT3, nb, f->v3_stride, dj);
  count_launches(1);
  if (!jl.empty()) {
    const dim3 g2((nb + 31) / 32, (nb + 31) / 32, (unsigned)jl.size());
    tsplit3_kernel<<<g2, blk, 0, s>>>(f->W, nb, f->L3, nb, f->l3_stride, dj + jv.size());
    count_launches(1);
  }
  DG_CUDA_TRY(cudaGetLastError());
  cudaFreeAsync(dj, s);  // (copies from pageable memory are staged before the calls return)
  return 0;
}

}  // namespace dg

using dg::grid_for;

extern "C" int dg_mixed_factor_ex(dg_mixed **out, int n, int nb, double *const *tiles,
                                  int precision, double shift, void *stream);

extern "C" int dg_mixed_factor(dg_mixed **out, int n, int nb, double *const *tiles, int precision,
                               void *stream) {
  return dg_mixed_factor_ex(out, n, nb, tiles, precision, 0.0, stream);
}

extern "C" int dg_mixed_factor_ex(dg_mixed **out, int n, int nb, double *const *tiles,
                                  int precision, double shift, void *stream) {
  DG_CHECK_ARG(out != nullptr, 1);
  DG_CHECK_ARG(n > 0, 2);
  DG_CHECK_ARG(nb >= 64 && nb % 64 == 0, 3);
  DG_CHECK_ARG(tiles != nullptr, 4);
  DG_CHECK_ARG(precision == DG_PREC_BF16 || precision == DG_PREC_BF16X3 ||
                   precision == DG_PREC_FP16 || precision == DG_PREC_FP16X3 ||
                   precision == DG_PREC_FP32 || precision == DG_PREC_BF16X6 ||
                   precision == DG_PREC_FP8,
               5);
  DG_CHECK_ARG(shift >= 0.0, 6);
  cudaStream_t s = (cudaStream_t)stream;
  dg_mixed *f = new dg_mixed();
  f->n = n; f->nb = nb; f->mt = (n + nb - 1) / nb; f->precision = precision;
  f->shift = shift;
  cudaGetDevice(&f->dev);
  const int mt = f->mt;
  const long long wsize = dg::panel_base(mt, n, nb) + (long long)nb * nb;
  const long long tmax = std::max(0LL, (long long)n - nb);
  auto fail = [&](int rc) {
    dg_mixed_destroy(f);
    return rc;
  };
  const bool fp16 = (precision == DG_PREC_FP16 || precision == DG_PREC_FP16X3);
  const bool fp8 = precision == DG_PREC_FP8;
  f->r3_stride = wsize;
  f->v3_stride = (long long)mt * nb * nb;
  f->l3_stride = std::max(1LL, dg::lp_base(mt, nb));
  struct Alloc { void **p; size_t bytes; };
  Alloc allocs[] = {
      {(void **)&f->W, sizeof(float) * (size_t)wsize},
      {(void **)&f->s, sizeof(double) * (size_t)n},
      {(void **)&f->tiles_dev, sizeof(double *) * (size_t)mt * mt},
      {(void **)&f->P_hi, fp16 ? 2 * 2 * (size_t)std::max(1LL, tmax) * nb : (size_t)256},
      {(void **)&f->P_lo, fp16 ? 2 * 2 * (size_t)std::max(1LL, tmax) * nb : (size_t)256},
      {(void **)&f->P8, fp8 ? 2 * (size_t)std::max(1LL, tmax) * nb : (size_t)256},
      {(void **)&f->s8, fp8 ? 2 * sizeof(float) * (size_t)std::max(1LL, tmax) : (size_t)256},
      {(void **)&f->diag_backup, sizeof(float) * (size_t)nb * nb},
      {(void **)&f->d64, sizeof(double) * (size_t)nb * nb},
      {(void **)&f->panel_max, sizeof(float) * (size_t)mt},
      {(void **)&f->alpha_dev, sizeof(float) * (size_t)mt},
      {(void **)&f->words, sizeof(int) * (size_t)(3 + 2 * mt)},
      {(void **)&f->Vinv, sizeof(float) * (size_t)mt * nb * nb},
      {(void **)&f->diag_scratch, dg::diag_chol_inv_scratch_bytes()},
      {(void **)&f->S3r, 3 * 2 * (size_t)std::max(1LL, tmax) * nb},
      {(void **)&f->R3, 3 * 2 * (size_t)f->r3_stride},
      {(void **)&f->V3, 3 * 2 * (size_t)f->v3_stride},
      {(void **)&f->VT3, 3 * 2 * (size_t)f->v3_stride},
      {(void **)&f->L3, 3 * 2 * (size_t)f->l3_stride},
  };
  f->stream = s;
  for (auto &a : allocs) {
    if (dg::pool_malloc_async(a.p, a.bytes, s) != cudaSuccess) {
      cudaGetLastError();
      dg_set_last_error(__FILE__, __LINE__, "device allocation for the mixed factor failed");
      return fail(DG_ERR_NOMEM);
    }
    f->bytes += a.bytes;
  }
  if (cudaMemcpyAsync(f->tiles_dev, tiles, sizeof(double *) * (size_t)mt * mt,
                      cudaMemcpyHostToDevice, s) != cudaSuccess)
    return fail(DG_ERR_CUDA);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  // the scaled FP32 copy first, on s: the factorization starts from it
  int rc = dg::mixed_prepare(f, s);
  if (rc) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return fail(rc);
  }
  // ||A||_inf (for the backward errors of the solve) and, with the emulated
  // FP64 engine, A's rows cut into the BF16 slices of the refinement's
  // emulated residual: both depend on A alone, so they run on a
  // low-priority stream beside the factorization, after the copy above
  // (which also reads A); ev_oz marks their completion.
  double *rows = nullptr, *dmax = nullptr;
  if (dg::pool_malloc_async((void **)&rows, sizeof(double) * (n + 1), s) != cudaSuccess) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return fail(DG_ERR_NOMEM);
  }
  dmax = rows + n;
  const bool oz = dg::get_f64_engine() == 2 && n <= 131072;
  const long long ldk = ((long long)n + 7) / 8 * 8;
  const size_t ba = 16 * (size_t)ldk * n;
  if (oz && dg::pool_malloc_async(&f->ozA, ba + 8 * (size_t)n, s) != cudaSuccess) {
    cudaGetLastError();  // no room: the solve cuts its own slices or uses the FP64 pipe
    f->ozA = nullptr;
  }
  {
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    cudaEvent_t ready;
    if (cudaStreamCreateWithPriority(&f->aux2, cudaStreamNonBlocking, least) != cudaSuccess ||
        cudaEventCreateWithFlags(&f->ev_oz, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&f->ev_gate, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      cudaFreeAsync(rows, s);
      return fail(DG_ERR_CUDA);
    }
    cudaEventRecord(ready, s);  // tile pointers, buffers and the copy of A are in place
    cudaStreamWaitEvent(f->aux2, ready, 0);
    cudaEventDestroy(ready);
  }
  // The factorization is queued first: the BF16 schedule records ev_gate at
  // mid-factorization, and the slicing of A on aux2 waits for it (for the
  // other schedules the event is never recorded and the wait is empty).
  if (!rc) rc = dg::mixed_factor_run(f, s);
  if (!rc) {
    cudaStreamWaitEvent(f->aux2, f->ev_gate, 0);
    cudaMemsetAsync(rows, 0, sizeof(double) * n, f->aux2);
    dg::row_abs_sum_kernel<<<dim3((n + 255) / 256, mt), 256, 0, f->aux2>>>(f->tiles_dev, n, nb, mt,
                                                                          rows);
    dg::colmax_kernel<<<1, 1024, 0, f->aux2>>>(rows, n, n, dmax);
    dg::count_launches(2);
    if (f->ozA) {
      f->oz_ldk = ldk;
      f->ozAs = (unsigned long long *)((char *)f->ozA + ba);
      f->bytes += ba + 8 * (size_t)n;
      rc = dg::oz_split_tile_rows((const double *const *)f->tiles_dev, n, nb, f->ozA, ldk,
                                  f->ozAs, nullptr, f->aux2);
    }
  }
  cudaEventRecord(f->ev_oz, f->aux2);
  if (!rc) rc = dg::mixed_transpose_columns(f, s);
  cudaEventRecord(e1, s);
  cudaStreamWaitEvent(s, f->ev_oz, 0);  // ||A||_inf is read below
  if (rc) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(rows, s);
    return fail(rc);
  }
  // the host reads ||A||_inf and the status words once, after the factorization
  int words[3];
  if (cudaMemcpyAsync(words, f->words, sizeof(words), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&f->normA, dmax, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(rows, s);
    return fail(DG_ERR_CUDA);
  }
  cudaFreeAsync(rows, s);
  cudaEventElapsedTime(&f->factor_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  f->retries = words[1];
  int info = words[0];
  if (words[2] != 0x7f7f7f7f && words[2] > 0) info = words[2];  // non-positive diagonal
  f->info = info;
  *out = f;
  if (info < 0) {
    dg_set_last_error(__FILE__, __LINE__, "a bounded device wait timed out in the trailing update");
    return info;
  }
  return info;
}

extern "C" void dg_mixed_destroy(dg_mixed *f) {
  if (!f) return;
  // the slices of A are cut on aux2: the frees below wait for them
  if (f->ev_oz && f->stream) cudaStreamWaitEvent(f->stream, f->ev_oz, 0);
  void *ps[] = {f->W, f->s, f->tiles_dev, f->P_hi, f->P_lo, f->P8, f->s8, f->diag_backup, f->d64,
                f->panel_max, f->alpha_dev, f->words, f->Vinv, f->diag_scratch, f->S3r,
                f->R3, f->V3, f->VT3, f->L3, f->ozA};
  for (void *p : ps)
    if (p) cudaFreeAsync(p, f->stream);  // stream-ordered: no device-wide synchronisation
  if (f->ev_next) cudaEventDestroy(f->ev_next);
  if (f->ev_panel) cudaEventDestroy(f->ev_panel);
  for (cudaEvent_t e : f->ev_row)
    if (e) cudaEventDestroy(e);
  for (cudaStream_t q : f->near_s)
    if (q) cudaStreamDestroy(q);
  for (cudaStream_t q : f->far_s)
    if (q) cudaStreamDestroy(q);
  if (f->ev_oz) cudaEventDestroy(f->ev_oz);
  if (f->ev_gate) cudaEventDestroy(f->ev_gate);
  if (f->aux) cudaStreamDestroy(f->aux);
  if (f->aux2) cudaStreamDestroy(f->aux2);
  delete f;
}

extern "C" int dg_mixed_info(const dg_mixed *f, dg_mixed_stats *st) {
  DG_CHECK_ARG(f != nullptr, 1);
  DG_CHECK_ARG(st != nullptr, 2);
  st->n = f->n;
  st->nb = f->nb;
  st->precision = f->precision;
  st->info = f->info;
  st->retries = f->retries;
  st->factor_ms = f->factor_ms;
  st->norm_inf = f->normA;
  st->device_bytes = (long long)f->bytes;
  st->shift = f->shift;
  return 0;
}

// ---------------------------------------------------------------------------
// refinement
// ---------------------------------------------------------------------------
namespace {

struct Work {
  double *R = nullptr, *V = nullptr;  // residual; GMRES basis
  float *Z = nullptr;
  double *cm = nullptr;               // column maxima scratch (3 r)
};

int correction(const dg_mixed *f, const double *R, long long ldr, double *X, long long ldx,
               float *Z, int r, cudaStream_t s) {
  const int n = f->n;
  dg::scale_to_f32_kernel<<<grid_for((long long)n * r), 256, 0, s>>>(R, ldr, f->s, Z, n, n, r);
  dg::count_launches(1);
  DG_TRY(dg::mixed_tri_solve(f, Z, Z + (size_t)n * r, n, r, s));
  dg::update_x_kernel<<<grid_for((long long)n * r), 256, 0, s>>>(X, ldx, f->s, Z, n, n, r);
  dg::count_launches(1);
  DG_CUDA_TRY(cudaGetLastError());
  return 0;
}

// With the emulated FP64 engine the residual's product runs on the tensor
// cores: the rows of A (the caller's tile grid) are cut into BF16 slices once
// per solve, X's columns every iteration, and R = B - A X is one emulated GEMM
// with K = n and FP64 accuracy.
struct OzResidual {
  void *a = nullptr, *x = nullptr;          // slices of A's rows / X's columns
  unsigned long long *as = nullptr, *xs = nullptr;
  long long ldk = 0;
};

// R = B - A X (FP64, A from the caller's tiles)
int residual(const dg_mixed *f, const double *B, long long ldb, const double *X, long long ldx,
             double *R, int r, cudaStream_t s, const OzResidual *oz) {
  const int n = f->n;
  DG_CUDA_TRY(cudaMemcpy2DAsync(R, sizeof(double) * n, B, sizeof(double) * ldb,
                                sizeof(double) * n, r, cudaMemcpyDeviceToDevice, s));
  if (oz && oz->a) {
    DG_TRY(dg::oz_split(X, ldx, 1, n, r, oz->x, oz->ldk, oz->ldk * r, oz->xs, nullptr, s));
    return dg::oz_gemm(n, r, n, -1.0, oz->a, oz->ldk, oz->ldk * n, oz->as, oz->x, oz->ldk,
                       oz->ldk * r, oz->xs, 1.0, R, n, 0, nullptr, s);
  }
  return dg::gemm_tiles_f64(n, f->nb, r, -1.0, (const double *const *)f->tiles_dev, X, ldx, 1.0, R,
                            n, nullptr, s);
}

int backward_errors(const dg_mixed *f, const double *B, long long ldb, const double *X,
                    long long ldx, const double *R, int r, double *cm, std::vector<double> &berr,
                    cudaStream_t s) {
  const int n = f->n;
  dg::colmax_kernel<<<r, 256, 0, s>>>(R, n, n, cm);
  dg::colmax_kernel<<<r, 256, 0, s>>>(X, ldx, n, cm + r);
  dg::colmax_kernel<<<r, 256, 0, s>>>(B, ldb, n, cm + 2 * r);
  dg::count_launches(3);
  std::vector<double> h(3 * (size_t)r);
  DG_CUDA_TRY(cudaMemcpyAsync(h.data(), cm, sizeof(double) * 3 * r, cudaMemcpyDeviceToHost, s));
  DG_CUDA_TRY(cudaStreamSynchronize(s));
  berr.resize(r);
  for (int j = 0; j < r; j++) {
    const double den = f->normA * h[r + j] + h[2 * r + j];
    berr[j] = den > 0 ? h[j] / den : (h[j] == 0 ? 0.0 : INFINITY);
  }
  return 0;
}

// ---- small batched vector kernels for GMRES (one column per CTA) ----
__global__ void dots_kernel(const double *U, long long ldu, const double *V, long long ldv, int n,
                            double *out) {
  const int j = blockIdx.x;
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += U[i + j * ldu] * V[i + j * ldv];
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) out[j] = acc;
  }
}

// out[i r + j] = V_i(:, j) . W(:, j) for the kk basis blocks V_i (stride vs):
// CTA (j, i).  The classical Gram-Schmidt projections of one GMRES step.
__global__ void multi_dots_kernel(const double *V, long long vs, const double *W, int n, int r,
                                  double *out) {
  const int j = blockIdx.x, i = blockIdx.y;
  const double *v = V + vs * i + (size_t)j * n, *w = W + (size_t)j * n;
  double acc = 0.0;
  for (int e = threadIdx.x; e < n; e += blockDim.x) acc = fma(v[e], w[e], acc);
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) out[(size_t)i * r + j] = acc;
  }
}

// W(:, j) -= sum_i h[i r + j] V_i(:, j), i < kk.
__global__ void multi_axpy_kernel(const double *V, long long vs, int kk, double *W, int n, int r,
                                  const double *h) {
  const long long total = (long long)n * r;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e / n);
    double acc = W[e];
    for (int i = 0; i < kk; i++) acc = fma(-h[(size_t)i * r + j], V[vs * i + e], acc);
    W[e] = acc;
  }
}

// V(:, j) = a[j] * U(:, j) + b[j] * V(:, j)   (coefficients from device memory)
__global__ void axpby_kernel(const double *U, long long ldu, double *V, long long ldv, int n, int r,
                             const double *a, const double *b, int neg_a) {
  const long long total = (long long)n * r;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    const double aj = neg_a ? -a[j] : a[j];
    const double bj = b ? b[j] : 1.0;
    V[i + j * ldv] = aj * U[i + j * ldu] + bj * V[i + j * ldv];
  }
}

__global__ void inv_kernel(const double *x, double *y, int r) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < r) y[j] = x[j] > 0 ? 1.0 / sqrt(x[j]) : 0.0;
}

// z = M^-1 y for FP64 y (M = the low-precision factor of A, with the scaling)
int precond(const dg_mixed *f, const double *Y, double *Zo, float *Z32, int r, cudaStream_t s) {
  const int n = f->n;
  DG_CUDA_TRY(cudaMemsetAsync(Zo, 0, sizeof(double) * (size_t)n * r, s));
  return correction(f, Y, n, Zo, n, Z32, r, s);
}

// Restarted GMRES(m) on A d = r0 (FP64), left preconditioned by the factor,
// each column an independent Krylov space.  x += d.  Returns iterations.
// Y = A V (FP64, n x r, ld n): the emulated product from A's slices when
// they exist, else the FP64 tile GEMM.
int matvec(const dg_mixed *f, const double *V, double *Y, int r, cudaStream_t s,
           const OzResidual *oz) {
  const int n = f->n;
  if (oz && oz->a) {
    DG_TRY(dg::oz_split(V, n, 1, n, r, oz->x, oz->ldk, oz->ldk * r, oz->xs, nullptr, s));
    return dg::oz_gemm(n, r, n, 1.0, oz->a, oz->ldk, oz->ldk * n, oz->as, oz->x, oz->ldk,
                       oz->ldk * r, oz->xs, 0.0, Y, n, 0, nullptr, s);
  }
  return dg::gemm_tiles_f64(n, f->nb, r, 1.0, (const double *const *)f->tiles_dev, V, n, 0.0, Y, n,
                            nullptr, s);
}

int gmres_ir(const dg_mixed *f, const double *R0, double *X, long long ldx, int r, int m,
             int max_iters, double inner_tol, cudaStream_t s, int *iters_out, const OzResidual *oz) {
  const int n = f->n;
  const size_t col = (size_t)n;
  double *V = nullptr, *W = nullptr, *D = nullptr, *sc = nullptr;
  float *Z32 = nullptr;
  if (dg::pool_malloc_async((void **)&V, sizeof(double) * col * r * (m + 1), s) != cudaSuccess ||
      dg::pool_malloc_async((void **)&W, sizeof(double) * col * r * 2, s) != cudaSuccess ||
      dg::pool_malloc_async((void **)&D, sizeof(double) * col * r, s) != cudaSuccess ||
      dg::pool_malloc_async((void **)&sc, sizeof(double) * r * (m + 4), s) != cudaSuccess ||
      dg::pool_malloc_async((void **)&Z32, sizeof(float) * col * r * 2, s) != cudaSuccess) {
    cudaGetLastError();
    return DG_ERR_NOMEM;
  }
  double *T = W + col * r;  // second scratch block
  double *hb = nullptr;      // the Gram-Schmidt coefficients, 2 (m + 1) r
  if (dg::pool_malloc_async((void **)&hb, sizeof(double) * 2 * (size_t)(m + 1) * r, s) !=
      cudaSuccess) {
    cudaGetLastError();
    cudaFreeAsync(V, s);
    cudaFreeAsync(W, s);
    cudaFreeAsync(D, s);
    cudaFreeAsync(sc, s);
    cudaFreeAsync(Z32, s);
    return DG_ERR_NOMEM;
  }
  std::vector<double> hh;
  auto Vk = [&](int k) { return V + col * r * k; };
  std::vector<double> H((size_t)(m + 1) * m * r), g((size_t)(m + 1) * r), hcol(r), cs(m * r), sn(m * r);
  int total_it = 0;
  int rc = 0;
  DG_CUDA_TRY(cudaMemsetAsync(D, 0, sizeof(double) * col * r, s));
  // z0 = M^-1 r0
  rc = precond(f, R0, Vk(0), Z32, r, s);
  std::vector<double> beta0(r);
  while (!rc && total_it < max_iters) {
    // beta = ||v0||, v0 /= beta
    dots_kernel<<<r, 256, 0, s>>>(Vk(0), n, Vk(0), n, n, sc);
    cudaMemcpyAsync(hcol.data(), sc, sizeof(double) * r, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    for (int j = 0; j < r; j++) {
      beta0[j] = std::sqrt(hcol[j]);
      g[j] = beta0[j];
      for (int i = 1; i <= m; i++) g[i * r + j] = 0.0;
    }
    inv_kernel<<<(r + 127) / 128, 128, 0, s>>>(sc, sc + r, r);
    cudaMemsetAsync(sc + 2 * r, 0, sizeof(double) * r, s);
    axpby_kernel<<<grid_for(col * r), 256, 0, s>>>(Vk(0), n, Vk(0), n, n, r, sc + r, sc + 2 * r, 0);
    dg::count_launches(3);
    int kdone = 0;
    for (int k = 0; k < m && total_it < max_iters; k++, total_it++) {
      // w = M^-1 A v_k
      rc = matvec(f, Vk(k), T, r, s, oz);
      if (rc) break;
      rc = precond(f, T, W, Z32, r, s);
      if (rc) break;
      // classical Gram-Schmidt twice (CGS2): the projections on all of
      // v_0..v_k in one launch, the update in one more, repeated once; the
      // host reads both sets of coefficients and the norm in one copy
      const int kk = k + 1;
      const long long vs = (long long)col * r;
      multi_dots_kernel<<<dim3(r, kk), 256, 0, s>>>(V, vs, W, n, r, hb);
      multi_axpy_kernel<<<grid_for(col * r), 256, 0, s>>>(V, vs, kk, W, n, r, hb);
      multi_dots_kernel<<<dim3(r, kk), 256, 0, s>>>(V, vs, W, n, r, hb + (size_t)kk * r);
      multi_axpy_kernel<<<grid_for(col * r), 256, 0, s>>>(V, vs, kk, W, n, r, hb + (size_t)kk * r);
      dots_kernel<<<r, 256, 0, s>>>(W, n, W, n, n, sc);
      dg::count_launches(5);
      hh.resize((size_t)2 * kk * r + r);
      cudaMemcpyAsync(hh.data(), hb, sizeof(double) * 2 * kk * r, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(hh.data() + 2 * kk * r, sc, sizeof(double) * r, cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      for (int i = 0; i <= k; i++)
        for (int j = 0; j < r; j++)
          H[((size_t)i * m + k) * r + j] = hh[(size_t)i * r + j] + hh[(size_t)(kk + i) * r + j];
      for (int j = 0; j < r; j++)
        H[((size_t)(k + 1) * m + k) * r + j] = std::sqrt(hh[(size_t)2 * kk * r + j]);
      inv_kernel<<<(r + 127) / 128, 128, 0, s>>>(sc, sc + r, r);
      cudaMemsetAsync(Vk(k + 1), 0, sizeof(double) * col * r, s);
      axpby_kernel<<<grid_for(col * r), 256, 0, s>>>(W, n, Vk(k + 1), n, n, r, sc + r, nullptr, 0);
      dg::count_launches(3);
      // Givens rotations on the host, per column
      double worst = 0.0;
      for (int j = 0; j < r; j++) {
        for (int i = 0; i < k; i++) {
          double &a = H[((size_t)i * m + k) * r + j], &b = H[((size_t)(i + 1) * m + k) * r + j];
          const double t = cs[i * r + j] * a + sn[i * r + j] * b;
          b = -sn[i * r + j] * a + cs[i * r + j] * b;
          a = t;
        }
        double &a = H[((size_t)k * m + k) * r + j], &b = H[((size_t)(k + 1) * m + k) * r + j];
        const double den = std::hypot(a, b);
        const double c = den > 0 ? a / den : 1.0, sv = den > 0 ? b / den : 0.0;
        cs[k * r + j] = c;
        sn[k * r + j] = sv;
        a = den;
        b = 0.0;
        g[(k + 1) * r + j] = -sv * g[k * r + j];
        g[k * r + j] = c * g[k * r + j];
        const double rel = beta0[j] > 0 ? std::fabs(g[(k + 1) * r + j]) / beta0[j] : 0.0;
        worst = std::max(worst, rel);
      }
      kdone = k + 1;
      if (worst <= inner_tol) break;
    }
    if (rc) break;
    // y = H^-1 g per column, D += V y
    std::vector<double> y((size_t)kdone * r);
    for (int j = 0; j < r; j++)
      for (int i = kdone - 1; i >= 0; i--) {
        double acc = g[i * r + j];
        for (int l = i + 1; l < kdone; l++) acc -= H[((size_t)i * m + l) * r + j] * y[l * r + j];
        const double h = H[((size_t)i * m + i) * r + j];
        y[i * r + j] = h != 0 ? acc / h : 0.0;
      }
    for (int i = 0; i < kdone; i++) {
      cudaMemcpyAsync(sc + 3 * r, &y[(size_t)i * r], sizeof(double) * r, cudaMemcpyHostToDevice, s);
      axpby_kernel<<<grid_for(col * r), 256, 0, s>>>(Vk(i), n, D, n, n, r, sc + 3 * r, nullptr, 0);
      dg::count_launches(1);
      cudaStreamSynchronize(s);
    }
    break;  // one cycle per outer refinement step; the outer loop restarts
  }
  if (!rc) {
    // x += d
    std::vector<double> ones(r, 1.0);
    cudaMemcpyAsync(sc, ones.data(), sizeof(double) * r, cudaMemcpyHostToDevice, s);
    axpby_kernel<<<grid_for(col * r), 256, 0, s>>>(D, n, X, ldx, n, r, sc, nullptr, 0);
    dg::count_launches(1);
    cudaStreamSynchronize(s);
  }
  cudaFreeAsync(V, s);
  cudaFreeAsync(W, s);
  cudaFreeAsync(D, s);
  cudaFreeAsync(sc, s);
  cudaFreeAsync(Z32, s);
  cudaFreeAsync(hb, s);
  *iters_out = total_it;
  return rc;
}

}  // namespace

extern "C" int dg_mixed_solve(const dg_mixed *f, int nrhs, const double *B, int ldb, double *X,
                              int ldx, const dg_ir_opts *opts, dg_ir_report *rep, void *stream) {
  DG_CHECK_ARG(f != nullptr, 1);
  DG_CHECK_ARG(nrhs > 0, 2);
  DG_CHECK_ARG(B != nullptr, 3);
  DG_CHECK_ARG(ldb >= f->n, 4);
  DG_CHECK_ARG(X != nullptr, 5);
  DG_CHECK_ARG(ldx >= f->n, 6);
  if (f->info != 0) {
    dg_set_last_error(__FILE__, __LINE__, "the factorization failed; no solve");
    return DG_ERR_STATE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int n = f->n, r = nrhs;
  dg_ir_opts o;
  o.tol = 1e-12; o.max_iter = 30; o.gmres = 0; o.restart = 30; o.gmres_inner_tol = 1e-4;
  if (opts) o = *opts;
  double *R = nullptr, *cm = nullptr;
  float *Z = nullptr;
  if (dg::pool_malloc_async((void **)&R, sizeof(double) * (size_t)n * r, s) != cudaSuccess ||
      dg::pool_malloc_async((void **)&cm, sizeof(double) * 3 * r, s) != cudaSuccess ||
      dg::pool_malloc_async((void **)&Z, sizeof(float) * (size_t)n * r * 2, s) != cudaSuccess) {
    cudaGetLastError();
    return DG_ERR_NOMEM;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  OzResidual oz;
  bool own_a = false;
  if (dg::get_f64_engine() == 2 && n <= 131072) {
    oz.ldk = ((long long)n + 7) / 8 * 8;
    const size_t ba = 16 * (size_t)oz.ldk * n, bx = 16 * (size_t)oz.ldk * r;
    if (f->ozA) {
      // A's slices were cut beside the factorization
      oz.a = f->ozA;
      oz.as = f->ozAs;
      DG_CUDA_TRY(cudaStreamWaitEvent(s, f->ev_oz, 0));
    } else if (dg::pool_malloc_async(&oz.a, ba + 8 * (size_t)n, s) == cudaSuccess) {
      own_a = true;
      oz.as = (unsigned long long *)((char *)oz.a + ba);
      if (dg::oz_split_tile_rows((const double *const *)f->tiles_dev, n, f->nb, oz.a, oz.ldk,
                                 oz.as, nullptr, s)) {
        cudaFreeAsync(oz.a, s);
        oz.a = nullptr;
        own_a = false;
      }
    } else {
      cudaGetLastError();
      oz.a = nullptr;
    }
    if (oz.a && dg::pool_malloc_async(&oz.x, bx + 8 * (size_t)r, s) == cudaSuccess) {
      oz.xs = (unsigned long long *)((char *)oz.x + bx);
    } else {
      cudaGetLastError();  // no room for the slices: the FP64 residual
      if (own_a) cudaFreeAsync(oz.a, s);
      oz.a = oz.x = nullptr;
      own_a = false;
    }
  }
  DG_CUDA_TRY(cudaMemset2DAsync(X, sizeof(double) * ldx, 0, sizeof(double) * n, r, s));
  DG_CUDA_TRY(cudaMemcpy2DAsync(R, sizeof(double) * n, B, sizeof(double) * ldb, sizeof(double) * n,
                                r, cudaMemcpyDeviceToDevice, s));
  std::vector<double> berr, prev;
  int it = 0, rc = 0, gm_iters = 0, outer = 0;
  bool converged = false, use_gmres = (o.gmres == 1);
  for (it = 0; it < o.max_iter; it++) {
    if (!use_gmres) {
      rc = correction(f, R, n, X, ldx, Z, r, s);
    } else {
      int gi = 0;
      rc = gmres_ir(f, R, X, ldx, r, o.restart, o.restart, o.gmres_inner_tol, s, &gi, &oz);
      gm_iters += gi;
    }
    if (rc) break;
    outer++;
    rc = residual(f, B, ldb, X, ldx, R, r, s, &oz);
    if (rc) break;
    rc = backward_errors(f, B, ldb, X, ldx, R, r, cm, berr, s);
    if (rc) break;
    double worst = 0.0;
    for (double b : berr) worst = std::max(worst, std::isfinite(b) ? b : INFINITY);
    if (worst <= o.tol) {
      converged = true;
      break;
    }
    // plain refinement stalls: the error no longer halves -> GMRES-IR
    if (!use_gmres && o.gmres == 0 && !prev.empty()) {
      double pw = 0.0;
      for (double b : prev) pw = std::max(pw, b);
      if (!(worst < 0.5 * pw)) use_gmres = true;
    }
    prev = berr;
  }
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(R, s);
  cudaFreeAsync(cm, s);
  cudaFreeAsync(Z, s);
  if (own_a) cudaFreeAsync(oz.a, s);
  if (oz.x) cudaFreeAsync(oz.x, s);
  if (rep) {
    rep->iterations = outer;
    rep->gmres_iterations = gm_iters;
    rep->used_gmres = use_gmres ? 1 : 0;
    rep->converged = converged ? 1 : 0;
    double worst = 0.0;
    for (double b : berr) worst = std::max(worst, b);
    rep->backward_error = worst;
    rep->solve_ms = ms;
  }
  if (rc) return rc;
  if (!converged) {
    dg_set_last_error(__FILE__, __LINE__, "iterative refinement did not reach the tolerance");
    return DG_ERR_NOCONVERGE;
  }
  return 0;
}

extern "C" int dg_gemm_f32_tc_tn(int m, int n, int k, float alpha, const float *A, int lda,
                                 const float *B, int ldb, float beta, float *C, int ldc,
                                 void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(k > 0 && k % 8 == 0, 3);
  DG_CHECK_ARG(lda >= k && lda % 8 == 0, 6);
  DG_CHECK_ARG(ldb >= k && ldb % 8 == 0, 8);
  DG_CHECK_ARG(ldc >= (m > 1 ? m : 1), 11);
  if (m == 0 || n == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t an = (size_t)lda * m, bn = (size_t)ldb * n;
  __nv_bfloat16 *buf = nullptr;
  DG_CUDA_TRY(dg::pool_malloc_async((void **)&buf, sizeof(__nv_bfloat16) * 3 * (an + bn), s));
  __nv_bfloat16 *a3 = buf, *b3 = buf + 3 * an;
  dg::split3_kernel<<<grid_for((long long)k * m), 256, 0, s>>>(
      A, (long long)k * m, a3, a3 + an, a3 + 2 * an, nullptr, nullptr, k, lda);
  dg::split3_kernel<<<grid_for((long long)k * n), 256, 0, s>>>(
      B, (long long)k * n, b3, b3 + bn, b3 + 2 * bn, nullptr, nullptr, k, ldb);
  dg::count_launches(2);
  dg::TcGemmArgs g;
  memset(&g, 0, sizeof g);
  g.m = m; g.n = n; g.k = k; g.terms = 6;
  g.a_hi = a3; g.a_mid = a3 + an; g.a_lo = a3 + 2 * an; g.lda = lda; g.a_rows = m;
  g.b_hi = b3; g.b_mid = b3 + bn; g.b_lo = b3 + 2 * bn; g.ldb = ldb; g.b_rows = n;
  g.alpha = alpha; g.beta = beta; g.c = C; g.ldc = ldc; g.layout = 0; g.upper = 0; g.bn = 128;
  int rc = dg::tc_gemm_bf16(g, s);
  cudaFreeAsync(buf, s);
  return rc;
}
