// FP64 GEMM emulated on the BF16 tensor cores (Ozaki's error-free splitting),
// for the FP64 tile updates of the plain path and the FP64 residual of
// refinement.  GB300 executes FP64 arithmetic at about 1.2 TFLOP/s, so the
// FP64 products are carried out on tcgen05 exactly, and only a short FP64
// accumulation per output element remains on the FP64 pipe.
//
// Splitting (oz_split_kernel): each operand vector v (a row of op(A) or a
// column of op(B), K values) is scaled by 2^-e with 2^(e-1) <= max|v| < 2^e,
// and cut into S = 8 slices of 7 bits:
//     v = 2^e * sum_{s=1..8} d_s 2^(-7 s) + r,   d_s integer, |d_s| <= 127,
//     |r| < 2^(e-56).
// Slice s is stored as the BF16 value d_s 2^(-7s): exact, since |d_s| has at
// most 7 significant bits and the factor is a power of two.
//
// Products (oz_gemm_kernel): C = alpha * 2^(ea_i + eb_j) * sum_{s+t<=9} A_s B_t'
// + beta * C, K <= 1024.  One product A_s B_t' sums K terms d_s d_t 2^(-7(s+t))
// with |d_s d_t| < 2^14, so its FP32 accumulation in TMEM is exact (the
// integer part stays below 2^24).  Products of level s+t <= 6 (15 of them)
// are accumulated separately, each exactly, and added in FP64; the 21
// products of levels 7..9 share one FP32 accumulator, whose rounding is below
// 2^-54 of |C|'s scale.  The dropped levels (>= 10) and the slicing remainder
// are below 2^-56.  The result has an FP64 GEMM's accuracy relative to
// 2^(ea_i + eb_j) K.
//
// CTA tile: 128 rows (TMEM lanes) x 64 columns, K in blocks of 64, 6 warps:
// warps 0-3 accumulate in FP64 (one row per thread, 64 doubles), warp 4
// issues the TMA loads, warp 5 the MMAs.  Job s (s = 1..8) streams A_s and
// the B_t it pairs with (t = 1..9-s) through two 80 KiB shared-memory stages
// (TMA, 128-byte swizzle); its exact products go to TMEM accumulators
// E_1..E_5 (64 columns each), its grouped products to G.  After a job with
// exact products warps 0-3 add E into their FP64 registers before the next
// job reuses E.
// All waits are bounded (1 s): a timeout records DG_ERR_TIMEOUT and the CTA
// drains and returns.
#include <cuda_bf16.h>

#include "dg_common.cuh"
#include "runtime.h"
#include "tc_ptx.cuh"

namespace dg {
namespace {

using namespace ptx;

constexpr int OZ_S = 8;           // slices per operand
constexpr int OZ_BM = 128, OZ_BN = 64, OZ_BK = 64;
constexpr int OZ_A_BYTES = OZ_BM * OZ_BK * 2;   // 16 KiB
constexpr int OZ_B_BYTES = OZ_BN * OZ_BK * 2;   // 8 KiB
constexpr int OZ_STAGE = OZ_A_BYTES + 8 * OZ_B_BYTES;  // 80 KiB
constexpr int OZ_STAGES = 2;
constexpr int OZ_SMEM = OZ_STAGES * OZ_STAGE + 1024 + 256;

struct OzParams {
  CUtensorMap a, b;       // 3-D maps: {K, rows, slice}
  const int *ea, *eb;     // exponents per A row / per B row
  double *c;
  long long ldc;
  int m, n, k;
  double alpha, beta;
  int tri;                // 1: store only i <= j, 2: only i >= j
  int *status;
};

__device__ __forceinline__ int n_pair(int s) { return 9 - s; }           // t = 1..9-s
__device__ __forceinline__ int n_exact(int s) { return s <= 5 ? 6 - s : 0; }  // t with s+t <= 6

__global__ void __launch_bounds__(192, 1) oz_gemm_kernel(const __grid_constant__ OzParams p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + OZ_STAGES * OZ_STAGE);
  uint64_t *empty = full + OZ_STAGES;
  uint64_t *ready = empty + OZ_STAGES;   // MMA -> epilogue: exact accumulators complete
  uint64_t *drained = ready + 1;         // epilogue -> MMA: exact accumulators read
  uint64_t *done = drained + 1;          // MMA -> epilogue: everything complete
  uint32_t *tmem_slot = (uint32_t *)(done + 1);
  int *abort_flag = (int *)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i0 = blockIdx.x * OZ_BM, j0 = blockIdx.y * OZ_BN;
  if ((p.tri == 1 && i0 > j0 + OZ_BN - 1) || (p.tri == 2 && j0 > i0 + OZ_BM - 1)) return;
  // one read of the status word decides for the whole CTA
  if (threadIdx.x == 0) *abort_flag = (p.status && *(volatile int *)p.status) ? 1 : 0;
  __syncthreads();
  if (*(volatile int *)abort_flag) return;
  __syncthreads();

  if (threadIdx.x == 0) {
    for (int s = 0; s < OZ_STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(ready, 1);
    mbar_init(drained, 128);
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t G = tmem;                    // columns 0..63
  const int nk = (p.k + OZ_BK - 1) / OZ_BK;

  if (warp == 4) {
    if (lane == 0) {
    // ---------------- TMA producer ----------------
    int it = 0;
    for (int s = 1; s <= OZ_S && !*(volatile int *)abort_flag; s++) {
      const int np = n_pair(s);
      const uint32_t bytes = OZ_A_BYTES + np * OZ_B_BYTES;
      for (int kb = 0; kb < nk; kb++, it++) {
        const int st = it % OZ_STAGES;
        if (it >= OZ_STAGES && !mbar_wait(&empty[st], ((it / OZ_STAGES) - 1) & 1)) {
          atomicExch(abort_flag, 1);
          break;
        }
        uint8_t *dst = smem + st * OZ_STAGE;
        mbar_expect_tx(&full[st], bytes);
        tma_load_3d(dst, &p.a, &full[st], kb * OZ_BK, i0, s - 1);
        for (int t = 1; t <= np; t++)
          tma_load_3d(dst + OZ_A_BYTES + (t - 1) * OZ_B_BYTES, &p.b, &full[st], kb * OZ_BK, j0,
                      t - 1);
      }
    }
    // drain the loads in flight
    for (int q = (it > OZ_STAGES ? it - OZ_STAGES : 0); q < it; q++)
      if (!mbar_wait(&full[q % OZ_STAGES], (q / OZ_STAGES) & 1)) atomicExch(abort_flag, 1);
    }
    __syncwarp();
  } else if (warp == 5) {
    if (lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t idesc = idesc_f16kind(OZ_BM, OZ_BN, false);
    const uint32_t sbase = smem_u32(smem);
    int it = 0, flushes = 0;
    bool g_started = false;
    for (int s = 1; s <= OZ_S; s++) {
      const int np = n_pair(s), ne = n_exact(s);
      // the exact accumulators must have been read by the previous flush
      if (ne > 0 && flushes > 0 && !mbar_wait(drained, (flushes - 1) & 1)) {
        atomicExch(abort_flag, 1);
        break;
      }
      bool ok = true;
      for (int kb = 0; kb < nk; kb++, it++) {
        const int st = it % OZ_STAGES;
        if (!mbar_wait(&full[st], (it / OZ_STAGES) & 1)) {
          atomicExch(abort_flag, 1);
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t sa = sbase + st * OZ_STAGE;
#pragma unroll
        for (int kk = 0; kk < OZ_BK / 16; kk++) {
          const uint64_t adesc = sw128_desc(sa + kk * 32);
          for (int t = 1; t <= np; t++) {
            const uint64_t bdesc = sw128_desc(sa + OZ_A_BYTES + (t - 1) * OZ_B_BYTES + kk * 32);
            if (t <= ne) {
              mma_bf16(tmem + 64 * t, adesc, bdesc, idesc, (kb | kk) ? 1u : 0u);
            } else {
              mma_bf16(G, adesc, bdesc, idesc, g_started ? 1u : 0u);
              g_started = true;
            }
          }
        }
        mma_commit(&empty[st]);
      }
      if (!ok) break;
      if (ne > 0) {
        mma_commit(ready);
        flushes++;
      }
    }
    mma_commit(done);
    }
    __syncwarp();
  }

  // ---------------- FP64 accumulation (warps 0-3) ----------------
  double acc[OZ_BN];
#pragma unroll
  for (int c = 0; c < OZ_BN; c++) acc[c] = 0.0;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  int flush = 0;
  for (int s = 1; s <= OZ_S && warp < 4; s++) {
    const int ne = n_exact(s);
    if (ne == 0) continue;
    if (!mbar_wait(ready, flush & 1)) {
      atomicExch(abort_flag, 1);
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    for (int t = 1; t <= ne; t++) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        float v[32];
        tmem_ld32(tmem + 64 * t + h * 32 + lane_base, v);
#pragma unroll
        for (int c = 0; c < 32; c++) acc[h * 32 + c] += (double)v[c];
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    mbar_arrive(drained);
    flush++;
  }
  const bool ok = mbar_wait(done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!ok) atomicExch(abort_flag, 1);
  __syncthreads();
  const bool aborted = *(volatile int *)abort_flag != 0;
  if (!aborted && nk > 0 && warp < 4) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
      float v[32];
      tmem_ld32(G + h * 32 + lane_base, v);
#pragma unroll
      for (int c = 0; c < 32; c++) acc[h * 32 + c] += (double)v[c];
    }
    const int row = i0 + warp * 32 + lane;
    if (row < p.m) {
      const int ea = p.ea[row];
      // 8 columns at a time: their reads of C are issued before the writes
#pragma unroll
      for (int c0 = 0; c0 < OZ_BN; c0 += 8) {
        double old[8];
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const int col = j0 + c0 + c;
          const bool in = col < p.n && !(p.tri == 1 && row > col) && !(p.tri == 2 && row < col);
          old[c] = (in && p.beta != 0.0) ? p.c[(size_t)row + (size_t)col * p.ldc] : 0.0;
        }
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const int col = j0 + c0 + c;
          if (col >= p.n || (p.tri == 1 && row > col) || (p.tri == 2 && row < col)) continue;
          double vout = p.alpha * ldexp(acc[c0 + c], ea + p.eb[col]);
          if (p.beta != 0.0) vout = fma(p.beta, old[c], vout);
          p.c[(size_t)row + (size_t)col * p.ldc] = vout;
        }
      }
    }
  }
  if (aborted && threadIdx.x == 0 && p.status) atomicCAS(p.status, 0, DG_ERR_TIMEOUT);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512)
                 : "memory");
}

// Splits `ncols` vectors of length K (element k of vector c at
// src[c*cstride + k*kstride]: columns of a column-major matrix have
// kstride 1, rows have cstride 1) into OZ_S BF16 slices: slice s of vector c
// at dst + s*sstride + c*ldk, and the exponent of vector c at e[c].  One CTA
// per vector.
__global__ void __launch_bounds__(128) oz_split_kernel(const double *src, long long cstride,
                                                      long long kstride, int K, int ncols,
                                                      __nv_bfloat16 *dst, long long ldk,
                                                      long long sstride, int *e,
                                                      const int *abort_flag) {
  if (abort_flag && *(volatile const int *)abort_flag) return;
  const int c = blockIdx.x;
  if (c >= ncols) return;
  const double *v = src + (size_t)c * cstride;
  double m = 0.0;
  for (int k = threadIdx.x; k < K; k += blockDim.x) m = fmax(m, fabs(v[(size_t)k * kstride]));
  __shared__ double red[4];
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  m = fmax(fmax(red[0], red[1]), fmax(red[2], red[3]));
  int ex = 0;
  if (m > 0.0) {
    frexp(m, &ex);  // m in [2^(ex-1), 2^ex)
  }
  if (threadIdx.x == 0) e[c] = ex;
  for (int k = threadIdx.x; k < ldk; k += blockDim.x) {
    double x = k < K ? ldexp(v[(size_t)k * kstride], -ex) : 0.0;  // |x| < 1
#pragma unroll
    for (int s = 0; s < OZ_S; s++) {
      x *= 128.0;
      const double d = trunc(x);
      x -= d;
      dst[(size_t)s * sstride + (size_t)c * ldk + k] =
          __float2bfloat16_rn(ldexpf((float)d, -7 * (s + 1)));
    }
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn oz_encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *q = nullptr;
    cudaDriverEntryPointQueryResult r;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &q, 12000, cudaEnableDefault,
                                         &r) == cudaSuccess &&
        r == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)q;
  }
  return fn;
}

// The map spans the slot's padded length ldk (the split zero-fills k >= K).
bool oz_map(CUtensorMap *map, const void *base, long long ldk, long long rows, long long sstride,
            int box_rows) {
  EncodeTiledFn enc = oz_encode_fn();
  if (!enc) return false;
  cuuint64_t dims[3] = {(cuuint64_t)ldk, (cuuint64_t)rows, (cuuint64_t)OZ_S};
  cuuint64_t strides[2] = {(cuuint64_t)ldk * 2, (cuuint64_t)sstride * 2};
  cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)base, dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

int oz_split(const double *src, long long cstride, long long kstride, int K, int ncols,
             void *slices, long long ldk, long long sstride, int *e, const int *abort_flag,
             cudaStream_t s) {
  if (ncols <= 0) return 0;
  oz_split_kernel<<<ncols, 128, 0, s>>>(src, cstride, kstride, K, ncols, (__nv_bfloat16 *)slices,
                                        ldk, sstride, e, abort_flag);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

int oz_gemm(int m, int n, int k, double alpha, const void *a_slices, long long lda_k,
            long long a_sstride, const int *ea, const void *b_slices, long long ldb_k,
            long long b_sstride, const int *eb, double beta, double *C, long long ldc, int tri,
            int *status, cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  if (k <= 0 || k > 1024 || lda_k % 8 || ldb_k % 8) return DG_ERR_UNSUPPORTED;
  OzParams p;
  memset(&p, 0, sizeof p);
  if (lda_k < k || ldb_k < k) return DG_ERR_UNSUPPORTED;
  if (!oz_map(&p.a, a_slices, lda_k, m, a_sstride, OZ_BM) ||
      !oz_map(&p.b, b_slices, ldb_k, n, b_sstride, OZ_BN)) {
    dg_set_last_error(__FILE__, __LINE__, "cuTensorMapEncodeTiled failed");
    return DG_ERR_CUDA;
  }
  p.ea = ea; p.eb = eb; p.c = C; p.ldc = ldc;
  p.m = m; p.n = n; p.k = k; p.alpha = alpha; p.beta = beta; p.tri = tri;
  p.status = status;
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr[dev & 63]) {
    DG_CUDA_TRY(cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     OZ_SMEM));
    attr[dev & 63] = true;
  }
  dim3 grid((m + OZ_BM - 1) / OZ_BM, (n + OZ_BN - 1) / OZ_BN);
  oz_gemm_kernel<<<grid, 192, OZ_SMEM, s>>>(p);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

}  // namespace dg

// Building block exposed for tests: C = alpha op(A) op(B) + beta C in FP64
// through the emulated path, with op(A) = A' (A is k x m) and op(B) = B
// (k x n), both column-major, k <= 1024.  Uses stream-ordered scratch.
extern "C" int dg_gemm_f64_emulated_tn(int m, int n, int k, double alpha, const double *A, int lda,
                                       const double *B, int ldb, double beta, double *C, int ldc,
                                       void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(k > 0 && k <= 1024, 3);
  DG_CHECK_ARG(lda >= k, 6);
  DG_CHECK_ARG(ldb >= k, 8);
  DG_CHECK_ARG(ldc >= (m > 1 ? m : 1), 11);
  if (m == 0 || n == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  const long long ldk = (k + 7) / 8 * 8;
  const long long sa = ldk * m, sb = ldk * n;
  void *buf = nullptr;
  const size_t bytes = 2 * (size_t)dg::OZ_S * (sa + sb) + 4 * (size_t)(m + n) + 256;
  DG_CUDA_TRY(cudaMallocAsync(&buf, bytes, s));
  __nv_bfloat16 *as = (__nv_bfloat16 *)buf;
  __nv_bfloat16 *bs = as + dg::OZ_S * sa;
  int *ea = (int *)(bs + dg::OZ_S * sb);
  int *eb = ea + m;
  int rc = dg::oz_split(A, lda, 1, k, m, as, ldk, sa, ea, nullptr, s);
  if (!rc) rc = dg::oz_split(B, ldb, 1, k, n, bs, ldk, sb, eb, nullptr, s);
  if (!rc)
    rc = dg::oz_gemm(m, n, k, alpha, as, ldk, sa, ea, bs, ldk, sb, eb, beta, C, ldc, 0, nullptr, s);
  cudaFreeAsync(buf, s);
  return rc;
}
