// FP64 GEMM emulated on the BF16 tensor cores (Ozaki's error-free splitting),
// for the FP64 tile updates of the plain path and the FP64 residual of
// refinement.  GB300 executes FP64 arithmetic at about 1.2 TFLOP/s, so the
// FP64 products are carried out on tcgen05 exactly, and only a short FP64
// accumulation per output element remains on the FP64 pipe.
//
// Splitting (oz_split_kernel): each operand vector v (a row of op(A) or a
// column of op(B), K values) is scaled by 2^-e with 2^(e-1) <= max|v| < 2^e,
// and cut into S = 8 slices by rounding to nearest:
//     v = 2^e * sum_{s=1..8} d_s 2^(-7 s) + r,   d_s integer,
//     |d_1| <= 128, |d_s| <= 64 (s >= 2), |r| <= 2^(e-57).
// Slice s is stored as the BF16 value d_s 2^(-7s): exact, since every
// integer of magnitude <= 256 has at most 8 significant bits.
//
// Products (oz_gemm_kernel): C = alpha * 2^(ea_i + eb_j) * sum_{s+t<=9} A_s B_t'
// + beta * C, K <= 1024.  A product A_s B_t' sums terms d_s d_t 2^(-7(s+t)).
// Level L = s + t collects the L - 1 products of that weight.  Over a window
// of 512 values of K the sum of level L <= 6 stays within 2^24 units of
// 2^(-7L) (level 6: (2*128*64 + 2*64*64 + 64*64) * 512 < 2^24; levels 2 and
// 3 within 2^24 over all 1024), so its FP32 accumulation in TMEM is exact.
// Levels 2..6 are read exactly after each window and summed as 64-bit
// integers in units of 2^-42 (|sum| < 2^53 over K = 1024, exact again in the
// final conversion to FP64).  Levels 7..9 accumulate in FP32 over the whole
// K; their rounding is below 2^-56 of |C|'s scale, and the dropped levels
// (>= 10) and the slicing remainder are below 2^-55.  The result has an FP64
// GEMM's accuracy relative to 2^(ea_i + eb_j) K.
//
// TMEM holds one 64-column accumulator per level, level L at columns
// 64 (L - 2) .. 64 (L - 1) - 1 (all 512 columns).  The B slices of a stage
// are stored one after the other, so B_t .. B_u form one operand of
// 64 (u - t + 1) rows, and A_s x [B_t .. B_u] is ONE MMA whose output
// columns fall exactly on levels s + t .. s + u.  Per 16 values of K that is
// 14 MMAs of N = 64..256: 8 onto levels 7..9 and 6 onto levels 2..6.
//
// CTA tile: 128 rows (TMEM lanes) x 64 columns.  K advances in stages of 32:
// one stage holds the 8 slices of the A tile and of the B tile (96 KiB, two
// 3-D TMA loads with 64-byte swizzle), and two stages are in flight.  6
// warps: warp 4 issues the TMA loads, warp 5 the MMAs (levels 7..9 first),
// warps 0-3 read levels 2..6 at the end of each window (one row per thread,
// 64 integers) while the next stage's MMAs onto levels 7..9 run.
// All waits are bounded (1 s): a timeout records DG_ERR_TIMEOUT and the CTA
// drains and returns.
#include <cuda_bf16.h>

#include "dg_common.cuh"
#include "runtime.h"
#include "tc_ptx.cuh"

namespace dg {
namespace {

using namespace ptx;

constexpr int OZ_S = 8;                                   // slices per operand
constexpr int kOzNonFinite = 1 << 30;                     // exponent of a non-finite vector
constexpr int OZ_BM = 128, OZ_BN = 64, OZ_BK = 32;        // K per stage
constexpr int OZ_WIN = 16;                                // stages per exact window (K 512)
constexpr int OZ_A_SLICE = OZ_BM * OZ_BK * 2;             // 8 KiB
constexpr int OZ_B_SLICE = OZ_BN * OZ_BK * 2;             // 4 KiB
constexpr int OZ_STAGE = OZ_S * (OZ_A_SLICE + OZ_B_SLICE);  // 96 KiB
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
  int *status;            // skip when non-zero; DG_ERR_TIMEOUT recorded here
  const int *abort2;      // skip when non-zero (read only)
};

__global__ void __launch_bounds__(192, 1) oz_gemm_kernel(const __grid_constant__ OzParams p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + OZ_STAGES * OZ_STAGE);
  uint64_t *empty = full + OZ_STAGES;
  uint64_t *ready = empty + OZ_STAGES;   // MMA -> readers: a window's exact sums complete
  uint64_t *drained = ready + 1;         // readers -> MMA: exact accumulators read
  uint64_t *done = drained + 1;          // MMA -> readers: everything complete
  uint32_t *tmem_slot = (uint32_t *)(done + 1);
  int *abort_flag = (int *)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i0 = blockIdx.x * OZ_BM, j0 = blockIdx.y * OZ_BN;
  if ((p.tri == 1 && i0 > j0 + OZ_BN - 1) || (p.tri == 2 && j0 > i0 + OZ_BM - 1)) return;
  // one read of the status word decides for the whole CTA
  if (threadIdx.x == 0)
    *abort_flag = aborted(p.status, p.abort2) ? 1 : 0;
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
  const int nst = (p.k + OZ_BK - 1) / OZ_BK;  // stages
  const int nwin = (nst + OZ_WIN - 1) / OZ_WIN;

  if (warp == 4) {
    if (lane == 0) {
      // ---------------- TMA producer ----------------
      int it = 0;
      for (; it < nst && !*(volatile int *)abort_flag; it++) {
        const int st = it % OZ_STAGES;
        if (it >= OZ_STAGES && !mbar_wait(&empty[st], ((it / OZ_STAGES) - 1) & 1)) {
          atomicExch(abort_flag, 1);
          break;
        }
        uint8_t *dst = smem + st * OZ_STAGE;
        mbar_expect_tx(&full[st], OZ_STAGE);
        tma_load_3d(dst, &p.a, &full[st], it * OZ_BK, i0, 0);
        tma_load_3d(dst + OZ_S * OZ_A_SLICE, &p.b, &full[st], it * OZ_BK, j0, 0);
      }
      // drain the loads in flight
      for (int q = (it > OZ_STAGES ? it - OZ_STAGES : 0); q < it; q++)
        if (!mbar_wait(&full[q % OZ_STAGES], (q / OZ_STAGES) & 1)) atomicExch(abort_flag, 1);
    }
    __syncwarp();
  } else if (warp == 5) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      const uint32_t idesc64 = idesc_f16kind(OZ_BM, OZ_BN, false);  // N = 64 c: + (8 (c-1)) << 17
      const uint32_t sbase = smem_u32(smem);
      for (int it = 0; it < nst; it++) {
        const int st = it % OZ_STAGES, w = it / OZ_WIN, wpos = it % OZ_WIN;
        if (!mbar_wait(&full[st], (it / OZ_STAGES) & 1)) {
          atomicExch(abort_flag, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // descriptors: base + (byte offset >> 4)
        const uint64_t da = sw64_desc(sbase + st * OZ_STAGE);
        const uint64_t db = sw64_desc(sbase + st * OZ_STAGE + OZ_S * OZ_A_SLICE);
        // A_s x [B_t .. B_u] onto levels s+t .. s+u (TMEM column 64 (s+t-2))
        auto mma_run = [&](int kk, int s_, int t, int u, uint32_t acc) {
          mma_bf16(tmem + 64 * (s_ + t - 2), da + (((s_ - 1) * OZ_A_SLICE + kk * 32) >> 4),
                   db + (((t - 1) * OZ_B_SLICE + kk * 32) >> 4),
                   idesc64 + ((uint32_t)(8 * (u - t)) << 17), acc);
        };
        // levels 7..9: t from max(1, 7 - s) to 9 - s; the first MMA sets them
#pragma unroll 1
        for (int kk = 0; kk < OZ_BK / 16; kk++)
#pragma unroll 1
          for (int s_ = 1; s_ <= OZ_S; s_++)
            mma_run(kk, s_, 7 - s_ > 1 ? 7 - s_ : 1, 9 - s_, (it == 0 && kk == 0 && s_ == 1) ? 0u : 1u);
        // levels 2..6: the previous window's sums must have been read
        if (wpos == 0 && w > 0 && !mbar_wait(drained, (w - 1) & 1)) {
          atomicExch(abort_flag, 1);
          break;
        }
        const uint32_t first = (wpos == 0) ? 0u : 1u;
#pragma unroll 1
        for (int kk = 0; kk < OZ_BK / 16; kk++) {
          const uint32_t a0 = (kk == 0) ? first : 1u;
          mma_run(kk, 1, 1, 4, a0);   // levels 2..5
          mma_run(kk, 1, 5, 5, a0);   // level 6
          mma_run(kk, 2, 1, 4, 1u);   // levels 3..6
          mma_run(kk, 3, 1, 3, 1u);   // levels 4..6
          mma_run(kk, 4, 1, 2, 1u);   // levels 5..6
          mma_run(kk, 5, 1, 1, 1u);   // level 6
        }
        mma_commit(&empty[st]);
        if (wpos == OZ_WIN - 1 || it == nst - 1) mma_commit(ready);
      }
      mma_commit(done);
    }
    __syncwarp();
  }

  // ---------------- exact sums (warps 0-3) ----------------
  long long acc[OZ_BN];
#pragma unroll
  for (int c = 0; c < OZ_BN; c++) acc[c] = 0;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  for (int w = 0; w < nwin && warp < 4; w++) {
    if (!mbar_wait(ready, w & 1)) {
      atomicExch(abort_flag, 1);
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
    for (int lvl = 2; lvl <= 6; lvl++) {
      const float up = __int_as_float((127 + 7 * lvl) << 23);  // 2^(7 lvl)
      const long long unit = 1LL << (7 * (6 - lvl));           // 2^(7 (6 - lvl))
#pragma unroll
      for (int h = 0; h < 2; h++) {
        float v[32];
        tmem_ld32(tmem + 64 * (lvl - 2) + h * 32 + lane_base, v);
#pragma unroll
        for (int c = 0; c < 32; c++) acc[h * 32 + c] += (long long)__float2int_rn(v[c] * up) * unit;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    mbar_arrive(drained);
  }
  const bool ok = mbar_wait(done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!ok) atomicExch(abort_flag, 1);
  __syncthreads();
  const bool aborted = *(volatile int *)abort_flag != 0;
  if (!aborted && nst > 0 && warp < 4) {
    const int row = i0 + warp * 32 + lane;
    const int ea = row < p.m ? p.ea[row] : 0;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      // levels 9, 8, 7 summed in FP32 (all lanes: the loads are warp-wide)
      float v[32], w[32];
      tmem_ld32(tmem + 64 * 7 + h * 32 + lane_base, v);
#pragma unroll 1
      for (int lvl = 8; lvl >= 7; lvl--) {
        tmem_ld32(tmem + 64 * (lvl - 2) + h * 32 + lane_base, w);
#pragma unroll
        for (int c = 0; c < 32; c++) v[c] = w[c] + v[c];
      }
      if (row >= p.m) continue;
      // 8 columns at a time: their reads of C are issued before the writes
#pragma unroll
      for (int c0 = 0; c0 < 32; c0 += 8) {
        double old[8];
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const int col = j0 + h * 32 + c0 + c;
          const bool in = col < p.n && !(p.tri == 1 && row > col) && !(p.tri == 2 && row < col);
          old[c] = (in && p.beta != 0.0) ? p.c[(size_t)row + (size_t)col * p.ldc] : 0.0;
        }
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const int col = j0 + h * 32 + c0 + c;
          if (col >= p.n || (p.tri == 1 && row > col) || (p.tri == 2 && row < col)) continue;
          const double x = fma((double)acc[h * 32 + c0 + c], 0x1p-42, (double)v[c0 + c]);
          const int eb = p.eb[col];
          double vout = (ea == kOzNonFinite || eb == kOzNonFinite)
                            ? __longlong_as_double(0x7FF8000000000000ll)
                            : p.alpha * ldexp(x, ea + eb);
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

// Splitting runs on integer arithmetic (the FP64 pipe is slow on this
// part): the exponent comes from the bits of max|v|, and the 56-bit integer
// X = round(v * 2^(56 - e)) (|X| <= 2^56) is cut into base-128 digits
// d_8 .. d_2 in [-64, 63] by rounding to nearest, leaving d_1 in [-128, 128].
// A vector holding an infinity or a NaN gets the exponent kOzNonFinite, and
// every output that uses it is NaN.
constexpr int SPLIT_V = 32;    // vectors per CTA
constexpr int SPLIT_K = 128;   // values of K per slicing CTA

__device__ __forceinline__ unsigned long long abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}

// frexp exponent of the non-negative double with bits b (0 for 0).
__device__ __forceinline__ int exponent_of(unsigned long long b) {
  const int eb = (int)(b >> 52);
  if (eb == 0x7FF) return kOzNonFinite;
  if (eb) return eb - 1022;
  if (b == 0) return 0;
  return (63 - __clzll((long long)b)) + 1 - 1074;  // subnormal: b * 2^-1074
}

// round(v * 2^(56 - ex)) for |v| < 2^ex.
__device__ __forceinline__ long long scaled56(double v, int ex) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int eb = (int)((b >> 52) & 0x7FF);
  unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  if (eb) mant |= 1ull << 52;
  // v = mant * 2^(max(eb, 1) - 1075)
  const int sh = (eb ? eb : 1) - 1019 - ex;  // <= 3
  long long r;
  if (sh >= 0) r = (long long)(mant << sh);
  else if (sh > -63) r = (long long)((mant + (1ull << (-sh - 1))) >> (-sh));
  else r = 0;
  return (b >> 63) ? -r : r;
}

// Exponent of each of `ncols` vectors of length K (element k of vector c at
// src[c*cstride + k*kstride]).  CTA: 32 x 8 threads over 32 vectors, reading
// along whichever of k or c is contiguous.
__global__ void __launch_bounds__(256) oz_exp_kernel(const double *src, long long cstride,
                                                    long long kstride, int K, int ncols, int *e,
                                                    const int *abort_flag, const int *abort2) {
  if (aborted(abort_flag, abort2)) return;
  __shared__ unsigned long long red[8][SPLIT_V + 1];
  const int tx = threadIdx.x, ty = threadIdx.y, c0 = blockIdx.x * SPLIT_V;
  if (kstride == 1) {  // columns: lanes along k, warp ty over vectors ty, ty+8, ...
    for (int vi = ty; vi < SPLIT_V; vi += 8) {
      const int c = c0 + vi;
      unsigned long long m = 0;
      if (c < ncols)
        for (int k = tx; k < K; k += 32) {
          const unsigned long long a = abs_bits(src[(size_t)c * cstride + k]);
          m = a > m ? a : m;
        }
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long q = __shfl_xor_sync(0xffffffffu, m, o);
        m = q > m ? q : m;
      }
      if (tx == 0 && c < ncols) e[c] = exponent_of(m);
    }
  } else {             // rows (or general strides): lanes along vectors
    const int c = c0 + tx;
    unsigned long long m = 0;
    if (c < ncols)
      for (int k = ty; k < K; k += 8) {
        const unsigned long long a = abs_bits(src[(size_t)c * cstride + (size_t)k * kstride]);
        m = a > m ? a : m;
      }
    red[ty][tx] = m;
    __syncthreads();
    if (ty == 0 && c < ncols) {
      for (int y = 1; y < 8; y++) m = red[y][tx] > m ? red[y][tx] : m;
      e[c] = exponent_of(m);
    }
  }
}

// Slices of the vectors [32 bx, 32 bx + 32) over k in [128 by, 128 by + 128)
// (k < ldk; zeros for k >= K): slice s (0-based) of vector c at
// dst + s*sstride + c*ldk.  Tiles of 32 x 32 values pass through shared
// memory so that both the reads and the writes are coalesced.
__global__ void __launch_bounds__(256) oz_slice_kernel(const double *src, long long cstride,
                                                      long long kstride, int K, int ncols,
                                                      __nv_bfloat16 *dst, long long ldk,
                                                      long long sstride, const int *e,
                                                      const int *abort_flag, const int *abort2) {
  if (aborted(abort_flag, abort2)) return;
  __shared__ double tile[SPLIT_V][33];
  __shared__ int ex[SPLIT_V];
  const int tx = threadIdx.x, ty = threadIdx.y, c0 = blockIdx.x * SPLIT_V;
  if (ty == 0) ex[tx] = (c0 + tx < ncols) ? e[c0 + tx] : 0;
  for (int kc = blockIdx.y * SPLIT_K; kc < (blockIdx.y + 1) * SPLIT_K && kc < ldk; kc += 32) {
    __syncthreads();
    if (kstride == 1) {
      for (int vi = ty; vi < SPLIT_V; vi += 8) {
        const int c = c0 + vi, k = kc + tx;
        tile[vi][tx] = (c < ncols && k < K) ? src[(size_t)c * cstride + k] : 0.0;
      }
    } else {
      for (int kk = ty; kk < 32; kk += 8) {
        const int c = c0 + tx, k = kc + kk;
        tile[tx][kk] = (c < ncols && k < K) ? src[(size_t)c * cstride + (size_t)k * kstride] : 0.0;
      }
    }
    __syncthreads();
    const int k = kc + tx;
    if (k >= ldk) continue;
    for (int vi = ty; vi < SPLIT_V; vi += 8) {
      const int c = c0 + vi;
      if (c >= ncols) continue;
      long long X = (ex[vi] == kOzNonFinite) ? 0 : scaled56(tile[vi][tx], ex[vi]);
      __nv_bfloat16 *out = dst + (size_t)c * ldk + k;
#pragma unroll
      for (int s = OZ_S; s >= 1; s--) {
        const long long d = (s > 1) ? ((X + 64) & 127) - 64 : X;
        X = (X - d) >> 7;
        const float w = __int_as_float((127 - 7 * s) << 23);  // 2^(-7 s)
        out[(size_t)(s - 1) * sstride] = __float2bfloat16_rn((float)d * w);
      }
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
  cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, (cuuint32_t)OZ_S};
  cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)base, dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

int oz_split(const double *src, long long cstride, long long kstride, int K, int ncols,
             void *slices, long long ldk, long long sstride, int *e, const int *abort_flag,
             cudaStream_t s, const int *abort2) {
  if (ncols <= 0) return 0;
  const dim3 blk(32, 8);
  const int nv = (ncols + SPLIT_V - 1) / SPLIT_V;
  oz_exp_kernel<<<nv, blk, 0, s>>>(src, cstride, kstride, K, ncols, e, abort_flag, abort2);
  DG_CUDA_TRY(cudaGetLastError());
  const dim3 grid(nv, (unsigned)((ldk + SPLIT_K - 1) / SPLIT_K));
  oz_slice_kernel<<<grid, blk, 0, s>>>(src, cstride, kstride, K, ncols, (__nv_bfloat16 *)slices,
                                       ldk, sstride, e, abort_flag, abort2);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(2);
  return 0;
}

int oz_gemm(int m, int n, int k, double alpha, const void *a_slices, long long lda_k,
            long long a_sstride, const int *ea, const void *b_slices, long long ldb_k,
            long long b_sstride, const int *eb, double beta, double *C, long long ldc, int tri,
            int *status, cudaStream_t s, const int *abort2) {
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
  p.abort2 = abort2;
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

static size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t oz_scratch_bytes(int m, int n, int k, bool same) {
  const size_t ldk = (size_t)(k + 7) / 8 * 8;
  size_t b = round256((size_t)OZ_S * ldk * m * 2) + round256((size_t)m * 4);
  if (!same) b += round256((size_t)OZ_S * ldk * n * 2) + round256((size_t)n * 4);
  return b;
}

int oz_gemm_general(char ta, char tb, int m, int n, int k, double alpha, const double *A,
                    long long lda, const double *B, long long ldb, double beta, double *C,
                    long long ldc, int tri, void *scratch, size_t bytes, int *status,
                    const int *abort2, cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  const bool tA = !(ta == 'N' || ta == 'n'), tB = !(tb == 'N' || tb == 'n');
  // the rows of op(A) are the columns of op(B): one set of slices (SYRK)
  const bool same = (A == B && lda == ldb && m == n && tA != tB);
  if (k <= 0 || k > 1024 || !scratch || oz_scratch_bytes(m, n, k, same) > bytes) return 1;
  const long long ldk = (k + 7) / 8 * 8;
  char *q = (char *)scratch;
  void *sa = q;
  q += round256((size_t)OZ_S * ldk * m * 2);
  int *ea = (int *)q;
  q += round256((size_t)m * 4);
  void *sb = sa;
  int *eb = ea;
  // row i of op(A), element p: A[i + p lda] ('N') or A[p + i lda] ('T')
  DG_TRY(oz_split(A, tA ? lda : 1, tA ? 1 : lda, k, m, sa, ldk, ldk * m, ea, status, s, abort2));
  if (!same) {
    sb = q;
    q += round256((size_t)OZ_S * ldk * n * 2);
    eb = (int *)q;
    // column j of op(B), element p: B[p + j ldb] ('N') or B[j + p ldb] ('T')
    DG_TRY(oz_split(B, tB ? 1 : ldb, tB ? ldb : 1, k, n, sb, ldk, ldk * n, eb, status, s, abort2));
  }
  return oz_gemm(m, n, k, alpha, sa, ldk, ldk * m, ea, sb, ldk, same ? ldk * m : ldk * n, eb, beta,
                 C, ldc, tri, status, s, abort2);
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
  const size_t bytes = dg::oz_scratch_bytes(m, n, k, false);
  void *buf = nullptr;
  DG_CUDA_TRY(cudaMallocAsync(&buf, bytes, s));
  int rc = dg::oz_gemm_general('T', 'N', m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, 0, buf,
                               bytes, nullptr, nullptr, s);
  cudaFreeAsync(buf, s);
  return rc;
}

// The two stages of dg_gemm_f64_emulated_tn as separate calls, for callers
// that reuse the slices of one operand across many products (the tiles of a
// factor, the matrix of a refinement residual).
extern "C" int dg_f64_slices(int k, int ncols, const double *src, long long cstride,
                             long long kstride, void *slices, int ldk, int *exps, void *stream) {
  DG_CHECK_ARG(k > 0 && k <= 1024, 1);
  DG_CHECK_ARG(ncols >= 0, 2);
  DG_CHECK_ARG(ldk >= k && ldk % 8 == 0, 7);
  DG_CHECK_ARG(((uintptr_t)slices & 15) == 0, 6);
  return dg::oz_split(src, cstride, kstride, k, ncols, slices, ldk, (long long)ldk * ncols, exps,
                      nullptr, (cudaStream_t)stream);
}

extern "C" int dg_gemm_f64_slices(int m, int n, int k, double alpha, const void *a_slices,
                                  int lda_k, const int *ea, const void *b_slices, int ldb_k,
                                  const int *eb, double beta, double *C, int ldc, int *status,
                                  void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(k > 0 && k <= 1024, 3);
  DG_CHECK_ARG(lda_k >= k && lda_k % 8 == 0, 6);
  DG_CHECK_ARG(ldb_k >= k && ldb_k % 8 == 0, 9);
  DG_CHECK_ARG(ldc >= (m > 1 ? m : 1), 13);
  return dg::oz_gemm(m, n, k, alpha, a_slices, lda_k, (long long)lda_k * m, ea, b_slices, ldb_k,
                     (long long)ldb_k * n, eb, beta, C, ldc, 0, status, (cudaStream_t)stream);
}
