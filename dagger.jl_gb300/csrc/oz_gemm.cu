// FP64 GEMM emulated on the BF16 tensor cores (Ozaki's error-free splitting),
// for the FP64 tile updates of the plain path and the FP64 residual of
// refinement.  GB300 executes FP64 arithmetic at about 1.1 TFLOP/s, so the
// FP64 products are carried out on tcgen05 exactly, the sums are formed in
// 64-bit integers, and one FP64 operation per output element remains.
//
// Splitting (oz_max_kernel, oz_slice_kernel): each operand vector v (a row of
// op(A) or a column of op(B), K values) is scaled by 2^-e with
// 2^(e-1) <= max|v| < 2^e and cut into S = 7 slices by rounding to nearest:
//     v = 2^e * sum_{s=1..7} d_s 2^(-8 s) + r,   d_s integer,
//     |d_1| <= 256, |d_s| <= 128 (s >= 2), |r| <= 2^(e-57).
// Slice s is stored as the BF16 value d_s 2^(-8s): exact, since every
// integer of magnitude <= 256 has at most 8 significant bits (the digits use
// the whole BF16 significand).  The split runs on integer arithmetic: the
// per-vector scale word is max|v|'s bit pattern (an atomic maximum over the
// vector), e follows from its exponent field, and X = round(v 2^(56-e))
// (|X| <= 2^56) is cut into balanced base-256 digits.
// A vector holding an infinity or a NaN makes every output that uses it NaN.
//
// Products (oz_gemm_kernel): C = alpha * 2^(ea_i + eb_j) * sum_{s+t<=8} A_s B_t'
// + beta * C, K <= 131072: 28 slice products.  A product A_s B_t' sums terms
// d_s d_t 2^(-8(s+t)).  Level L = s + t collects the L - 1 products of that
// weight.  Over a window of 160 values of K the sum of level L <= 5 stays
// within 2^24 units of 2^(-8L) (level 5: (2*256*128 + 2*128*128) * 160 < 2^24),
// so its FP32 accumulation in TMEM is exact.  Levels 2..5 are read exactly
// after each window and summed as 64-bit integers in units of 2^-40
// (|sum| < 2^50 K / 1024).  Levels 6..8 accumulate in FP32 over the whole K
// (their rounding is below 2^-55 K of |C|'s scale, the dropped levels >= 9
// below 2^-55 K, the slicing remainders below 2^-56 K) and join the integer
// sum at 2^-51 (2^-44 at the largest K).  The 62-bit total is rounded once
// to FP64 by integer arithmetic, with 2^(ea_i + eb_j) folded into the
// exponent, and added to beta C.  The result has an FP64 GEMM's accuracy
// relative to 2^(ea_i + eb_j) K.
//
// TMEM holds one 64-column accumulator per level, level L at columns
// 64 (L - 2) .. 64 (L - 1) - 1 (448 columns).  The B slices of a stage are
// stored one after the other, so B_t .. B_u form one operand of
// 64 (u - t + 1) rows, and A_s x [B_t .. B_u] is ONE MMA whose output
// columns fall exactly on levels s + t .. s + u.  Per 16 values of K that is
// 11 MMAs of N = 64..256: 7 onto levels 6..8 and 4 onto levels 2..5.
//
// CTA tile: 128 rows (TMEM lanes) x 64 columns.  K advances in stages of 32:
// one stage holds the 7 slices of the A tile and of the B tile (84 KiB, two
// 3-D TMA loads with 64-byte swizzle), and two stages are in flight.  18
// warps: warp 16 issues the TMA loads, warp 17 the MMAs (levels 6..8 first),
// warps 0-15 (four per TMEM lane quarter, 16 columns each) read levels 2..5
// at the end of each window while the next stage's MMAs onto levels 6..8
// run, and at the end of a block they form its outputs (several warps per
// scheduler, so the integer epilogue's latency is hidden).  A CTA may own
// several output blocks: the producer and the issuer then run on into the
// next block as soon as the readers have emptied TMEM, so that one block's
// outputs are formed while the next block's products run.
// All waits are bounded (1 s): a timeout records DG_ERR_TIMEOUT and the CTA
// drains and returns.
#include <cuda_bf16.h>
#include <limits.h>

#include <atomic>

#include "dg_common.cuh"
#include "runtime.h"
#include "tc_ptx.cuh"

namespace dg {
namespace {

using namespace ptx;

constexpr int OZ_S = kOzSlices;                           // slices per operand (7)
constexpr int kOzNonFinite = 1 << 30;                     // exponent of a non-finite vector
#ifndef OZ_STAGE_K
#define OZ_STAGE_K 32
#endif
constexpr int OZ_BM = 128, OZ_BN = 64, OZ_BK = OZ_STAGE_K;  // K per stage (16 or 32)
constexpr int OZ_WIN = 160 / OZ_BK;                       // stages per exact window (K 160)
constexpr int OZ_A_SLICE = OZ_BM * OZ_BK * 2;             // 8 KiB at K 32
constexpr int OZ_B_SLICE = OZ_BN * OZ_BK * 2;             // 4 KiB at K 32
constexpr int OZ_STAGE = OZ_S * (OZ_A_SLICE + OZ_B_SLICE);  // 84 KiB at K 32
constexpr int OZ_STAGES = (220 * 1024 - 1536) / OZ_STAGE;  // 2 at K 32, 5 at K 16
static_assert(OZ_BK == 16 || OZ_BK == 32, "stage K is 16 (32-byte swizzle) or 32 (64-byte)");
constexpr int OZ_SMEM = OZ_STAGES * OZ_STAGE + 1024 + 512;
// Fraction bits kept below 2^-40 when levels 6..8 join the integer sum: 11
// for K <= 1024, one fewer per doubling of K, so |sum| * 2^guard stays below
// 2^62 (|sum| < 2^50 K / 1024).  K may reach kOzMaxK.
constexpr int kOzMaxK = 131072;
constexpr int OZ_READERS = 16;                            // reader warps: 4 per TMEM lane quarter
constexpr int OZ_RCOLS = OZ_BN / (OZ_READERS / 4);        // columns per reader thread (16)
constexpr int OZ_PRODUCER = OZ_READERS, OZ_ISSUER = OZ_READERS + 1;
constexpr int OZ_THREADS = 32 * (OZ_READERS + 2);

struct OzParams {
  CUtensorMap a, b;                 // 3-D maps: {K, rows, slice}
  const unsigned long long *ma, *mb;  // scale words per A row / per B row
  double *c;
  long long ldc;
  int m, n, k;
  double alpha, beta;
  int tri;                // 1: store only i <= j, 2: only i >= j
  int *status;            // skip when non-zero; DG_ERR_TIMEOUT recorded here
  const int *abort2;      // skip when non-zero (read only)
  const double *dscale;   // when set, beta of row i (dmode 1) / column j (dmode 2) is dscale[.]
  int dmode;
  int guard;              // fraction bits below 2^-40 of the integer sum
  int blocks;             // 128 x 64 output blocks of the stored part
};

// frexp exponent of the non-negative double with bits b (0 for 0).
__device__ __forceinline__ int exponent_of(unsigned long long b) {
  const int eb = (int)(b >> 52);
  if (eb >= 0x7FF) return kOzNonFinite;
  if (eb) return eb - 1022;
  if (b == 0) return 0;
  return (63 - __clzll((long long)b)) + 1 - 1074;  // subnormal: b * 2^-1074
}

// Results outside the normal range (overflow, subnormal): the library's
// scaling, kept out of line so that the common path stays integer-only.
__device__ __noinline__ double scale_slow(unsigned long long sign, int p, unsigned long long mant,
                                          int E) {
  return ldexp(__longlong_as_double((long long)(sign | ((unsigned long long)(p + 1023) << 52) |
                                                (mant & 0xFFFFFFFFFFFFFull))),
               E);
}

// T * 2^E as a double, rounded to nearest even once (T < 2^63 in magnitude).
__device__ __forceinline__ double int_to_double_scaled(long long T, int E) {
  if (T == 0) return 0.0;
  const unsigned long long sign = T < 0 ? (1ull << 63) : 0ull;
  unsigned long long u = T < 0 ? 0ull - (unsigned long long)T : (unsigned long long)T;
  int p = 63 - __clzll((long long)u);  // leading bit
  unsigned long long mant;
  if (p <= 52) {
    mant = u << (52 - p);
  } else {
    const int sh = p - 52;
    mant = u >> sh;
    const unsigned long long rem = u & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (mant & 1))) mant++;
    if (mant >> 53) {
      mant >>= 1;
      p++;
    }
  }
  const int biased = p + E + 1023;
  if (biased >= 1 && biased <= 2046)
    return __longlong_as_double(
        (long long)(sign | ((unsigned long long)biased << 52) | (mant & 0xFFFFFFFFFFFFFull)));
  return scale_slow(sign, p, mant, E);
}

// Output blocks (128 x 64) that hold part of the stored triangle in block
// column bj: row blocks lo .. lo + count - 1 (all mblk of them when tri = 0).
__host__ __device__ __forceinline__ int oz_col_blocks(int tri, int bj, int mblk, int &lo) {
  int hi = mblk;
  lo = 0;
  if (tri == 1) {  // i <= j: rows below (64 bj + 63) only
    const int h = (bj * OZ_BN + OZ_BN - 1) / OZ_BM + 1;
    hi = h < mblk ? h : mblk;
  } else if (tri == 2) {  // i >= j: rows from 64 bj on
    lo = (bj * OZ_BN) / OZ_BM;
  }
  return hi > lo ? hi - lo : 0;
}

// Row blocks per group of the full-matrix walk: the CTAs of one wave share
// the slices of 1024 rows of A and of the few block columns of B they are at.
constexpr int OZ_GROUP = 8;

// Origin of the v-th output block of the stored part.  Full C: groups of
// OZ_GROUP row blocks, each walked column by column (row blocks fastest), so
// that the blocks in flight at once read a compact set of slices from L2
// (going down whole block columns of a tall C streams all of A through L2
// once per block column).  One triangle: column by column.
__device__ __forceinline__ void oz_block(const OzParams &p, int v, int mblk, int nblk, int &i0,
                                         int &j0) {
  if (p.tri == 0) {
    const int g = v / (OZ_GROUP * nblk), local = v - g * (OZ_GROUP * nblk);
    const int rows = min(OZ_GROUP, mblk - g * OZ_GROUP);
    i0 = (g * OZ_GROUP + local % rows) * OZ_BM;
    j0 = (local / rows) * OZ_BN;
    return;
  }
  i0 = j0 = 0;
  for (int bj = 0; bj < nblk; bj++) {
    int lo;
    const int c = oz_col_blocks(p.tri, bj, mblk, lo);
    if (v < c) {
      i0 = (lo + v) * OZ_BM;
      j0 = bj * OZ_BN;
      return;
    }
    v -= c;
  }
}

// The same decision in every lane of a warp (the TMEM loads are warp-wide).
__device__ __forceinline__ bool warp_aborted(const int *flag) {
  return __any_sync(0xffffffffu, *(const volatile int *)flag != 0);
}

// One CTA computes the output blocks v = blockIdx.x, + gridDim.x, ... of
// the stored part (p.blocks of them).  Its TMA producer and MMA issuer run
// ahead across block boundaries: the next block's stages are loaded while
// the current block's last MMAs run, and its MMAs start as soon as the
// readers have taken the current block's accumulators out of TMEM, so that
// the outputs are formed (C read, integer sum rounded, C written) while the
// tensor cores work on the next block.
__global__ void __launch_bounds__(OZ_THREADS, 1) oz_gemm_kernel(const __grid_constant__ OzParams p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + OZ_STAGES * OZ_STAGE);
  uint64_t *empty = full + OZ_STAGES;
  uint64_t *ready = empty + OZ_STAGES;   // MMA -> readers: a window's exact sums complete
  uint64_t *drained = ready + 1;         // readers -> MMA: a window's accumulators read
  uint64_t *done = drained + 1;          // MMA -> readers: every MMA of the CTA complete
  uint32_t *tmem_slot = (uint32_t *)(done + 1);
  int *abort_flag = (int *)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mblk = (p.m + OZ_BM - 1) / OZ_BM, nblk = (p.n + OZ_BN - 1) / OZ_BN;
  // one read of the status words decides for the whole CTA
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
    mbar_init(drained, 32 * OZ_READERS);
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
  const int nst = (p.k + OZ_BK - 1) / OZ_BK;  // stages per block
  const int nwin = (nst + OZ_WIN - 1) / OZ_WIN;

  if (warp == OZ_PRODUCER) {
    if (lane == 0) {
      // ---------------- TMA producer ----------------
      int g = 0;  // stages loaded, over all blocks
      bool stop = false;
      for (int v = blockIdx.x; v < p.blocks && !stop; v += gridDim.x) {
        int i0, j0;
        oz_block(p, v, mblk, nblk, i0, j0);
        for (int it = 0; it < nst; it++, g++) {
          const int st = g % OZ_STAGES;
          if (*(volatile int *)abort_flag ||
              (g >= OZ_STAGES && !mbar_wait(&empty[st], ((g / OZ_STAGES) - 1) & 1))) {
            atomicExch(abort_flag, 1);
            stop = true;
            break;
          }
          uint8_t *dst = smem + st * OZ_STAGE;
          mbar_expect_tx(&full[st], OZ_STAGE);
          tma_load_3d(dst, &p.a, &full[st], it * OZ_BK, i0, 0);
          tma_load_3d(dst + OZ_S * OZ_A_SLICE, &p.b, &full[st], it * OZ_BK, j0, 0);
        }
      }
      // drain the loads in flight
      for (int q = (g > OZ_STAGES ? g - OZ_STAGES : 0); q < g; q++)
        if (!mbar_wait(&full[q % OZ_STAGES], (q / OZ_STAGES) & 1)) atomicExch(abort_flag, 1);
    }
    __syncwarp();
  } else if (warp == OZ_ISSUER) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      const uint32_t idesc64 = idesc_f16kind(OZ_BM, OZ_BN, false);  // N = 64 c: + (8 (c-1)) << 17
      const uint32_t sbase = smem_u32(smem);
      int g = 0, gw = 0;  // stages and windows issued, over all blocks
      bool stop = false, any = false;
      for (int v = blockIdx.x; v < p.blocks && !stop; v += gridDim.x) {
        for (int it = 0; it < nst; it++, g++) {
          const int st = g % OZ_STAGES, wpos = it % OZ_WIN;
          if (!mbar_wait(&full[st], (g / OZ_STAGES) & 1)) {
            atomicExch(abort_flag, 1);
            stop = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          // descriptors: base + (byte offset >> 4)
          const uint32_t sa = sbase + st * OZ_STAGE, sb = sa + OZ_S * OZ_A_SLICE;
          const uint64_t da = OZ_BK == 32 ? sw64_desc(sa) : sw32_desc(sa);
          const uint64_t db = OZ_BK == 32 ? sw64_desc(sb) : sw32_desc(sb);
          // A_s x [B_t .. B_u] onto levels s+t .. s+u (TMEM column 64 (s+t-2))
          auto mma_run = [&](int kk, int s_, int t, int u, uint32_t acc) {
            mma_bf16(tmem + 64 * (s_ + t - 2), da + (((s_ - 1) * OZ_A_SLICE + kk * 32) >> 4),
                     db + (((t - 1) * OZ_B_SLICE + kk * 32) >> 4),
                     idesc64 + ((uint32_t)(8 * (u - t)) << 17), acc);
          };
          // a new block resets levels 6..8 too: the previous block's sums
          // (all levels) must have been read
          if (it == 0 && gw > 0) {
            if (!mbar_wait(drained, (gw - 1) & 1)) {
              atomicExch(abort_flag, 1);
              stop = true;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          }
          any = true;
          // levels 6..8: t from max(1, 6 - s) to 8 - s; the block's first MMA
          // (s = 1, levels 6..8) sets them
#pragma unroll
          for (int kk = 0; kk < OZ_BK / 16; kk++)
#pragma unroll
            for (int s_ = 1; s_ <= OZ_S; s_++)
              mma_run(kk, s_, 6 - s_ > 1 ? 6 - s_ : 1, 8 - s_,
                      (it == 0 && kk == 0 && s_ == 1) ? 0u : 1u);
          // levels 2..5: the previous window's sums must have been read
          if (wpos == 0 && it > 0) {
            if (!mbar_wait(drained, (gw - 1) & 1)) {
              atomicExch(abort_flag, 1);
              stop = true;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          }
          const uint32_t first = (wpos == 0) ? 0u : 1u;
#pragma unroll
          for (int kk = 0; kk < OZ_BK / 16; kk++) {
            const uint32_t a0 = (kk == 0) ? first : 1u;
            mma_run(kk, 1, 1, 4, a0);   // levels 2..5
            mma_run(kk, 2, 1, 3, 1u);   // levels 3..5
            mma_run(kk, 3, 1, 2, 1u);   // levels 4..5
            mma_run(kk, 4, 1, 1, 1u);   // level 5
          }
          mma_commit(&empty[st]);
          if (wpos == OZ_WIN - 1 || it == nst - 1) {
            mma_commit(ready);
            gw++;
          }
        }
      }
      if (any)
        mma_commit(done);
      else
        mbar_arrive(done);
    }
    __syncwarp();
  } else {
    // ---------------- readers ----------------
    // reader warp w: TMEM lanes 32 (w mod 4) .. + 31 (one output row per
    // thread), columns cb .. cb + 15 with cb = 16 (w / 4)
    const int cb = (warp >> 2) * OZ_RCOLS;
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    // levels 8, 7, 6 summed in FP32 join the integer sum at 2^-(40 + guard)
    // (|v| < 2^-21 K / 1024, so |v| 2^(40 + guard) < 2^30)
    const float unit6 = __int_as_float((127 + 40 + p.guard) << 23);
    int gw = 0;  // windows read, over all blocks
    for (int v = blockIdx.x; v < p.blocks; v += gridDim.x) {
      int i0, j0;
      oz_block(p, v, mblk, nblk, i0, j0);
      // the block's C into L2 while its products run
      for (int line = threadIdx.x; line < OZ_BN * (OZ_BM / 16); line += 32 * OZ_READERS) {
        const int col = j0 + line / (OZ_BM / 16), row = i0 + 16 * (line % (OZ_BM / 16));
        if (col < p.n && row < p.m)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(p.c + (size_t)row + (size_t)col * p.ldc));
      }
      long long acc[OZ_RCOLS];
#pragma unroll
      for (int c = 0; c < OZ_RCOLS; c++) acc[c] = 0;
      bool ok = !warp_aborted(abort_flag);
      for (int w = 0; w < nwin; w++, gw++) {
        if (ok) {
          ok = __all_sync(0xffffffffu, mbar_wait(ready, gw & 1));
          if (!ok) atomicExch(abort_flag, 1);
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (ok) {
#pragma unroll
          // level L holds an integer below 2^24 in units of 2^(-8L): to 32
          // bits, then shifted to units of 2^-40 (two levels per TMEM wait)
#pragma unroll
          for (int lvl = 2; lvl <= 5; lvl += 2) {
            const float up = __int_as_float((127 + 8 * lvl) << 23);  // 2^(8 lvl)
            const int sh = 8 * (5 - lvl);                            // x 2^(8 (5 - lvl))
#pragma unroll
            for (int ch = 0; ch < OZ_RCOLS; ch += 16) {
              float x[16], y[16];
              tmem_ld16x2(tmem + 64 * (lvl - 2) + cb + ch + lane_base,
                          tmem + 64 * (lvl - 1) + cb + ch + lane_base, x, y);
#pragma unroll
              for (int c = 0; c < 16; c++)
                acc[ch + c] +=
                    (long long)((unsigned long long)(long long)__float2int_rn(x[c] * up) << sh) +
                    (long long)((unsigned long long)(long long)__float2int_rn(y[c] * (up * 256.0f))
                                << (sh - 8));
            }
          }
          if (w == nwin - 1) {
#pragma unroll
            for (int ch = 0; ch < OZ_RCOLS; ch += 16) {
              float x[16], y[16];
              tmem_ld16(tmem + 64 * 6 + cb + ch + lane_base, x);
              tmem_ld16(tmem + 64 * 5 + cb + ch + lane_base, y);
#pragma unroll
              for (int c = 0; c < 16; c++) x[c] = y[c] + x[c];
              tmem_ld16(tmem + 64 * 4 + cb + ch + lane_base, y);
#pragma unroll
              for (int c = 0; c < 16; c++)
                acc[ch + c] = (long long)((unsigned long long)acc[ch + c] << p.guard) +
                              (long long)__float2int_rn((y[c] + x[c]) * unit6);
            }
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        mbar_arrive(drained);
      }
      const int row = i0 + (warp & 3) * 32 + lane;
      if (!ok || row >= p.m) continue;
      // the block's outputs, while the tensor cores run the next block
      const int ea = exponent_of(p.ma[row]);
      const bool fast = (p.alpha == -1.0 && p.beta == 1.0);
#pragma unroll
      for (int ch = 0; ch < OZ_RCOLS; ch += 8) {
        double old[8];
        int eb[8];
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const int col = j0 + cb + ch + c;
          const bool in = col < p.n && !(p.tri == 1 && row > col) && !(p.tri == 2 && row < col);
          old[c] = (in && (p.beta != 0.0 || p.dmode)) ? p.c[(size_t)row + (size_t)col * p.ldc] : 0.0;
          eb[c] = col < p.n ? exponent_of(p.mb[col]) : 0;
        }
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const int col = j0 + cb + ch + c;
          if (col >= p.n || (p.tri == 1 && row > col) || (p.tri == 2 && row < col)) continue;
          double vout;
          if (ea == kOzNonFinite || eb[c] == kOzNonFinite) {
            vout = __longlong_as_double(0x7FF8000000000000ll);
          } else {
            const double x = int_to_double_scaled(acc[ch + c], ea + eb[c] - 40 - p.guard);
            if (fast)
              vout = old[c] - x;
            else if (p.dmode)
              vout = fma(p.dscale[p.dmode == 1 ? row : col], old[c], p.alpha * x);
            else
              vout = (p.beta != 0.0) ? fma(p.alpha, x, p.beta * old[c]) : p.alpha * x;
          }
          p.c[(size_t)row + (size_t)col * p.ldc] = vout;
        }
      }
    }
  }

  // every MMA complete before TMEM is freed
  if (threadIdx.x == 0 && !mbar_wait(done, 0)) atomicExch(abort_flag, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (*(volatile int *)abort_flag != 0 && threadIdx.x == 0 && p.status)
    atomicCAS(p.status, 0, DG_ERR_TIMEOUT);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512)
                 : "memory");
}

// ---------------------------------------------------------------------------
// splitting
// ---------------------------------------------------------------------------
constexpr int SPLIT_V = 32;    // vectors per CTA
constexpr int MAX_K = 256;     // values of K per scale CTA
constexpr int SPLIT_K = 64;    // values of K per slicing CTA

// Where the split reads: element k of vector c at p[c*cs + k*ks], or, for a
// tile grid (tiles != nullptr), row c and column k of the n x n matrix whose
// nb x nb tile (i, j) is tiles[i + j*mt] (column-major, ld = its row count).
struct OzSrc {
  const double *p;
  long long cs, ks;
  const double *const *tiles;
  int nb, mt, n;
  int lg;  // log2(nb) when nb is a power of two (the tile index is a shift), else -1
  __device__ __forceinline__ double at(int c, int k) const {
    if (!tiles) return p[(size_t)c * cs + (size_t)k * ks];
    const int ti = lg >= 0 ? c >> lg : c / nb, tj = lg >= 0 ? k >> lg : k / nb;
    const int ld = min(nb, n - ti * nb);
    return tiles[ti + (size_t)tj * mt][(size_t)(c - ti * nb) + (size_t)(k - tj * nb) * ld];
  }
  // lanes along the contiguous direction: k for columns, c for rows and tiles
  __device__ __forceinline__ bool k_contiguous() const { return !tiles && ks == 1; }
};

__device__ __forceinline__ unsigned long long abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
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

// Scale words of `ncols` vectors of length K (element k of vector c at
// src[c*cstride + k*kstride]): the maximum of |v|'s bit pattern, by atomic
// maximum over CTAs of 32 vectors x 256 values of K (the words start at 0).
// CTA: 32 x 8 threads reading along whichever of k or c is contiguous.
__global__ void __launch_bounds__(256) oz_max_kernel(OzSrc src, int K, int ncols,
                                                    unsigned long long *mb, int zero_diag,
                                                    const int *abort_flag, const int *abort2) {
  if (aborted(abort_flag, abort2)) return;
  __shared__ unsigned long long red[8][SPLIT_V + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int c0 = blockIdx.x * SPLIT_V, k0 = blockIdx.y * MAX_K;
  const int k1 = min(K, k0 + MAX_K);
  if (src.k_contiguous()) {  // columns: lanes along k, warp ty over vectors ty, ty+8, ...
#pragma unroll
    for (int i = 0; i < SPLIT_V / 8; i++) {
      const int c = c0 + ty + 8 * i;
      unsigned long long m = 0;
      if (c < ncols) {
        const double *v = src.p + (size_t)c * src.cs;
#pragma unroll
        for (int j = 0; j < MAX_K / 32; j++) {
          const int k = k0 + tx + 32 * j;
          const unsigned long long a = (k < k1 && !(zero_diag && k == c)) ? abs_bits(v[k]) : 0ull;
          m = a > m ? a : m;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long q = __shfl_xor_sync(0xffffffffu, m, o);
        m = q > m ? q : m;
      }
      if (tx == 0 && c < ncols && m) atomicMax(mb + c, m);
    }
  } else {             // rows (or general strides): lanes along vectors, warps along k
    const int c = c0 + tx;
    unsigned long long m = 0;
    if (c < ncols) {
#pragma unroll 8
      for (int k = k0 + ty; k < k1; k += 8) {
        const unsigned long long a = (zero_diag && k == c) ? 0ull : abs_bits(src.at(c, k));
        m = a > m ? a : m;
      }
    }
    red[ty][tx] = m;
    __syncthreads();
    if (ty == 0 && c < ncols) {
      for (int y = 1; y < 8; y++) m = red[y][tx] > m ? red[y][tx] : m;
      if (m) atomicMax(mb + c, m);
    }
  }
}

// Slices of the vectors [32 bx, 32 bx + 32) over k in [64 by, 64 by + 64)
// (k < ldk; zeros for k >= K): slice s (0-based) of vector c at
// dst + s*sstride + c*ldk.  The 32 x 64 values pass through shared memory so
// that the reads are coalesced in either orientation; each thread then cuts 8
// consecutive values of one vector into 7 slices and writes 16 bytes per slice.
__global__ void __launch_bounds__(256) oz_slice_kernel(OzSrc src, int K, int ncols,
                                                      __nv_bfloat16 *dst, long long ldk,
                                                      long long sstride,
                                                      const unsigned long long *mb,
                                                      double *diag_out, const int *abort_flag,
                                                      const int *abort2) {
  if (aborted(abort_flag, abort2)) return;
  __shared__ double tile[SPLIT_V][SPLIT_K + 1];
  __shared__ int ex[SPLIT_V];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
  const int c0 = blockIdx.x * SPLIT_V, kc = blockIdx.y * SPLIT_K;
  if (ty == 0) ex[tx] = (c0 + tx < ncols) ? exponent_of(mb[c0 + tx]) : 0;
  if (src.k_contiguous()) {
    for (int vi = ty; vi < SPLIT_V; vi += 8) {
      const int c = c0 + vi;
#pragma unroll
      for (int h = 0; h < SPLIT_K; h += 32) {
        const int k = kc + h + tx;
        tile[vi][h + tx] = (c < ncols && k < K) ? src.p[(size_t)c * src.cs + k] : 0.0;
      }
    }
  } else {
    const int c = c0 + tx;
#pragma unroll
    for (int kk = ty; kk < SPLIT_K; kk += 8) {
      const int k = kc + kk;
      tile[tx][kk] = (c < ncols && k < K) ? src.at(c, k) : 0.0;
    }
  }
  __syncthreads();
  const int vi = tid >> 3, k0 = 8 * (tid & 7);  // 8 values of one vector
  const int c = c0 + vi;
  if (c >= ncols || kc + k0 >= ldk) return;
  // diag_out: element c of vector c goes there instead of into the slices
  const int kd = (diag_out && c >= kc + k0 && c < kc + k0 + 8) ? c - kc - k0 : -1;
  if (kd >= 0) {
    diag_out[c] = tile[vi][k0 + kd];
    tile[vi][k0 + kd] = 0.0;
  }
  const int e = ex[vi];
  uint32_t packed[OZ_S][4];  // slice s: 8 BF16 values
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    uint32_t lo[OZ_S], hi[OZ_S];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      long long X = (e == kOzNonFinite) ? 0 : scaled56(tile[vi][k0 + j + h], e);
#pragma unroll
      for (int s_ = OZ_S; s_ >= 1; s_--) {
        const long long d = (s_ > 1) ? ((X + 128) & 255) - 128 : X;
        X = (X - d) >> 8;
        // d 2^(-8 s) has at most 8 significant bits: its BF16 is the FP32's top half
        const uint32_t b =
            __float_as_uint((float)(int)d * __int_as_float((127 - 8 * s_) << 23)) >> 16;
        if (h == 0) lo[s_ - 1] = b; else hi[s_ - 1] = b;
      }
    }
#pragma unroll
    for (int s_ = 0; s_ < OZ_S; s_++) packed[s_][j >> 1] = lo[s_] | (hi[s_] << 16);
  }
  __nv_bfloat16 *out = dst + (size_t)c * ldk + kc + k0;
#pragma unroll
  for (int s_ = 0; s_ < OZ_S; s_++)
    *reinterpret_cast<uint4 *>(out + (size_t)s_ * sstride) =
        make_uint4(packed[s_][0], packed[s_][1], packed[s_][2], packed[s_][3]);
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
             CU_TENSOR_MAP_INTERLEAVE_NONE,
             OZ_BK == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

static int split_from(const OzSrc &src, int K, int ncols, void *slices, long long ldk,
                      long long sstride, unsigned long long *scales, const int *abort_flag,
                      cudaStream_t s, const int *abort2, double *diag_out) {
  if (ncols <= 0) return 0;
  DG_CUDA_TRY(cudaMemsetAsync(scales, 0, sizeof(unsigned long long) * (size_t)ncols, s));
  const dim3 blk(32, 8);
  const int nv = (ncols + SPLIT_V - 1) / SPLIT_V;
  oz_max_kernel<<<dim3(nv, (K + MAX_K - 1) / MAX_K), blk, 0, s>>>(
      src, K, ncols, scales, diag_out ? 1 : 0, abort_flag, abort2);
  DG_CUDA_TRY(cudaGetLastError());
  const dim3 grid(nv, (unsigned)((ldk + SPLIT_K - 1) / SPLIT_K));
  oz_slice_kernel<<<grid, blk, 0, s>>>(src, K, ncols, (__nv_bfloat16 *)slices, ldk, sstride,
                                       scales, diag_out, abort_flag, abort2);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(2);
  return 0;
}

int oz_split(const double *src, long long cstride, long long kstride, int K, int ncols,
             void *slices, long long ldk, long long sstride, unsigned long long *scales,
             const int *abort_flag, cudaStream_t s, const int *abort2, double *diag_out) {
  OzSrc q;
  q.p = src; q.cs = cstride; q.ks = kstride; q.tiles = nullptr; q.nb = q.mt = q.n = 0; q.lg = -1;
  return split_from(q, K, ncols, slices, ldk, sstride, scales, abort_flag, s, abort2, diag_out);
}

int oz_split_tile_rows(const double *const *tiles_dev, int n, int nb, void *slices, long long ldk,
                       unsigned long long *scales, const int *abort_flag, cudaStream_t s) {
  if (n > kOzMaxK) return DG_ERR_UNSUPPORTED;
  OzSrc q;
  q.p = nullptr; q.cs = q.ks = 0; q.tiles = tiles_dev; q.nb = nb; q.mt = (n + nb - 1) / nb; q.n = n;
  q.lg = -1;
  for (int l = 0; l < 31; l++)
    if ((1 << l) == nb) q.lg = l;
  return split_from(q, n, n, slices, ldk, ldk * n, scales, abort_flag, s, nullptr, nullptr);
}

int oz_gemm(int m, int n, int k, double alpha, const void *a_slices, long long lda_k,
            long long a_sstride, const unsigned long long *ma, const void *b_slices,
            long long ldb_k, long long b_sstride, const unsigned long long *mb, double beta,
            double *C, long long ldc, int tri, int *status, cudaStream_t s, const int *abort2,
            const double *dscale, int dmode, int blocks_per_cta) {
  if (m <= 0 || n <= 0) return 0;
  if (k <= 0 || k > kOzMaxK || lda_k % 8 || ldb_k % 8) return DG_ERR_UNSUPPORTED;
  if (lda_k < k || ldb_k < k) return DG_ERR_UNSUPPORTED;
  OzParams p;
  memset(&p, 0, sizeof p);
  if (!oz_map(&p.a, a_slices, lda_k, m, a_sstride, OZ_BM) ||
      !oz_map(&p.b, b_slices, ldb_k, n, b_sstride, OZ_BN)) {
    dg_set_last_error(__FILE__, __LINE__, "cuTensorMapEncodeTiled failed");
    return DG_ERR_CUDA;
  }
  p.ma = ma; p.mb = mb; p.c = C; p.ldc = ldc;
  p.m = m; p.n = n; p.k = k; p.alpha = alpha; p.beta = beta; p.tri = tri;
  p.status = status;
  p.abort2 = abort2;
  p.dscale = dscale;
  p.dmode = dscale ? dmode : 0;
  p.guard = 11;
  for (long long kk = 1024; kk < k; kk *= 2) p.guard--;
  static std::atomic<bool> attr[64];  // zero-initialised: false
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr[dev & 63]) {
    DG_CUDA_TRY(cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     OZ_SMEM));
    attr[dev & 63] = true;
  }
  const int mblk = (m + OZ_BM - 1) / OZ_BM, nblk = (n + OZ_BN - 1) / OZ_BN;
  long long blocks = 0;
  for (int bj = 0; bj < nblk; bj++) {
    int lo;
    blocks += oz_col_blocks(tri, bj, mblk, lo);
  }
  if (blocks == 0) return 0;
  if (blocks > INT_MAX) return DG_ERR_UNSUPPORTED;
  p.blocks = (int)blocks;
  int per = blocks_per_cta;
  if (per <= 0) {  // one wave: ceil(blocks / SMs) blocks per CTA
    const int sms = dg_num_sms();
    per = (int)((blocks + sms - 1) / sms);
  }
  const long long ctas = (blocks + per - 1) / per;
  oz_gemm_kernel<<<(unsigned)ctas, OZ_THREADS, OZ_SMEM, s>>>(p);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

static size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t oz_scratch_bytes(int m, int n, int k, bool same) {
  const size_t ldk = (size_t)(k + 7) / 8 * 8;
  size_t b = round256((size_t)OZ_S * ldk * m * 2) + round256((size_t)m * 8);
  if (!same) b += round256((size_t)OZ_S * ldk * n * 2) + round256((size_t)n * 8);
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
  if (k <= 0 || k > kOzMaxK || !scratch || oz_scratch_bytes(m, n, k, same) > bytes) return 1;
  const long long ldk = (k + 7) / 8 * 8;
  char *q = (char *)scratch;
  void *sa = q;
  q += round256((size_t)OZ_S * ldk * m * 2);
  unsigned long long *ma = (unsigned long long *)q;
  q += round256((size_t)m * 8);
  void *sb = sa;
  unsigned long long *mb = ma;
  // row i of op(A), element p: A[i + p lda] ('N') or A[p + i lda] ('T')
  DG_TRY(oz_split(A, tA ? lda : 1, tA ? 1 : lda, k, m, sa, ldk, ldk * m, ma, status, s, abort2));
  if (!same) {
    sb = q;
    q += round256((size_t)OZ_S * ldk * n * 2);
    mb = (unsigned long long *)q;
    // column j of op(B), element p: B[p + j ldb] ('N') or B[j + p ldb] ('T')
    DG_TRY(oz_split(B, tB ? 1 : ldb, tB ? ldb : 1, k, n, sb, ldk, ldk * n, mb, status, s, abort2));
  }
  return oz_gemm(m, n, k, alpha, sa, ldk, ldk * m, ma, sb, ldk, same ? ldk * m : ldk * n, mb, beta,
                 C, ldc, tri, status, s, abort2, nullptr, 0, 0);
}

}  // namespace dg

// Building block exposed for tests: C = alpha op(A) op(B) + beta C in FP64
// through the emulated path, with op(A) = A' (A is k x m) and op(B) = B
// (k x n), both column-major, k <= 131072.  Uses stream-ordered scratch.
extern "C" int dg_gemm_f64_emulated_tn(int m, int n, int k, double alpha, const double *A, int lda,
                                       const double *B, int ldb, double beta, double *C, int ldc,
                                       void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(k > 0 && k <= dg::kOzMaxK, 3);
  DG_CHECK_ARG(lda >= k, 6);
  DG_CHECK_ARG(ldb >= k, 8);
  DG_CHECK_ARG(ldc >= (m > 1 ? m : 1), 11);
  if (m == 0 || n == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = dg::oz_scratch_bytes(m, n, k, false);
  void *buf = nullptr;
  DG_CUDA_TRY(dg::pool_malloc_async(&buf, bytes, s));
  int rc = dg::oz_gemm_general('T', 'N', m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, 0, buf,
                               bytes, nullptr, nullptr, s);
  cudaFreeAsync(buf, s);
  return rc;
}

// The two stages of dg_gemm_f64_emulated_tn as separate calls, for callers
// that reuse the slices of one operand across many products (the tiles of a
// factor, the matrix of a refinement residual).
extern "C" int dg_f64_slices(int k, int ncols, const double *src, long long cstride,
                             long long kstride, void *slices, int ldk, void *scales,
                             void *stream) {
  DG_CHECK_ARG(k > 0 && k <= dg::kOzMaxK, 1);
  DG_CHECK_ARG(ncols >= 0, 2);
  DG_CHECK_ARG(ldk >= k && ldk % 8 == 0, 7);
  DG_CHECK_ARG(((uintptr_t)slices & 15) == 0, 6);
  DG_CHECK_ARG(((uintptr_t)scales & 7) == 0, 8);
  return dg::oz_split(src, cstride, kstride, k, ncols, slices, ldk, (long long)ldk * ncols,
                      (unsigned long long *)scales, nullptr, (cudaStream_t)stream);
}

extern "C" int dg_gemm_f64_slices(int m, int n, int k, double alpha, const void *a_slices,
                                  int lda_k, const void *a_scales, const void *b_slices, int ldb_k,
                                  const void *b_scales, double beta, double *C, int ldc,
                                  int *status, void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(k > 0 && k <= dg::kOzMaxK, 3);
  DG_CHECK_ARG(lda_k >= k && lda_k % 8 == 0, 6);
  DG_CHECK_ARG(ldb_k >= k && ldb_k % 8 == 0, 9);
  DG_CHECK_ARG(ldc >= (m > 1 ? m : 1), 13);
  return dg::oz_gemm(m, n, k, alpha, a_slices, lda_k, (long long)lda_k * m,
                     (const unsigned long long *)a_scales, b_slices, ldb_k, (long long)ldb_k * n,
                     (const unsigned long long *)b_scales, beta, C, ldc, 0, status,
                     (cudaStream_t)stream, nullptr, nullptr, 0, 0);
}
