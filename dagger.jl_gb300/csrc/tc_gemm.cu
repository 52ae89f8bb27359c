// BF16 tensor-core GEMM on tcgen05 with TMEM accumulators and TMA-staged
// operands: the trailing SYRK/GEMM update of the mixed-precision Cholesky.
//
//   C(i, j) <- alpha * sum_t sum_p A_t(p, i) * B_t(p, j) + beta * C(i, j)
//
// A and B are "K-major" BF16 panels: row i of the panel holds the K values
// A(0..K-1, i) contiguously (a column-major nb x n tile of the factor's row
// panel is already in this order).  With `terms` = 3 the operands are given
// as hi/lo BF16 pairs (x = hi + lo, lo = bf16(x - hi)) and the three products
// hi*hi + hi*lo + lo*hi accumulate into the same FP32 TMEM accumulator,
// carrying about 16 significant bits per operand instead of 8.
//
// With `terms` = 6 each operand is given as three BF16 slices (x = hi + mid
// + lo, each slice the rounding of what the previous ones leave) and the six
// products whose slice orders sum to at most 4 (hh, hm, mh, hl, mm, lh)
// accumulate together: about 24 significant bits, an FP32-accurate product
// on the BF16 tensor cores (the panel solve of the mixed factor).
//
// FP8 form (persistent kernel only): E4M3 operands, each vector scaled by a
// power of two so that its largest magnitude lies in [128, 256) before the
// rounding (split_e4m3), one kind::f8f6f4 product (K = 32 per instruction, at
// twice the BF16 rate), and the two vectors' scales applied in the epilogue.
// Each operand value carries 4 significant bits.
//
// One CTA computes a 128 x BN tile of C with 4 warps:
//   warp 0, one thread   TMA producer: per K-block of 64, loads the A and B
//                        slabs (128B-swizzled, 1024-byte aligned stages) and
//                        arms the stage's "full" mbarrier with the byte count
//   warp 1, one thread   MMA issuer: waits "full", issues 4 (x terms)
//                        tcgen05.mma kind::f16 (M=128, N=BN, K=16) into TMEM,
//                        and tcgen05.commit's the stage's "empty" mbarrier so
//                        the producer can refill it; a final commit arms
//                        the accumulator barrier
//   warps 0-3            epilogue: tcgen05.ld 32x32b.x32 of their 32 TMEM
//                        lanes (rows), then a coalesced read-modify-write of C
// Output addressing: plain column-major C, or the packed upper row-panel
// layout of the mixed factor (row panel r holds columns r*nb..n-1 of rows
// r*nb..r*nb+nb-1, column-major with leading dimension nb), where only the
// upper triangle (i <= j) is updated.
//
// Every mbarrier wait is bounded by the global timer (about 2 s).  A wait that
// gives up records DG_ERR_TIMEOUT in the status word, stops issuing, drains
// the copies and MMAs already issued (again bounded), frees its TMEM and
// returns; nothing traps.
#include <cuda.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <atomic>

#include "dg_common.cuh"
#include "runtime.h"
#include "tc_gemm.h"
#include "tc_ptx.cuh"

namespace dg {
namespace {

constexpr int BM = 128, BK = 64;

using namespace ptx;

template <int BN, int TERMS>
struct Smem {
  static constexpr int A_BYTES = BM * BK * 2;
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int SLICES = TERMS == 1 ? 1 : (TERMS == 3 ? 2 : 3);
  static constexpr int STAGE_BYTES = SLICES * (A_BYTES + B_BYTES);
  static constexpr int STAGES = TERMS == 1 ? 4 : (TERMS == 3 ? (BN == 128 ? 3 : 2) : 2);
  static constexpr int TOTAL = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
};

template <int BN, int TERMS>
__global__ void __launch_bounds__(128, 1) tc_gemm_kernel(const __grid_constant__ TcParams p) {
  using S = Smem<BN, TERMS>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + S::STAGES * S::STAGE_BYTES);
  uint64_t *empty = full + S::STAGES;
  uint64_t *accum = empty + S::STAGES;
  uint32_t *tmem_slot = (uint32_t *)(accum + 1);
  int *abort_flag = (int *)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int bi = blockIdx.x, bj = blockIdx.y;
  const int i0 = bi * BM, j0 = bj * BN;
  // tiles wholly below the diagonal of an upper-triangular update do nothing
  if (p.upper && i0 > j0 + BN - 1) return;
  if (p.status && *(volatile int *)p.status) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S::STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const int nk = (p.k + BK - 1) / BK;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer ----------------
    int issued = 0;
    for (int kb = 0; kb < nk; kb++) {
      const int s = kb % S::STAGES;
      const uint32_t round = kb / S::STAGES;
      if (kb >= S::STAGES && !mbar_wait(&empty[s], (round - 1) & 1)) {
        atomicExch(abort_flag, 1);
        break;
      }
      if (*(volatile int *)abort_flag) break;
      uint8_t *st = smem + s * S::STAGE_BYTES;
      mbar_expect_tx(&full[s], S::STAGE_BYTES);
      const int kx = kb * BK;
      tma_load_2d(st, &p.a_hi, &full[s], kx, p.a_row0 + i0);
      tma_load_2d(st + S::A_BYTES, &p.b_hi, &full[s], kx, p.b_row0 + j0);
      if (TERMS >= 3) {
        tma_load_2d(st + S::A_BYTES + S::B_BYTES, &p.a_lo, &full[s], kx, p.a_row0 + i0);
        tma_load_2d(st + 2 * S::A_BYTES + S::B_BYTES, &p.b_lo, &full[s], kx, p.b_row0 + j0);
      }
      if (TERMS == 6) {
        tma_load_2d(st + 2 * S::A_BYTES + 2 * S::B_BYTES, &p.a_mid, &full[s], kx, p.a_row0 + i0);
        tma_load_2d(st + 3 * S::A_BYTES + 2 * S::B_BYTES, &p.b_mid, &full[s], kx, p.b_row0 + j0);
      }
      issued++;
    }
    // drain: every load issued must land before the CTA may exit
    for (int kb = (issued > S::STAGES ? issued - S::STAGES : 0); kb < issued; kb++)
      if (!mbar_wait(&full[kb % S::STAGES], (kb / S::STAGES) & 1)) atomicExch(abort_flag, 1);
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t idesc = p.idesc;
    const uint32_t sbase = smem_u32(smem);
    int done = 0;
    for (int kb = 0; kb < nk; kb++) {
      const int s = kb % S::STAGES;
      if (!mbar_wait(&full[s], (kb / S::STAGES) & 1)) {
        atomicExch(abort_flag, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t st = sbase + s * S::STAGE_BYTES;
#pragma unroll
      for (int kk = 0; kk < BK / 16; kk++) {
        const uint32_t koff = kk * 32;  // 16 BF16 along K inside the swizzled row
        const uint64_t a = sw128_desc(st + koff);
        const uint64_t b = sw128_desc(st + S::A_BYTES + koff);
        mma_bf16(tmem, a, b, idesc, (kb | kk) ? 1u : 0u);
        if (TERMS >= 3) {
          const uint64_t alo = sw128_desc(st + S::A_BYTES + S::B_BYTES + koff);
          const uint64_t blo = sw128_desc(st + 2 * S::A_BYTES + S::B_BYTES + koff);
          if (TERMS == 3) {
            mma_bf16(tmem, a, blo, idesc, 1u);
            mma_bf16(tmem, alo, b, idesc, 1u);
          } else {
            // slice orders: hi 1, mid 2, lo 3; the products with order sum <= 4
            const uint64_t amid = sw128_desc(st + 2 * S::A_BYTES + 2 * S::B_BYTES + koff);
            const uint64_t bmid = sw128_desc(st + 3 * S::A_BYTES + 2 * S::B_BYTES + koff);
            mma_bf16(tmem, a, bmid, idesc, 1u);
            mma_bf16(tmem, amid, b, idesc, 1u);
            mma_bf16(tmem, a, blo, idesc, 1u);
            mma_bf16(tmem, amid, bmid, idesc, 1u);
            mma_bf16(tmem, alo, b, idesc, 1u);
          }
        }
      }
      mma_commit(&empty[s]);
      done++;
    }
    mma_commit(accum);
    (void)done;
  }
  __syncwarp();

  // ---------------- epilogue (all 4 warps) ----------------
  const bool ok = mbar_wait(accum, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!ok) atomicExch(abort_flag, 1);
  __syncthreads();
  const bool aborted = *(volatile int *)abort_flag != 0;
  const float alpha = p.alpha_dev ? *p.alpha_dev : p.alpha;
  if (!aborted && nk > 0) {
    const int row = i0 + warp * 32 + lane;  // TMEM lane == row of the tile
    for (int c0 = 0; c0 < BN; c0 += 32) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
      if (row >= p.m) continue;
      // Each lane owns one row; the 32 columns of the chunk are 32 separate
      // coalesced warp accesses.  All reads of C are issued before any write
      // so the read-modify-writes overlap instead of serialising.
      float *cp0;
      long long cstride;
      if (p.layout == 0) {
        cp0 = p.c + (size_t)row + (size_t)(j0 + c0) * p.ldc;
        cstride = p.ldc;
      } else {
        // packed upper row panels; global indices shifted by the trailing offset
        const long long gi = p.off + row;
        const long long r = gi / p.nb;
        const long long base = (long long)p.nb * (r * p.ntot - p.nb * r * (r - 1) / 2);
        cp0 = p.c + base + (gi - r * p.nb) + (p.off + j0 + c0 - r * p.nb) * p.nb;
        cstride = p.nb;
      }
      const bool upper = p.layout == 1 || p.upper;
      const bool read_c = p.layout == 1 || p.beta != 0.f;
      float old[32];
#pragma unroll
      for (int c = 0; c < 32; c++) {
        const int col = j0 + c0 + c;
        const bool in = col < p.n && !(upper && row > col);
        old[c] = (in && read_c) ? cp0[(size_t)c * cstride] : 0.f;
      }
#pragma unroll
      for (int c = 0; c < 32; c++) {
        const int col = j0 + c0 + c;
        if (col >= p.n || (upper && row > col)) continue;
        const float b = p.layout == 1 ? 1.f : p.beta;
        cp0[(size_t)c * cstride] = read_c ? fmaf(alpha, v[c], b * old[c]) : alpha * v[c];
      }
    }
  }
  if (aborted && threadIdx.x == 0 && p.status) atomicCAS(p.status, 0, DG_ERR_TIMEOUT);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN)
                 : "memory");
}

// ---------------------------------------------------------------------------
// Persistent form: one CTA per SM walks the output tiles (column by column of
// tiles, so the CTAs running together share a B tile in L2) with two TMEM
// accumulators, so the epilogue of one tile (TMEM -> registers -> the C
// read-modify-write) overlaps the products of the next.
//   warp 0, one thread   TMA producer over every tile's K blocks
//   warp 1, one thread   MMA issuer: waits for an empty accumulator, issues
//                        the tile's products into it, commits "accumulator
//                        full"
//   warps 2-5            epilogue: wait "full", read their TMEM lane quarter,
//                        update C, arrive on "accumulator empty"
// Every wait is bounded as in the one-tile kernel; a wait that gives up stops
// all three roles, drains what was issued, and records DG_ERR_TIMEOUT.
// ---------------------------------------------------------------------------
template <int BN, int TERMS>
struct SmemP {
  static constexpr int A_BYTES = BM * BK * 2;
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int SLICES = TERMS == 1 ? 1 : 2;
  static constexpr int STAGE_BYTES = SLICES * (A_BYTES + B_BYTES);
  static constexpr int STAGES = (196608 / STAGE_BYTES) < 8 ? (196608 / STAGE_BYTES) : 8;
  static constexpr int TOTAL = STAGES * STAGE_BYTES + 1024 + 256;
};

// F8: E4M3 operands (kind::f8f6f4).  A stage then holds 128 values of K per
// row (the same 128 bytes), and each product is scaled in the epilogue by
// the two vectors' power-of-two scales.
template <int BN, int TERMS, bool F8>
__global__ void __launch_bounds__(192, 1) tc_gemm_persist_kernel(const __grid_constant__ TcParams p) {
  using S = SmemP<BN, TERMS>;
  static_assert(!F8 || TERMS == 1, "the FP8 form has one product");
  constexpr int KE = F8 ? 2 * BK : BK;  // K values per stage
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + S::STAGES * S::STAGE_BYTES);
  uint64_t *empty = full + S::STAGES;
  uint64_t *accf = empty + S::STAGES;  // [2] accumulator full
  uint64_t *acce = accf + 2;           // [2] accumulator empty
  uint64_t *drain = acce + 2;
  uint32_t *tmem_slot = (uint32_t *)(drain + 1);
  int *abort_flag = (int *)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (p.status && *(volatile int *)p.status) return;
  const int mtiles = (p.m + BM - 1) / BM, ntiles = (p.n + BN - 1) / BN;
  const int total = mtiles * ntiles;
  const int nk = (p.k + KE - 1) / KE;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S::STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 4);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(2 * BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer ----------------
    uint32_t it = 0;
    bool stop = false;
    for (int t = blockIdx.x; t < total && !stop; t += gridDim.x) {
      const int i0 = (t % mtiles) * BM, j0 = (t / mtiles) * BN;
      if (p.upper && i0 > j0 + BN - 1) continue;
      for (int kb = 0; kb < nk; kb++, it++) {
        const int s = it % S::STAGES;
        if (it >= (uint32_t)S::STAGES && !mbar_wait(&empty[s], ((it / S::STAGES) - 1) & 1)) {
          atomicExch(abort_flag, 1);
          stop = true;
          break;
        }
        if (*(volatile int *)abort_flag) {
          stop = true;
          break;
        }
        uint8_t *st = smem + s * S::STAGE_BYTES;
        mbar_expect_tx(&full[s], S::STAGE_BYTES);
        const int kx = kb * KE;
        tma_load_2d(st, &p.a_hi, &full[s], kx, p.a_row0 + i0);
        tma_load_2d(st + S::A_BYTES, &p.b_hi, &full[s], kx, p.b_row0 + j0);
        if (TERMS == 3) {
          tma_load_2d(st + S::A_BYTES + S::B_BYTES, &p.a_lo, &full[s], kx, p.a_row0 + i0);
          tma_load_2d(st + 2 * S::A_BYTES + S::B_BYTES, &p.b_lo, &full[s], kx, p.b_row0 + j0);
        }
      }
    }
    // every load issued must land before the CTA may exit
    for (uint32_t q = (it > (uint32_t)S::STAGES ? it - S::STAGES : 0); q < it; q++)
      if (!mbar_wait(&full[q % S::STAGES], (q / S::STAGES) & 1)) atomicExch(abort_flag, 1);
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t sbase = smem_u32(smem);
    uint32_t it = 0, lt = 0;
    bool stop = false;
    for (int t = blockIdx.x; t < total && !stop; t += gridDim.x) {
      const int i0 = (t % mtiles) * BM, j0 = (t / mtiles) * BN;
      if (p.upper && i0 > j0 + BN - 1) continue;
      const uint32_t buf = lt & 1;
      if (!mbar_wait(&acce[buf], ((lt >> 1) & 1) ^ 1)) {
        atomicExch(abort_flag, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t d = tmem + buf * BN;
      for (int kb = 0; kb < nk; kb++, it++) {
        const int s = it % S::STAGES;
        if (*(volatile int *)abort_flag || !mbar_wait(&full[s], (it / S::STAGES) & 1)) {
          atomicExch(abort_flag, 1);
          stop = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = sbase + s * S::STAGE_BYTES;
#pragma unroll
        for (int kk = 0; kk < BK / 16; kk++) {
          const uint32_t koff = kk * 32;
          const uint64_t a = sw128_desc(st + koff);
          const uint64_t b = sw128_desc(st + S::A_BYTES + koff);
          if (F8)
            mma_f8(d, a, b, p.idesc, (kb | kk) ? 1u : 0u);
          else
            mma_bf16(d, a, b, p.idesc, (kb | kk) ? 1u : 0u);
          if (TERMS == 3) {
            const uint64_t alo = sw128_desc(st + S::A_BYTES + S::B_BYTES + koff);
            const uint64_t blo = sw128_desc(st + 2 * S::A_BYTES + S::B_BYTES + koff);
            mma_bf16(d, a, blo, p.idesc, 1u);
            mma_bf16(d, alo, b, p.idesc, 1u);
          }
        }
        mma_commit(&empty[s]);
      }
      if (stop) break;
      mma_commit(&accf[buf]);
      lt++;
    }
    // all products issued by this thread are complete before TMEM is freed
    mma_commit(drain);
    if (!mbar_wait(drain, 0)) atomicExch(abort_flag, 1);
  } else if (warp >= 2) {
    // ---------------- epilogue ----------------
    const int q = warp & 3;  // the TMEM lane quarter this warp may read
    const float alpha = p.alpha_dev ? *p.alpha_dev : p.alpha;
    const bool upper = p.layout == 1 || p.upper;
    const bool read_c = p.layout == 1 || p.beta != 0.f;
    const float beta = p.layout == 1 ? 1.f : p.beta;
    uint32_t lt = 0;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
      const int i0 = (t % mtiles) * BM, j0 = (t / mtiles) * BN;
      if (p.upper && i0 > j0 + BN - 1) continue;
      const uint32_t buf = lt & 1;
      if (*(volatile int *)abort_flag || !mbar_wait(&accf[buf], (lt >> 1) & 1)) {
        atomicExch(abort_flag, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int row = i0 + q * 32 + lane;
      // FP8: the row's scale joins alpha, the columns' are applied one by one
      const float arow = (F8 && row < p.m) ? alpha * p.a_scale[p.a_row0 + row] : alpha;
      long long r_panel = 0, base = 0;
      if (p.layout == 1) {
        const long long gi = p.off + row;
        r_panel = gi / p.nb;
        base = (long long)p.nb * (r_panel * p.ntot - p.nb * r_panel * (r_panel - 1) / 2) +
               (gi - r_panel * p.nb);
      }
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + buf * BN + c0, v);
        if (row >= p.m || j0 + c0 >= p.n) continue;
        float *cp0;
        long long cstride;
        if (p.layout == 0) {
          cp0 = p.c + (size_t)row + (size_t)(j0 + c0) * p.ldc;
          cstride = p.ldc;
        } else {
          cp0 = p.c + base + (p.off + j0 + c0 - r_panel * p.nb) * p.nb;
          cstride = p.nb;
        }
        float old[32];
#pragma unroll
        for (int c = 0; c < 32; c++) {
          const int col = j0 + c0 + c;
          const bool in = col < p.n && !(upper && row > col);
          old[c] = (in && read_c) ? cp0[(size_t)c * cstride] : 0.f;
        }
#pragma unroll
        for (int c = 0; c < 32; c++) {
          const int col = j0 + c0 + c;
          if (col >= p.n || (upper && row > col)) continue;
          const float a = F8 ? arow * p.b_scale[p.b_row0 + col] : alpha;
          cp0[(size_t)c * cstride] = read_c ? fmaf(a, v[c], beta * old[c]) : a * v[c];
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[buf]);
      lt++;
    }
  }
  __syncthreads();
  if (*(volatile int *)abort_flag && threadIdx.x == 0 && p.status)
    atomicCAS(p.status, 0, DG_ERR_TIMEOUT);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN)
                 : "memory");
}

// cuTensorMapEncodeTiled is a driver API call; it is resolved through the
// runtime's entry-point query so the library does not link libcuda (it then
// loads on machines without a driver, e.g. for ABI checks).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

enum OperandType { OP_BF16, OP_FP16, OP_E4M3 };

// 2-D map of a K-major operand (kdim values per vector, ldk between vectors)
// whose boxes are 128 bytes of K by box_rows vectors, 128-byte swizzle.
bool encode_map(CUtensorMap *map, const void *base, int kdim, int rows, int ldk, int box_rows,
                OperandType type) {
  EncodeTiledFn cuTensorMapEncodeTiled = encode_fn();
  if (!cuTensorMapEncodeTiled) return false;
  const int esize = type == OP_E4M3 ? 1 : 2;
  cuuint64_t dims[2] = {(cuuint64_t)kdim, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ldk * esize};
  cuuint32_t box[2] = {(cuuint32_t)(128 / esize), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  const CUtensorMapDataType dt = type == OP_E4M3   ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                 : type == OP_FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                   : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  CUresult r = cuTensorMapEncodeTiled(map, dt, 2, (void *)base, dims, strides, box, estr,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <int BN, int TERMS>
int launch(const TcParams &p, cudaStream_t s) {
  using S = Smem<BN, TERMS>;
  static std::atomic<bool> attr_set[64];  // zero-initialised: false
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr_set[dev & 63]) {
    DG_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_kernel<BN, TERMS>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, S::TOTAL));
    attr_set[dev & 63] = true;
  }
  dim3 grid((p.m + BM - 1) / BM, (p.n + BN - 1) / BN);
  tc_gemm_kernel<BN, TERMS><<<grid, 128, S::TOTAL, s>>>(p);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

template <int BN, int TERMS, bool F8 = false>
int launch_persist(const TcParams &p, int tiles_per_cta, cudaStream_t s) {
  using S = SmemP<BN, TERMS>;
  static std::atomic<bool> attr_set[64];  // zero-initialised: false
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr_set[dev & 63]) {
    DG_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_persist_kernel<BN, TERMS, F8>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, S::TOTAL));
    attr_set[dev & 63] = true;
  }
  const long long mt = (p.m + BM - 1) / BM, nt = (p.n + BN - 1) / BN;
  long long tiles = mt * nt;
  if (p.upper) {  // tiles not wholly below the diagonal
    tiles = 0;
    for (long long bj = 0; bj < nt; bj++)
      tiles += std::min(mt, (bj * BN + BN - 1) / BM + 1);
  }
  if (tiles <= 0) return 0;
  long long grid = dg_num_sms();
  if (tiles_per_cta > 0) grid = std::max(grid, (tiles + tiles_per_cta - 1) / tiles_per_cta);
  grid = std::min<long long>(std::min<long long>(grid, tiles), 1 << 30);
  tc_gemm_persist_kernel<BN, TERMS, F8><<<(unsigned)grid, 192, S::TOTAL, s>>>(p);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

}  // namespace

// One warp per vector (column of a column-major K x ncols FP32 operand):
// scale = 2^(e - 8) with 2^(e-1) <= max|v| < 2^e, dst = e4m3(v / scale)
// rounded to nearest (largest magnitude in [128, 256), below E4M3's 448), the
// vector's scale stored for the epilogue.  A zero vector keeps scale 1; a
// vector with an infinity or NaN gets a NaN scale, so every product that uses
// it is NaN.
__global__ void e4m3_kernel(const float *src, long long ld, int k, int ncols, uint8_t *dst,
                            long long ldd, float *scale, const int *a1, const int *a2) {
  if (aborted(a1, a2)) return;
  const long long col = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (col >= ncols) return;
  const float *v = src + col * ld;
  float mx = 0.f;
  int bad = 0;
  for (int i = lane; i < k; i += 32) {
    const float x = v[i];
    bad |= !isfinite(x);
    mx = fmaxf(mx, fabsf(x));
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  bad = __any_sync(0xffffffffu, bad);
  int e = 0;
  frexpf(mx, &e);
  const int sh = mx > 0.f ? min(8 - e, 127) : 0;
  const float up = ldexpf(1.f, sh);
  uint8_t *d = dst + col * ldd;
  for (int i = lane; i < k; i += 32)
    d[i] = (uint8_t)__nv_cvt_float_to_fp8(v[i] * up, __NV_SATFINITE, __NV_E4M3);
  if (lane == 0) scale[col] = bad ? __int_as_float(0x7fc00000) : ldexpf(1.f, -sh);
}

int split_e4m3(const float *src, long long ld, int k, int ncols, uint8_t *dst, long long ldd,
               float *scale, const int *a1, const int *a2, cudaStream_t s) {
  if (ncols <= 0 || k <= 0) return 0;
  const long long threads = 32LL * ncols;
  e4m3_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(src, ld, k, ncols, dst, ldd,
                                                                scale, a1, a2);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

int tc_gemm_bf16(const TcGemmArgs &g, cudaStream_t s) {
  if (g.m <= 0 || g.n <= 0) return 0;
  if (g.terms != 1 && g.terms != 3 && g.terms != 6) return DG_ERR_UNSUPPORTED;
  // K itself may be ragged: the tensor maps' K extent is g.k and the last
  // block's columns past it are filled with zeros by TMA (only the row
  // strides need 16-byte multiples)
  const int lmul = g.fp8 ? 16 : 8;
  if (g.k <= 0 || g.lda % lmul != 0 || g.ldb % lmul != 0) return DG_ERR_UNSUPPORTED;
  if (((uintptr_t)g.a_hi | (uintptr_t)g.b_hi) & 15) return DG_ERR_UNSUPPORTED;
  if (g.fp8 && (g.terms != 1 || !g.a_scale || !g.b_scale)) return DG_ERR_UNSUPPORTED;
  if (g.terms >= 3 && (((uintptr_t)g.a_lo | (uintptr_t)g.b_lo) & 15)) return DG_ERR_UNSUPPORTED;
  if (g.terms == 6 && (((uintptr_t)g.a_mid | (uintptr_t)g.b_mid) & 15)) return DG_ERR_UNSUPPORTED;
  const int bn = (g.bn == 256 && g.terms != 6) ? 256 : 128;
  TcParams p;
  memset(&p, 0, sizeof p);
  const OperandType ty = g.fp8 ? OP_E4M3 : g.fp16 ? OP_FP16 : OP_BF16;
  if (!encode_map(&p.a_hi, g.a_hi, g.k, g.a_rows, g.lda, BM, ty) ||
      !encode_map(&p.b_hi, g.b_hi, g.k, g.b_rows, g.ldb, bn, ty)) {
    dg_set_last_error(__FILE__, __LINE__, "cuTensorMapEncodeTiled failed");
    return DG_ERR_CUDA;
  }
  if (g.terms >= 3 && (!encode_map(&p.a_lo, g.a_lo, g.k, g.a_rows, g.lda, BM, ty) ||
                       !encode_map(&p.b_lo, g.b_lo, g.k, g.b_rows, g.ldb, bn, ty))) {
    dg_set_last_error(__FILE__, __LINE__, "cuTensorMapEncodeTiled failed");
    return DG_ERR_CUDA;
  }
  if (g.terms == 6 && (!encode_map(&p.a_mid, g.a_mid, g.k, g.a_rows, g.lda, BM, ty) ||
                       !encode_map(&p.b_mid, g.b_mid, g.k, g.b_rows, g.ldb, bn, ty))) {
    dg_set_last_error(__FILE__, __LINE__, "cuTensorMapEncodeTiled failed");
    return DG_ERR_CUDA;
  }
  p.m = g.m; p.n = g.n; p.k = g.k;
  p.a_row0 = g.a_row0; p.b_row0 = g.b_row0;
  p.alpha = g.alpha; p.beta = g.beta;
  p.c = g.c; p.ldc = g.ldc;
  p.layout = g.layout; p.upper = g.upper;
  p.off = g.off; p.nb = g.nb; p.ntot = g.ntot;
  p.status = g.status;
  p.idesc = g.fp8 ? idesc_e4m3(BM, bn) : idesc_f16kind(BM, bn, g.fp16 != 0);
  p.alpha_dev = g.alpha_dev;
  p.a_scale = g.a_scale;
  p.b_scale = g.b_scale;
  const int tpc = g.tiles_per_cta;
  if (g.fp8)
    return bn == 256 ? launch_persist<256, 1, true>(p, tpc, s)
                     : launch_persist<128, 1, true>(p, tpc, s);
  if (g.terms == 6) return launch<128, 6>(p, s);
  if (g.terms == 1)
    return bn == 256 ? launch_persist<256, 1>(p, tpc, s) : launch_persist<128, 1>(p, tpc, s);
  return bn == 256 ? launch_persist<256, 3>(p, tpc, s) : launch_persist<128, 3>(p, tpc, s);
}

}  // namespace dg

// Building-block entry: C = alpha * A' B + beta * C with 16-bit K-major
// operands (A is k x m column-major, B is k x n column-major) and FP32 C.
extern "C" int dg_gemm_tc_tn(int m, int n, int k, int terms, int fp16, const void *a_hi,
                             const void *a_lo, int lda, const void *b_hi, const void *b_lo, int ldb,
                             float alpha, float beta, float *C, int ldc, int bn, int *status,
                             void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(k > 0 && k % 8 == 0, 3);
  DG_CHECK_ARG(terms == 1 || terms == 3, 4);
  DG_CHECK_ARG(lda >= k && lda % 8 == 0, 8);
  DG_CHECK_ARG(ldb >= k && ldb % 8 == 0, 11);
  DG_CHECK_ARG(ldc >= (m > 1 ? m : 1), 15);
  dg::TcGemmArgs g;
  memset(&g, 0, sizeof g);
  g.m = m; g.n = n; g.k = k; g.terms = terms;
  g.a_hi = a_hi; g.a_lo = a_lo; g.lda = lda; g.a_rows = m;
  g.b_hi = b_hi; g.b_lo = b_lo; g.ldb = ldb; g.b_rows = n;
  g.alpha = alpha; g.beta = beta; g.c = C; g.ldc = ldc;
  g.layout = 0; g.upper = 0; g.bn = bn; g.status = status; g.fp16 = fp16;
  return dg::tc_gemm_bf16(g, (cudaStream_t)stream);
}

// Building-block entry of the FP8 form: C = alpha * A' B + beta * C with FP32
// K-major operands (A is k x m column-major, B is k x n) cut to E4M3 with a
// power-of-two scale per vector (split_e4m3) and multiplied on kind::f8f6f4.
// Allocates stream-ordered scratch for the 8-bit operands and the scales.
extern "C" int dg_gemm_f8_tc_tn(int m, int n, int k, float alpha, const float *A, int lda,
                                const float *B, int ldb, float beta, float *C, int ldc,
                                void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(k > 0, 3);
  DG_CHECK_ARG(lda >= k, 6);
  DG_CHECK_ARG(ldb >= k, 8);
  DG_CHECK_ARG(ldc >= (m > 1 ? m : 1), 11);
  if (m == 0 || n == 0) return 0;
  DG_CHECK_ARG(A != nullptr, 5);
  DG_CHECK_ARG(B != nullptr, 7);
  DG_CHECK_ARG(C != nullptr, 10);
  cudaStream_t s = (cudaStream_t)stream;
  const long long ldk = (k + 15) / 16 * 16;
  const size_t abytes = ((size_t)ldk * m + 255) & ~(size_t)255;
  const size_t bbytes = ((size_t)ldk * n + 255) & ~(size_t)255;
  const size_t sbytes = ((sizeof(float) * ((size_t)m + n)) + 255) & ~(size_t)255;
  uint8_t *buf = nullptr;
  DG_CUDA_TRY(dg::pool_malloc_async((void **)&buf, abytes + bbytes + sbytes, s));
  uint8_t *a8 = buf, *b8 = buf + abytes;
  float *sa = (float *)(buf + abytes + bbytes), *sb = sa + m;
  int rc = dg::split_e4m3(A, lda, k, m, a8, ldk, sa, nullptr, nullptr, s);
  if (!rc) rc = dg::split_e4m3(B, ldb, k, n, b8, ldk, sb, nullptr, nullptr, s);
  if (!rc) {
    dg::TcGemmArgs g;
    memset(&g, 0, sizeof g);
    g.m = m; g.n = n; g.k = k; g.terms = 1; g.fp8 = 1;
    g.a_hi = a8; g.lda = (int)ldk; g.a_rows = m;
    g.b_hi = b8; g.ldb = (int)ldk; g.b_rows = n;
    g.a_scale = sa; g.b_scale = sb;
    g.alpha = alpha; g.beta = beta; g.c = C; g.ldc = ldc;
    g.bn = 128;
    rc = dg::tc_gemm_bf16(g, s);
  }
  cudaFreeAsync(buf, s);
  return rc;
}
