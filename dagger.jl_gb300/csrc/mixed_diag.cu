// Diagonal block of the mixed-precision factor: the FP32 Cholesky factor
// U (A = U'U) of one n x n block (n <= 1024) and its inverse V = U^-1, in one
// cooperative launch.
//
// The mixed factorization's critical path is, per block step, the
// factorization of the diagonal block and the solve of its row panel.  Done
// as a recursion of small launches (64 x 64 leaves, recursive TRSMs and
// GEMMs) that chain took several milliseconds per step; here it is one
// launch of G CTAs working on the L2-resident block with a grid barrier per
// 32-column step:
//
//   step j (blocks of 32 rows/columns, bj = j * 32):
//     CTA 0        finishes the diagonal tile (j+1, j+1): its last update
//                  -= U(j, j+1)' U(j, j+1), then all its threads factor it and
//                  invert the 32 x 32 factor in shared memory (one barrier
//                  per column)
//     CTAs 1..G-1  update the other tiles (r, c), j+1 <= r <= c, by
//                  -= U(j, r)' U(j, c), forming the row-panel blocks
//                  U(j, r) = I_j' A(j, r) on the fly from the inverse I_j of
//                  the diagonal factor (so no barrier separates the panel
//                  solve from the update); each CTA works on four tiles at
//                  once, one per group of 64 threads with 4 x 4 outputs per
//                  thread (half a shared-memory load per FMA)
//     grid barrier
//   then every off-diagonal block of U is formed, U(j, c) = I_j' A(j, c),
//   and V = U^-1 by recursive doubling over the 32-block inverses:
//     V12 = -V11 U12 V22, levels of 32, 64, ..., 512 (two barriers each).
//
// Blocks past n are read as the identity and never written, so a ragged last
// block needs no special case.  Every barrier wait is bounded (DG_ERR_TIMEOUT
// in the status word, then every CTA returns).  A pivot that is not positive
// (or NaN) records the LAPACK-style info (atomicCAS of offset + column + 1)
// and stops the launch; the caller's FP64 retry then refactors the block and
// a second launch in "inverse only" mode forms V from the retried factor.
#include <math.h>

#include <algorithm>
#include <atomic>

#include "dg_common.cuh"
#include "runtime.h"
#include "tc_ptx.cuh"

namespace dg {
namespace {

constexpr int DB = 32;            // sub-block order
constexpr int DT = 256;           // threads per CTA
constexpr int GT = 64;            // threads per group (one 32 x 32 tile product)
constexpr int NG = DT / GT;       // groups per CTA
constexpr int DP = DB + 1;        // padded shared-memory column
constexpr int TS = DB * DP;       // floats per shared tile
constexpr int kDiagMaxN = 1024;
constexpr int kDiagMaxGrid = 64;   // the chain shares the GPU with the bulk update
// shared memory: the CTA's I_j, then five tiles per group
constexpr int kDiagSmem = (1 + NG * 5) * TS * (int)sizeof(float);

struct DiagArgs {
  float *D;            // the block, column-major, ld
  long long ld;
  int n;
  float *V;            // inverse, column-major, ldv (upper; zero below)
  long long ldv;
  float *I;            // [nblk][32 x 32] inverses of the diagonal 32-blocks
  float *T;            // doubling scratch (512 x 512)
  unsigned *bar;       // barrier counter (zero at launch)
  int *fail;           // set when a pivot fails (zero at launch)
  int *info;           // first failed column, 1-based plus info_off
  int info_off;
  int *status;         // sticky error word; non-zero on entry = skip
  const int *run_if;   // mode 1: run only when *run_if != 0
  int mode;            // 0 = factor + inverse, 1 = inverse of a factored block
};

__device__ __forceinline__ unsigned ld_acq(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_rel(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier number `epoch` (1, 2, ...); false when the launch must stop
// (a timeout here or elsewhere, or a failed pivot).
__device__ bool grid_sync(const DiagArgs &a, unsigned epoch, int *s_stop) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    red_rel(a.bar, 1u);
    const unsigned target = gridDim.x * epoch;
    int stop = 0;
    if (ld_acq(a.bar) < target) {
      const uint64_t t0 = ptx::globaltimer();
      while (ld_acq(a.bar) < target) {
        if (*(volatile int *)a.status) {
          stop = 1;
          break;
        }
        if (ptx::globaltimer() - t0 > ptx::kWaitNs) {
          atomicCAS(a.status, 0, DG_ERR_TIMEOUT);
          stop = 1;
          break;
        }
      }
    }
    if (*(volatile int *)a.fail || *(volatile int *)a.status) stop = 1;
    *s_stop = stop;
  }
  __syncthreads();
  return *s_stop == 0;
}

// Element (r, c) of an n x n matrix with the identity outside it.
__device__ __forceinline__ float rd_pad(const float *M, long long ld, int n, int r, int c) {
  if (r < n && c < n) return __ldcg(M + r + (size_t)c * ld);
  return r == c ? 1.f : 0.f;
}

__device__ __forceinline__ void gsync(int grp) {
  asm volatile("bar.sync %0, %1;" ::"r"(grp + 1), "r"(GT) : "memory");
}

// 32 x 32 tile at (r0, c0) of M into shared t[c * DP + r] (identity padded),
// by the 64 threads of a group (l = thread within the group).
__device__ __forceinline__ void load_tile(float *t, const float *M, long long ld, int n, int r0,
                                          int c0, int l) {
  const int r = l & 31;
#pragma unroll
  for (int q = 0; q < 16; q++) {
    const int c = (l >> 5) + 2 * q;
    t[c * DP + r] = rd_pad(M, ld, n, r0 + r, c0 + c);
  }
}

__device__ __forceinline__ void store_tile(const float *t, float *M, long long ld, int n, int r0,
                                           int c0, bool upper_only, int l) {
  const int r = l & 31;
#pragma unroll
  for (int q = 0; q < 16; q++) {
    const int c = (l >> 5) + 2 * q;
    if (r0 + r < n && c0 + c < n && (!upper_only || r <= c))
      __stcg(M + (r0 + r) + (size_t)(c0 + c) * ld, t[c * DP + r]);
  }
}

// acc[i][j] (+)= sum_p X(p, r0 + i) Y(p, c0 + j): X' Y on this thread's 4 x 4
// outputs, r0 = (l & 7) * 4, c0 = (l >> 3) * 4.
__device__ __forceinline__ void mma_tn(float (&acc)[4][4], const float *x, const float *y, int l) {
  const int r0 = (l & 7) * 4, c0 = (l >> 3) * 4;
#pragma unroll 4
  for (int p = 0; p < DB; p++) {
    float xv[4], yv[4];
#pragma unroll
    for (int i = 0; i < 4; i++) xv[i] = x[(r0 + i) * DP + p];
#pragma unroll
    for (int j = 0; j < 4; j++) yv[j] = y[(c0 + j) * DP + p];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = fmaf(xv[i], yv[j], acc[i][j]);
  }
}

// acc[i][j] (+)= sum_p X(r0 + i, p) Y(p, c0 + j): X Y.
__device__ __forceinline__ void mma_nn(float (&acc)[4][4], const float *x, const float *y, int l) {
  const int r0 = (l & 7) * 4, c0 = (l >> 3) * 4;
#pragma unroll 4
  for (int p = 0; p < DB; p++) {
    float xv[4], yv[4];
#pragma unroll
    for (int i = 0; i < 4; i++) xv[i] = x[p * DP + r0 + i];
#pragma unroll
    for (int j = 0; j < 4; j++) yv[j] = y[(c0 + j) * DP + p];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = fmaf(xv[i], yv[j], acc[i][j]);
  }
}

__device__ __forceinline__ void zero(float (&acc)[4][4]) {
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
}

// t = acc (sign 0) or t += sign * acc on this thread's outputs.
__device__ __forceinline__ void put(float *t, const float (&acc)[4][4], int l, float sign = 0.f) {
  const int r0 = (l & 7) * 4, c0 = (l >> 3) * 4;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      float *e = t + (c0 + j) * DP + r0 + i;
      *e = sign == 0.f ? acc[i][j] : fmaf(sign, acc[i][j], *e);
    }
}

// Barrier over the NT threads of the calling set: the whole CTA (NT = DT)
// or one group (NT = GT, named barrier grp + 1).
template <int NT>
__device__ __forceinline__ void tsync(int grp) {
  if (NT == DT) __syncthreads();
  else gsync(grp);
}

// Cholesky factor and inverse of the 32 x 32 tile T (shared, T[c * DP + r] =
// element (r, c), upper triangle read), by NT threads (tid in 0..NT-1).
// Right-looking with one barrier per column: step j reads pivot d = T(j, j)
// and row j unscaled, s = rsqrt(d) (the hardware approximation: about 2^-22
// relative, far below what the mixed form's operands carry), and updates
// T(r, c) -= (s T(j, r)) (s T(j, c)) for j < r <= c; row j's scaling by s
// (U(j, :), the diagonal d s = sqrt(d)) waits until step j + 1, which no
// longer reads it.  The inverse X = U^-1 (into W) is formed by recursive
// doubling from 1 / U(j, j) = s kept per column (five levels of block
// products).  piv: 32 floats of shared scratch.  factor = false only
// inverts (T already holds U).  Returns the first failed column or -1 (valid
// in every calling thread); on failure T is left partly factored and W unset.
template <int NT>
__device__ int tile_chol_inv(float *T, float *W, float *piv, bool factor, int tid, int grp) {
  constexpr int PER = DB * DB / NT;
  tsync<NT>(grp);
  if (factor) {
    for (int j = 0; j < DB; j++) {
      const float d = T[j * DP + j];
      if (!(d > 0.f)) return j;  // the same value in every thread: a uniform exit
      const float sj = rsqrtf(d);
      if (tid == 0) piv[j] = sj;
      const float pm = j > 0 ? piv[j - 1] : 0.f;
#pragma unroll
      for (int q = 0; q < PER; q++) {
        const int e = tid + NT * q, r = e & 31, c = e >> 5;
        if (r > j && r <= c)
          T[c * DP + r] = fmaf(-(T[r * DP + j] * sj), T[c * DP + j] * sj, T[c * DP + r]);
        if (r == j - 1 && c >= r) T[c * DP + r] *= pm;
      }
      tsync<NT>(grp);
    }
    const float pl = piv[DB - 1];
#pragma unroll
    for (int q = 0; q < PER; q++) {
      const int e = tid + NT * q, r = e & 31, c = e >> 5;
      if (r == DB - 1 && c >= r) T[c * DP + r] *= pl;
    }
  } else if (tid < DB) {
    piv[tid] = 1.0f / T[tid * DP + tid];
  }
  // W = U^-1 by recursive doubling over the diagonal blocks: W starts as
  // diag(1 / U(j, j)) (piv), and level b turns every 2b x 2b diagonal block
  // into its inverse from the two b x b inverses on its diagonal,
  // V12 = -V11 (U12 V22): three barriers per level, five levels, where a
  // back substitution takes one barrier per column.
#pragma unroll
  for (int q = 0; q < PER; q++) {
    const int e = tid + NT * q, r = e & 31, c = e >> 5;
    W[c * DP + r] = r == c ? piv[r] : 0.f;
    if (r > c) T[c * DP + r] = 0.f;  // the factor is upper triangular
  }
  tsync<NT>(grp);
  for (int b = 1; b < DB; b <<= 1) {
    // X = U12 V22, into the places of V12 (rows below i0 + b: no V22 reads)
#pragma unroll
    for (int q = 0; q < PER; q++) {
      const int e = tid + NT * q, r = e & 31, c = e >> 5;
      const int i0 = r & ~(2 * b - 1);
      if ((c & ~(2 * b - 1)) == i0 && r - i0 < b && c - i0 >= b) {
        float x = 0.f;
        for (int t = i0 + b; t <= c; t++) x = fmaf(T[t * DP + r], W[c * DP + t], x);
        W[c * DP + r] = x;
      }
    }
    tsync<NT>(grp);
    float y[PER];
#pragma unroll
    for (int q = 0; q < PER; q++) {
      const int e = tid + NT * q, r = e & 31, c = e >> 5;
      const int i0 = r & ~(2 * b - 1);
      y[q] = 0.f;
      if ((c & ~(2 * b - 1)) == i0 && r - i0 < b && c - i0 >= b)
        for (int t = r; t < i0 + b; t++) y[q] = fmaf(-W[t * DP + r], W[c * DP + t], y[q]);
    }
    tsync<NT>(grp);
#pragma unroll
    for (int q = 0; q < PER; q++) {
      const int e = tid + NT * q, r = e & 31, c = e >> 5;
      const int i0 = r & ~(2 * b - 1);
      if ((c & ~(2 * b - 1)) == i0 && r - i0 < b && c - i0 >= b) W[c * DP + r] = y[q];
    }
    tsync<NT>(grp);
  }
  return -1;
}

// Tile `idx` (0-based, row-major) of the upper triangle of an m x m tile grid.
__device__ __forceinline__ void upper_tile(int idx, int m, int &rr, int &cc) {
  rr = 0;
  while (idx >= m - rr) {
    idx -= m - rr;
    rr++;
  }
  cc = rr + idx;
}

__global__ void __launch_bounds__(DT, 1) diag_chol_inv_kernel(const DiagArgs a) {
  extern __shared__ float smem[];
  __shared__ int s_stop;
  __shared__ float s_piv[NG][DB];
  // (every CTA takes the same decision: the status word can change during
  // the launch, but a CTA that returns here leaves the others' barrier
  // waits to see it and stop)
  if (*(volatile int *)a.status) return;
  if (a.mode == 1 && (!a.run_if || *(volatile const int *)a.run_if == 0)) return;
  const int n = a.n, nblk = (n + DB - 1) / DB;
  const int G = gridDim.x, g = blockIdx.x;
  const int grp = threadIdx.x / GT, l = threadIdx.x % GT;
  float *sI = smem;
  float *g0 = smem + TS * (1 + 5 * grp);  // this group's five tiles
  float *tA = g0, *tB = g0 + TS, *tC = g0 + 2 * TS, *tU = g0 + 3 * TS, *tV = g0 + 4 * TS;
  unsigned epoch = 0;
  const int ngroups = G * NG;             // every group of the grid
  const int gid = g * NG + grp;

  if (a.mode == 0) {
    // group 0's tiles, used by the whole of CTA 0 for the critical chain
    float *cA = smem + TS, *cC = smem + 3 * TS, *cU = smem + 4 * TS, *cV = smem + 5 * TS;
    // ---- block 0 (CTA 0) ----
    if (g == 0) {
      if (grp == 0) load_tile(cC, a.D, a.ld, n, 0, 0, l);
      const int f = tile_chol_inv<DT>(cC, sI, s_piv[0], true, threadIdx.x, 0);
      if (f >= 0) {
        if (threadIdx.x == 0) {
          atomicCAS(a.info, 0, a.info_off + f + 1);
          atomicExch(a.fail, 1);
        }
      } else if (grp == 0) {
        store_tile(cC, a.D, a.ld, n, 0, 0, true, l);
      } else if (grp == 1) {
        store_tile(sI, a.I, DB, DB, 0, 0, false, l);
      }
    }
    if (!grid_sync(a, ++epoch, &s_stop)) return;
    // ---- steps ----
    for (int j = 0; j + 1 < nblk; j++) {
      const int bj = j * DB;
      if (g == 0) {
        // CTA 0: the critical chain (sI holds I_j from the previous step)
        if (grp == 0) load_tile(cA, a.D, a.ld, n, bj, bj + DB, l);       // A(j, j+1)
        if (grp == 1) load_tile(cC, a.D, a.ld, n, bj + DB, bj + DB, l);  // tile (j+1, j+1)
        __syncthreads();
        if (grp == 0) {
          float acc[4][4];
          zero(acc);
          mma_tn(acc, sI, cA, l);                                 // U(j, j+1)
          put(cU, acc, l);
          gsync(0);
          zero(acc);
          mma_tn(acc, cU, cU, l);
          put(cC, acc, l, -1.f);
        }
        const int f = tile_chol_inv<DT>(cC, cV, s_piv[0], true, threadIdx.x, 0);
        if (f >= 0) {
          if (threadIdx.x == 0) {
            atomicCAS(a.info, 0, a.info_off + bj + DB + f + 1);
            atomicExch(a.fail, 1);
          }
        } else {
          if (grp == 0) store_tile(cC, a.D, a.ld, n, bj + DB, bj + DB, true, l);
          if (grp == 1) store_tile(cV, a.I + (size_t)(j + 1) * DB * DB, DB, DB, 0, 0, false, l);
          for (int e = threadIdx.x; e < TS; e += DT) sI[e] = cV[e];  // I_(j+1) for the next step
        }
      } else {
        // the other tiles (rr, cc), j+1 <= rr <= cc < nblk, (rr, cc) != (j+1, j+1),
        // one per group of CTAs 1 .. G-1
        const int m = nblk - 1 - j;
        const int ntiles = m * (m + 1) / 2 - 1;
        if (ntiles > 0) {
          __syncthreads();
          for (int e = threadIdx.x; e < TS; e += DT) {
            const int c = e / DP, r = e - c * DP;
            if (r < DB) sI[e] = __ldcg(a.I + (size_t)j * DB * DB + r + c * DB);
          }
          __syncthreads();
          const int wgid = gid - NG, nw = ngroups - NG;  // worker groups
          for (int t = wgid; t < ntiles; t += nw) {
            int rr, cc;
            upper_tile(t + 1, m, rr, cc);
            const int R0 = (j + 1 + rr) * DB, C0 = (j + 1 + cc) * DB;
            gsync(grp);
            load_tile(tA, a.D, a.ld, n, bj, R0, l);  // A(j, rr)
            load_tile(tB, a.D, a.ld, n, bj, C0, l);  // A(j, cc)
            load_tile(tC, a.D, a.ld, n, R0, C0, l);  // A(rr, cc)
            gsync(grp);
            float acc[4][4];
            zero(acc);
            mma_tn(acc, sI, tA, l);
            put(tU, acc, l);
            zero(acc);
            mma_tn(acc, sI, tB, l);
            put(tV, acc, l);
            gsync(grp);
            zero(acc);
            mma_tn(acc, tU, tV, l);
            put(tC, acc, l, -1.f);
            gsync(grp);
            store_tile(tC, a.D, a.ld, n, R0, C0, rr == cc, l);
          }
        }
      }
      if (!grid_sync(a, ++epoch, &s_stop)) return;
    }
    // ---- the off-diagonal blocks of U: U(j, c) = I_j' A(j, c) ----
    {
      const int nb2 = nblk * (nblk - 1) / 2;
      for (int t = gid; t < nb2; t += ngroups) {
        int jj, idx;
        upper_tile(t, nblk - 1, jj, idx);  // row jj of the strict upper grid
        const int cc = idx + 1;
        gsync(grp);
        load_tile(tV, a.I + (size_t)jj * DB * DB, DB, DB, 0, 0, l);
        load_tile(tA, a.D, a.ld, n, jj * DB, cc * DB, l);
        gsync(grp);
        float acc[4][4];
        zero(acc);
        mma_tn(acc, tV, tA, l);
        put(tC, acc, l);
        gsync(grp);
        store_tile(tC, a.D, a.ld, n, jj * DB, cc * DB, false, l);
      }
    }
  } else {
    // ---- mode 1: inverses of the diagonal 32-blocks of a factored block ----
    for (int jj = gid; jj < nblk; jj += ngroups) {
      gsync(grp);
      load_tile(tC, a.D, a.ld, n, jj * DB, jj * DB, l);
      tile_chol_inv<GT>(tC, tV, s_piv[grp], false, l, grp);
      store_tile(tV, a.I + (size_t)jj * DB * DB, DB, DB, 0, 0, false, l);
    }
    if (!grid_sync(a, ++epoch, &s_stop)) return;  // every I_j before V is assembled
  }
  // ---- V: I_j on the diagonal, zero below ----
  for (int t = gid; t < nblk * nblk; t += ngroups) {
    const int rb = t % nblk, cb = t / nblk;
    if (rb < cb) continue;
    gsync(grp);
    if (rb == cb) {
      load_tile(tC, a.I + (size_t)rb * DB * DB, DB, DB, 0, 0, l);
    } else {
      for (int e = l; e < TS; e += GT) tC[e] = 0.f;
    }
    gsync(grp);
    store_tile(tC, a.V, a.ldv, n, rb * DB, cb * DB, false, l);
  }
  if (!grid_sync(a, ++epoch, &s_stop)) return;
  // ---- recursive doubling: V12 = -V11 U12 V22 ----
  int npad = DB;
  while (npad < n) npad *= 2;
  for (int sz = DB; sz < npad; sz *= 2) {
    const int nodes = npad / (2 * sz), sb = sz / DB;
    const int per = sb * sb;
    // phase 1: T_q = V11 U12 (V11 upper: k-blocks kb >= rb)
    for (int t = gid; t < nodes * per; t += ngroups) {
      const int q = t / per, rb = (t % per) % sb, cb = (t % per) / sb;
      const int b0 = q * 2 * sz;
      if (b0 + sz >= n) continue;
      float acc[4][4];
      zero(acc);
      for (int kb = rb; kb < sb; kb++) {
        gsync(grp);
        load_tile(tA, a.V, a.ldv, n, b0 + rb * DB, b0 + kb * DB, l);
        load_tile(tB, a.D, a.ld, n, b0 + kb * DB, b0 + sz + cb * DB, l);
        gsync(grp);
        mma_nn(acc, tA, tB, l);
      }
      float *Tq = a.T + (size_t)q * sz * sz;
      const int r0 = (l & 7) * 4, c0 = (l >> 3) * 4;
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int jx = 0; jx < 4; jx++)
          __stcg(Tq + (rb * DB + r0 + i) + (size_t)(cb * DB + c0 + jx) * sz, acc[i][jx]);
    }
    if (!grid_sync(a, ++epoch, &s_stop)) return;
    // phase 2: V12 = -T_q V22 (V22 upper: k-blocks kb <= cb)
    for (int t = gid; t < nodes * per; t += ngroups) {
      const int q = t / per, rb = (t % per) % sb, cb = (t % per) / sb;
      const int b0 = q * 2 * sz;
      if (b0 + sz >= n) continue;
      const float *Tq = a.T + (size_t)q * sz * sz;
      float acc[4][4];
      zero(acc);
      for (int kb = 0; kb <= cb; kb++) {
        gsync(grp);
        {
          const int r = l & 31;
#pragma unroll
          for (int qq = 0; qq < 16; qq++) {
            const int c = (l >> 5) + 2 * qq;
            tA[c * DP + r] = __ldcg(Tq + (rb * DB + r) + (size_t)(kb * DB + c) * sz);
          }
        }
        load_tile(tB, a.V, a.ldv, n, b0 + sz + kb * DB, b0 + sz + cb * DB, l);
        gsync(grp);
        mma_nn(acc, tA, tB, l);
      }
      gsync(grp);
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int jx = 0; jx < 4; jx++) acc[i][jx] = -acc[i][jx];
      put(tC, acc, l);
      gsync(grp);
      store_tile(tC, a.V, a.ldv, n, b0 + rb * DB, b0 + sz + cb * DB, false, l);
    }
    if (sz * 2 < npad && !grid_sync(a, ++epoch, &s_stop)) return;
  }
}

}  // namespace

size_t diag_chol_inv_scratch_bytes() {
  // barrier word + fail word | 32 inverses of 32 x 32 | doubling scratch 512 x 512
  return 256 + sizeof(float) * (size_t)(kDiagMaxN / DB) * DB * DB +
         sizeof(float) * (size_t)(kDiagMaxN / 2) * (kDiagMaxN / 2);
}

int diag_chol_inv_f32(float *D, long long ld, int n, float *V, long long ldv, void *scratch,
                      int *info, int info_off, int *status, const int *run_if, int mode,
                      cudaStream_t s) {
  if (n <= 0) return 0;
  if (n > kDiagMaxN || ld < n || ldv < n) return DG_ERR_UNSUPPORTED;
  char *sc = (char *)scratch;
  DiagArgs a;
  a.D = D;
  a.ld = ld;
  a.n = n;
  a.V = V;
  a.ldv = ldv;
  a.bar = (unsigned *)sc;
  a.fail = (int *)(sc + 4);
  a.I = (float *)(sc + 256);
  a.T = a.I + (size_t)(kDiagMaxN / DB) * DB * DB;
  a.info = info;
  a.info_off = info_off;
  a.status = status;
  a.run_if = run_if;
  a.mode = mode;
  const int nblk = (n + DB - 1) / DB;
  // CTA 0 runs the chain; enough worker groups for the first step's tiles
  int G = std::min(kDiagMaxGrid, std::max(2, 1 + (nblk * (nblk + 1) / 2 + NG - 1) / NG));
  G = std::min(G, dg_num_sms());
  static std::atomic<bool> attr_set[64];  // zero-initialised: false
  int dev = 0;
  DG_CUDA_TRY(cudaGetDevice(&dev));
  if (!attr_set[dev & 63]) {
    DG_CUDA_TRY(cudaFuncSetAttribute(diag_chol_inv_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, kDiagSmem));
    attr_set[dev & 63] = true;
  }
  DG_CUDA_TRY(cudaMemsetAsync(sc, 0, 8, s));
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.gridDim = dim3(G);
  cfg.blockDim = dim3(DT);
  cfg.dynamicSmemBytes = kDiagSmem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  DG_CUDA_TRY(cudaLaunchKernelEx(&cfg, diag_chol_inv_kernel, a));
  count_launches(1);
  return 0;
}

}  // namespace dg

// Building block of the mixed form (no counterpart in the reference): the
// FP32 factor U (A = U'U, upper) of one n x n block in place and V = U^-1,
// both column-major; *info_host = the 1-based column of the first pivot that
// is not positive (0 when none).  Synchronises `stream`.
extern "C" int dg_potrf_inv_f32(int n, float *A, int lda, float *V, int ldv, int *info_host,
                                void *stream) {
  DG_CHECK_ARG(n >= 0 && n <= 1024, 1);
  DG_CHECK_ARG(A != nullptr || n == 0, 2);
  DG_CHECK_ARG(lda >= (n > 1 ? n : 1), 3);
  DG_CHECK_ARG(V != nullptr || n == 0, 4);
  DG_CHECK_ARG(ldv >= (n > 1 ? n : 1), 5);
  DG_CHECK_ARG(info_host != nullptr, 6);
  *info_host = 0;
  if (n == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  char *buf = nullptr;
  const size_t sb = dg::diag_chol_inv_scratch_bytes();
  DG_CUDA_TRY(dg::pool_malloc_async((void **)&buf, sb + 256, s));
  int *words = (int *)(buf + sb);  // [0] info, [1] status
  DG_CUDA_TRY(cudaMemsetAsync(words, 0, 8, s));
  int rc = dg::diag_chol_inv_f32(A, lda, n, V, ldv, buf, words, 0, words + 1, nullptr, 0, s);
  int h[2] = {0, 0};
  if (!rc) {
    DG_CUDA_TRY(cudaMemcpyAsync(h, words, 8, cudaMemcpyDeviceToHost, s));
  }
  DG_CUDA_TRY(cudaFreeAsync(buf, s));
  DG_CUDA_TRY(cudaStreamSynchronize(s));
  if (rc) return rc;
  if (h[1]) {
    dg_set_last_error(__FILE__, __LINE__, "a bounded grid barrier wait timed out");
    return h[1];
  }
  *info_host = h[0];
  return h[0];
}
