// Tiled LU (src/array/lu.jl, linalg.jl:264-308) on GB300: the pivoted
// factorization of one block column (the panel), the row interchanges that
// the panel's pivots make in the other block columns, and the permutation of
// a right-hand side before the triangular solves.
//
// Panel: the tiles of block column k from the diagonal down are gathered into
// one column-major buffer and factored there, recursively like LAPACK's
// getrf2 (left half, then the right half's top rows solved with the unit
// lower L11 and the rest updated by one GEMM, then the right half), with
// leaves of 32 columns.  The reference factors the same panel either with one
// LAPACK getrf (factor_panel_lapack!, lu.jl:263-304) or, on GPUs, column by
// column as four kinds of tasks per column (search_and_update_ipiv!,
// swaprows_panel!, update_panel_diag!, update_panel_offdiag!, lu.jl:24-127);
// here a leaf is ONE launch of up to 96 CTAs (about 384 rows each, so most
// SMs stay free for the trailing updates): every CTA keeps a contiguous range
// of the strip's rows in shared memory, and the grid agrees on each column's
// pivot through one grid barrier per column (a counter in global memory;
// every wait is bounded and records DG_ERR_TIMEOUT; the launch is
// cooperative, so all CTAs are co-resident), with the rank-1 updates
// of the later columns deferred into the barrier waits.  The
// result is LAPACK's: the pivot of a column is the first row of largest
// magnitude (idamax), multipliers are scaled by the reciprocal of the pivot
// when it is at least the smallest normal number, and an exactly zero pivot
// sets info to its (1-based) column and leaves its column unscaled.
//
// Interchanges in the other block columns (swaprows_trail!, lu.jl:129-185):
// the reference swaps rows tile pair by tile pair, in pivot order.  A panel's
// interchanges are one permutation of at most 2 nb rows, so one kernel per
// panel turns them into a (destination, source) row list, and each block
// column applies it in one launch: every warp gathers one column's listed
// rows into shared memory and writes them back permuted.
#include <float.h>
#include <limits.h>

#include <mutex>

#include "dg_common.cuh"
#include "runtime.h"
#include "tc_ptx.cuh"

namespace dg {
namespace {

#ifndef DG_LU_LEAF_W
#define DG_LU_LEAF_W 32
#endif
constexpr int kLeafW = DG_LU_LEAF_W;    // columns of one leaf launch (16 or 32)
static_assert(kLeafW == 16 || kLeafW == 32, "a leaf is 16 or 32 columns wide");
constexpr int kLeafThreads = 256;
constexpr int kLeafWarps = kLeafThreads / 32;
constexpr int kLeafMaxRows = 768;      // rows one CTA keeps in shared memory
constexpr int kLeafMaxGrid = 96;       // CTAs of a leaf launch at most (their candidate rows
                                       // sit in shared memory beside the strip)
#ifndef DG_LU_LEAF_ROWS
#define DG_LU_LEAF_ROWS 384
#endif
constexpr int kLeafRowsTarget = DG_LU_LEAF_ROWS;  // rows per CTA a leaf aims for
constexpr int kLeafSwapMax = 2 * kLeafW;
constexpr int kListHash = 4096;        // >= 4 x the pivots of the widest panel
constexpr int kMaxPanelPivots = 1024;
constexpr int kLaswpWarps = 4;
constexpr int kPermSmemRows = 40960;   // composite permutation kept in shared memory
constexpr int kPermChunk = 4096;

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

struct LeafArgs {
  double *P;
  long long ld;
  int nrows;        // rows from the leaf's diagonal to the panel's end
  int c0;           // first column (and first row) of the leaf in the panel
  int wl;           // leaf columns (<= kLeafW)
  int wp;           // panel columns: the interchanges also go to the others
  int R;            // rows per CTA
  int nopiv;
  int *lpiv;        // lpiv[c0 + j] = panel row of column c0 + j's pivot
  int *info;        // atomicMin(info, info_offset + c0 + j + 1) on an exact zero pivot
  int info_offset;
  unsigned *counter;  // grid barrier arrivals, zero at launch
  int *status;        // DG_ERR_TIMEOUT when a barrier wait gave up
  double *sval;     // [2][G] candidate magnitudes (by column parity)
  int *sidx;        // [2][G] candidate rows
  double *srow;     // [2][G][kLeafW] candidate rows' values
  double *jrow;     // [2][kLeafW] the diagonal row's values
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// The larger magnitude wins, then the smaller row: the first maximum, as
// idamax.  A NaN never wins.
__device__ __forceinline__ bool better(double v, int i, double bv, int bi) {
  return v > bv || (v == bv && i < bi);
}

__device__ __forceinline__ void warp_best(double &bv, int &bi) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const double ov = __shfl_down_sync(0xffffffffu, bv, o);
    const int oi = __shfl_down_sync(0xffffffffu, bi, o);
    if (better(ov, oi, bv, bi)) {
      bv = ov;
      bi = oi;
    }
  }
}

__device__ __forceinline__ void red_release_add(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One leaf: columns c0 .. c0+wl-1 of the panel, rows c0 .. c0+nrows-1.
// Row r (counted from the leaf's diagonal) belongs to CTA r / R.  Step j:
// every CTA publishes its candidate row (and the diagonal row's owner that
// row), arrives at the grid barrier and, while warp 0 waits, applies the
// previous pivot's rank-1 update to columns j+1.. (deferred one step); then
// the pivot is read from all candidates, rows j and p trade places, the
// multipliers are scaled and only column j+1 is updated.  The critical path
// of a column carries one column of FP64 work; the rest overlaps the wait.
// A published row gets the deferred update on the fly (the same fma as the
// deferred pass), so every CTA sees fully updated pivot rows.
__global__ void __launch_bounds__(kLeafThreads, 1) lu_leaf_kernel(LeafArgs a) {
  extern __shared__ double sm[];  // column c of this CTA's rows at sm + c*R, then crow
  double *crow = sm + (size_t)a.wl * a.R;  // [G][kLeafW] the candidate rows
  __shared__ double cval[kLeafMaxGrid];
  __shared__ int cidx[kLeafMaxGrid];
  __shared__ double prow[kLeafW];   // the current column's pivot row
  __shared__ double dprow[kLeafW];  // the pivot row of the deferred update
  __shared__ double jrow_s[kLeafW]; // the displaced diagonal row (the pivot's owner)
  __shared__ double wv[kLeafWarps];
  __shared__ int wi[kLeafWarps];
  __shared__ int piv[kLeafW];
  __shared__ int spos[kLeafSwapMax], scont[kLeafSwapMax];
  __shared__ int s_best, s_stop, s_n;
  const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int R = a.R, r0 = g * R;
  const int rn = max(0, min(R, a.nrows - r0));
  if (*(volatile int *)a.status) return;  // an earlier launch timed out
  double *D = a.P + (size_t)a.c0 * a.ld + a.c0;  // the leaf's diagonal element
  for (int c = 0; c < a.wl; c++)
    for (int r = tid; r < rn; r += kLeafThreads)
      sm[c * R + r] = D[(size_t)(r0 + r) + (size_t)c * a.ld];
  __syncthreads();
  const int jmax = min(a.wl, a.nrows);
  int dj = -1;  // the pivot whose update of columns dj+2.. is pending
  for (int j = 0; j < jmax; j++) {
    const int par = j & 1;
    double *sval = a.sval + par * G;
    int *sidx = a.sidx + par * G;
    double *srow = a.srow + (size_t)par * G * kLeafW;
    double *jrow = a.jrow + par * kLeafW;
    // the value of row r (local), column c with the pending update applied
    auto current = [&](int r, int c) {
      double v = sm[c * R + r];
      if (dj >= 0 && c >= dj + 2) v = fma(-sm[dj * R + r], dprow[c], v);
      return v;
    };
    // 1. this CTA's candidate: its first row of largest |a(r, j)|, r >= j
    if (!a.nopiv) {
      double bv = -1.0;
      int bi = INT_MAX;
      for (int r = tid; r < rn; r += kLeafThreads) {
        const int gr = r0 + r;
        if (gr < j) continue;
        const double v = fabs(sm[j * R + r]);
        if (better(v, gr, bv, bi)) {
          bv = v;
          bi = gr;
        }
      }
      warp_best(bv, bi);
      if (lane == 0) {
        wv[warp] = bv;
        wi[warp] = bi;
      }
      __syncthreads();
      bv = wv[0];
      bi = wi[0];
      for (int w = 1; w < kLeafWarps; w++)
        if (better(wv[w], wi[w], bv, bi)) {
          bv = wv[w];
          bi = wi[w];
        }
      if (tid == 0) {
        __stcg(&sval[g], bv);
        __stcg(&sidx[g], bi);
      }
      if (bi != INT_MAX && tid < a.wl) __stcg(&srow[(size_t)g * kLeafW + tid], current(bi - r0, tid));
    }
    if (j >= r0 && j < r0 + rn && tid < a.wl) __stcg(&jrow[tid], current(j - r0, tid));
    // 2. arrive; the deferred update runs while warp 0 waits (bounded)
    __syncthreads();
    if (tid == 0) red_release_add(a.counter, 1u);
    if (dj >= 0 && warp > 0) {
      for (int r = tid - 32; r < rn; r += kLeafThreads - 32) {
        if (r0 + r <= dj) continue;
        const double l = sm[dj * R + r];
        for (int c = dj + 2; c < a.wl; c++) sm[c * R + r] = fma(-l, dprow[c], sm[c * R + r]);
      }
    }
    if (tid == 0) {
      const unsigned target = (unsigned)G * (unsigned)(j + 1);
      int stop = 0;
      if (ld_acquire_u32(a.counter) < target) {
        const uint64_t t0 = ptx::globaltimer();
        while (ld_acquire_u32(a.counter) < target) {
          if (*(volatile int *)a.status) {
            stop = 1;
            break;
          }
          if (ptx::globaltimer() - t0 > ptx::kWaitNs) {
            atomicExch(a.status, DG_ERR_TIMEOUT);
            stop = 1;
            break;
          }
        }
      }
      s_stop = stop;
    }
    __syncthreads();
    if (s_stop) return;
    // 3. every candidate record and the diagonal row in one round trip, then
    //    the column's pivot, the same in every CTA
    if (!a.nopiv) {
      for (int e = tid; e < G * kLeafW; e += kLeafThreads) crow[e] = __ldcg(&srow[e]);
      for (int q = tid; q < G; q += kLeafThreads) {
        cval[q] = __ldcg(&sval[q]);
        cidx[q] = __ldcg(&sidx[q]);
      }
    }
    if (tid >= kLeafThreads - kLeafW && tid - (kLeafThreads - kLeafW) < a.wl)
      jrow_s[tid - (kLeafThreads - kLeafW)] = __ldcg(&jrow[tid - (kLeafThreads - kLeafW)]);
    __syncthreads();
    if (warp == 0) {
      double bv = -1.0;
      int bi = INT_MAX;
      if (!a.nopiv) {
        for (int q = lane; q < G; q += 32)
          if (cidx[q] != INT_MAX && better(cval[q], cidx[q], bv, bi)) {
            bv = cval[q];
            bi = cidx[q];
          }
        warp_best(bv, bi);
      }
      if (lane == 0) s_best = (bi == INT_MAX) ? j : bi;
    }
    __syncthreads();
    const int p = s_best;
    if (tid < a.wl) prow[tid] = (p == j) ? jrow_s[tid] : crow[(p / R) * kLeafW + tid];
    if (tid == 0) piv[j] = p;
    __syncthreads();
    // 4. rows j and p trade places
    if (p != j && tid < a.wl) {
      if (j >= r0 && j < r0 + rn) sm[tid * R + (j - r0)] = prow[tid];
      if (p >= r0 && p < r0 + rn) sm[tid * R + (p - r0)] = jrow_s[tid];
    }
    if (g == 0 && tid == 0) {
      a.lpiv[a.c0 + j] = a.c0 + p;
      if (prow[j] == 0.0) atomicMin(a.info, a.info_offset + a.c0 + j + 1);
    }
    __syncthreads();
    // 5. multipliers below the diagonal; column j+1 now, the others deferred
    const double pv = prow[j];
    const bool scale = (pv != 0.0);
    const bool recip = a.nopiv || fabs(pv) >= DBL_MIN;
    const double rinv = scale ? 1.0 / pv : 0.0;
    for (int r = tid; r < rn; r += kLeafThreads) {
      if (r0 + r <= j) continue;
      double l = sm[j * R + r];
      if (scale) {
        l = recip ? l * rinv : l / pv;
        sm[j * R + r] = l;
      }
      if (j + 1 < a.wl) sm[(j + 1) * R + r] = fma(-l, prow[j + 1], sm[(j + 1) * R + r]);
    }
    if (tid < a.wl) dprow[tid] = prow[tid];
    dj = j;
    __syncthreads();
  }
  // the last pivot's deferred update
  if (dj >= 0) {
    for (int r = tid; r < rn; r += kLeafThreads) {
      if (r0 + r <= dj) continue;
      const double l = sm[dj * R + r];
      for (int c = dj + 2; c < a.wl; c++) sm[c * R + r] = fma(-l, dprow[c], sm[c * R + r]);
    }
  }
  __syncthreads();
  for (int c = 0; c < a.wl; c++)
    for (int r = tid; r < rn; r += kLeafThreads)
      D[(size_t)(r0 + r) + (size_t)c * a.ld] = sm[c * R + r];
  if (a.nopiv || a.wp <= a.wl) return;
  // The leaf's interchanges in the panel's other columns, as one permutation
  // of at most 2 wl rows: row spos[i] receives the row that was at scont[i].
  if (tid == 0) {
    int n = 0;
    for (int j = 0; j < jmax; j++) {
      const int x = j, y = piv[j];
      if (x == y) continue;
      int ix = -1, iy = -1;
      for (int q = 0; q < n; q++) {
        if (spos[q] == x) ix = q;
        if (spos[q] == y) iy = q;
      }
      if (ix < 0) {
        spos[n] = x;
        scont[n] = x;
        ix = n++;
      }
      if (iy < 0) {
        spos[n] = y;
        scont[n] = y;
        iy = n++;
      }
      const int t = scont[ix];
      scont[ix] = scont[iy];
      scont[iy] = t;
    }
    s_n = n;
  }
  __syncthreads();
  const int n = s_n;
  if (n == 0) return;
  const int others = a.wp - a.wl;
  for (int q = g * kLeafWarps + warp; q < others; q += G * kLeafWarps) {
    const int col = q < a.c0 ? q : q + a.wl;
    double *cp = a.P + (size_t)col * a.ld + a.c0;
    double v0 = 0.0, v1 = 0.0;
    if (lane < n) v0 = cp[scont[lane]];
    if (lane + 32 < n) v1 = cp[scont[lane + 32]];
    __syncwarp();
    if (lane < n) cp[spos[lane]] = v0;
    if (lane + 32 < n) cp[spos[lane + 32]] = v1;
  }
}

// A panel's npiv pivots (panel rows, lpiv[p] >= p) as ipiv (global, 1-based:
// row0 + lpiv[p] + 1) and as the (destination, source) list of the rows the
// interchanges move: lists[0] = count, destinations at lists + 1, sources at
// lists + 1 + cap.  One CTA; thread 0 replays the interchanges on the
// contents of the first npiv rows (an array) and of the rows below them that
// the pivots reach (a hash table).
__global__ void __launch_bounds__(256) lu_lists_kernel(const int *lpiv, int npiv, int row0,
                                                       long long *ipiv, int *lists, int cap) {
  __shared__ int top[kMaxPanelPivots];
  __shared__ int hkey[kListHash], hval[kListHash];
  __shared__ int cnt;
  const int tid = threadIdx.x;
  for (int p = tid; p < npiv; p += blockDim.x) {
    top[p] = p;
    ipiv[p] = (long long)row0 + lpiv[p] + 1;
  }
  for (int h = tid; h < kListHash; h += blockDim.x) hkey[h] = -1;
  if (tid == 0) cnt = 0;
  __syncthreads();
  if (tid == 0) {
    for (int p = 0; p < npiv; p++) {
      const int r = lpiv[p];
      if (r == p) continue;
      int *cell;
      if (r < npiv) {
        cell = &top[r];
      } else {
        unsigned h = ((unsigned)r * 2654435761u) >> 20;
        while (hkey[h] != -1 && hkey[h] != r) h = (h + 1) & (kListHash - 1);
        if (hkey[h] == -1) {
          hkey[h] = r;
          hval[h] = r;
        }
        cell = &hval[h];
      }
      const int t = top[p];
      top[p] = *cell;
      *cell = t;
    }
  }
  __syncthreads();
  int *dst = lists + 1, *src = lists + 1 + cap;
  for (int p = tid; p < npiv; p += blockDim.x)
    if (top[p] != p) {
      const int i = atomicAdd(&cnt, 1);
      dst[i] = p;
      src[i] = top[p];
    }
  for (int h = tid; h < kListHash; h += blockDim.x)
    if (hkey[h] >= 0 && hval[h] != hkey[h]) {
      const int i = atomicAdd(&cnt, 1);
      dst[i] = hkey[h];
      src[i] = hval[h];
    }
  __syncthreads();
  if (tid == 0) lists[0] = cnt;
}

struct TileColumn {
  double *t[kMaxTileRows];
};

// Row r of a block column held as ntiles tiles of nb rows (the last one
// last_rows), column col: tile r / nb, ld = the tile's rows.
__device__ __forceinline__ double *tile_elem(const TileColumn &tc, int ntiles, int nb,
                                             int last_rows, int r, int col) {
  const int ti = r / nb;
  const int ld = (ti == ntiles - 1) ? last_rows : nb;
  return tc.t[ti] + (r - ti * nb) + (size_t)col * ld;
}

// One warp per column: the listed rows are read into shared memory, then
// written to their destinations.
__global__ void __launch_bounds__(kLaswpWarps * 32) lu_laswp_kernel(TileColumn tc, int ntiles, int nb,
                                                                   int last_rows, int ncols,
                                                                   const int *lists, int cap) {
  extern __shared__ double buf[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int col = blockIdx.x * kLaswpWarps + warp;
  const int n = min(lists[0], cap);
  if (col >= ncols || n <= 0) return;
  const int *dst = lists + 1, *src = lists + 1 + cap;
  double *b = buf + (size_t)warp * cap;
  for (int t = lane; t < n; t += 32) b[t] = *tile_elem(tc, ntiles, nb, last_rows, src[t], col);
  __syncwarp();
  for (int t = lane; t < n; t += 32) *tile_elem(tc, ntiles, nb, last_rows, dst[t], col) = b[t];
}

// perm[t] = the row that npiv interchanges (ipiv, global and 1-based) move
// to position t of an n-row array: apply_ipiv_rows! (linalg.jl:279-308) as
// one permutation.  One CTA; thread 0 replays the interchanges on a copy in
// shared memory (n <= kPermSmemRows) or in perm itself, the pivots staged
// through shared memory in chunks.
__global__ void __launch_bounds__(256) lu_perm_kernel(const long long *ipiv, int npiv, int n,
                                                      int *perm, int in_smem) {
  extern __shared__ int sp[];
  int *chunk = sp;
  int *w = in_smem ? sp + kPermChunk : perm;
  for (int t = threadIdx.x; t < n; t += blockDim.x) w[t] = t;
  __syncthreads();
  for (int p0 = 0; p0 < npiv; p0 += kPermChunk) {
    const int len = min(kPermChunk, npiv - p0);
    for (int q = threadIdx.x; q < len; q += blockDim.x) {
      const long long r = ipiv[p0 + q] - 1;
      chunk[q] = (r >= 0 && r < n) ? (int)r : -1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int q = 0; q < len; q++) {
        const int p = p0 + q, r = chunk[q];
        if (r < 0 || r == p || p >= n) continue;
        const int x = w[p];
        w[p] = w[r];
        w[r] = x;
      }
    }
    __syncthreads();
  }
  if (in_smem)
    for (int t = threadIdx.x; t < n; t += blockDim.x) perm[t] = w[t];
}

// X (n x ncols, ld n) = rows perm[0..n) of the tiled block column.
__global__ void __launch_bounds__(256) lu_rows_gather_kernel(TileColumn tc, int ntiles, int nb,
                                                             int last_rows, int n, int ncols,
                                                             const int *perm, double *X) {
  const long long total = (long long)n * ncols;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int t = (int)(e % n), c = (int)(e / n);
    X[e] = *tile_elem(tc, ntiles, nb, last_rows, perm[t], c);
  }
}

__global__ void lu_ipiv_kernel(const int *lpiv, int npiv, int row0, long long *ipiv) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < npiv) ipiv[p] = (long long)row0 + lpiv[p] + 1;
}

__global__ void lu_iota_kernel(long long *ipiv, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ipiv[i] = i + 1;
}

std::once_flag g_attr_once;
void set_attributes() {
  std::call_once(g_attr_once, [] {
    cudaFuncSetAttribute(lu_leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (kLeafW * kLeafMaxRows + kLeafMaxGrid * kLeafW) * 8);
    cudaFuncSetAttribute(lu_laswp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kLaswpWarps * 2 * kMaxPanelPivots * 8);
    cudaFuncSetAttribute(lu_perm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (kPermChunk + kPermSmemRows) * 4);
  });
}

struct Leaf {
  unsigned *counter;
  double *sval;
  int *sidx;
  double *srow;
  double *jrow;
};

Leaf leaf_scratch(void *p) {
  char *q = (char *)p;
  Leaf l;
  l.counter = (unsigned *)q;
  q += 256;
  l.sval = (double *)q;
  q += round256((size_t)2 * kLeafMaxGrid * 8);
  l.sidx = (int *)q;
  q += round256((size_t)2 * kLeafMaxGrid * 4);
  l.srow = (double *)q;
  q += round256((size_t)2 * kLeafMaxGrid * kLeafW * 8);
  l.jrow = (double *)q;
  return l;
}

struct PanelCtx {
  double *P;
  long long ld;
  int mrows, wp, nopiv;
  int *lpiv, *info, info_offset, *status;
  void *leaf;
  void *oz;
  size_t oz_bytes;
  cudaStream_t s;
};

int leaf_launch(const PanelCtx &c, int c0, int wl) {
  const int nrows = c.mrows - c0;
  // about kLeafRowsTarget rows per CTA: enough rows to keep the per-column
  // barrier cheap and leave most SMs to concurrent work, few enough that the
  // deferred FP64 updates hide behind the barrier waits
  int G = max((nrows + kLeafMaxRows - 1) / kLeafMaxRows, (nrows + kLeafRowsTarget - 1) / kLeafRowsTarget);
  G = min(G, min(dg_num_sms(), kLeafMaxGrid));
  if (G < 1) G = 1;
  const int R = (nrows + G - 1) / G;
  if (R > kLeafMaxRows) return DG_ERR_UNSUPPORTED;
  Leaf l = leaf_scratch(c.leaf);
  DG_CUDA_TRY(cudaMemsetAsync(l.counter, 0, sizeof(unsigned), c.s));
  LeafArgs a;
  a.P = c.P;
  a.ld = c.ld;
  a.nrows = nrows;
  a.c0 = c0;
  a.wl = wl;
  a.wp = c.wp;
  a.R = R;
  a.nopiv = c.nopiv;
  a.lpiv = c.lpiv;
  a.info = c.info;
  a.info_offset = c.info_offset;
  a.counter = l.counter;
  a.status = c.status;
  a.sval = l.sval;
  a.sidx = l.sidx;
  a.srow = l.srow;
  a.jrow = l.jrow;
  // A cooperative launch: the G CTAs are scheduled together, so the
  // per-column grid barrier never waits for a CTA that other kernels of the
  // region (the look-ahead trailing updates on other streams) keep from
  // starting.  The attribute is kept when the launch is captured into the
  // region's graph.
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.gridDim = dim3(G);
  cfg.blockDim = dim3(kLeafThreads);
  cfg.dynamicSmemBytes = ((size_t)wl * R + (size_t)G * kLeafW) * 8;
  cfg.stream = c.s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  DG_CUDA_TRY(cudaLaunchKernelEx(&cfg, lu_leaf_kernel, a));
  count_launches(1);
  return 0;
}

// getrf2's recursion over panel columns c0 .. c0+n-1 (rows c0 .. mrows-1).
int panel_rec(const PanelCtx &c, int c0, int n) {
  const int nrows = c.mrows - c0;
  if (n <= 0 || nrows <= 0) return 0;
  if (n <= kLeafW) return leaf_launch(c, c0, n);
  const int n1 = (n / 2 + kLeafW - 1) / kLeafW * kLeafW, n2 = n - n1;
  DG_TRY(panel_rec(c, c0, n1));
  const long long ld = c.ld;
  double *A11 = c.P + c0 + (size_t)c0 * ld;
  double *A12 = c.P + c0 + (size_t)(c0 + n1) * ld;
  const int k1 = min(n1, nrows);  // rows of L11 (fewer when the panel is wide)
  // A12 = L11^-1 A12 (trsm 'L', 'L', 'N', 'U')
  if (c.oz)
    DG_TRY(trsm_f64_oz('L', 'L', 'N', 'U', k1, n2, 1.0, A11, (int)ld, A12, (int)ld, c.oz,
                       c.oz_bytes, c.status, c.s));
  else
    DG_TRY(trsm_f64('L', 'L', 'N', 'U', k1, n2, 1.0, A11, (int)ld, A12, (int)ld, c.status, c.s));
  if (nrows <= n1) return 0;
  double *A21 = c.P + (c0 + n1) + (size_t)c0 * ld;
  double *A22 = c.P + (c0 + n1) + (size_t)(c0 + n1) * ld;
  DG_TRY(gemm_update_f64('N', 'N', nrows - n1, n2, n1, -1.0, A21, ld, A12, ld, 1.0, A22, ld, c.oz,
                         c.oz_bytes, c.status, c.s));
  return panel_rec(c, c0 + n1, n2);
}

TileColumn tile_column(double *const *tiles, int ntiles) {
  TileColumn tc;
  memset(&tc, 0, sizeof tc);
  for (int i = 0; i < ntiles; i++) tc.t[i] = tiles[i];
  return tc;
}

}  // namespace

void lu_prepare() { set_attributes(); }

size_t lu_leaf_scratch_bytes() {
  return 256 + round256((size_t)2 * kLeafMaxGrid * 8) + round256((size_t)2 * kLeafMaxGrid * 4) +
         round256((size_t)2 * kLeafMaxGrid * kLeafW * 8) + round256((size_t)2 * kLeafW * 8);
}

int lu_panel_f64(double *P, long long ld, int mrows, int wcols, bool pivot, int *lpiv, int *info,
                 int info_offset, void *leaf_scratch, int *status, void *oz, size_t oz_bytes,
                 long long *ipiv_out, int *lists, int list_cap, cudaStream_t s) {
  if (mrows <= 0 || wcols <= 0) return 0;
  const int npiv = mrows < wcols ? mrows : wcols;
  if (pivot && lists && (npiv > kMaxPanelPivots || 2 * npiv > list_cap)) return DG_ERR_UNSUPPORTED;
  if (ld < mrows || ld > 2147483647LL) return DG_ERR_UNSUPPORTED;
  set_attributes();
  PanelCtx c;
  c.P = P;
  c.ld = ld;
  c.mrows = mrows;
  c.wp = wcols;
  c.nopiv = pivot ? 0 : 1;
  c.lpiv = lpiv;
  c.info = info;
  c.info_offset = info_offset;
  c.status = status;
  c.leaf = leaf_scratch;
  c.oz = oz;
  c.oz_bytes = oz_bytes;
  c.s = s;
  DG_TRY(panel_rec(c, 0, wcols));
  if (!pivot) return 0;
  if (lists)
    lu_lists_kernel<<<1, 256, 0, s>>>(lpiv, npiv, info_offset, ipiv_out, lists, list_cap);
  else
    lu_ipiv_kernel<<<(npiv + 255) / 256, 256, 0, s>>>(lpiv, npiv, info_offset, ipiv_out);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

int lu_laswp_tiles(double *const *tiles, int ntiles, int nb, int rows, int ncols, const int *lists,
                   int list_cap, cudaStream_t s) {
  if (ntiles <= 0 || ncols <= 0 || rows <= 0) return 0;
  if (ntiles > kMaxTileRows || list_cap > 2 * kMaxPanelPivots) return DG_ERR_UNSUPPORTED;
  set_attributes();
  const int last_rows = rows - (ntiles - 1) * nb;
  if (last_rows <= 0 || last_rows > nb) return DG_ERR_UNSUPPORTED;
  const int grid = (ncols + kLaswpWarps - 1) / kLaswpWarps;
  lu_laswp_kernel<<<grid, kLaswpWarps * 32, (size_t)kLaswpWarps * list_cap * 8, s>>>(
      tile_column(tiles, ntiles), ntiles, nb, last_rows, ncols, lists, list_cap);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

int lu_perm(const long long *ipiv, int npiv, int n, int *perm, cudaStream_t s) {
  if (n <= 0) return 0;
  set_attributes();
  const int in_smem = n <= kPermSmemRows ? 1 : 0;
  const size_t smem = (size_t)(kPermChunk + (in_smem ? n : 0)) * 4;
  lu_perm_kernel<<<1, 256, smem, s>>>(ipiv, npiv, n, perm, in_smem);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

int lu_rows_tiles(double *const *tiles, int ntiles, int nb, int n, int ncols, const int *perm,
                  double *X, cudaStream_t s) {
  if (n <= 0 || ncols <= 0) return 0;
  if (ntiles > kMaxTileRows) return DG_ERR_UNSUPPORTED;
  const int last_rows = n - (ntiles - 1) * nb;
  if (last_rows <= 0 || last_rows > nb) return DG_ERR_UNSUPPORTED;
  const long long total = (long long)n * ncols;
  const int grid = (int)std::min<long long>((total + 255) / 256, (long long)dg_num_sms() * 8);
  lu_rows_gather_kernel<<<grid, 256, 0, s>>>(tile_column(tiles, ntiles), ntiles, nb, last_rows, n,
                                             ncols, perm, X);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  for (int i = 0; i < ntiles; i++) {
    const int rows = (i == ntiles - 1) ? last_rows : nb;
    DG_CUDA_TRY(cudaMemcpy2DAsync(tiles[i], (size_t)rows * 8, X + (size_t)i * nb, (size_t)n * 8,
                                  (size_t)rows * 8, ncols, cudaMemcpyDeviceToDevice, s));
  }
  return 0;
}

int lu_iota(long long *ipiv, int n, cudaStream_t s) {
  if (n <= 0) return 0;
  lu_iota_kernel<<<(n + 255) / 256, 256, 0, s>>>(ipiv, n);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

}  // namespace dg
