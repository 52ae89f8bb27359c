// Pre-factorization checks on a tiled matrix:
//   ishermitian(::DArray) (src/array/linalg.jl:90-124 of Dagger.jl): each
//     diagonal tile must equal its transpose exactly; each off-diagonal pair
//     (i, j), i > j, passes when ||A_ij - A_ji'||_F <= sqrt(eps) *
//     max(||A_ij||_F, ||A_ji||_F) (is_cross_hermitian, linalg.jl:43-48).
//   chkfinite(::DArray) (linalg.jl:138-148): every element finite.
// One launch covers all tile pairs and fills the GPU: CTA (strip, i, j) with
// i >= j compares a 32-row strip of tile (i, j) with the matching 32 columns
// of tile (j, i) through 32 x 33 shared-memory transposes (both reads
// coalesced) and stores its three sums of squares in a per-strip slot; a
// second launch adds each pair's slots in strip order (so the outcome does
// not depend on scheduling) and raises the flag when the pair fails.
// Stdlib's ishermitian compares with ==, so a NaN anywhere in a diagonal
// tile fails the check as well.  chkfinite splits each tile's contiguous
// elements into chunks of kFiniteChunk per CTA.
#include <math.h>

#include <algorithm>

#include "dg_common.cuh"
#include "runtime.h"

namespace {

__device__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (warp == 0) {
    s = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return s;  // valid in thread 0
}

constexpr int kFiniteChunk = 16384;

// Slot of pair (i, j), i >= j, in the lower-triangle packed order.
__device__ __forceinline__ size_t pair_index(int i, int j) {
  return (size_t)i * (i + 1) / 2 + j;
}

__global__ void __launch_bounds__(256) herm_pair_kernel(const double *const *tiles, int n, int nb,
                                                        int mt, int strips, double *part,
                                                        int *flag) {
  const int strip = blockIdx.x, i = blockIdx.y, j = blockIdx.z;
  if (i < j) return;
  __shared__ double xs[32][33], ys[32][33];
  __shared__ double red[8];
  const int ri = min(nb, n - i * nb), rj = min(nb, n - j * nb);
  const int r0 = strip * 32;
  const bool diag = i == j;
  double *slot = part + (pair_index(i, j) * strips + strip) * 3;
  if (r0 >= ri) {  // ragged last tile row: an empty strip adds nothing
    if (!diag && threadIdx.x == 0) slot[0] = slot[1] = slot[2] = 0.0;
    return;
  }
  const double *X = tiles[i + (size_t)j * mt];  // ri x rj, ld ri
  const double *Y = tiles[j + (size_t)i * mt];  // rj x ri, ld rj
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  double d2 = 0.0, x2 = 0.0, y2 = 0.0;
  int mism = 0;
  for (int c0 = 0; c0 < rj; c0 += 32) {
    __syncthreads();
#pragma unroll
    for (int c = ty; c < 32; c += 8) {
      int r = r0 + tx, cc = c0 + c;
      xs[c][tx] = (r < ri && cc < rj) ? X[(size_t)r + (size_t)cc * ri] : 0.0;
      // Y(cc', r') with cc' = c0 + tx, r' = r0 + c: coalesced along cc'
      int yr = c0 + tx, yc = r0 + c;
      ys[tx][c] = (yr < rj && yc < ri) ? Y[(size_t)yr + (size_t)yc * rj] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int c = ty; c < 32; c += 8) {
      int r = r0 + tx, cc = c0 + c;
      if (r < ri && cc < rj) {
        double x = xs[c][tx], y = ys[c][tx];  // X(r, cc) and Y(cc, r)
        if (diag) {
          if (!(x == y)) mism = 1;
        } else {
          double d = x - y;
          d2 += d * d;
          x2 += x * x;
          y2 += y * y;
        }
      }
    }
  }
  if (diag) {
    if (__syncthreads_or(mism) && threadIdx.x == 0) atomicOr(flag, 1);
    return;
  }
  d2 = block_sum(d2, red);
  x2 = block_sum(x2, red);
  y2 = block_sum(y2, red);
  if (threadIdx.x == 0) {
    slot[0] = d2;
    slot[1] = x2;
    slot[2] = y2;
  }
}

// One thread per off-diagonal pair: is_cross_hermitian on the strip sums.
__global__ void herm_decide_kernel(const double *part, int mt, int strips, int *flag) {
  const size_t npairs = (size_t)mt * (mt + 1) / 2;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npairs;
       p += (size_t)gridDim.x * blockDim.x) {
    // i from the packed index: the largest i with i (i + 1) / 2 <= p
    int i = (int)((sqrt(8.0 * (double)p + 1.0) - 1.0) * 0.5);
    while ((size_t)(i + 1) * (i + 2) / 2 <= p) ++i;
    while ((size_t)i * (i + 1) / 2 > p) --i;
    const int j = (int)(p - (size_t)i * (i + 1) / 2);
    if (i == j) continue;
    double d2 = 0.0, x2 = 0.0, y2 = 0.0;
    const double *q = part + p * strips * 3;
    for (int s = 0; s < strips; ++s) {
      d2 += q[3 * s];
      x2 += q[3 * s + 1];
      y2 += q[3 * s + 2];
    }
    const double rtol = sqrt(2.220446049250313e-16);
    // NaN in either norm makes the comparison false, as in Julia
    if (!(sqrt(d2) <= rtol * fmax(sqrt(x2), sqrt(y2)))) atomicOr(flag, 1);
  }
}

// grid (chunks, mt, nt): chunk c of tile (i, j)'s ri * cj contiguous elements
__global__ void __launch_bounds__(256) finite_kernel(const double *const *tiles, int m, int n,
                                                     int mb, int nb, int mt, int *flag) {
  const int i = blockIdx.y, j = blockIdx.z;
  const int ri = min(mb, m - i * mb), cj = min(nb, n - j * nb);
  const size_t total = (size_t)ri * cj;
  const size_t e0 = (size_t)blockIdx.x * kFiniteChunk;
  if (e0 >= total) return;
  const size_t e1 = e0 + kFiniteChunk < total ? e0 + kFiniteChunk : total;
  const double *X = tiles[i + (size_t)j * mt];
  int bad = 0;
#pragma unroll 8
  for (size_t e = e0 + threadIdx.x; e < e1; e += 256)
    if (!isfinite(X[e])) bad = 1;
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

// herm: n x n with Blocks(nb, nb); otherwise m x n with Blocks(mb, nb).
int run_check(bool herm, int m, int n, int mb, int nb, double *const *tiles, cudaStream_t s) {
  const int mt = (m + mb - 1) / mb, nt = (n + nb - 1) / nb;
  DG_CHECK_ARG(mt <= 65535 && nt <= 65535, 2);
  const size_t ntiles = (size_t)mt * nt;
  const int strips = (mb + 31) / 32;
  const size_t chunks = ((size_t)mb * nb + kFiniteChunk - 1) / kFiniteChunk;
  DG_CHECK_ARG(chunks <= 0x7fffffffu, 3);
  const size_t npairs = herm ? (size_t)mt * (mt + 1) / 2 : 0;
  // one stream-ordered block per call: the flag, the strip sums of every
  // pair, then the tile pointer grid
  const size_t part_off = 256;
  const size_t ptr_off = part_off + ((npairs * strips * 3 * sizeof(double) + 255) & ~(size_t)255);
  char *buf = nullptr;
  DG_CUDA_TRY(dg::pool_malloc_async((void **)&buf, ptr_off + sizeof(double *) * ntiles, s));
  int *flag = (int *)buf;
  double *part = (double *)(buf + part_off);
  const double **dptrs = (const double **)(buf + ptr_off);
  DG_CUDA_TRY(cudaMemcpyAsync(dptrs, tiles, sizeof(double *) * ntiles, cudaMemcpyHostToDevice, s));
  DG_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), s));
  if (herm) {
    herm_pair_kernel<<<dim3(strips, mt, mt), 256, 0, s>>>(dptrs, n, nb, mt, strips, part, flag);
    DG_CUDA_TRY(cudaGetLastError());
    if (mt > 1) {
      const int blocks = (int)std::min<size_t>((npairs + 255) / 256, 4096);
      herm_decide_kernel<<<blocks, 256, 0, s>>>(part, mt, strips, flag);
      DG_CUDA_TRY(cudaGetLastError());
    }
    dg::count_launches(mt > 1 ? 2 : 1);
  } else {
    finite_kernel<<<dim3((unsigned)chunks, mt, nt), 256, 0, s>>>(dptrs, m, n, mb, nb, mt, flag);
    DG_CUDA_TRY(cudaGetLastError());
    dg::count_launches(1);
  }
  int h = 0;
  DG_CUDA_TRY(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  DG_CUDA_TRY(cudaFreeAsync(buf, s));
  DG_CUDA_TRY(cudaStreamSynchronize(s));
  return h ? 0 : 1;
}

}  // namespace

extern "C" int dg_ishermitian_tiled(int n, int nb, double *const *tiles, void *stream) {
  DG_CHECK_ARG(n >= 0, 1);
  DG_CHECK_ARG(nb > 0, 2);
  if (n == 0) return 1;
  DG_CHECK_ARG(tiles != nullptr, 3);
  return run_check(true, n, n, nb, nb, tiles, (cudaStream_t)stream);
}

extern "C" int dg_chkfinite_tiled(int n, int nb, double *const *tiles, void *stream) {
  DG_CHECK_ARG(n >= 0, 1);
  DG_CHECK_ARG(nb > 0, 2);
  if (n == 0) return 1;
  DG_CHECK_ARG(tiles != nullptr, 3);
  return run_check(false, n, n, nb, nb, tiles, (cudaStream_t)stream);
}

extern "C" int dg_chkfinite_tiled_mn(int m, int n, int mb, int nb, double *const *tiles,
                                     void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(mb > 0, 3);
  DG_CHECK_ARG(nb > 0, 4);
  if (m == 0 || n == 0) return 1;
  DG_CHECK_ARG(tiles != nullptr, 5);
  return run_check(false, m, n, mb, nb, tiles, (cudaStream_t)stream);
}
