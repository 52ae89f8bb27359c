// Pre-factorization checks on a tiled matrix:
//   ishermitian(::DArray) (src/array/linalg.jl:90-124 of Dagger.jl): each
//     diagonal tile must equal its transpose exactly; each off-diagonal pair
//     (i, j), i > j, passes when ||A_ij - A_ji'||_F <= sqrt(eps) *
//     max(||A_ij||_F, ||A_ji||_F) (is_cross_hermitian, linalg.jl:43-48).
//   chkfinite(::DArray) (linalg.jl:138-148): every element finite.
// One launch covers all tile pairs: CTA (i, j) with i >= j compares tile
// (i, j) with the transpose of tile (j, i) through 32 x 33 shared-memory
// transposes (both reads coalesced), reduces its three sums of squares and
// raises a device flag when the pair fails.  Stdlib's ishermitian compares
// with ==, so a NaN anywhere in a diagonal tile fails the check as well.
#include <math.h>

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

__global__ void __launch_bounds__(256) herm_pair_kernel(const double *const *tiles, int n, int nb,
                                                        int mt, int *flag) {
  const int i = blockIdx.x, j = blockIdx.y;
  if (i < j) return;
  __shared__ double xs[32][33], ys[32][33];
  __shared__ double red[8];
  const int ri = min(nb, n - i * nb), rj = min(nb, n - j * nb);
  const double *X = tiles[i + (size_t)j * mt];  // ri x rj, ld ri
  const double *Y = tiles[j + (size_t)i * mt];  // rj x ri, ld rj
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  double d2 = 0.0, x2 = 0.0, y2 = 0.0;
  int mism = 0;
  for (int r0 = 0; r0 < ri; r0 += 32)
    for (int c0 = 0; c0 < rj; c0 += 32) {
      __syncthreads();
      for (int c = ty; c < 32; c += 8) {
        int r = r0 + tx, cc = c0 + c;
        xs[c][tx] = (r < ri && cc < rj) ? X[(size_t)r + (size_t)cc * ri] : 0.0;
        // Y(cc', r') with cc' = c0 + tx, r' = r0 + c: coalesced along cc'
        int yr = c0 + tx, yc = r0 + c;
        ys[tx][c] = (yr < rj && yc < ri) ? Y[(size_t)yr + (size_t)yc * rj] : 0.0;
      }
      __syncthreads();
      for (int c = ty; c < 32; c += 8) {
        int r = r0 + tx, cc = c0 + c;
        if (r < ri && cc < rj) {
          double x = xs[c][tx], y = ys[c][tx];  // X(r, cc) and Y(cc, r)
          if (i == j) {
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
  if (i == j) {
    if (__syncthreads_or(mism) && threadIdx.x == 0) atomicOr(flag, 1);
    return;
  }
  d2 = block_sum(d2, red);
  x2 = block_sum(x2, red);
  y2 = block_sum(y2, red);
  if (threadIdx.x == 0) {
    const double rtol = sqrt(2.220446049250313e-16);
    // NaN in either norm makes the comparison false, as in Julia
    if (!(sqrt(d2) <= rtol * fmax(sqrt(x2), sqrt(y2)))) atomicOr(flag, 1);
  }
}

__global__ void finite_kernel(const double *const *tiles, int m, int n, int mb, int nb, int mt,
                              int *flag) {
  const int i = blockIdx.x, j = blockIdx.y;
  const int ri = min(mb, m - i * mb), cj = min(nb, n - j * nb);
  const double *X = tiles[i + (size_t)j * mt];
  int bad = 0;
  for (size_t e = threadIdx.x; e < (size_t)ri * cj; e += blockDim.x)
    if (!isfinite(X[e])) bad = 1;
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

// herm: n x n with Blocks(nb, nb); otherwise m x n with Blocks(mb, nb).
int run_check(bool herm, int m, int n, int mb, int nb, double *const *tiles, cudaStream_t s) {
  const int mt = (m + mb - 1) / mb, nt = (n + nb - 1) / nb;
  DG_CHECK_ARG(mt <= 65535 && nt <= 65535, 2);
  int *flag = nullptr;
  int rc = dg::device_state().scratch_int(&flag);
  if (rc) return rc;
  // the tile pointer grid is staged through a small device buffer
  const double **dptrs = nullptr;
  size_t bytes = sizeof(double *) * (size_t)mt * nt;
  DG_CUDA_TRY(dg::pool_malloc_async((void **)&dptrs, bytes, s));
  DG_CUDA_TRY(cudaMemcpyAsync(dptrs, tiles, bytes, cudaMemcpyHostToDevice, s));
  DG_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), s));
  dim3 grid(mt, nt);
  if (herm)
    herm_pair_kernel<<<grid, 256, 0, s>>>(dptrs, n, nb, mt, flag);
  else
    finite_kernel<<<grid, 256, 0, s>>>(dptrs, m, n, mb, nb, mt, flag);
  DG_CUDA_TRY(cudaGetLastError());
  dg::count_launches(1);
  int h = 0;
  DG_CUDA_TRY(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  DG_CUDA_TRY(cudaFreeAsync(dptrs, s));
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
