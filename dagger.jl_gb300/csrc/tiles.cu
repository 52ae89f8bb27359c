// Tile copies of copytri! (src/array/mul.jl:368-425), which makes the result
// of syrk_dagger! a full symmetric matrix: an off-diagonal tile receives the
// transpose of its mirror tile (copytile!), a diagonal tile its upper
// triangle mirrored into the lower one (copydiagtile!, the diagonal kept).
#include "dg_common.cuh"

namespace dg {
namespace {

// dst (cols x rows, ldd) = src (rows x cols, lds)'; 32 x 32 blocks through
// shared memory, reads and writes along columns.
__global__ void __launch_bounds__(256) tile_transpose_kernel(const double *__restrict__ src,
                                                             long long lds, int rows, int cols,
                                                             double *__restrict__ dst,
                                                             long long ldd) {
  __shared__ double buf[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
#pragma unroll
  for (int q = ty; q < 32; q += 8) {
    const int r = r0 + tx, c = c0 + q;
    buf[q][tx] = (r < rows && c < cols) ? src[(size_t)r + (size_t)c * lds] : 0.0;
  }
  __syncthreads();
#pragma unroll
  for (int q = ty; q < 32; q += 8) {
    const int c = c0 + tx, r = r0 + q;  // dst(c, r) = src(r, c)
    if (r < rows && c < cols) dst[(size_t)c + (size_t)r * ldd] = buf[tx][q];
  }
}

// A(i, j) = A(j, i) for i > j (n x n, lda): the upper triangle mirrored.
__global__ void __launch_bounds__(256) tile_mirror_kernel(double *A, long long lda, int n) {
  __shared__ double buf[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int bi = blockIdx.x, bj = blockIdx.y;  // target block (bi, bj), bi >= bj
  if (bi < bj) return;
  const int r0 = bj * 32, c0 = bi * 32;  // source block rows r0.., columns c0.. (upper side)
#pragma unroll
  for (int q = ty; q < 32; q += 8) {
    const int r = r0 + tx, c = c0 + q;
    buf[q][tx] = (r < n && c < n) ? A[(size_t)r + (size_t)c * lda] : 0.0;
  }
  __syncthreads();
#pragma unroll
  for (int q = ty; q < 32; q += 8) {
    const int i = c0 + tx, j = r0 + q;  // A(i, j) = A(j, i) with j = r, i = c
    if (i < n && j < n && i > j) A[(size_t)i + (size_t)j * lda] = buf[tx][q];
  }
}

}  // namespace

int tile_transpose(const double *src, long long lds, int rows, int cols, double *dst,
                   long long ldd, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return 0;
  const dim3 grid((rows + 31) / 32, (cols + 31) / 32), blk(32, 8);
  if (grid.y > 65535) return DG_ERR_UNSUPPORTED;
  tile_transpose_kernel<<<grid, blk, 0, s>>>(src, lds, rows, cols, dst, ldd);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

int tile_mirror_upper(double *A, long long lda, int n, cudaStream_t s) {
  if (n <= 1) return 0;
  const dim3 grid((n + 31) / 32, (n + 31) / 32), blk(32, 8);
  if (grid.y > 65535) return DG_ERR_UNSUPPORTED;
  tile_mirror_kernel<<<grid, blk, 0, s>>>(A, lda, n);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

}  // namespace dg
