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

// ---------------------------------------------------------------------------
// Re-blocking copy: copyto!(buffer, A) between two tilings of one m x n matrix
// (copy_buffered / darray_copyto!, src/array/copy.jl:11-37 of Dagger.jl).
// Source and destination are tile grids (column-major grid, tile (i, j) =
// tiles[i + j*mt], each tile column-major with leading dimension equal to its
// row count).  One CTA copies a 32 x 32 block of the matrix: each warp walks
// columns, lane l reads row r0 + l of the source tile and writes the same row
// of the destination tile, so reads and writes are coalesced runs within one
// tile column (a block that straddles a tile edge splits the run).  8 bytes
// read and 8 written per element: an HBM-bound copy.
// ---------------------------------------------------------------------------
namespace dg {
namespace {

__global__ void __launch_bounds__(256) reblock_kernel(int m, int n, int smb, int snb, int smt,
                                                      const double *const *__restrict__ src,
                                                      int dmb, int dnb, int dmt,
                                                      double *const *__restrict__ dst) {
  const int r = blockIdx.x * 32 + threadIdx.x;
  if (r >= m) return;
  const int si = r / smb, sr = r - si * smb, di = r / dmb, dr = r - di * dmb;
  const int sld = min(smb, m - si * smb), dld = min(dmb, m - di * dmb);
  for (int q = threadIdx.y; q < 32; q += 8) {
    const int c = blockIdx.y * 32 + q;
    if (c >= n) break;
    const int sj = c / snb, sc = c - sj * snb, dj = c / dnb, dc = c - dj * dnb;
    const double v = src[si + (size_t)sj * smt][sr + (size_t)sc * sld];
    dst[di + (size_t)dj * dmt][dr + (size_t)dc * dld] = v;
  }
}

}  // namespace
}  // namespace dg

extern "C" int dg_copy_reblock(int m, int n, int src_mb, int src_nb, double *const *src_tiles,
                               int dst_mb, int dst_nb, double *const *dst_tiles, void *stream) {
  DG_CHECK_ARG(m >= 0, 1);
  DG_CHECK_ARG(n >= 0, 2);
  DG_CHECK_ARG(src_mb > 0, 3);
  DG_CHECK_ARG(src_nb > 0, 4);
  DG_CHECK_ARG(dst_mb > 0, 6);
  DG_CHECK_ARG(dst_nb > 0, 7);
  if (m == 0 || n == 0) return 0;
  DG_CHECK_ARG(src_tiles != nullptr, 5);
  DG_CHECK_ARG(dst_tiles != nullptr, 8);
  const int smt = (m + src_mb - 1) / src_mb, snt = (n + src_nb - 1) / src_nb;
  const int dmt = (m + dst_mb - 1) / dst_mb, dnt = (n + dst_nb - 1) / dst_nb;
  const dim3 grid((m + 31) / 32, (n + 31) / 32), blk(32, 8);
  DG_CHECK_ARG(grid.y <= 65535, 2);
  cudaStream_t s = (cudaStream_t)stream;
  // both pointer grids staged through one stream-ordered device buffer
  const size_t ns = (size_t)smt * snt, nd = (size_t)dmt * dnt;
  double **dptrs = nullptr;
  DG_CUDA_TRY(dg::pool_malloc_async((void **)&dptrs, sizeof(double *) * (ns + nd), s));
  DG_CUDA_TRY(cudaMemcpyAsync(dptrs, src_tiles, sizeof(double *) * ns, cudaMemcpyHostToDevice, s));
  DG_CUDA_TRY(
      cudaMemcpyAsync(dptrs + ns, dst_tiles, sizeof(double *) * nd, cudaMemcpyHostToDevice, s));
  dg::reblock_kernel<<<grid, blk, 0, s>>>(m, n, src_mb, src_nb, smt, dptrs, dst_mb, dst_nb, dmt,
                                          dptrs + ns);
  DG_CUDA_TRY(cudaGetLastError());
  dg::count_launches(1);
  // stream-ordered: the host pointer grids were staged by the pageable copies
  // before they returned, so the caller may free them at once
  DG_CUDA_TRY(cudaFreeAsync(dptrs, s));
  return 0;
}
