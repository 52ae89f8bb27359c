// Host-to-tile upload for the factorization region: tile (i, j) of a matrix
// held row-major in pinned host memory (element (r, c) at host[r*ldh + c],
// the layout of a C-contiguous array) is read by the kernel over the host
// link through unified addressing and transposed in shared memory into the
// column-major tile (leading dimension = its row count).  The copy engines
// and kernel reads reach the same link bandwidth on GB300 (about 211 GB/s),
// so reading from the kernel costs nothing and folds the re-tiling into the
// transfer.  As graph tasks the uploads overlap the factorization: a tile's
// first task waits only for its own upload, the way Dagger moves a CPU chunk
// to the GPU processor when the first task that needs it runs
// (ext/CUDAExt.jl:329-348).
#include "dg_common.cuh"

namespace dg {
namespace {

// CTA: 32 x 8 threads over a 32-column strip of the tile, 64 rows at a time
// (8 loads of 8 bytes per thread in flight, 16 KiB per CTA, to cover the host
// link's latency); reads along host rows (256 B per warp), writes along tile
// columns.  One CTA per 32 columns: a 1024-wide tile is 32 CTAs, light enough
// to run beside the factorization's kernels.
__global__ void __launch_bounds__(256) upload_tile_kernel(const double *__restrict__ host,
                                                          long long ldh, int rows, int cols,
                                                          double *__restrict__ tile) {
  __shared__ double buf[64][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int cb = blockIdx.x * 32, c = cb + tx;
  for (int rb = 0; rb < rows; rb += 64) {
    double v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int r = rb + ty + 8 * q;
      v[q] = (r < rows && c < cols) ? host[(size_t)r * ldh + c] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < 8; q++) buf[ty + 8 * q][tx] = v[q];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int cc = cb + ty + 8 * q;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int r = rb + 32 * h + tx;
        if (r < rows && cc < cols) tile[(size_t)r + (size_t)cc * rows] = buf[32 * h + tx][ty + 8 * q];
      }
    }
    __syncthreads();
  }
}

}  // namespace

int upload_tile(const double *host, long long ldh, int rows, int cols, double *tile,
                cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return 0;
  const dim3 grid((cols + 31) / 32), blk(32, 8);
  upload_tile_kernel<<<grid, blk, 0, s>>>(host, ldh, rows, cols, tile);
  DG_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}

// Whether a kernel may read p: device, managed or page-locked host memory
// (pageable host memory is not addressable from the GPU).
bool device_readable(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged ||
         (a.type == cudaMemoryTypeHost && a.devicePointer == p);
}

}  // namespace dg
