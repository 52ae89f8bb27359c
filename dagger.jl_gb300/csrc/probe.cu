// Pipe-throughput probe used by the benchmark to state its FP64 roofline.
//
// The device's FP64 rate is not in the measured-peaks record (which covers
// HBM copy bandwidth and BF16 tensor throughput), so the benchmark measures
// it in the same run: every thread of a grid of (SMs x 8) CTAs runs
// sixteen independent fused multiply-add chains for `iters` steps, enough
// independent work to keep the FP64 pipe of every SM busy.  The result
// depends on the SM clock at the time, like any peak.
#include "dg_common.cuh"

namespace {

__global__ void __launch_bounds__(256) fma_chains_f64(int iters, double seed, double *out) {
  double a[16];
#pragma unroll
  for (int j = 0; j < 16; j++) a[j] = seed + threadIdx.x + j;
  const double m = 0.9999999, c = 1e-7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 16; j++) a[j] = fma(a[j], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 16; j++) s += a[j];
  if (s == 12345.678) out[0] = s;  // keeps the chains live; never true in practice
}

}  // namespace

extern "C" int dg_probe_fp64_fma_tflops(int iters, double *tflops, void *stream) {
  DG_CHECK_ARG(iters > 0, 1);
  DG_CHECK_ARG(tflops != nullptr, 2);
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = dg_num_sms() * 8, threads = 256;
  double *sink = nullptr;
  DG_CUDA_TRY(cudaMallocAsync((void **)&sink, sizeof(double), s));
  cudaEvent_t e0, e1;
  DG_CUDA_TRY(cudaEventCreate(&e0));
  DG_CUDA_TRY(cudaEventCreate(&e1));
  fma_chains_f64<<<blocks, threads, 0, s>>>(iters / 4 + 1, 1.0, sink);  // warm-up
  float best = 0.f;
  for (int rep = 0; rep < 3; rep++) {
    DG_CUDA_TRY(cudaEventRecord(e0, s));
    fma_chains_f64<<<blocks, threads, 0, s>>>(iters, 1.0, sink);
    DG_CUDA_TRY(cudaEventRecord(e1, s));
    DG_CUDA_TRY(cudaGetLastError());
    DG_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep == 0 || ms < best) best = ms;
  }
  dg::count_launches(4);
  const float ms = best;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(sink, s);
  const double flops = 2.0 * 16.0 * (double)iters * blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return 0;
}
