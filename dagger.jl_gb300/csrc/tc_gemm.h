// Internal interface of the tcgen05 BF16 / FP16 / FP8 GEMM (tc_gemm.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace dg {

// Kernel parameters (passed as one __grid_constant__ struct so the tensor
// maps stay in parameter space, as TMA requires).
struct TcParams {
  CUtensorMap a_hi, b_hi, a_lo, b_lo, a_mid, b_mid;
  int m, n, k;
  int a_row0, b_row0;  // first panel row of the A / B operand
  float alpha, beta;
  float *c;
  long long ldc;
  int layout;          // 0 = column-major C (ldc); 1 = packed upper row panels
  int upper;           // update only i <= j
  long long off;       // layout 1: global index of row/column 0 of this update
  int nb;              // layout 1: row-panel height
  long long ntot;      // layout 1: order of the whole matrix
  int *status;         // device status word: non-zero on entry = skip; timeout recorded
  uint32_t idesc;      // tcgen05 instruction descriptor (operand types, M, N)
  const float *alpha_dev;  // when set, alpha is read from device memory
  // FP8 operands: the product of output (i, j) is multiplied by
  // a_scale[a_row0 + i] * b_scale[b_row0 + j] (the vectors' power-of-two
  // scales); null for 16-bit operands
  const float *a_scale, *b_scale;
};

struct TcGemmArgs {
  int m, n, k, terms;                 // terms: 1 (bf16), 3 (hi/lo split) or 6 (hi/mid/lo)
  int fp8;                            // terms 1 with E4M3 operands (one byte per value,
                                      // lda / ldb in values, multiples of 16) and the
                                      // per-vector scales a_scale / b_scale
  const float *a_scale, *b_scale;
  const void *a_hi, *a_lo;            // K-major BF16 panels
  const void *a_mid, *b_mid;          // terms 6: the middle slices
  int lda, a_rows, a_row0;
  const void *b_hi, *b_lo;
  int ldb, b_rows, b_row0;
  float alpha, beta;
  float *c;
  long long ldc;
  int layout, upper;
  long long off;
  int nb;
  long long ntot;
  int bn;                             // 128 or 256 columns per CTA tile
  int *status;
  int fp16;                           // operands are FP16 instead of BF16
  const float *alpha_dev;             // optional device-resident alpha
  int tiles_per_cta;                  // 0: one wave (a CTA per SM walks all tiles); else about
                                      // that many tiles per CTA, so that CTAs finish and
                                      // launches of other streams can take their SMs
};

int tc_gemm_bf16(const TcGemmArgs &g, cudaStream_t s);

// E4M3 copy of ncols FP32 vectors of length k (vector c at src + c * ld), a
// power-of-two scale per vector (dst values = v / scale[c], the largest in
// [128, 256)), dst vector c at dst + c * ldd.  Skips when *a1 or *a2 is
// non-zero (either may be null).
int split_e4m3(const float *src, long long ld, int k, int ncols, uint8_t *dst, long long ldd,
               float *scale, const int *a1, const int *a2, cudaStream_t s);

}  // namespace dg
