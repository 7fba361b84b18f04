// FP64 instruction-rate probe: the denominator of the FP64-pipe roofline the
// FP64 sweeps report next to their HBM fraction.  Every thread runs kChains
// independent fused multiply-add chains, so the pipe, not latency, sets the
// rate; the sums are stored so the chains cannot be removed.
#include "fpm_internal.h"

namespace fpm {

namespace {
constexpr int kChains = 8, kIters = 1024;
}

__global__ void k_fp64_rate(double* out, double m) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) a[c] = 1.0 + 1e-9 * (t + c);
  for (int it = 0; it < kIters; it++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) a[c] = __fma_rn(a[c], m, 1e-3);
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += a[c];
  out[t] = s;
}

// Blocks x threads of one probe launch; out holds blocks * threads doubles.
void fp64_rate_shape(int sms, int* blocks, int* threads) {
  *blocks = sms * 8;
  *threads = 256;
}

cudaError_t fp64_rate_probe(double* out, int blocks, int threads, cudaStream_t st, double* instr_per_s) {
  cudaEvent_t e0, e1;
  cudaError_t e = cudaEventCreate(&e0);
  if (e != cudaSuccess) return e;
  e = cudaEventCreate(&e1);
  if (e != cudaSuccess) {
    cudaEventDestroy(e0);
    return e;
  }
  float best = 1e30f;
  for (int rep = 0; rep < 3 && e == cudaSuccess; rep++) {
    cudaEventRecord(e0, st);
    k_fp64_rate<<<blocks, threads, 0, st>>>(out, 0.999999); note_launch();
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;  // the first launch warms up
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *instr_per_s = (double)blocks * threads * kChains * kIters / (best * 1e-3);
  return e;
}

}  // namespace fpm
