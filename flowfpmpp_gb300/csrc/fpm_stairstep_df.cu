// FP64 -> double-float (f32 pair) conversion of flat arrays.
//
// GB300 issues FP64 FMAs at about 1/58 of its FP32 rate, which makes an FP64
// Jacobi sweep ALU-bound at roughly a third of HBM bandwidth.  The fast
// sweep (fpm_jacobi_tma.cu) therefore keeps phi, src and rdiag as hi + lo
// float pairs (8 bytes per value, the same traffic as FP64, 48-bit
// significand) and evaluates the sweep with error-free FP32 transforms.
#include "fpm_internal.h"

namespace fpm {

__global__ void k_to_df(const double* __restrict__ x, float2* __restrict__ y, long long n) {
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x)
    y[m] = df_from_double(x[m]);
}
cudaError_t launch_to_df(const double* x, float2* y, long long n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  long long nb = (n + 255) / 256;
  if (nb > 152LL * 32) nb = 152LL * 32;
  k_to_df<<<(unsigned)nb, 256, 0, st>>>(x, y, n); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
