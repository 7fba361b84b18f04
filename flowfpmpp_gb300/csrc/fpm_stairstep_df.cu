// Weighted-Jacobi sweep in double-float (f32 pair) arithmetic.
//
// GB300 issues FP64 FMAs at about 1/58 of its FP32 rate, which makes the FP64
// sweep of src/fpm_stairstep_mpi_3d.f90:384-399 ALU-bound at roughly a third
// of HBM bandwidth.  This kernel keeps phi, src and rdiag as hi+lo float
// pairs (8 bytes per value, the same traffic as FP64) and evaluates
//   b = 0.2 a + rdiag (src + cw a_w + ce a_e + cs a_s + cn a_n + cb a_b + ct a_t)
// in the reference's order with error-free FP32 transforms, so a sweep costs
// only FP32 instructions and stays HBM-bound.  The representation carries a
// 48-bit significand; after thousands of sweeps the field agrees with the
// FP64 oracle to about 1e-14 relative (tested to 1e-12).
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
  k_to_df<<<(unsigned)nb, 256, 0, st>>>(x, y, n);
  return cudaGetLastError();
}

__global__ void k_from_df_interior(Dims d, const float2* __restrict__ x, double* __restrict__ y) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  if (i > d.nx || j > d.ny) return;
  for (int k = blockIdx.z + 1; k <= d.nz; k += gridDim.z) {
    const long long p = d.ph(i, j, k);
    y[p] = df_to_double(x[p]);
  }
}
cudaError_t launch_from_df_interior(const Dims& d, const float2* x, double* y, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_from_df_interior<<<L.grid, L.block, 0, st>>>(d, x, y);
  return cudaGetLastError();
}

// coef_df holds cw, ce (nx) | cs, cn (ny) | cb, ct (nz) as double-float.
__global__ void k_jacobi_df(Dims d, const float2* __restrict__ a, float2* __restrict__ b,
                            const float2* __restrict__ src, const float2* __restrict__ rdiag,
                            const float2* __restrict__ coef) {
  const float2* cw = coef;
  const float2* ce = cw + d.nx;
  const float2* cs = ce + d.nx;
  const float2* cn = cs + d.ny;
  const float2* cb = cn + d.ny;
  const float2* ct = cb + d.nz;
  const float2 p2 = make_float2(0.2f, -2.9802322831784522e-09f);  // 0.2 split as hi + lo
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  if (i > d.nx || j > d.ny) return;
  const float2 cwi = cw[i - 1], cei = ce[i - 1], csj = cs[j - 1], cnj = cn[j - 1];
  const long long px = d.nx + 2, pl = d.plane();
  for (int k = blockIdx.z + 1; k <= d.nz; k += gridDim.z) {
    const long long cc = d.in(i, j, k), p = d.ph(i, j, k);
    const long long pb = k > 1 ? p - pl : p, pt = k < d.nz ? p + pl : p;
    float2 s = src[cc];
    s = df_fma(cwi, a[p - 1], s);
    s = df_fma(cei, a[p + 1], s);
    s = df_fma(csj, a[p - px], s);
    s = df_fma(cnj, a[p + px], s);
    s = df_fma(cb[k - 1], a[pb], s);
    s = df_fma(ct[k - 1], a[pt], s);
    const float2 t = df_mul(p2, a[p]);
    b[p] = df_fma(rdiag[cc], s, t);
  }
}
cudaError_t launch_jacobi_df(const Dims& d, const float2* a, float2* b, const float2* src, const float2* rdiag,
                             const float2* coef_df, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_jacobi_df<<<L.grid, L.block, 0, st>>>(d, a, b, src, rdiag, coef_df);
  return cudaGetLastError();
}

}  // namespace fpm
