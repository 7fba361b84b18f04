// Shared device helpers: Fortran-layout indexing, correctly rounded FP64
// arithmetic without contraction, double-float (f32 pair) arithmetic, and
// deterministic block / grid reductions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fpm {

// ---------------------------------------------------------------- layout
// Stair-step fields follow the reference's Fortran layout, x fastest:
//   padded  (0:nx+1, 0:ny+1, 1:nz): phi, next (search direction), solid
//   interior (1:nx, 1:ny, 1:nz):    rhs, src, diag, rdiag, r, flow fields
//   faces   xlo/xhi(ny,nz), ylo/yhi(nx,nz), zlo/zhi(nx,ny)
//   axes    xc(0:nx+1), yc(0:ny+1), zc(1:nz), dx(1:nx), dy(1:ny), dz(1:nz)
struct Dims {
  int nx, ny, nz;
  __host__ __device__ __forceinline__ long long ph(int i, int j, int k) const {  // k is 1-based
    return (long long)i + (long long)(nx + 2) * ((long long)j + (long long)(ny + 2) * (long long)(k - 1));
  }
  __host__ __device__ __forceinline__ long long in(int i, int j, int k) const {
    return (long long)(i - 1) + (long long)nx * ((long long)(j - 1) + (long long)ny * (long long)(k - 1));
  }
  __host__ __device__ __forceinline__ long long xf(int j, int k) const { return (long long)(j - 1) + (long long)ny * (k - 1); }
  __host__ __device__ __forceinline__ long long yf(int i, int k) const { return (long long)(i - 1) + (long long)nx * (k - 1); }
  __host__ __device__ __forceinline__ long long zf(int i, int j) const { return (long long)(i - 1) + (long long)nx * (j - 1); }
  __host__ __device__ __forceinline__ long long plane() const { return (long long)(nx + 2) * (ny + 2); }
  __host__ __device__ __forceinline__ long long npad() const { return plane() * nz; }
  __host__ __device__ __forceinline__ long long ncell() const { return (long long)nx * ny * nz; }
};

// ---------------------------------------------------------------- exact FP64
// Separately rounded operations: the compiler may not fuse these into FMAs,
// so a kernel written with them reproduces a -ffp-contract=off CPU build bit
// for bit when it evaluates the same expression in the same order.
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// ---------------------------------------------------------------- double-float
// A value is hi + lo with |lo| <= ulp(hi)/2 (float2: x = hi, y = lo), giving a
// 48-bit significand.  Error-free transforms follow Dekker / Knuth (TwoSum)
// and use the hardware FMA for the exact product.
__device__ __forceinline__ float2 df_make(float h, float l) { return make_float2(h, l); }

// (a * b) + c, all double-float; relative error about 2^-46.
__device__ __forceinline__ float2 df_fma(float2 a, float2 b, float2 c) {
  float p = a.x * b.x;
  float pe = fmaf(a.x, b.x, -p);
  pe = fmaf(a.x, b.y, pe);
  pe = fmaf(a.y, b.x, pe);
  float s = p + c.x;
  float bb = s - p;
  float e = (p - (s - bb)) + (c.x - bb);
  e += pe + c.y;
  float h = s + e;
  return make_float2(h, e - (h - s));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  float s = a.x + b.x;
  float bb = s - a.x;
  float e = (a.x - (s - bb)) + (b.x - bb);
  e += a.y + b.y;
  float h = s + e;
  return make_float2(h, e - (h - s));
}
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  float p = a.x * b.x;
  float pe = fmaf(a.x, b.x, -p);
  pe = fmaf(a.x, b.y, pe);
  pe = fmaf(a.y, b.x, pe);
  float h = p + pe;
  return make_float2(h, pe - (h - p));
}
// FP64 <-> double-float.  Splitting uses FP64 conversions, so kernels only do
// it outside the sweep loop (operator build and the final write-back).
__host__ __device__ __forceinline__ float2 df_from_double(double x) {
  float h = (float)x;
  float l = (float)(x - (double)h);
  return make_float2(h, l);
}
__host__ __device__ __forceinline__ double df_to_double(float2 v) { return (double)v.x + (double)v.y; }

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ int lin_tid() { return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z); }
__device__ __forceinline__ int lin_nthreads() { return blockDim.x * blockDim.y * blockDim.z; }
__device__ __forceinline__ int lin_bid() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }
__device__ __forceinline__ int lin_nblocks() { return gridDim.x * gridDim.y * gridDim.z; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide reduction of NS sums and NM maxima (maxima of non-negative values;
// fmax drops NaN like the reference's max()).  Result valid in thread 0.  The
// shuffle tree and the warp order are fixed, so results are reproducible.
template <int NS, int NM>
__device__ __forceinline__ void block_reduce(double (&s)[NS > 0 ? NS : 1], double (&m)[NM > 0 ? NM : 1]) {
  __shared__ double sh[(NS + NM) > 0 ? (NS + NM) : 1][32];
  int tid = lin_tid(), lane = tid & 31, warp = tid >> 5;
  int nwarp = (lin_nthreads() + 31) >> 5;
#pragma unroll
  for (int n = 0; n < NS; n++) s[n] = warp_sum(s[n]);
#pragma unroll
  for (int n = 0; n < NM; n++) m[n] = warp_max(m[n]);
  if (lane == 0) {
#pragma unroll
    for (int n = 0; n < NS; n++) sh[n][warp] = s[n];
#pragma unroll
    for (int n = 0; n < NM; n++) sh[NS + n][warp] = m[n];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int n = 0; n < NS; n++) s[n] = warp_sum(lane < nwarp ? sh[n][lane] : 0.0);
#pragma unroll
    for (int n = 0; n < NM; n++) m[n] = warp_max(lane < nwarp ? sh[NS + n][lane] : 0.0);
  }
  __syncthreads();
}

// Grid-wide deterministic reduction.  Each block stores its partials; the last
// block to finish (ticket counter) combines them in block order and writes
// out[0..NS) = sums, out[NS..NS+NM) = maxima.  partials holds
// (NS+NM) * nblocks doubles; *ticket starts at 0 and the last block resets it.
// Returns true (in every thread of the last block) so callers can append a
// scalar epilogue executed once per launch after the reduction is complete.
template <int NS, int NM>
__device__ bool grid_reduce(double (&s)[NS > 0 ? NS : 1], double (&m)[NM > 0 ? NM : 1], double* partials,
                            unsigned int* ticket, double* out) {
  __shared__ bool am_last;
  const int nb = lin_nblocks(), bid = lin_bid(), tid = lin_tid();
  block_reduce<NS, NM>(s, m);
  if (tid == 0) {
#pragma unroll
    for (int n = 0; n < NS; n++) partials[(size_t)n * nb + bid] = s[n];
#pragma unroll
    for (int n = 0; n < NM; n++) partials[(size_t)(NS + n) * nb + bid] = m[n];
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    am_last = (t == (unsigned int)nb - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double as[NS > 0 ? NS : 1], am[NM > 0 ? NM : 1];
#pragma unroll
  for (int n = 0; n < NS; n++) as[n] = 0.0;
#pragma unroll
  for (int n = 0; n < NM; n++) am[n] = 0.0;
  for (int b = tid; b < nb; b += lin_nthreads()) {
#pragma unroll
    for (int n = 0; n < NS; n++) as[n] += __ldcg(partials + (size_t)n * nb + b);
#pragma unroll
    for (int n = 0; n < NM; n++) am[n] = fmax(am[n], __ldcg(partials + (size_t)(NS + n) * nb + b));
  }
  block_reduce<NS, NM>(as, am);
  if (tid == 0) {
#pragma unroll
    for (int n = 0; n < NS; n++) out[n] = as[n];
#pragma unroll
    for (int n = 0; n < NM; n++) out[NS + n] = am[n];
    *ticket = 0u;
    __threadfence();
  }
  __syncthreads();
  return true;
}

}  // namespace fpm
