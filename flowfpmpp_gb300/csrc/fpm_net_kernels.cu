// Learned initial guess / preconditioner: the 3-D convolution kernels.
//
// Activations are channels-last BF16: voxel v = i + nx (j + ny k) (x fastest,
// the solver's own cell order), channel c at v * C + c.  A 3x3x3 convolution
// with zero padding is an implicit GEMM, M = voxels, N = output channels,
// K = 27 taps x input channels, run on the tensor cores with
// mma.sync.m16n8k16 (BF16 operands, FP32 accumulation).
//
// Forward / backward-data tile: a CTA of 4 warps owns 4 rows (j) x 32 voxels
// (i) of one plane k; each warp owns one row (two m16 tiles) and all output
// channels.  For every 16-channel slice of the input the CTA stages in shared
// memory, with cp.async (zero fill outside the grid), the 6 x 3 neighbouring
// rows of 34 voxels and the slice's weights for all 27 taps, then runs the
// 27 taps out of shared memory with ldmatrix.  Rows of 32 bytes are stored
// with their two 16-byte halves swapped on every other group of four rows,
// so the 8-row ldmatrix phases hit distinct banks.
//
// The input of a convolution may be the concatenation of a tensor A at the
// same resolution and a tensor B at half resolution read with nearest-
// neighbour upsampling (the decoder's skip connection), fused into the loads.
//
// Weight gradient: dW[t][co][ci] = sum_v dY[v][co] X[v + t][ci], an M = co,
// N = ci, K = voxel GEMM; both operands are read transposed out of shared
// memory (ldmatrix.trans).
#include <cuda_bf16.h>

#include "fpm_internal.h"
#include "fpm_net.h"

namespace fpm {
namespace net {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::);
  asm volatile("cp.async.wait_group 0;\n" ::);
}
__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int kRows = 4;             // rows (j) per CTA, one per warp
constexpr int kTx = 32;              // voxels (i) per row
constexpr int kHaloRows = 18;        // (kRows + 2) x 3 planes
constexpr int kHaloVox = kTx + 2;    // 34
constexpr int kActBytes = kHaloRows * kHaloVox * 32;

// Byte offset of 16-byte half h of 32-byte row r (swizzled).
__device__ __forceinline__ int sw32(int r, int h) { return (r * 2 + (h ^ ((r >> 2) & 1))) * 16; }

// Stage the 16-channel slice `slice` of the (possibly concatenated) input
// around the CTA's tile: 6 rows x 3 planes x 34 voxels.
__device__ __forceinline__ void stage_input(const ConvArgs& a, int slice, int i0, int j0, int k0, char* act) {
  const int c0 = slice * 16;
  const bool from_a = c0 < a.ca;
  const int hx = a.nx >> 1, hy = a.ny >> 1;
  for (int idx = threadIdx.x + threadIdx.y * 32; idx < kHaloRows * kHaloVox * 2; idx += 128) {
    const int row = idx / (kHaloVox * 2), rem = idx - row * (kHaloVox * 2);
    const int vox = rem >> 1, h = rem & 1;
    const int dj = row % 6 - 1, dk = row / 6 - 1;
    const int i = i0 - 1 + vox, j = j0 + dj, k = k0 + dk;
    const bool ok = i >= 0 && i < a.nx && j >= 0 && j < a.ny && k >= 0 && k < a.nz;
    const __nv_bfloat16* src;
    if (from_a) {
      src = a.a + ((long long)(ok ? i + (long long)a.nx * (j + (long long)a.ny * k) : 0) * a.ca + c0 + 8 * h);
    } else {
      const long long vb = ok ? (i >> 1) + (long long)hx * ((j >> 1) + (long long)hy * (k >> 1)) : 0;
      src = a.b + (vb * a.cb + (c0 - a.ca) + 8 * h);
    }
    cp_async16(act + sw32(row * kHaloVox + vox, h), src, ok);
  }
}

// out[v][co] = epilogue(bias[co] + sum_t sum_ci in[v + t][ci] w[t][co][ci]).
template <int COUT>
__global__ void __launch_bounds__(128) k_conv(ConvArgs a) {
  constexpr int NT = COUT / 8;
  extern __shared__ __align__(128) char smem[];
  char* act = smem;
  char* wts = smem + kActBytes;
  const int warp = threadIdx.y, lane = threadIdx.x;
  const int i0 = blockIdx.x * kTx, j0 = blockIdx.y * kRows, k0 = blockIdx.z;
  float acc[2][NT][4];
#pragma unroll
  for (int m = 0; m < 2; m++)
#pragma unroll
    for (int n = 0; n < NT; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[m][n][q] = 0.f;

  const int nslices = a.cin / 16;
  for (int s = 0; s < nslices; s++) {
    stage_input(a, s, i0, j0, k0, act);
    const __nv_bfloat16* wsrc = a.w + (long long)s * 27 * COUT * 16;
    for (int idx = threadIdx.x + threadIdx.y * 32; idx < 27 * COUT * 2; idx += 128) {
      const int row = idx >> 1, h = idx & 1;  // row = t * COUT + co
      cp_async16(wts + sw32(row, h), wsrc + row * 16 + 8 * h, true);
    }
    cp_async_wait_all();
    __syncthreads();
#pragma unroll 1
    for (int t = 0; t < 27; t++) {
      const int di = t % 3 - 1, dj = (t / 3) % 3 - 1, dk = t / 9 - 1;
      const int row = (warp + 1 + dj) + 6 * (dk + 1);
      unsigned af[2][4];
#pragma unroll
      for (int m = 0; m < 2; m++) {
        const int vox = 1 + di + 16 * m + (lane & 15);
        ldsm_x4(af[m], act + sw32(row * kHaloVox + vox, lane >> 4));
      }
#pragma unroll
      for (int p = 0; p < NT / 2; p++) {
        const int mi = lane >> 3;
        const int co = 16 * p + (mi >> 1) * 8 + (lane & 7);
        unsigned bf[4];
        ldsm_x4(bf, wts + sw32(t * COUT + co, mi & 1));
#pragma unroll
        for (int m = 0; m < 2; m++) {
          mma_bf16(acc[m][2 * p], af[m], bf[0], bf[1]);
          mma_bf16(acc[m][2 * p + 1], af[m], bf[2], bf[3]);
        }
      }
    }
    __syncthreads();
  }

  // Epilogue.
  const int g = lane >> 2, t4 = lane & 3;
  const int j = j0 + warp, k = k0;
  if (j >= a.ny) return;
#pragma unroll
  for (int m = 0; m < 2; m++) {
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int i = i0 + 16 * m + g + 8 * half;
      if (i >= a.nx) continue;
      const long long v = i + (long long)a.nx * (j + (long long)a.ny * k);
#pragma unroll
      for (int n = 0; n < NT; n++) {
        const int co = 8 * n + 2 * t4;
        float x0 = acc[m][n][2 * half], x1 = acc[m][n][2 * half + 1];
        if (a.mode == kConvBf16) {
          if (a.bias) {
            x0 += a.bias[co];
            x1 += a.bias[co + 1];
          }
          if (a.relu) {
            x0 = fmaxf(x0, 0.f);
            x1 = fmaxf(x1, 0.f);
          }
          *reinterpret_cast<__nv_bfloat162*>(a.y + v * COUT + co) = __floats2bfloat162_rn(x0, x1);
        } else if (a.mode == kConvF32) {
          if (a.bias) {
            x0 += a.bias[co];
            x1 += a.bias[co + 1];
          }
          *reinterpret_cast<float2*>(a.yf + v * COUT + co) = make_float2(x0, x1);
        } else {  // kConvGrad: split into the gradients of A and of B (upsampling adjoint)
          if (co < a.csplit) {
            float* p = a.ga + v * a.csplit + co;
            p[0] += x0;
            p[1] += x1;
          } else {
            const int cbn = COUT - a.csplit;
            const long long vb = (i >> 1) + (long long)(a.nx >> 1) * ((j >> 1) + (long long)(a.ny >> 1) * (k >> 1));
            float* p = a.gb + vb * cbn + (co - a.csplit);
            atomicAdd(p, x0);
            atomicAdd(p + 1, x1);
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------- weight gradient
// One CTA: one 16-channel input slice, one plane offset dk, a run of
// `tiles_per_cta` voxel tiles (4 rows x 32 voxels of one plane each).  Output
// tiles (9 taps (di, dj) x COUT/16, each 16 co x 16 ci) are dealt round-robin
// to the 4 warps.  Rows in shared memory are padded to an odd number of
// 16-byte units so the 8-row ldmatrix phases hit distinct banks.
template <int COUT>
__global__ void __launch_bounds__(128) k_conv_wgrad(WgradArgs w) {
  constexpr int MT = COUT / 16;
  constexpr int NTILE = 9 * MT;
  constexpr int PER_WARP = (NTILE + 3) / 4;
  constexpr int DY_STRIDE = COUT * 2 + 16;   // bytes per voxel row of dY
  constexpr int X_STRIDE = 48;               // bytes per voxel row of the input slice
  extern __shared__ __align__(128) char smem[];
  char* dys = smem;                                  // [128][DY_STRIDE]
  char* xs = smem + kRows * kTx * DY_STRIDE;         // [6][34][X_STRIDE]
  const ConvArgs& a = w.conv;
  const int warp = threadIdx.y, lane = threadIdx.x;
  const int slice = blockIdx.y, dk = (int)blockIdx.z - 1;
  const int tiles_x = (a.nx + kTx - 1) / kTx, tiles_y = (a.ny + kRows - 1) / kRows;
  const long long ntiles = (long long)tiles_x * tiles_y * a.nz;
  float acc[PER_WARP][2][4];
#pragma unroll
  for (int q = 0; q < PER_WARP; q++)
#pragma unroll
    for (int n = 0; n < 2; n++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[q][n][e] = 0.f;

  const long long t_begin = (long long)blockIdx.x * w.tiles_per_cta;
  const long long t_end = min(ntiles, t_begin + w.tiles_per_cta);
  const int c0 = slice * 16;
  const bool from_a = c0 < a.ca;
  const int hx = a.nx >> 1, hy = a.ny >> 1;
  for (long long tile = t_begin; tile < t_end; tile++) {
    const int tx = (int)(tile % tiles_x);
    const int ty = (int)((tile / tiles_x) % tiles_y);
    const int k0 = (int)(tile / ((long long)tiles_x * tiles_y));
    const int i0 = tx * kTx, j0 = ty * kRows;
    // dY tile: 128 voxels x COUT channels (zero outside the grid).
    for (int idx = threadIdx.x + threadIdx.y * 32; idx < kRows * kTx * (COUT / 8); idx += 128) {
      const int vox = idx / (COUT / 8), ch = idx - vox * (COUT / 8);
      const int i = i0 + (vox & 31), j = j0 + (vox >> 5);
      const bool ok = i < a.nx && j < a.ny;
      const long long v = ok ? i + (long long)a.nx * (j + (long long)a.ny * k0) : 0;
      cp_async16(dys + vox * DY_STRIDE + ch * 16, w.dy + v * COUT + ch * 8, ok);
    }
    // input slice: 6 rows x 34 voxels at plane k0 + dk.
    for (int idx = threadIdx.x + threadIdx.y * 32; idx < 6 * kHaloVox * 2; idx += 128) {
      const int row = idx / (kHaloVox * 2), rem = idx - row * (kHaloVox * 2);
      const int vox = rem >> 1, h = rem & 1;
      const int i = i0 - 1 + vox, j = j0 + row - 1, k = k0 + dk;
      const bool ok = i >= 0 && i < a.nx && j >= 0 && j < a.ny && k >= 0 && k < a.nz;
      const __nv_bfloat16* src;
      if (from_a) {
        src = a.a + ((long long)(ok ? i + (long long)a.nx * (j + (long long)a.ny * k) : 0) * a.ca + c0 + 8 * h);
      } else {
        const long long vb = ok ? (i >> 1) + (long long)hx * ((j >> 1) + (long long)hy * (k >> 1)) : 0;
        src = a.b + (vb * a.cb + (c0 - a.ca) + 8 * h);
      }
      cp_async16(xs + (row * kHaloVox + vox) * X_STRIDE + h * 16, src, ok);
    }
    cp_async_wait_all();
    __syncthreads();
#pragma unroll 1
    for (int ks = 0; ks < 8; ks++) {  // 16 voxels per step: row ks / 2, voxels 16 (ks % 2) ..
      const int r = ks >> 1, vb = 16 * (ks & 1);
      const int mi = lane >> 3;
#pragma unroll
      for (int q = 0; q < PER_WARP; q++) {
        const int id = warp + 4 * q;
        if (id >= NTILE) break;
        const int mt = id % MT, tap = id / MT;  // tap = (dj+1)*3 + (di+1)
        const int di = tap % 3 - 1, dj = tap / 3 - 1;
        unsigned af[4], bf[4];
        // A = dY^T (co x voxel): matrices (co lo, v 0-7), (co hi, v 0-7), (co lo, v 8-15), (co hi, v 8-15)
        ldsm_x4_t(af, dys + (r * 32 + vb + (lane & 7) + 8 * (mi >> 1)) * DY_STRIDE + (2 * mt + (mi & 1)) * 16);
        // B = X (voxel x ci): matrices (ci lo, v 0-7), (ci lo, v 8-15), (ci hi, v 0-7), (ci hi, v 8-15)
        ldsm_x4_t(bf, xs + ((r + 1 + dj) * kHaloVox + 1 + di + vb + (lane & 7) + 8 * (mi & 1)) * X_STRIDE +
                          (mi >> 1) * 16);
        mma_bf16(acc[q][0], af, bf[0], bf[1]);
        mma_bf16(acc[q][1], af, bf[2], bf[3]);
      }
    }
    __syncthreads();
  }
  const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int q = 0; q < PER_WARP; q++) {
    const int id = warp + 4 * q;
    if (id >= NTILE) break;
    const int mt = id % MT, tap = id / MT;
    const int t = (dk + 1) * 9 + tap;
#pragma unroll
    for (int nt = 0; nt < 2; nt++) {
      const int ci = c0 + 8 * nt + 2 * t4;
#pragma unroll
      for (int half = 0; half < 2; half++) {
        const int co = 16 * mt + g + 8 * half;
        float* p = w.dw + ((long long)t * COUT + co) * a.cin + ci;
        atomicAdd(p, acc[q][nt][2 * half]);
        atomicAdd(p + 1, acc[q][nt][2 * half + 1]);
      }
    }
  }
}

// ---------------------------------------------------------------- launchers
static size_t conv_smem(int cout) { return (size_t)kActBytes + (size_t)27 * cout * 32; }
static size_t wgrad_smem(int cout) { return (size_t)kRows * kTx * (cout * 2 + 16) + 6 * kHaloVox * 48; }

template <int COUT>
static cudaError_t launch_conv_t(const ConvArgs& a, cudaStream_t st) {
  static bool attr = false;
  const size_t sm = conv_smem(COUT);
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_conv<COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const dim3 grid((a.nx + kTx - 1) / kTx, (a.ny + kRows - 1) / kRows, a.nz);
  k_conv<COUT><<<grid, dim3(32, kRows), sm, st>>>(a);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_conv(const ConvArgs& a, int cout, cudaStream_t st) {
  if (a.cin % 16 || a.cin < 16) return cudaErrorInvalidValue;
  switch (cout) {
    case 16: return launch_conv_t<16>(a, st);
    case 32: return launch_conv_t<32>(a, st);
    case 48: return launch_conv_t<48>(a, st);
    case 64: return launch_conv_t<64>(a, st);
    case 80: return launch_conv_t<80>(a, st);
    case 112: return launch_conv_t<112>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

template <int COUT>
static cudaError_t launch_wgrad_t(const WgradArgs& w, cudaStream_t st) {
  static bool attr = false;
  const size_t sm = wgrad_smem(COUT);
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_conv_wgrad<COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const ConvArgs& a = w.conv;
  const long long ntiles = (long long)((a.nx + kTx - 1) / kTx) * ((a.ny + kRows - 1) / kRows) * a.nz;
  const dim3 grid((unsigned)((ntiles + w.tiles_per_cta - 1) / w.tiles_per_cta), a.cin / 16, 3);
  k_conv_wgrad<COUT><<<grid, dim3(32, kRows), sm, st>>>(w);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_conv_wgrad(const WgradArgs& w, int cout, cudaStream_t st) {
  if (w.conv.cin % 16 || w.conv.cin < 16 || w.tiles_per_cta < 1) return cudaErrorInvalidValue;
  switch (cout) {
    case 16: return launch_wgrad_t<16>(w, st);
    case 32: return launch_wgrad_t<32>(w, st);
    case 48: return launch_wgrad_t<48>(w, st);
    case 64: return launch_wgrad_t<64>(w, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace net
}  // namespace fpm
