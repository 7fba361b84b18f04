// Learned initial guess / preconditioner: the 3-D convolution kernels.
//
// Activations are channels-last BF16: voxel v = i + nx (j + ny k) (x fastest,
// the solver's own cell order), channel c at v * C + c.  A 3x3x3 convolution
// with zero padding is an implicit GEMM, M = voxels, N = output channels,
// K = 27 taps x input channels, run on the tensor cores: layers whose rows
// are multiples of 128 voxels on tcgen05.mma with tensor-memory accumulators
// and TMA-staged operands (k_conv_tc, below), the others and the weight
// gradients with mma.sync.m16n8k16 (BF16 operands, FP32 accumulation).
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

#include <cstdlib>

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

// ---------------------------------------------------------------- tcgen05 convolution
// The same convolution on the fifth-generation tensor cores for rows of 128
// voxels (nx a multiple of 128).  A CTA owns the 128 voxels i0 .. i0+127 of
// TJ x TK rows (j0 .. j0+TJ-1, k0 .. k0+TK-1), M = 128 voxels, N = COUT, and
// accumulates each output row in its own tensor-memory (TMEM) columns (FP32,
// lane = voxel).  Per 16-channel input slice the CTA stages the (TJ+2) x
// (TK+2) neighbouring rows of 130 voxels and the slice's weights for the 27
// taps in the K-major no-swizzle operand layout (core matrices of 8 rows x
// 16 bytes, the two 8-channel halves of the slice in separate arrays):
// channels of the same-resolution input A arrive by two 4-D TMA boxes
// {8 channels, 130 voxels, TJ+2, TK+2} (zero fill outside the grid), the
// upsampled half-resolution input B and the weights by cp.async.  One thread
// then issues 27 tcgen05.mma (M128 x N COUT x K16, BF16) per output row: tap
// (di, dj, dk) of row (tj, tk) reads staged row (tj+1+dj, tk+1+dk) from voxel
// 1 + di, so the shifted operands cost nothing and every staged row serves
// up to nine output rows.  A commit to an mbarrier tells the CTA when the
// operands may be overwritten; the epilogue reads the accumulators with
// tcgen05.ld (warp w owns TMEM lanes 32w .. 32w+31).  Tiles are sized so that
// two CTAs fit an SM (shared memory and 512 TMEM columns).  Waits are bounded:
// a timeout sets g_conv_tc_err, waits (bounded) for the copies and MMAs in
// flight and returns after freeing the tensor memory.
namespace {
constexpr int kTcM = 128;                     // voxels per row
constexpr int kTcVox = kTcM + 2;              // staged voxels per neighbour row
constexpr int kTcRowBytes = kTcVox * 16;      // one 8-channel half of a staged row
constexpr unsigned kTcSpin = 1u << 20;

// Output rows (TJ x TK) per CTA and TMEM columns per output row (CS) for the
// layer widths that run on this kernel (the full- and half-resolution layers
// of the network); other widths stay on the mma.sync kernel.
template <int COUT>
struct TcTile {
  static constexpr bool on = false;
};
template <>
struct TcTile<16> { static constexpr bool on = true; static constexpr int TJ = 4, TK = 2, CS = 16; };
template <>
struct TcTile<32> { static constexpr bool on = true; static constexpr int TJ = 2, TK = 2, CS = 32; };
template <>
struct TcTile<48> { static constexpr bool on = true; static constexpr int TJ = 2, TK = 2, CS = 64; };
template <>
struct TcTile<80> { static constexpr bool on = true; static constexpr int TJ = 1, TK = 1, CS = 128; };

template <int COUT>
struct TcCfg {
  static constexpr int TJ = TcTile<COUT>::TJ, TK = TcTile<COUT>::TK, CS = TcTile<COUT>::CS;
  static constexpr int kRowsIn = (TJ + 2) * (TK + 2);
  static constexpr int kLoaded = kRowsIn * kTcRowBytes;        // bytes of one staged half
  static constexpr int kHalf = (kLoaded + 127) / 128 * 128;    // 128-byte aligned TMA destination
  static constexpr int kAct = 2 * kHalf;
  static constexpr int kWts = 27 * 2 * COUT * 16;
  static constexpr int kSmem = kAct + kWts;
  static constexpr int kAcc = TJ * TK * CS;
  static constexpr int kCols = kAcc <= 32 ? 32 : kAcc <= 64 ? 64 : kAcc <= 128 ? 128 : kAcc <= 256 ? 256 : 512;
  static_assert(COUT % 16 == 0 && COUT >= 16 && COUT <= 256 && CS >= COUT, "N of an M=128 MMA");
  static_assert(kAcc <= 512, "TMEM columns");
};

__device__ int g_conv_tc_err;

__device__ __forceinline__ uint64_t tc_desc(unsigned saddr, unsigned lbo, unsigned sbo) {
  // K-major, no swizzle: start, leading (K) and stride (M/N) byte offsets in
  // 16-byte units, descriptor version 1 (bits 46-47)
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
__device__ __forceinline__ bool tc_wait(unsigned bar, unsigned parity) {
  for (unsigned it = 0; it < kTcSpin; ++it) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(1000u)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void tc_load_4d(unsigned dst, const CUtensorMap* map, int c, int i, int j, int k,
                                           unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c), "r"(i), "r"(j), "r"(k), "r"(bar)
      : "memory");
}
}  // namespace

template <int COUT>
__global__ void __launch_bounds__(128) k_conv_tc(ConvArgs a, const __grid_constant__ CUtensorMap tm_a) {
  using C = TcCfg<COUT>;
  extern __shared__ __align__(128) char smem[];
  char* act = smem;                // [2 halves][TK+2][TJ+2][130 voxels][16 B]
  char* wts = smem + C::kAct;      // [27 taps][2 halves][COUT][16 B]
  __shared__ __align__(8) uint64_t bars[2];  // 0: the slice's TMA boxes, 1: the slice's MMAs
  __shared__ unsigned tmem_base_s;
  __shared__ float bias_s[COUT];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int c = tid; c < COUT; c += 128) bias_s[c] = a.bias ? a.bias[c] : 0.f;
  const int i0 = blockIdx.x * kTcM, j0 = blockIdx.y * C::TJ, k0 = blockIdx.z * C::TK;
  const unsigned bar_ld = smem_u32(&bars[0]), bar_mma = smem_u32(&bars[1]);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_ld) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_mma) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tm_a)) : "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(C::kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = tmem_base_s;
  // instruction descriptor: F32 accumulator, BF16 A and B, both K-major, N, M
  constexpr unsigned kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(COUT >> 3) << 17) |
                              ((unsigned)(kTcM >> 4) << 24);
  const int hx = a.nx >> 1, hy = a.ny >> 1;
  const int nslices = a.cin / 16;
  bool ok = true, mma_pending = false, ld_pending = false;
  unsigned ph_ld = 0, ph_mma = 0;
  for (int s = 0; s < nslices; s++) {
    // the previous slice's MMAs must be done before its operands are overwritten
    if (mma_pending && tc_wait(bar_mma, ph_mma)) {
      ph_mma ^= 1u;
      mma_pending = false;
    }
    if (__syncthreads_or(mma_pending)) {
      ok = false;
      break;
    }
    const int c0 = s * 16;
    const bool from_a = c0 < a.ca;
    if (from_a) {
      if (tid == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_ld), "r"(2 * C::kLoaded)
                     : "memory");
        tc_load_4d(smem_u32(act), &tm_a, c0, i0 - 1, j0 - 1, k0 - 1, bar_ld);
        tc_load_4d(smem_u32(act + C::kHalf), &tm_a, c0 + 8, i0 - 1, j0 - 1, k0 - 1, bar_ld);
      }
      ld_pending = true;
    } else {
      // upsampled half-resolution input: row by row, voxel i reads B at i >> 1
      for (int row = 0; row < C::kRowsIn; row++) {
        const int jj = j0 - 1 + row % (C::TJ + 2), kk = k0 - 1 + row / (C::TJ + 2);
        const bool rin = jj >= 0 && jj < a.ny && kk >= 0 && kk < a.nz;
        const __nv_bfloat16* brow =
            rin ? a.b + (long long)hx * ((jj >> 1) + (long long)hy * (kk >> 1)) * a.cb + (c0 - a.ca) : a.b;
        char* drow = act + row * kTcRowBytes;
        for (int c = tid; c < kTcVox * 2; c += 128) {
          const int vox = c >> 1, h = c & 1, i = i0 - 1 + vox;
          const bool in = rin && i >= 0 && i < a.nx;
          cp_async16(drow + h * C::kHalf + vox * 16, in ? brow + (long long)(i >> 1) * a.cb + 8 * h : a.b, in);
        }
      }
    }
    const __nv_bfloat16* wsrc = a.w + (long long)s * 27 * COUT * 16;
    for (int idx = tid; idx < 27 * COUT * 2; idx += 128) {
      const int r = idx >> 1, h = idx & 1;  // r = t * COUT + co
      const int t = r / COUT, co = r - t * COUT;
      cp_async16(wts + (t * 2 + h) * COUT * 16 + co * 16, wsrc + r * 16 + 8 * h, true);
    }
    cp_async_wait_all();
    // the cp.async operands were written through the generic proxy; the MMA
    // reads them through the async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (ld_pending && tc_wait(bar_ld, ph_ld)) {
      ph_ld ^= 1u;
      ld_pending = false;
    }
    if (__syncthreads_or(ld_pending)) {
      ok = false;
      break;
    }
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const unsigned act_a = smem_u32(act), wts_a = smem_u32(wts);
      for (int o = 0; o < C::TJ * C::TK; o++) {
        const int tj = o % C::TJ, tk = o / C::TJ;
        const unsigned d = tmem + (unsigned)(o * C::CS);
        for (int t = 0; t < 27; t++) {
          const int di = t % 3, dj = (t / 3) % 3, dk = t / 9;  // offsets + 1
          const int row = (tj + dj) + (C::TJ + 2) * (tk + dk);
          const uint64_t ad = tc_desc(act_a + row * kTcRowBytes + di * 16, C::kHalf, 128);
          const uint64_t bd = tc_desc(wts_a + (t * 2) * COUT * 16, COUT * 16, 128);
          const unsigned acc = (s > 0 || t > 0) ? 1u : 0u;
          asm volatile(
              "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
              "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc)
              : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_mma)
                   : "memory");
    }
    mma_pending = true;
  }
  if (ok && mma_pending && tc_wait(bar_mma, ph_mma)) {
    ph_mma ^= 1u;
    mma_pending = false;
  }
  if (__syncthreads_or(!ok || mma_pending)) {
    if (tid == 0) {
      atomicExch(&g_conv_tc_err, 1);
      // bounded waits for the work still in flight before the memory is released
      if (mma_pending) tc_wait(bar_mma, ph_mma);
      if (ld_pending) tc_wait(bar_ld, ph_ld);
    }
  } else {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // epilogue: voxel i of this warp's 32 TMEM lanes, every output row of the tile
    const int i = i0 + 32 * warp + lane;
    for (int o = 0; o < C::TJ * C::TK; o++) {
      const int j = j0 + o % C::TJ, k = k0 + o / C::TJ;
      if (j >= a.ny || k >= a.nz) continue;  // uniform over the CTA
      const long long v = i + (long long)a.nx * (j + (long long)a.ny * k);
#pragma unroll
      for (int c16 = 0; c16 < COUT / 16; c16++) {
        float x[16];
        unsigned r[16];
        const unsigned taddr = tmem + ((unsigned)(32 * warp) << 16) + (unsigned)(o * C::CS + 16 * c16);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int e = 0; e < 16; e++) x[e] = __uint_as_float(r[e]);
        const int cb = 16 * c16;
        if (a.mode == kConvBf16) {
          unsigned q[8];
#pragma unroll
          for (int e = 0; e < 16; e += 2) {
            float x0 = x[e] + bias_s[cb + e], x1 = x[e + 1] + bias_s[cb + e + 1];
            if (a.relu) {
              x0 = fmaxf(x0, 0.f);
              x1 = fmaxf(x1, 0.f);
            }
            const __nv_bfloat162 h2 = __floats2bfloat162_rn(x0, x1);
            q[e / 2] = *reinterpret_cast<const unsigned*>(&h2);
          }
          uint4* dst = reinterpret_cast<uint4*>(a.y + v * COUT + cb);
          dst[0] = make_uint4(q[0], q[1], q[2], q[3]);
          dst[1] = make_uint4(q[4], q[5], q[6], q[7]);
        } else if (a.mode == kConvF32) {
          float4* dst = reinterpret_cast<float4*>(a.yf + v * COUT + cb);
#pragma unroll
          for (int e = 0; e < 4; e++)
            dst[e] = make_float4(x[4 * e] + bias_s[cb + 4 * e], x[4 * e + 1] + bias_s[cb + 4 * e + 1],
                                 x[4 * e + 2] + bias_s[cb + 4 * e + 2], x[4 * e + 3] + bias_s[cb + 4 * e + 3]);
        } else if (cb < a.csplit) {  // csplit is a multiple of 16: the chunk is all A
          float4* g = reinterpret_cast<float4*>(a.ga + v * a.csplit + cb);
#pragma unroll
          for (int e = 0; e < 4; e++) {
            float4 t = g[e];
            t.x += x[4 * e];
            t.y += x[4 * e + 1];
            t.z += x[4 * e + 2];
            t.w += x[4 * e + 3];
            g[e] = t;
          }
        } else {
          // the 2x2x2 sum into the half-resolution B: lanes 2m and 2m + 1 hold
          // voxels i and i + 1 of the same half-resolution voxel
#pragma unroll
          for (int e = 0; e < 16; e++) x[e] += __shfl_xor_sync(0xffffffffu, x[e], 1);
          if (!(lane & 1)) {
            const long long vb = (i >> 1) + (long long)hx * ((j >> 1) + (long long)hy * (k >> 1));
            float4* g = reinterpret_cast<float4*>(a.gb + vb * (COUT - a.csplit) + (cb - a.csplit));
#pragma unroll
            for (int e = 0; e < 4; e++)
              atomicAdd(g + e, make_float4(x[4 * e], x[4 * e + 1], x[4 * e + 2], x[4 * e + 3]));
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::kCols) : "memory");
}

// ---------------------------------------------------------------- launchers
static size_t conv_smem(int cout) { return (size_t)kActBytes + (size_t)27 * cout * 32; }
static size_t wgrad_smem(int cout) { return (size_t)kRows * kTx * (cout * 2 + 16) + 6 * kHaloVox * 48; }

static bool tc_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("FPM_CONV_TC");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <int COUT>
static cudaError_t launch_conv_tc(const ConvArgs& a, cudaStream_t st) {
  using C = TcCfg<COUT>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_conv_tc<COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  // the same-resolution input as {ca channels, nx, ny, nz}, box {8, 130, TJ+2, TK+2}
  CUtensorMap tm;
  const uint64_t cs = 2ull * a.ca;
  const uint64_t dims[4] = {(uint64_t)a.ca, (uint64_t)a.nx, (uint64_t)a.ny, (uint64_t)a.nz};
  const uint64_t strides[3] = {cs, cs * a.nx, cs * a.nx * a.ny};
  const uint32_t box[4] = {8, (uint32_t)kTcVox, (uint32_t)(C::TJ + 2), (uint32_t)(C::TK + 2)};
  if (!tma_encode(&tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(a.a), dims, strides, box))
    return cudaErrorInvalidValue;
  const dim3 grid(a.nx / kTcM, (a.ny + C::TJ - 1) / C::TJ, (a.nz + C::TK - 1) / C::TK);
  k_conv_tc<COUT><<<grid, 128, C::kSmem, st>>>(a, tm);
  note_launch();
  return cudaGetLastError();
}

template <int COUT>
static cudaError_t launch_conv_t(const ConvArgs& a, cudaStream_t st) {
  if constexpr (TcTile<COUT>::on) {
    if (tc_enabled() && a.nx % kTcM == 0 && (a.mode != kConvGrad || a.csplit % 16 == 0))
      return launch_conv_tc<COUT>(a, st);
  }
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

// Reads and clears the tcgen05 convolution's timeout flag.
cudaError_t conv_tc_error(cudaStream_t st, int* flag) {
  cudaError_t e = cudaMemcpyFromSymbolAsync(flag, g_conv_tc_err, sizeof(int), 0, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess || *flag == 0) return e;
  const int zero = 0;
  return cudaMemcpyToSymbolAsync(g_conv_tc_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st);
}

}  // namespace net
}  // namespace fpm
