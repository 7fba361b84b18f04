// Weighted-Jacobi sweep (src/fpm_stairstep_mpi_3d.f90:384-399) in
// double-float arithmetic, streamed through shared memory by TMA.
//
// Each CTA owns a TX x TY column of interior cells and marches k through a
// chunk of planes.  One elected thread keeps a ring of phi planes (tile plus
// one-cell x-y halo; 4 deep) and a ring of (src, rdiag) planes (3 deep) in
// flight with cp.async.bulk.tensor, completion tracked by mbarriers; every
// thread reads its seven phi values and its src/rdiag from shared memory, so
// global memory sees each field once per sweep (the x-y halo re-reads hit L2)
// and the DRAM stream never waits on a dependent load.  A thread owns CY rows
// of its column; with CY even, row pairs run through the packed FP32x2
// instructions.  Tile shape, ring depths and planes per CTA are template and
// launch parameters chosen by the host autotuner.
//
// Internal layout (owned by this module, not the caller's):
//   phi   float2 (hi, lo), padded (0:nx+1, 0:ny+1, 1:nz) with x pitch PX even
//   sr    (src_hi, src_lo, rdiag_hi, rdiag_lo) per interior cell, x fastest
// The pitch keeps every TMA row start on a 16-byte boundary: the phi box
// starts at x = TX*bx (TX even) and spans TX+2 elements of 8 bytes.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "fpm_internal.h"
#include "fpm_tma.cuh"

namespace fpm {

namespace {

using tma::mbar_expect_tx;
using tma::mbar_init;
using tma::mbar_wait;
using tma::smem_u32;
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t bar) {
  tma::load_3d(dst, map, x, y, z, bar);
}

}  // namespace

// 0.2 as hi + lo.
#define DF_POINT2 make_float2(0.2f, -2.9802322831784522e-09f)

// Unnormalised double-float accumulator: value = s + e.  Adding an exact
// product c*a costs 12 FP32 operations (TwoProd with FMA, TwoSum into s, the
// two error terms into e); normalisation is deferred to the end of the sum.
struct DfAcc {
  float s, e;
};
__device__ __forceinline__ void acc_prod(DfAcc& A, float2 c, float2 a) {
  const float p = c.x * a.x;
  float pe = fmaf(c.x, a.x, -p);
  pe = fmaf(c.x, a.y, pe);
  pe = fmaf(c.y, a.x, pe);
  const float s = A.s + p;
  const float bb = s - A.s;
  const float t = (A.s - (s - bb)) + (p - bb);
  A.s = s;
  A.e += t + pe;
}
__device__ __forceinline__ float2 acc_norm(const DfAcc& A) {
  const float h = A.s + A.e;
  return make_float2(h, A.e - (h - A.s));
}
// b = 0.2 a + rdiag * s for double-float a, rdiag, s.
__device__ __forceinline__ float2 df_jacobi_finish(float2 a, float2 rd, float2 s) {
  const float2 P2 = DF_POINT2;
  const float p = P2.x * a.x;
  float pe = fmaf(P2.x, a.x, -p);
  pe = fmaf(P2.x, a.y, pe);
  pe = fmaf(P2.y, a.x, pe);
  const float q = rd.x * s.x;
  float qe = fmaf(rd.x, s.x, -q);
  qe = fmaf(rd.x, s.y, qe);
  qe = fmaf(rd.y, s.x, qe);
  const float u = p + q;
  const float bb = u - p;
  const float t = (p - (u - bb)) + (q - bb);
  const float e = t + (pe + qe);
  const float h = u + e;
  return make_float2(h, e - (h - u));
}

// Packed FP32x2 form of the same arithmetic for two cells at once (lane 0 and
// lane 1 are two rows of one column).  Each packed instruction rounds every
// lane like its scalar FP32 counterpart, so a lane computes exactly what the
// scalar TwoProd / TwoSum sequence computes without FMA contraction.  The
// product error is carried negated (fma with -c against +p), which avoids a
// separate negation of p and leaves every rounding unchanged.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// A double-float coefficient pair: high parts, and both parts negated.
struct DfCoef2 {
  float2 h, nh, nl;
};
__device__ __forceinline__ DfCoef2 coef2(float2 c0, float2 c1) {
  return DfCoef2{make_float2(c0.x, c1.x), make_float2(-c0.x, -c1.x), make_float2(-c0.y, -c1.y)};
}
struct DfAcc2 {
  float2 s, e;
};
// A += c * a for lane-wise double-float c and a = (ah, al).
__device__ __forceinline__ void acc_prod2(DfAcc2& A, const DfCoef2& c, float2 ah, float2 al) {
  const float2 p = __fmul2_rn(c.h, ah);
  float2 npe = __ffma2_rn(c.nh, ah, p);
  npe = __ffma2_rn(c.nh, al, npe);
  npe = __ffma2_rn(c.nl, ah, npe);
  const float2 s = add2(A.s, p);
  const float2 bb = sub2(s, A.s);
  const float2 t = add2(sub2(A.s, sub2(s, bb)), sub2(p, bb));
  A.s = s;
  A.e = add2(A.e, sub2(t, npe));
}
// b = 0.2 a + rd * s, lane-wise; returns (hi, lo) pairs in *bh, *bl.
__device__ __forceinline__ void df_jacobi_finish2(float2 ah, float2 al, float2 rdh, float2 rdl, const DfAcc2& A,
                                                  float2* bh, float2* bl) {
  const float2 P2 = DF_POINT2;
  const float2 sh = add2(A.s, A.e);
  const float2 sl = sub2(A.e, sub2(sh, A.s));
  const float2 p = __fmul2_rn(make_float2(P2.x, P2.x), ah);
  float2 npe = __ffma2_rn(make_float2(-P2.x, -P2.x), ah, p);
  npe = __ffma2_rn(make_float2(-P2.x, -P2.x), al, npe);
  npe = __ffma2_rn(make_float2(-P2.y, -P2.y), ah, npe);
  const float2 m1 = make_float2(-1.f, -1.f);
  const float2 q = __fmul2_rn(rdh, sh);
  float2 nqe = __ffma2_rn(__fmul2_rn(rdh, m1), sh, q);
  nqe = __ffma2_rn(__fmul2_rn(rdh, m1), sl, nqe);
  nqe = __ffma2_rn(__fmul2_rn(rdl, m1), sh, nqe);
  const float2 u = add2(p, q);
  const float2 bb = sub2(u, p);
  const float2 t = add2(sub2(p, sub2(u, bb)), sub2(q, bb));
  const float2 e = sub2(t, add2(npe, nqe));
  const float2 h = add2(u, e);
  *bh = h;
  *bl = sub2(e, sub2(h, u));
}

// One plane of a thread's column: rows jbase + r*TYB (r < CY) of column i,
// from the phi planes k-1 (pm), k (pc), k+1 (pp) and the (src, rdiag) plane in
// shared memory; writes phi' at outp + px * r*TYB.
template <int TX, int TYB, int CY>
__device__ __forceinline__ void df_plane(const float2* pm, const float2* pc, const float2* pp, const float4* srp,
                                         float2* outp, long long px, int tx, int tyb, int jbase, int ny, float2 cwi,
                                         float2 cei, const float2 (&csj)[CY], const float2 (&cnj)[CY], float2 cbk,
                                         float2 ctk) {
  constexpr int PW = TX + 2;
  if constexpr (CY % 2 == 0) {
    // Rows r and r+1 of the column share one packed computation.
    const DfCoef2 CW = coef2(cwi, cwi), CE = coef2(cei, cei), CB = coef2(cbk, cbk), CT = coef2(ctk, ctk);
#pragma unroll
    for (int r = 0; r < CY; r += 2) {
      const int j = jbase + r * TYB;
      if (j <= ny) {
        const int c0 = (tx + 1) + PW * (tyb + r * TYB + 1), c1 = c0 + PW * TYB;
        const float4 s0 = srp[tx + TX * (tyb + r * TYB)], s1 = srp[tx + TX * (tyb + (r + 1) * TYB)];
        const float2 a0 = pc[c0], a1 = pc[c1];
        DfAcc2 A{make_float2(s0.x, s1.x), make_float2(s0.y, s1.y)};
        float2 v0 = pc[c0 - 1], v1 = pc[c1 - 1];
        acc_prod2(A, CW, make_float2(v0.x, v1.x), make_float2(v0.y, v1.y));
        v0 = pc[c0 + 1], v1 = pc[c1 + 1];
        acc_prod2(A, CE, make_float2(v0.x, v1.x), make_float2(v0.y, v1.y));
        v0 = pc[c0 - PW], v1 = pc[c1 - PW];
        acc_prod2(A, coef2(csj[r], csj[r + 1]), make_float2(v0.x, v1.x), make_float2(v0.y, v1.y));
        v0 = pc[c0 + PW], v1 = pc[c1 + PW];
        acc_prod2(A, coef2(cnj[r], cnj[r + 1]), make_float2(v0.x, v1.x), make_float2(v0.y, v1.y));
        v0 = pm[c0], v1 = pm[c1];
        acc_prod2(A, CB, make_float2(v0.x, v1.x), make_float2(v0.y, v1.y));
        v0 = pp[c0], v1 = pp[c1];
        acc_prod2(A, CT, make_float2(v0.x, v1.x), make_float2(v0.y, v1.y));
        float2 bh, bl;
        df_jacobi_finish2(make_float2(a0.x, a1.x), make_float2(a0.y, a1.y), make_float2(s0.z, s1.z),
                          make_float2(s0.w, s1.w), A, &bh, &bl);
        outp[px * (r * TYB)] = make_float2(bh.x, bl.x);
        if (j + TYB <= ny) outp[px * ((r + 1) * TYB)] = make_float2(bh.y, bl.y);
      }
    }
  } else {
#pragma unroll
    for (int r = 0; r < CY; r++) {
      const int j = jbase + r * TYB;
      if (j <= ny) {
        const int c0 = (tx + 1) + PW * (tyb + r * TYB + 1);
        const float4 sr = srp[tx + TX * (tyb + r * TYB)];
        const float2 ac = pc[c0];
        DfAcc A{sr.x, sr.y};
        acc_prod(A, cwi, pc[c0 - 1]);
        acc_prod(A, cei, pc[c0 + 1]);
        acc_prod(A, csj[r], pc[c0 - PW]);
        acc_prod(A, cnj[r], pc[c0 + PW]);
        acc_prod(A, cbk, pm[c0]);
        acc_prod(A, ctk, pp[c0]);
        outp[px * (r * TYB)] = df_jacobi_finish(ac, make_float2(sr.z, sr.w), acc_norm(A));
      }
    }
  }
}

// One CTA: TX x (TYB*CY) interior cells; thread (tx, tyb) owns rows
// tyb + r*TYB (r < CY) of its column, so a warp reads contiguous rows of the
// shared-memory plane.  kPhiStages / kSrStages are the ring depths: planes in
// flight ahead of the compute are kPhiStages - 2 of phi and kSrStages - 1 of
// (src, rdiag).
template <int TX, int TYB, int CY, int kPhiStages, int kSrStages>
__global__ void __launch_bounds__(TX* TYB, 1024 / (TX * TYB)) k_jacobi_df_tma(const __grid_constant__ CUtensorMap tm_phi,
                                                             const __grid_constant__ CUtensorMap tm_sr,
                                                             float2* __restrict__ out,
                                                             const float2* __restrict__ coef, int nx, int ny, int nz,
                                                             long long px, int kchunk, int* err) {
  constexpr int TY = TYB * CY, PW = TX + 2, PH = TY + 2;
  constexpr uint32_t kPhiBytes = PW * PH * 8, kSrBytes = TX * TY * 16;
  constexpr uint32_t kPhiStage = (kPhiBytes + 127) / 128 * 128;
  extern __shared__ __align__(128) unsigned char smem[];
  float4* sr_s = reinterpret_cast<float4*>(smem + kPhiStages * kPhiStage);
  uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(sr_s) + kSrStages * kSrBytes);
  const uint32_t phi_base = smem_u32(smem), sr_base = smem_u32(sr_s), bar_base = smem_u32(bars);

  const int tid = threadIdx.x, tx = tid % TX, tyb = tid / TX;
  const int bx = blockIdx.x, by = blockIdx.y;
  const int k0 = blockIdx.z * kchunk + 1;
  const int k1 = min(nz, k0 + kchunk - 1);
  const int i = TX * bx + tx + 1;
  const int jbase = TY * by + tyb + 1;

  if (tid == 0) {
    for (int s = 0; s < kPhiStages + kSrStages; s++) mbar_init(bar_base + 8 * s, 1);
    tma::mbar_init_fence();
  }
  __syncthreads();

  // Plane p of phi goes to ring slot (p - (k0-1)) % kPhiStages; its n-th use
  // of the slot completes phase n.  (src, rdiag) plane p goes to slot
  // (p - k0) % kSrStages.
  auto issue_phi = [&](int p) {
    const int u = p - (k0 - 1), s = u % kPhiStages;
    const uint32_t bar = bar_base + 8 * s;
    mbar_expect_tx(bar, kPhiBytes);
    tma_load_3d(phi_base + s * kPhiStage, &tm_phi, TX * bx, TY * by, p - 1, bar);
  };
  auto issue_sr = [&](int p) {
    const int s = (p - k0) % kSrStages;
    const uint32_t bar = bar_base + 8 * (kPhiStages + s);
    mbar_expect_tx(bar, kSrBytes);
    tma_load_3d(sr_base + s * kSrBytes, &tm_sr, 2 * TX * bx, TY * by, p - 1, bar);
  };
  auto phi_ready = [&](int p) {
    const int u = p - (k0 - 1);
    return mbar_wait(bar_base + 8 * (u % kPhiStages), (uint32_t)((u / kPhiStages) & 1));
  };
  auto sr_ready = [&](int p) {
    const int u = p - k0;
    return mbar_wait(bar_base + 8 * (kPhiStages + u % kSrStages), (uint32_t)((u / kSrStages) & 1));
  };

  int next_phi = k0 - 1, next_sr = k0;
  if (tid == 0) {
    for (; next_phi <= k0 + kPhiStages - 2 && next_phi <= k1 + 1; next_phi++) issue_phi(next_phi);
    for (; next_sr <= k0 + kSrStages - 1 && next_sr <= k1; next_sr++) issue_sr(next_sr);
  }

  const bool col = i <= nx;
  float2 cwi = make_float2(0.f, 0.f), cei = cwi;
  if (col) {
    cwi = coef[i - 1];
    cei = coef[nx + i - 1];
  }
  float2 csj[CY], cnj[CY];
#pragma unroll
  for (int r = 0; r < CY; r++) {
    const int j = jbase + r * TYB;
    csj[r] = j <= ny ? coef[2 * nx + j - 1] : make_float2(0.f, 0.f);
    cnj[r] = j <= ny ? coef[2 * nx + ny + j - 1] : make_float2(0.f, 0.f);
  }
  const float2* cb = coef + 2 * nx + 2 * ny;
  const float2* ct = cb + nz;
  const long long plane = px * (long long)(ny + 2);
  float2* outp = out + (long long)i + px * (long long)jbase + plane * (long long)(k0 - 1);

  bool failed = false;
  int kfail = k0;
  bool ok = phi_ready(k0 - 1) && phi_ready(k0);
  for (int k = k0; k <= k1; k++) {
    ok = ok && phi_ready(k + 1) && sr_ready(k);
    if (ok && col) {
      const int um = k - 1 - (k0 - 1);
      const float2* pm = reinterpret_cast<const float2*>(smem + (um % kPhiStages) * kPhiStage);
      const float2* pc = reinterpret_cast<const float2*>(smem + ((um + 1) % kPhiStages) * kPhiStage);
      const float2* pp = reinterpret_cast<const float2*>(smem + ((um + 2) % kPhiStages) * kPhiStage);
      const float4* srp = sr_s + ((k - k0) % kSrStages) * (TX * TY);
      // z neighbours clamp at the domain ends like a(i,j,max(k-1,1)); there
      // cb(1) = ct(nz) = 0, so reading the zero-filled plane gives the same sum.
      df_plane<TX, TYB, CY>(pm, pc, pp, srp, outp, px, tx, tyb, jbase, ny, cwi, cei, csj, cnj, cb[k - 1], ct[k - 1]);
    }
    outp += plane;
    if (__syncthreads_or(!ok)) {
      failed = true;
      kfail = k;
      break;
    }
    if (tid == 0) {
      if (next_phi <= k1 + 1) issue_phi(next_phi++);
      if (next_sr <= k1) issue_sr(next_sr++);
    }
  }
  if (failed && tid == 0) {
    atomicExch(err, 1);
    // Drain the copies still in flight (bounded) before the CTA exits:
    // phases already complete return at once.
    for (int p = kfail - 1; p < next_phi; p++) phi_ready(p);
    for (int p = kfail; p < next_sr; p++) sr_ready(p);
  }
}

// ---------------------------------------------------------------- packing
__global__ void k_pack_phi_df(Dims d, const double* __restrict__ phi, float2* __restrict__ out, long long px) {
  const long long n = d.npad();
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x) {
    const long long i = m % (d.nx + 2), r = m / (d.nx + 2);  // r = j + (ny+2)(k-1)
    out[i + px * r] = df_from_double(phi[m]);
  }
}
__global__ void k_unpack_phi_df(Dims d, const float2* __restrict__ in, double* __restrict__ phi, long long px) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  if (i > d.nx || j > d.ny) return;
  for (int k = blockIdx.z + 1; k <= d.nz; k += gridDim.z)
    phi[d.ph(i, j, k)] = df_to_double(in[(long long)i + px * ((long long)j + (long long)(d.ny + 2) * (k - 1))]);
}
__global__ void k_pack_sr(long long n, const double* __restrict__ src, const double* __restrict__ rdiag,
                          float4* __restrict__ out) {
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x) {
    const float2 s = df_from_double(src[m]), r = df_from_double(rdiag[m]);
    out[m] = make_float4(s.x, s.y, r.x, r.y);
  }
}

// ---------------------------------------------------------------- host side
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

bool tma_encode_3d(CUtensorMap* map, CUtensorMapDataType type, void* base, uint64_t d0, uint64_t d1, uint64_t d2,
                   uint64_t stride1_bytes, uint64_t stride2_bytes, uint32_t b0, uint32_t b1) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {d0, d1, d2};
  cuuint64_t strides[2] = {stride1_bytes, stride2_bytes};
  cuuint32_t box[3] = {b0, b1, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, type, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}
bool tma_encode(CUtensorMap* map, CUtensorMapDataType type, int rank, void* base, const uint64_t* dims,
                const uint64_t* strides, const uint32_t* box) {
  auto fn = encode_fn();
  if (!fn || rank < 1 || rank > 5) return false;
  cuuint64_t d[5], st[4];
  cuuint32_t b[5], estr[5];
  for (int r = 0; r < rank; r++) {
    d[r] = dims[r];
    b[r] = box[r];
    estr[r] = 1;
    if (r > 0) st[r - 1] = strides[r - 1];
  }
  CUresult res = fn(map, type, (cuuint32_t)rank, base, d, st, b, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return res == CUDA_SUCCESS;
}
static bool encode_3d(CUtensorMap* map, void* base, uint64_t d0, uint64_t d1, uint64_t d2, uint64_t stride1_bytes,
                      uint64_t stride2_bytes, uint32_t b0, uint32_t b1) {
  return tma_encode_3d(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, base, d0, d1, d2, stride1_bytes, stride2_bytes, b0, b1);
}

// Tile shapes the autotuner chooses from: (id, TX, TYB, CY, phi ring depth,
// (src, rdiag) ring depth).
#define FPM_DF_SHAPES(X)  \
  X(0, 64, 4, 2, 4, 3)    \
  X(1, 32, 8, 2, 4, 3)    \
  X(2, 64, 2, 4, 4, 3)    \
  X(3, 32, 4, 4, 4, 3)    \
  X(4, 128, 2, 2, 4, 3)   \
  X(5, 64, 4, 1, 4, 3)    \
  X(6, 32, 8, 1, 4, 3)    \
  X(7, 64, 8, 1, 4, 3)    \
  X(8, 32, 4, 2, 4, 3)    \
  X(9, 64, 2, 2, 4, 3)    \
  X(10, 32, 2, 4, 4, 3)

struct TileShape {
  int tx, tyb, cy;  // tile = tx x (tyb*cy); threads = tx*tyb
};
#define FPM_DF_SHAPE_ROW(id, tx, tyb, cy, ps, ss) {tx, tyb, cy},
static const TileShape kShapes[] = {FPM_DF_SHAPES(FPM_DF_SHAPE_ROW)};
#undef FPM_DF_SHAPE_ROW
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

template <int TX, int TYB, int CY, int PS, int SS>
static size_t shape_smem() {
  constexpr size_t ty = TYB * CY;
  constexpr size_t phi = ((TX + 2) * (ty + 2) * 8 + 127) / 128 * 128;
  return PS * phi + SS * (size_t)TX * ty * 16 + (PS + SS) * 8;
}

// Resident CTAs per SM of a tile shape's sweep kernel (shared memory and
// registers), for wave-aligned chunk choices.
template <int TX, int TYB, int CY, int PS, int SS>
static int shape_occupancy() {
  const size_t smem = shape_smem<TX, TYB, CY, PS, SS>();
  if (cudaFuncSetAttribute(k_jacobi_df_tma<TX, TYB, CY, PS, SS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return 1;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_jacobi_df_tma<TX, TYB, CY, PS, SS>, TX * TYB, smem) !=
      cudaSuccess)
    return 1;
  return n < 1 ? 1 : n;
}

template <int TX, int TYB, int CY, int PS, int SS>
static cudaError_t launch_shape(const JacobiDfPlan& pl, const float2* src_phi, float2* dst_phi, cudaStream_t st) {
  const CUtensorMap& tm = (src_phi == pl.a) ? pl.tm_a : pl.tm_b;
  const size_t smem = shape_smem<TX, TYB, CY, PS, SS>();
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_jacobi_df_tma<TX, TYB, CY, PS, SS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  constexpr int TY = TYB * CY;
  dim3 grid((pl.nx + TX - 1) / TX, (pl.ny + TY - 1) / TY, (pl.nz + pl.kchunk - 1) / pl.kchunk);
  k_jacobi_df_tma<TX, TYB, CY, PS, SS><<<grid, TX * TYB, smem, st>>>(tm, pl.tm_sr, dst_phi, pl.coef, pl.nx, pl.ny,
                                                                     pl.nz, pl.px, pl.kchunk, pl.err); note_launch();
  return cudaGetLastError();
}

cudaError_t jacobi_df_sweep(const JacobiDfPlan& pl, const float2* src_phi, float2* dst_phi, cudaStream_t st) {
#define FPM_DF_LAUNCH(id, tx, tyb, cy, ps, ss) \
  case id: return launch_shape<tx, tyb, cy, ps, ss>(pl, src_phi, dst_phi, st);
  switch (pl.shape) {
    FPM_DF_SHAPES(FPM_DF_LAUNCH)
    default: return cudaErrorInvalidValue;
  }
#undef FPM_DF_LAUNCH
}

int jacobi_df_num_shapes() { return kNumShapes; }

int jacobi_df_ctas_per_sm(int shape) {
#define FPM_DF_OCC(id, tx, tyb, cy, ps, ss) \
  case id: return shape_occupancy<tx, tyb, cy, ps, ss>();
  switch (shape) {
    FPM_DF_SHAPES(FPM_DF_OCC)
    default: return 1;
  }
#undef FPM_DF_OCC
}

// Packs FP64 phi / src / rdiag / coefficients into the internal double-float
// arrays.  a/b/sr/coef/err are allocated by the caller: a and b hold
// px*(ny+2)*nz float2, sr nx*ny*nz float4, coef 2(nx+ny+nz) float2.
cudaError_t jacobi_df_pack(JacobiDfPlan& pl, const double* phi, const double* src, const double* rdiag,
                           const double* coef64, cudaStream_t st) {
  const Dims d{pl.nx, pl.ny, pl.nz};
  const size_t nphi = sizeof(float2) * pl.px * (pl.ny + 2) * (size_t)pl.nz;
  long long nb = (d.npad() + 255) / 256;
  if (nb > 152LL * 32) nb = 152LL * 32;
  cudaError_t e = cudaMemsetAsync(pl.a, 0, nphi, st);
  if (e != cudaSuccess) return e;
  k_pack_phi_df<<<(unsigned)nb, 256, 0, st>>>(d, phi, pl.a, pl.px); note_launch();
  e = cudaMemcpyAsync(pl.b, pl.a, nphi, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  const long long nc = d.ncell();
  long long nb2 = (nc + 255) / 256;
  if (nb2 > 152LL * 32) nb2 = 152LL * 32;
  k_pack_sr<<<(unsigned)nb2, 256, 0, st>>>(nc, src, rdiag, pl.sr); note_launch();
  e = launch_to_df(coef64, pl.coef, 2LL * (pl.nx + pl.ny + pl.nz), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(pl.err, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Tensor maps for the plan's current tile shape.
cudaError_t jacobi_df_encode(JacobiDfPlan& pl) {
  const TileShape sh = kShapes[(pl.shape >= 0 && pl.shape < kNumShapes) ? pl.shape : 0];
  const uint64_t pitch1 = (uint64_t)pl.px * 8, pitch2 = pitch1 * (uint64_t)(pl.ny + 2);
  const int ty = sh.tyb * sh.cy;
  if (!encode_3d(&pl.tm_a, pl.a, pl.nx + 2, pl.ny + 2, pl.nz, pitch1, pitch2, sh.tx + 2, ty + 2) ||
      !encode_3d(&pl.tm_b, pl.b, pl.nx + 2, pl.ny + 2, pl.nz, pitch1, pitch2, sh.tx + 2, ty + 2) ||
      !encode_3d(&pl.tm_sr, pl.sr, 2ULL * pl.nx, pl.ny, pl.nz, 16ULL * pl.nx, 16ULL * pl.nx * pl.ny, 2 * sh.tx, ty))
    return cudaErrorInvalidValue;
  return cudaSuccess;
}

void jacobi_df_shape(int shape, int* tx, int* ty) {
  const TileShape sh = kShapes[(shape >= 0 && shape < kNumShapes) ? shape : 0];
  *tx = sh.tx;
  *ty = sh.tyb * sh.cy;
}

cudaError_t jacobi_df_unpack(const JacobiDfPlan& pl, const float2* cur, double* phi, cudaStream_t st) {
  const Dims d{pl.nx, pl.ny, pl.nz};
  Launch L = cells_launch(d);
  k_unpack_phi_df<<<L.grid, L.block, 0, st>>>(d, cur, phi, pl.px); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
