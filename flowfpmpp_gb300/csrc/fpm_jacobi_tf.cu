// Weighted-Jacobi sweep (src/fpm_stairstep_mpi_3d.f90:384-399) with FP64
// storage and triple-float arithmetic, streamed through shared memory by TMA.
//
// GB300 issues FP64 at about 0.53 T instructions/s (1.7 per clock and SM),
// which bounds an FP64 sweep (8 fused multiply-adds per cell) at about three
// times the HBM time.  This kernel keeps phi, src and rdiag in FP64 in HBM
// (32 bytes per cell and sweep, as the FP64 sweep) but evaluates
//   b = 0.2 a + rdiag (src + cw a_w + ce a_e + cs a_s + cn a_n + cb a_b + ct a_t)
// on the FP32 pipe: every FP64 input is split exactly into three FP32 limbs
// (24 + 23 + 6 significant bits) with integer operations, products are
// expanded into exact FMA-based TwoProd terms down to 2^-72 of the product,
// and sums run through three accumulators (levels 2^0, 2^-24, 2^-48 of the
// result) with error-free TwoSum on the first two, so the rounding of the
// expression before its final FP64 rounding is about 2^-60 relative -- finer
// than the FP64 evaluation's (whose separately rounded steps each contribute
// 2^-53).  The result leaves as the FP64 value nearest the three limbs (two
// FP64 additions, the first exact).
//
// Pipeline (shared with the double-float kernel): one thread keeps a ring of
// FP64 phi planes (tile plus one-cell x-y halo) and a ring of (src, rdiag)
// planes in flight with cp.async.bulk.tensor on mbarriers (bounded waits: a
// timeout sets the error flag, drains the CTA's copies and returns).  A phi
// plane is split into limbs once, when it lands, into a ring of three limb
// planes (k-1, k, k+1), so each value is split once per sweep instead of at
// each of its seven uses.  A thread owns two rows of its column and computes
// them together with the packed FP32x2 instructions (each lane rounds like the
// scalar instruction).
//
// Values with magnitude below 2^-74 keep only their leading limb(s) (their
// relative precision drops; the absolute error stays below 2^-98); magnitudes
// of 2^127 and above become infinities (they never occur in a stair-step
// solve); NaN stays NaN.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cmath>

#include "fpm_internal.h"
#include "fpm_tma.cuh"

namespace fpm {

namespace {

// Exact split of an FP64 value into h + m + l (same sign, |m| < 2^-23 |h|,
// |l| < 2^-46 |h|): h = the leading 24 significant bits, m = the next 23, l =
// the last 6.  Integer and FP32 operations only.
struct Limbs {
  float h, m, l;
};
__device__ __forceinline__ Limbs split3(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
  const int e = (int)((hi32 >> 20) & 0x7FFu);
  Limbs r{0.f, 0.f, 0.f};
  const unsigned sign = hi32 & 0x80000000u;
  if (e < 897) return r;  // zero, or below 2^-126
  if (e > 1150) {         // 2^127 and above: infinity; NaN stays NaN (bit operations, no conversion)
    const bool nan = e == 2047 && ((hi32 & 0xFFFFFu) | lo32) != 0u;
    r.h = __uint_as_float(sign | 0x7F800000u | (nan ? 0x400000u : 0u));
    return r;
  }
  r.h = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | ((hi32 & 0xFFFFFu) << 3) | (lo32 >> 29));
  const unsigned rem = lo32 & 0x1FFFFFFFu;  // 29 bits below h
  // n as an exact FP32 integer: (2^23 + n) - 2^23 for n < 2^23
  if (e >= 943) {
    const float mid = __uint_as_float(0x4B000000u | (rem >> 6)) - 8388608.0f;
    r.m = __uint_as_float(__float_as_uint(mid * __uint_as_float((unsigned)(e - 942) << 23)) | sign);
  }
  if (e >= 949) {
    const float lo = __uint_as_float(0x4B000000u | (rem & 63u)) - 8388608.0f;
    r.l = __uint_as_float(__float_as_uint(lo * __uint_as_float((unsigned)(e - 948) << 23)) | sign);
  }
  return r;
}

// FP32 -> FP64 by bit assembly (exact; zero and subnormals give a signed zero;
// infinities and NaN map to themselves).  Only integer operations: the
// conversion instruction runs on the FP64 pipe, and even a rarely taken
// branch to it is predicated into every call.
__device__ __forceinline__ double f32_bits_to_f64(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned sign = u & 0x80000000u;
  // exponent: zero/subnormal -> 0, infinity/NaN -> 2047, else rebiased
  const unsigned eo = e == 0u ? 0u : (e == 0xFFu ? 2047u : e + 896u);
  const unsigned hi = e == 0u ? sign : sign | (eo << 20) | ((u & 0x7FFFFFu) >> 3);
  const unsigned lo = e == 0u ? 0u : (u << 29);
  return __hiloint2double((int)hi, (int)lo);
}

// ---- packed two-lane arithmetic (lane 0 and lane 1 are two rows) ----------
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// s + e = a + b exactly (Knuth's TwoSum).
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = add2(a, b);
  const float2 bb = sub2(s, a);
  e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

struct TF2 {  // three limbs per lane
  float2 h, m, l;
};

// Three-level accumulator: value = s0 + s1 + s2 with s0 at the result's scale,
// s1 at 2^-24 of it and s2 at 2^-48; additions into s0 and s1 are error-free,
// their errors move one level down.
struct Acc3 {
  float2 s0, s1, s2;
  __device__ __forceinline__ void add1(float2 x) {
    float2 e;
    two_sum2(s1, x, s1, e);
    s2 = add2(s2, e);
  }
  __device__ __forceinline__ void add0(float2 x) {
    float2 e;
    two_sum2(s0, x, s0, e);
    add1(e);
  }
  // c * a for limbs c, a: c.h a.h exactly (TwoProd), c.h a.m and c.m a.h
  // exactly, the terms of order 2^-48 by FMAs (rounding 2^-72 of the product).
  __device__ __forceinline__ void add_prod(const TF2& c, const TF2& a) {
    const float2 p = mul2(c.h, a.h);
    const float2 pe = fma2(c.h, a.h, neg2(p));
    const float2 q1 = mul2(c.h, a.m);
    const float2 f1 = fma2(c.h, a.m, neg2(q1));
    const float2 q2 = mul2(c.m, a.h);
    const float2 f2 = fma2(c.m, a.h, neg2(q2));
    const float2 t = fma2(c.h, a.l, fma2(c.m, a.m, fma2(c.l, a.h, add2(f1, f2))));
    add0(p);
    add1(pe);
    add1(q1);
    add1(q2);
    s2 = add2(s2, t);
  }
};

__device__ __forceinline__ TF2 tf2_from(const Limbs& a, const Limbs& b) {
  return TF2{make_float2(a.h, b.h), make_float2(a.m, b.m), make_float2(a.l, b.l)};
}
__device__ __forceinline__ TF2 tf2_uniform(float4 c) {
  return TF2{make_float2(c.x, c.x), make_float2(c.y, c.y), make_float2(c.z, c.z)};
}

}  // namespace

// One CTA: TX x (TYB*CY) interior cells (CY even); thread (tx, tyb) owns rows
// tyb + r*TYB (r < CY) of its column, computed two at a time.  kPhiStages /
// kSrStages: FP64 phi and (src, rdiag) ring depths; the limb ring holds the
// planes k-1, k, k+1.
template <int TX, int TYB, int CY, int kPhiStages, int kSrStages>
__global__ void __launch_bounds__(TX* TYB) k_jacobi_tf_tma(const __grid_constant__ CUtensorMap tm_phi,
                                                          const __grid_constant__ CUtensorMap tm_sr,
                                                          double* __restrict__ out, const float4* __restrict__ coef,
                                                          float4 point2, int nx, int ny, int nz, long long px,
                                                          int kchunk, int* err) {
  static_assert(CY % 2 == 0, "rows are computed in pairs");
  constexpr int TY = TYB * CY, PW = TX + 2, PH = TY + 2, NT = TX * TYB;
  constexpr uint32_t kPhiBytes = PW * PH * 8, kSrBytes = TX * TY * 16;
  constexpr uint32_t kPhiStage = (kPhiBytes + 127) / 128 * 128;
  constexpr uint32_t kLimbPlane = (PW * PH * 4 + 127) / 128 * 128;  // one limb array of one plane
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* sr_raw = smem + kPhiStages * kPhiStage;
  float* limbs = reinterpret_cast<float*>(sr_raw + kSrStages * kSrBytes);  // 3 planes x 3 arrays
  uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(limbs) + 9 * kLimbPlane);
  const uint32_t phi_base = tma::smem_u32(smem), sr_base = tma::smem_u32(sr_raw), bar_base = tma::smem_u32(bars);

  const int tid = threadIdx.x, tx = tid % TX, tyb = tid / TX;
  const int bx = blockIdx.x, by = blockIdx.y;
  const int k0 = blockIdx.z * kchunk + 1;
  const int k1 = min(nz, k0 + kchunk - 1);
  const int i = TX * bx + tx + 1;
  const int jbase = TY * by + tyb + 1;

  if (tid == 0) {
    for (int s = 0; s < kPhiStages + kSrStages; s++) tma::mbar_init(bar_base + 8 * s, 1);
    tma::mbar_init_fence();
  }
  __syncthreads();

  auto issue_phi = [&](int p) {
    const int s = (p - (k0 - 1)) % kPhiStages;
    const uint32_t bar = bar_base + 8 * s;
    tma::mbar_expect_tx(bar, kPhiBytes);
    tma::load_3d(phi_base + s * kPhiStage, &tm_phi, TX * bx, TY * by, p - 1, bar);
  };
  auto issue_sr = [&](int p) {
    const int s = (p - k0) % kSrStages;
    const uint32_t bar = bar_base + 8 * (kPhiStages + s);
    tma::mbar_expect_tx(bar, kSrBytes);
    tma::load_3d(sr_base + s * kSrBytes, &tm_sr, 2 * TX * bx, TY * by, p - 1, bar);
  };
  auto phi_ready = [&](int p) {
    const int u = p - (k0 - 1);
    return tma::mbar_wait(bar_base + 8 * (u % kPhiStages), (uint32_t)((u / kPhiStages) & 1));
  };
  auto sr_ready = [&](int p) {
    const int u = p - k0;
    return tma::mbar_wait(bar_base + 8 * (kPhiStages + u % kSrStages), (uint32_t)((u / kSrStages) & 1));
  };
  // limb arrays of plane p: h, m, l
  auto limb = [&](int p, int which) { return limbs + (size_t)(3 * ((p - (k0 - 1)) % 3) + which) * (kLimbPlane / 4); };
  // split a landed FP64 plane into its limb plane
  auto transform = [&](int p) {
    const double* src = reinterpret_cast<const double*>(smem + ((p - (k0 - 1)) % kPhiStages) * kPhiStage);
    float* H = limb(p, 0);
    float* M = limb(p, 1);
    float* L = limb(p, 2);
    for (int e = tid; e < PW * PH; e += NT) {
      const Limbs s = split3(src[e]);
      H[e] = s.h;
      M[e] = s.m;
      L[e] = s.l;
    }
  };

  int next_phi = k0 - 1, next_sr = k0;
  if (tid == 0) {
    for (; next_phi <= k0 + kPhiStages - 2 && next_phi <= k1 + 1; next_phi++) issue_phi(next_phi);
    for (; next_sr <= k0 + kSrStages - 1 && next_sr <= k1; next_sr++) issue_sr(next_sr);
  }

  const bool col = i <= nx;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 cwi = col ? coef[i - 1] : z4, cei = col ? coef[nx + i - 1] : z4;
  float4 csj[CY], cnj[CY];
#pragma unroll
  for (int r = 0; r < CY; r++) {
    const int j = jbase + r * TYB;
    csj[r] = j <= ny ? coef[2 * nx + j - 1] : z4;
    cnj[r] = j <= ny ? coef[2 * nx + ny + j - 1] : z4;
  }
  const float4* cb = coef + 2 * nx + 2 * ny;
  const float4* ct = cb + nz;
  const TF2 P2 = tf2_uniform(point2);
  const long long plane = px * (long long)(ny + 2);
  double* outp = out + (long long)i + px * (long long)jbase + plane * (long long)(k0 - 1);

  bool failed = false;
  int kfail = k0;
  bool ok = phi_ready(k0 - 1) && phi_ready(k0);
  if (ok) {
    transform(k0 - 1);
    transform(k0);
  }
  for (int k = k0; k <= k1; k++) {
    ok = ok && phi_ready(k + 1) && sr_ready(k);
    if (ok) transform(k + 1);
    __syncthreads();
    if (ok && col) {
      const float *Hb = limb(k - 1, 0), *Mb = limb(k - 1, 1), *Lb = limb(k - 1, 2);
      const float *Hc = limb(k, 0), *Mc = limb(k, 1), *Lc = limb(k, 2);
      const float *Ht = limb(k + 1, 0), *Mt = limb(k + 1, 1), *Lt = limb(k + 1, 2);
      const double2* srp = reinterpret_cast<const double2*>(sr_raw + ((k - k0) % kSrStages) * kSrBytes);
      const TF2 CW = tf2_uniform(cwi), CE = tf2_uniform(cei), CB = tf2_uniform(cb[k - 1]), CT = tf2_uniform(ct[k - 1]);
#pragma unroll
      for (int r = 0; r < CY; r += 2) {
        const int j = jbase + r * TYB;
        if (j > ny) continue;
        const int c0 = (tx + 1) + PW * (tyb + r * TYB + 1), c1 = c0 + PW * TYB;
        auto at = [&](const float* H, const float* M, const float* L, int d) {
          return TF2{make_float2(H[c0 + d], H[c1 + d]), make_float2(M[c0 + d], M[c1 + d]),
                     make_float2(L[c0 + d], L[c1 + d])};
        };
        const double2 sr0 = srp[tx + TX * (tyb + r * TYB)], sr1 = srp[tx + TX * (tyb + (r + 1) * TYB)];
        const TF2 S = tf2_from(split3(sr0.x), split3(sr1.x));
        const TF2 RD = tf2_from(split3(sr0.y), split3(sr1.y));
        const TF2 CS{make_float2(csj[r].x, csj[r + 1].x), make_float2(csj[r].y, csj[r + 1].y),
                     make_float2(csj[r].z, csj[r + 1].z)};
        const TF2 CN{make_float2(cnj[r].x, cnj[r + 1].x), make_float2(cnj[r].y, cnj[r + 1].y),
                     make_float2(cnj[r].z, cnj[r + 1].z)};
        // src + cw a_w + ce a_e + cs a_s + cn a_n + cb a_b + ct a_t
        Acc3 A{S.h, S.m, S.l};
        A.add_prod(CW, at(Hc, Mc, Lc, -1));
        A.add_prod(CE, at(Hc, Mc, Lc, 1));
        A.add_prod(CS, at(Hc, Mc, Lc, -PW));
        A.add_prod(CN, at(Hc, Mc, Lc, PW));
        // z neighbours clamp at the domain ends like a(i,j,max(k-1,1)); there
        // cb(1) = ct(nz) = 0, so the zero-filled plane gives the same sum
        A.add_prod(CB, at(Hb, Mb, Lb, 0));
        A.add_prod(CT, at(Ht, Mt, Lt, 0));
        // the sum as limbs, then 0.2 a + rdiag * sum
        TF2 sum;
        float2 t;
        two_sum2(A.s0, A.s1, sum.h, t);
        two_sum2(t, A.s2, sum.m, sum.l);
        Acc3 B{make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        B.add_prod(P2, at(Hc, Mc, Lc, 0));
        B.add_prod(RD, sum);
        // nearest FP64: s0 + s1 is exact in FP64 (48 significant bits)
        const double b0 = __dadd_rn(__dadd_rn(f32_bits_to_f64(B.s0.x), f32_bits_to_f64(B.s1.x)),
                                    f32_bits_to_f64(B.s2.x));
        const double b1 = __dadd_rn(__dadd_rn(f32_bits_to_f64(B.s0.y), f32_bits_to_f64(B.s1.y)),
                                    f32_bits_to_f64(B.s2.y));
        outp[px * (r * TYB)] = b0;
        if (j + TYB <= ny) outp[px * ((r + 1) * TYB)] = b1;
      }
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
    for (int p = kfail - 1; p < next_phi; p++) phi_ready(p);
    for (int p = kfail; p < next_sr; p++) sr_ready(p);
  }
}

}  // namespace fpm

namespace fpm {

// ---------------------------------------------------------------- packing
// phi (caller layout, x pitch nx+2) -> internal layout (x pitch px, even)
__global__ void k_pack_phi_tf(Dims d, const double* __restrict__ phi, double* __restrict__ out, long long px) {
  const long long n = d.npad();
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x) {
    const long long i = m % (d.nx + 2), r = m / (d.nx + 2);
    out[i + px * r] = phi[m];
  }
}
__global__ void k_unpack_phi_tf(Dims d, const double* __restrict__ in, double* __restrict__ phi, long long px) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  if (i > d.nx || j > d.ny) return;
  for (int k = blockIdx.z + 1; k <= d.nz; k += gridDim.z)
    phi[d.ph(i, j, k)] = in[(long long)i + px * ((long long)j + (long long)(d.ny + 2) * (k - 1))];
}
__global__ void k_pack_sr_tf(long long n, const double* __restrict__ src, const double* __restrict__ rdiag,
                             double2* __restrict__ out) {
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x)
    out[m] = make_double2(src[m], rdiag[m]);
}
__global__ void k_pack_coef_tf(const double* __restrict__ c, float4* __restrict__ out, long long n) {
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x) {
    const Limbs s = split3(c[m]);
    out[m] = make_float4(s.h, s.m, s.l, 0.f);
  }
}

// ---------------------------------------------------------------- host side
// Tile shapes: (id, TX, TYB, CY, phi ring depth, (src, rdiag) ring depth).
#define FPM_TF_SHAPES(X) \
  X(0, 32, 8, 2, 4, 3)   \
  X(1, 32, 4, 2, 4, 3)   \
  X(2, 64, 4, 2, 4, 3)   \
  X(3, 32, 4, 4, 4, 3)   \
  X(4, 64, 2, 2, 4, 3)   \
  X(5, 32, 8, 2, 3, 2)

struct TfShape {
  int tx, tyb, cy;
};
#define FPM_TF_SHAPE_ROW(id, tx, tyb, cy, ps, ss) {tx, tyb, cy},
static const TfShape kTfShapes[] = {FPM_TF_SHAPES(FPM_TF_SHAPE_ROW)};
#undef FPM_TF_SHAPE_ROW
constexpr int kNumTfShapes = sizeof(kTfShapes) / sizeof(kTfShapes[0]);

template <int TX, int TYB, int CY, int PS, int SS>
static size_t tf_smem() {
  constexpr size_t ty = TYB * CY;
  constexpr size_t phi = ((TX + 2) * (ty + 2) * 8 + 127) / 128 * 128;
  constexpr size_t limb = ((TX + 2) * (ty + 2) * 4 + 127) / 128 * 128;
  return PS * phi + SS * (size_t)TX * ty * 16 + 9 * limb + (PS + SS) * 8;
}

template <int TX, int TYB, int CY, int PS, int SS>
static cudaError_t tf_launch(const JacobiTfPlan& pl, const double* src_phi, double* dst_phi, cudaStream_t st) {
  const CUtensorMap& tm = (src_phi == pl.a) ? pl.tm_a : pl.tm_b;
  const size_t smem = tf_smem<TX, TYB, CY, PS, SS>();
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_jacobi_tf_tma<TX, TYB, CY, PS, SS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  constexpr int TY = TYB * CY;
  dim3 grid((pl.nx + TX - 1) / TX, (pl.ny + TY - 1) / TY, (pl.nz + pl.kchunk - 1) / pl.kchunk);
  k_jacobi_tf_tma<TX, TYB, CY, PS, SS><<<grid, TX * TYB, smem, st>>>(tm, pl.tm_sr, dst_phi, pl.coef, pl.point2, pl.nx,
                                                                     pl.ny, pl.nz, pl.px, pl.kchunk, pl.err);
  note_launch();
  return cudaGetLastError();
}

cudaError_t jacobi_tf_sweep(const JacobiTfPlan& pl, const double* src_phi, double* dst_phi, cudaStream_t st) {
#define FPM_TF_LAUNCH(id, tx, tyb, cy, ps, ss) \
  case id: return tf_launch<tx, tyb, cy, ps, ss>(pl, src_phi, dst_phi, st);
  switch (pl.shape) {
    FPM_TF_SHAPES(FPM_TF_LAUNCH)
    default: return cudaErrorInvalidValue;
  }
#undef FPM_TF_LAUNCH
}

int jacobi_tf_num_shapes() { return kNumTfShapes; }

void jacobi_tf_shape(int shape, int* tx, int* ty) {
  const TfShape sh = kTfShapes[(shape >= 0 && shape < kNumTfShapes) ? shape : 0];
  *tx = sh.tx;
  *ty = sh.tyb * sh.cy;
}

// 0.2 as FP64 split into limbs on the host (the device split's arithmetic:
// truncated leading 24 bits, then 23, then the rest).
static float4 point2_limbs() {
  const double x = 0.2;
  const float h = (float)x;  // 0.2 rounds up to FP32: take the truncation instead
  float ht = h;
  if ((double)ht > x) ht = std::nextafter(ht, 0.f);
  const double r1 = x - (double)ht;
  float m = (float)r1;
  if (std::fabs((double)m) > std::fabs(r1)) m = std::nextafter(m, 0.f);
  const double r2 = r1 - (double)m;
  return make_float4(ht, m, (float)r2, 0.f);
}

cudaError_t jacobi_tf_pack(JacobiTfPlan& pl, const double* phi, const double* src, const double* rdiag,
                           const double* coef64, cudaStream_t st) {
  const Dims d{pl.nx, pl.ny, pl.nz};
  const size_t nphi = sizeof(double) * pl.px * (pl.ny + 2) * (size_t)pl.nz;
  long long nb = (d.npad() + 255) / 256;
  if (nb > 152LL * 32) nb = 152LL * 32;
  cudaError_t e = cudaMemsetAsync(pl.a, 0, nphi, st);
  if (e != cudaSuccess) return e;
  k_pack_phi_tf<<<(unsigned)nb, 256, 0, st>>>(d, phi, pl.a, pl.px); note_launch();
  e = cudaMemcpyAsync(pl.b, pl.a, nphi, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  const long long nc = d.ncell();
  long long nb2 = (nc + 255) / 256;
  if (nb2 > 152LL * 32) nb2 = 152LL * 32;
  k_pack_sr_tf<<<(unsigned)nb2, 256, 0, st>>>(nc, src, rdiag, reinterpret_cast<double2*>(pl.sr)); note_launch();
  const long long ncoef = 2LL * (pl.nx + pl.ny + pl.nz);
  k_pack_coef_tf<<<(unsigned)((ncoef + 255) / 256), 256, 0, st>>>(coef64, pl.coef, ncoef); note_launch();
  pl.point2 = point2_limbs();
  e = cudaMemsetAsync(pl.err, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t jacobi_tf_encode(JacobiTfPlan& pl) {
  const TfShape sh = kTfShapes[(pl.shape >= 0 && pl.shape < kNumTfShapes) ? pl.shape : 0];
  const uint64_t pitch1 = (uint64_t)pl.px * 8, pitch2 = pitch1 * (uint64_t)(pl.ny + 2);
  const int ty = sh.tyb * sh.cy;
  if (!tma_encode_3d(&pl.tm_a, CU_TENSOR_MAP_DATA_TYPE_UINT64, pl.a, pl.nx + 2, pl.ny + 2, pl.nz, pitch1, pitch2,
                     sh.tx + 2, ty + 2) ||
      !tma_encode_3d(&pl.tm_b, CU_TENSOR_MAP_DATA_TYPE_UINT64, pl.b, pl.nx + 2, pl.ny + 2, pl.nz, pitch1, pitch2,
                     sh.tx + 2, ty + 2) ||
      !tma_encode_3d(&pl.tm_sr, CU_TENSOR_MAP_DATA_TYPE_UINT64, pl.sr, 2ULL * pl.nx, pl.ny, pl.nz, 16ULL * pl.nx,
                     16ULL * pl.nx * pl.ny, 2 * sh.tx, ty))
    return cudaErrorInvalidValue;
  return cudaSuccess;
}

cudaError_t jacobi_tf_unpack(const JacobiTfPlan& pl, const double* cur, double* phi, cudaStream_t st) {
  const Dims d{pl.nx, pl.ny, pl.nz};
  Launch L = cells_launch(d);
  k_unpack_phi_tf<<<L.grid, L.block, 0, st>>>(d, cur, phi, pl.px); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
