// Force densities of several influence potentials in one pass
// (compute_stairstep_fpm_terms_3d, src/fpm_stairstep_mpi_3d.f90:426-497,
// for phi_x, phi_y, phi_z at once).
//
// The nine flow fields and the solid flag are read once per cell for all
// potentials: 9*8 + 4 + NP*(8 + 40) bytes per cell (220 for three
// potentials, against 3 x 124 for three separate calls).  On GB300 the FP64
// pipe (about 0.53 T instructions/s) would bound the ~25 FP64 operations per
// cell and potential at several times the HBM time, so the per-cell
// arithmetic is double-float (f32 pairs, 48-bit significand, error-free
// transforms on the FP32 pipe): every FP64 input is split into (hi, lo) with
// integer operations (the FP64 <-> FP32 conversion instructions run on the
// FP64 pipe), and each output leaves as RN(hi + lo) with one FP64 addition of
// the two parts rebuilt as FP64 by bit assembly.  The densities
// are accurate to about 1e-14 relative; the integrals are summed per thread
// in double-float along z and combined across threads and blocks in FP64.
// The separately rounded FP64 kernel (k_terms) stays the bit-identical
// single-potential path.
#include "fpm_internal.h"

namespace fpm {

namespace {

// FP64 -> (hi, lo) with hi the FP64 value truncated to 24 bits and lo the
// next 23 bits of the remainder: hi + lo is within 2^-46 relative of x.
// Integer and FP32 operations only.  Magnitudes below 2^-126 become zero (far below
// any tolerance of the densities); magnitudes of 2^127 and above become
// infinities and NaN stays NaN.  (The conversion instructions run on the FP64
// pipe, and even a rarely taken branch to one is predicated into every call.)
__device__ __forceinline__ float2 split_f64(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
  const int e = (int)((hi32 >> 20) & 0x7FFu);
  const unsigned sign = hi32 & 0x80000000u;
  if (e < 897) return make_float2(0.f, 0.f);
  if (e > 1150) {  // 2^127 and above: infinity; NaN stays NaN (bit operations, no conversion)
    const bool nan = e == 2047 && ((hi32 & 0xFFFFFu) | lo32) != 0u;
    return make_float2(__uint_as_float(sign | 0x7F800000u | (nan ? 0x400000u : 0u)), 0.f);
  }
  const float h = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | ((hi32 & 0xFFFFFu) << 3) | (lo32 >> 29));
  float l = 0.f;
  if (e >= 943) {  // the scale 2^(e-1069) of the remainder's top 23 bits is a normal float
    // top 23 of the 29 remainder bits as an exact FP32 integer (2^23 + n - 2^23,
    // FP32 pipe; the integer-to-float conversion instruction is not), scaled
    const float n = __uint_as_float(0x4B000000u | ((lo32 & 0x1FFFFFFFu) >> 6)) - 8388608.0f;
    l = n * __uint_as_float((unsigned)(e - 942) << 23);
    l = __uint_as_float(__float_as_uint(l) | sign);
  }
  return make_float2(h, l);
}

// FP32 -> FP64 by bit assembly (exact; the conversion instruction runs on the
// FP64 pipe).  Zero and subnormal inputs give a signed zero (a subnormal FP32
// value is far below the densities' tolerance); infinities and NaN map to
// themselves.
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned sign = u & 0x80000000u;
  const unsigned eo = e == 0u ? 0u : (e == 0xFFu ? 2047u : e + 896u);
  const unsigned hi = e == 0u ? sign : sign | (eo << 20) | ((u & 0x7FFFFFu) >> 3);
  const unsigned lo = e == 0u ? 0u : (u << 29);
  return __hiloint2double((int)hi, (int)lo);
}

// RN(hi + lo) of a double-float value: one FP64 addition.
__device__ __forceinline__ double df_to_f64(float2 v) { return __dadd_rn(f32_to_f64(v.x), f32_to_f64(v.y)); }

__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 df_sub(float2 a, float2 b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ float2 df_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

}  // namespace

struct TermsMultiArgs {
  const double* phi[kMaxRhs];
  Faces f[kMaxRhs];
  float2 bg[kMaxRhs][3];
  double* out[kMaxRhs][5];  // gx, gy, gz, vortex, advection
};

// Per-axis tables: the spacing reciprocals 1/(c_m - c_{m-1}) (m >= 1; entry 0
// unused) and the cell widths as double-float, and whether the cell centre
// lies strictly inside the integration bounds.
struct TermsTables {
  float2 *rx, *ry, *rz, *wx, *wy, *wz;
  unsigned char *inx, *iny, *inz;
};

__global__ void k_terms_tables(Dims d, Axes ax, double b0, double b1, double b2, double b3, double b4, double b5,
                               TermsTables t) {
  const int n = (d.nx + 2) + (d.ny + 2) + d.nz;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    if (s < d.nx + 2) {
      const int i = s;
      t.rx[i] = i >= 1 ? df_from_double(ddiv(1.0, dsub(ax.xc[i], ax.xc[i - 1]))) : make_float2(0.f, 0.f);
      if (i >= 1 && i <= d.nx) {
        t.wx[i - 1] = df_from_double(ax.dx[i - 1]);
        t.inx[i - 1] = ax.xc[i] > b0 && ax.xc[i] < b1;
      }
    } else if (s < d.nx + 2 + d.ny + 2) {
      const int j = s - (d.nx + 2);
      t.ry[j] = j >= 1 ? df_from_double(ddiv(1.0, dsub(ax.yc[j], ax.yc[j - 1]))) : make_float2(0.f, 0.f);
      if (j >= 1 && j <= d.ny) {
        t.wy[j - 1] = df_from_double(ax.dy[j - 1]);
        t.iny[j - 1] = ax.yc[j] > b2 && ax.yc[j] < b3;
      }
    } else {
      const int k = s - (d.nx + 2) - (d.ny + 2);  // 0-based: zc[k], dz[k]
      t.rz[k] = k >= 1 ? df_from_double(ddiv(1.0, dsub(ax.zc[k], ax.zc[k - 1]))) : make_float2(0.f, 0.f);
      t.wz[k] = df_from_double(ax.dz[k]);
      t.inz[k] = ax.zc[k] > b4 && ax.zc[k] < b5;
    }
  }
}

// One thread per (i, j) column over a strided set of planes (the cell loop of
// the other stair-step kernels), all potentials of a cell in the same thread
// so that the flow fields and the solid flags are loaded once.  Face
// gradients follow face_gradients (src/fpm_stairstep_mpi_3d.f90:472-497):
// outer face value | body_grad at a solid neighbour | (phi_nb - phi) /
// (c_nb - c).  (One warp per potential with the flow shared through L1 was
// measured slower for three potentials: 1.89 against 1.59 ms at 256^2 x 128.)
// Four blocks per SM (64 registers, a few spilled) instead of the compiler's
// 122 registers at two: the cell's long arithmetic phase runs with no loads
// in flight, so more resident warps pay (three potentials at 384^2 x 192:
// 4.71 -> 3.81 ms; three and five blocks measured 4.10 and 4.26 ms).
constexpr int kTermsRows = 8;

template <int NP>
__global__ void __launch_bounds__(256, 4) k_terms_multi(Dims d, TermsMultiArgs A, Flow fl,
                                                      const int32_t* __restrict__ solid, TermsTables t,
                                                      double* partials, unsigned int* ticket, double* totals) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * kTermsRows + threadIdx.y + 1;
  const bool inxy = (i <= d.nx) && (j <= d.ny);
  float2 sv[NP], sa[NP];  // sum over this thread's planes of dz * density (inside cells only)
#pragma unroll
  for (int m = 0; m < NP; m++) sv[m] = sa[m] = make_float2(0.f, 0.f);
  const long long px = d.nx + 2, pl = d.plane();
  float2 rxw = make_float2(0.f, 0.f), rxe = rxw, rys = rxw, ryn = rxw;
  bool colin = false;
  if (inxy) {
    rxw = t.rx[i];
    rxe = t.rx[i + 1];
    rys = t.ry[j];
    ryn = t.ry[j + 1];
    colin = t.inx[i - 1] && t.iny[j - 1];
  }
  for (int k = blockIdx.z + 1; k <= d.nz && inxy; k += gridDim.z) {
    const long long p = d.ph(i, j, k), cc = d.in(i, j, k);
    const bool fluid = solid[p] == 0;
    const bool sw = solid[p - 1] != 0, se = solid[p + 1] != 0, ss = solid[p - px] != 0, sn = solid[p + px] != 0;
    const bool sb = k > 1 && solid[p - pl] != 0, st = k < d.nz && solid[p + pl] != 0;
    const float hm = fluid ? 0.5f : 0.f;
    const float2 u = split_f64(fl.u[cc]), v = split_f64(fl.v[cc]), w = split_f64(fl.w[cc]);
    const float2 ox = split_f64(fl.ox[cc]), oy = split_f64(fl.oy[cc]), oz = split_f64(fl.oz[cc]);
    const float2 cx = df_sub(df_mul(w, oy), df_mul(v, oz));
    const float2 cy = df_sub(df_mul(u, oz), df_mul(w, ox));
    const float2 cz = df_sub(df_mul(v, ox), df_mul(u, oy));
    const float2 ax = split_f64(fl.ax[cc]), ay = split_f64(fl.ay[cc]), az = split_f64(fl.az[cc]);
    const float2 rzb = k > 1 ? t.rz[k - 1] : make_float2(0.f, 0.f);
    const float2 rzt = k < d.nz ? t.rz[k] : make_float2(0.f, 0.f);
    const bool inside = colin && t.inz[k - 1];
    const float2 wzk = t.wz[k - 1];
#pragma unroll
    for (int m = 0; m < NP; m++) {
      const double* ph = A.phi[m];
      const Faces& f = A.f[m];
      const float2 pc = split_f64(ph[p]);
      float2 g0, g1, g2, g3, g4, g5;
      if (i == 1) g0 = split_f64(f.xlo[d.xf(j, k)]);
      else if (sw) g0 = A.bg[m][0];
      else g0 = df_mul(df_sub(pc, split_f64(ph[p - 1])), rxw);
      if (i == d.nx) g1 = split_f64(f.xhi[d.xf(j, k)]);
      else if (se) g1 = A.bg[m][0];
      else g1 = df_mul(df_sub(split_f64(ph[p + 1]), pc), rxe);
      if (j == 1) g2 = split_f64(f.ylo[d.yf(i, k)]);
      else if (ss) g2 = A.bg[m][1];
      else g2 = df_mul(df_sub(pc, split_f64(ph[p - px])), rys);
      if (j == d.ny) g3 = split_f64(f.yhi[d.yf(i, k)]);
      else if (sn) g3 = A.bg[m][1];
      else g3 = df_mul(df_sub(split_f64(ph[p + px]), pc), ryn);
      if (k == 1) g4 = split_f64(f.zlo[d.zf(i, j)]);
      else if (sb) g4 = A.bg[m][2];
      else g4 = df_mul(df_sub(pc, split_f64(ph[p - pl])), rzb);
      if (k == d.nz) g5 = split_f64(f.zhi[d.zf(i, j)]);
      else if (st) g5 = A.bg[m][2];
      else g5 = df_mul(df_sub(split_f64(ph[p + pl]), pc), rzt);
      const float2 gx = df_scale(df_add(g0, g1), hm);
      const float2 gy = df_scale(df_add(g2, g3), hm);
      const float2 gz = df_scale(df_add(g4, g5), hm);
      const float2 vort = df_neg(df_add(df_add(df_mul(cx, gx), df_mul(cy, gy)), df_mul(cz, gz)));
      const float2 adv = df_neg(df_add(df_add(df_mul(ax, gx), df_mul(ay, gy)), df_mul(az, gz)));
      A.out[m][0][cc] = df_to_f64(gx);
      A.out[m][1][cc] = df_to_f64(gy);
      A.out[m][2][cc] = df_to_f64(gz);
      A.out[m][3][cc] = df_to_f64(vort);
      A.out[m][4][cc] = df_to_f64(adv);
      if (inside) {
        sv[m] = df_add(sv[m], df_mul(wzk, vort));
        sa[m] = df_add(sa[m], df_mul(wzk, adv));
      }
    }
  }
  // this column's sums times dx_i dy_j, then the deterministic grid reduction
  double s[2 * NP], mx[1] = {0.0};
  float2 wxy = make_float2(0.f, 0.f);
  if (inxy) wxy = df_mul(t.wx[i - 1], t.wy[j - 1]);
#pragma unroll
  for (int m = 0; m < NP; m++) {
    s[2 * m] = inxy ? df_to_f64(df_mul(wxy, sv[m])) : 0.0;
    s[2 * m + 1] = inxy ? df_to_f64(df_mul(wxy, sa[m])) : 0.0;
  }
  double out[2 * NP];
  if (grid_reduce<2 * NP, 0>(s, mx, partials, ticket, out) && lin_tid() == 0) {
#pragma unroll
    for (int n = 0; n < 2 * NP; n++) totals[n] = out[n];
  }
}

cudaError_t launch_terms_multi(const Dims& d, int np, const double* const* phi, const Flow& fl,
                               const int32_t* solid, const double* bg, const Axes& ax, const Faces* faces,
                               const double bounds[6], double* const* outs, void* tables, double* partials,
                               unsigned int* ticket, double* totals, cudaStream_t st) {
  if (np < 1 || np > kMaxRhs) return cudaErrorInvalidValue;
  TermsTables t;
  char* q = static_cast<char*>(tables);
  auto take = [&](size_t bytes) {
    void* r = q;
    q += (bytes + 255) / 256 * 256;
    return r;
  };
  t.rx = static_cast<float2*>(take(sizeof(float2) * (d.nx + 2)));
  t.ry = static_cast<float2*>(take(sizeof(float2) * (d.ny + 2)));
  t.rz = static_cast<float2*>(take(sizeof(float2) * d.nz));
  t.wx = static_cast<float2*>(take(sizeof(float2) * d.nx));
  t.wy = static_cast<float2*>(take(sizeof(float2) * d.ny));
  t.wz = static_cast<float2*>(take(sizeof(float2) * d.nz));
  t.inx = static_cast<unsigned char*>(take(d.nx));
  t.iny = static_cast<unsigned char*>(take(d.ny));
  t.inz = static_cast<unsigned char*>(take(d.nz));
  const int nt = (d.nx + 2) + (d.ny + 2) + d.nz;
  k_terms_tables<<<(nt + 255) / 256, 256, 0, st>>>(d, ax, bounds[0], bounds[1], bounds[2], bounds[3], bounds[4],
                                                   bounds[5], t);
  note_launch();
  TermsMultiArgs A;
  for (int m = 0; m < np; m++) {
    A.phi[m] = phi[m];
    A.f[m] = faces[m];
    for (int c = 0; c < 3; c++) A.bg[m][c] = df_from_double(bg[3 * m + c]);
    for (int c = 0; c < 5; c++) A.out[m][c] = outs[5 * m + c];
  }
  const dim3 grid = terms_multi_grid(d), block(32, kTermsRows, 1);
  switch (np) {
    case 1: k_terms_multi<1><<<grid, block, 0, st>>>(d, A, fl, solid, t, partials, ticket, totals); break;
    case 2: k_terms_multi<2><<<grid, block, 0, st>>>(d, A, fl, solid, t, partials, ticket, totals); break;
    case 3: k_terms_multi<3><<<grid, block, 0, st>>>(d, A, fl, solid, t, partials, ticket, totals); break;
    default: k_terms_multi<4><<<grid, block, 0, st>>>(d, A, fl, solid, t, partials, ticket, totals); break;
  }
  note_launch();
  return cudaGetLastError();
}

// Grid of k_terms_multi: (32 x kTermsRows)-cell tiles, z-strided chunks
// giving about 16 blocks per SM over the grid.
dim3 terms_multi_grid(const Dims& d) {
  const int gx = (d.nx + 31) / 32, gy = (d.ny + kTermsRows - 1) / kTermsRows;
  const long long xy = (long long)gx * gy;
  long long gz = (152LL * 16 + xy - 1) / xy;
  if (gz < 1) gz = 1;
  if (gz > d.nz) gz = d.nz;
  return dim3(gx, gy, (unsigned)gz);
}

// Bytes of the per-axis tables launch_terms_multi carves from `tables`.
size_t terms_multi_table_bytes(const Dims& d) {
  auto r = [](size_t b) { return (b + 255) / 256 * 256; };
  return r(8 * (d.nx + 2)) + r(8 * (d.ny + 2)) + r(8 * (size_t)d.nz) + r(8 * (size_t)d.nx) + r(8 * (size_t)d.ny) +
         r(8 * (size_t)d.nz) + r(d.nx) + r(d.ny) + r(d.nz);
}

}  // namespace fpm
