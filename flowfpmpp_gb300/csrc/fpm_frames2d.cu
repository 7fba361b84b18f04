// Batched uneven 2-D frames: for every frame of a batch, the reference's 2-D
// use of the stair-step solver (examples/flapping_foil_fpm.f90:61-81: nz = 2,
// dz = 0.5, zero outer data, body_grad = e_x and e_y, compatibility, PCG to
// the tolerance) followed by fpm_partition_terms_2d
// (src/fpm_partition_2d.f90:35-154) for both directions.
//
// All frames run in the same launches: every kernel walks a tile list (32 x 8
// columns of one frame, both z layers per thread), and every per-frame
// reduction is segmented: a tile writes its partial sums, and the last tile
// of its frame to finish (per-frame ticket) combines the frame's partials in
// tile order and updates that frame's scalars.  The solve is the mixed
// scheme: FP64 true residual, max-norm test and phi update; FP32 diagonal PCG
// in between, with per-frame, per-direction active flags so converged frames
// drop out of the work without a host round trip.
#include "fpm_internal.h"

namespace fpm {

namespace {

constexpr int kR = 2;  // right-hand sides per frame (phi_x, phi_y)

// 1 / (dz (zc(2) - zc(1))) for dz = 0.5, zc = (0.25, 0.75).
constexpr double kCz = 4.0;

struct TileRef {
  int tile, f, i, j;  // global tile id, frame, 1-based cell indices of this thread's column
  bool live;
};

// Block -> tile: the identity, or an entry of a compacted list of the tiles of
// the frames still iterating (all tiles of a frame are in it or none).
__device__ __forceinline__ TileRef tile_ref(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame,
                                            const int* __restrict__ tiles) {
  TileRef t;
  t.tile = tiles ? tiles[blockIdx.x] : (int)blockIdx.x;
  t.f = tile_frame[t.tile];
  const Frame2& F = fr[t.f];
  const int idx = t.tile - F.tile0;
  t.i = (idx % F.tiles_x) * 32 + threadIdx.x + 1;
  t.j = (idx / F.tiles_x) * 8 + threadIdx.y + 1;
  t.live = t.i <= F.nx && t.j <= F.ny;
  return t;
}

__device__ __forceinline__ long long ph(const Frame2& F, int i, int j, int k) {
  return F.opad + i + (long long)(F.nx + 2) * (j + (long long)(F.ny + 2) * (k - 1));
}
__device__ __forceinline__ long long in(const Frame2& F, int i, int j, int k) {
  return F.oint + (i - 1) + (long long)F.nx * ((j - 1) + (long long)F.ny * (k - 1));
}
__device__ __forceinline__ long long c2(const Frame2& F, int i, int j) {
  return F.o2 + (i - 1) + (long long)F.nx * (j - 1);
}

// Segmented reduction of NS sums and NM maxima over the tiles of one frame.
// Returns true in the last tile of the frame, with out[] holding the results.
template <int NS, int NM>
__device__ bool seg_reduce(double (&s)[NS > 0 ? NS : 1], double (&m)[NM > 0 ? NM : 1], const Frame2& F, int f,
                           double* partials, unsigned int* tickets, double* out, int tile) {
  __shared__ bool am_last;
  constexpr int N = NS + NM;
  block_reduce<NS, NM>(s, m);
  const int tid = lin_tid();
  if (tid == 0) {
#pragma unroll
    for (int n = 0; n < NS; n++) partials[(size_t)tile * N + n] = s[n];
#pragma unroll
    for (int n = 0; n < NM; n++) partials[(size_t)tile * N + NS + n] = m[n];
    __threadfence();
    const unsigned int t = atomicAdd(&tickets[f], 1u);
    am_last = (t == (unsigned int)F.ntiles - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double as[NS > 0 ? NS : 1], am[NM > 0 ? NM : 1];
#pragma unroll
  for (int n = 0; n < NS; n++) as[n] = 0.0;
#pragma unroll
  for (int n = 0; n < NM; n++) am[n] = 0.0;
  for (int b = tid; b < F.ntiles; b += lin_nthreads()) {
    const double* p = partials + (size_t)(F.tile0 + b) * N;
#pragma unroll
    for (int n = 0; n < NS; n++) as[n] += __ldcg(p + n);
#pragma unroll
    for (int n = 0; n < NM; n++) am[n] = fmax(am[n], __ldcg(p + NS + n));
  }
  block_reduce<NS, NM>(as, am);
  if (tid == 0) {
#pragma unroll
    for (int n = 0; n < NS; n++) out[n] = as[n];
#pragma unroll
    for (int n = 0; n < NM; n++) out[NS + n] = am[n];
    tickets[f] = 0u;
    __threadfence();
  }
  __syncthreads();
  return true;
}

struct F2Pair {
  float s = 0.f, e = 0.f;
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = a * b;
    const float pe = fmaf(a, b, -p);
    const float t = s + p;
    const float bb = t - s;
    e += ((s - (t - bb)) + (p - bb)) + pe;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)e; }
};

}  // namespace

// ---------------------------------------------------------------- compatibility
// enforce_stairstep_compatibility_3d (src/fpm_stairstep_mpi_3d.f90:41-92) with
// rhs = 0 and zero outer data: correction = -(body flux) / (fluid outer area),
// for body_grad = e_x (r = 0) and e_y (r = 1).
__global__ void k_b2_compat(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  const Frame2& F = fr[t.f];
  double s[3] = {0.0, 0.0, 0.0}, m[1] = {0.0};
  if (t.live) {
    const double dxi = b.dx[F.ox + t.i - 1], dyj = b.dy[F.oy + t.j - 1];
    for (int k = 1; k <= 2; k++) {
      if (b.solid3[ph(F, t.i, t.j, k)] != 0) continue;
      const double ayz = dmul(dyj, 0.5), axz = dmul(dxi, 0.5), axy = dmul(dxi, dyj);
      if (t.i == 1) s[2] += ayz;
      else if (b.solid3[ph(F, t.i - 1, t.j, k)] != 0) s[0] -= ayz;
      if (t.i == F.nx) s[2] += ayz;
      else if (b.solid3[ph(F, t.i + 1, t.j, k)] != 0) s[0] += ayz;
      if (t.j == 1) s[2] += axz;
      else if (b.solid3[ph(F, t.i, t.j - 1, k)] != 0) s[1] -= axz;
      if (t.j == F.ny) s[2] += axz;
      else if (b.solid3[ph(F, t.i, t.j + 1, k)] != 0) s[1] += axz;
      s[2] += axy;  // k == 1 bottom or k == 2 top face (the other z face is fluid)
    }
  }
  double out[3];
  if (seg_reduce<3, 0>(s, m, F, t.f, b.partials, b.tickets, out, t.tile) && lin_tid() == 0) {
    const double area = out[2];
    for (int r = 0; r < kR; r++) b.corr[t.f * kR + r] = area > 0 ? -out[r] / area : 0.0;
    if (!(area > 0)) atomicExch(b.err, 2);
  }
}

// ---------------------------------------------------------------- operator
// build_operator (src/fpm_stairstep_mpi_3d.f90:336-379) per frame, both
// directions: outer faces carry +-corr (xlo = -c, xhi = +c, ...), body faces
// body_grad; diag, rdiag = 1/(V diag) shared by both directions.
__global__ void k_b2_build(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  if (!t.live) return;
  const Frame2& F = fr[t.f];
  const int i = t.i, j = t.j, nx = F.nx, ny = F.ny;
  const double* xc = b.xc + F.ox;
  const double* yc = b.yc + F.oy;
  const double dxi = b.dx[F.ox + i - 1], dyj = b.dy[F.oy + j - 1], dzk = 0.5;
  const double cw = i == 1 ? 0.0 : ddiv(1.0, dmul(dxi, dsub(xc[i], xc[i - 1])));
  const double ce = i == nx ? 0.0 : ddiv(1.0, dmul(dxi, dsub(xc[i + 1], xc[i])));
  const double cs = j == 1 ? 0.0 : ddiv(1.0, dmul(dyj, dsub(yc[j], yc[j - 1])));
  const double cn = j == ny ? 0.0 : ddiv(1.0, dmul(dyj, dsub(yc[j + 1], yc[j])));
  if (j == 1) {
    b.cw32[F.ox + i - 1] = (float)cw;
    b.ce32[F.ox + i - 1] = (float)ce;
  }
  if (i == 1) {
    b.cs32[F.oy + j - 1] = (float)cs;
    b.cn32[F.oy + j - 1] = (float)cn;
  }
  for (int k = 1; k <= 2; k++) {
    const long long c = in(F, i, j, k);
    double s[kR] = {0.0, 0.0}, d = 0.0, wall = -1.0;
    if (b.solid3[ph(F, i, j, k)] == 0) {
      const double bg[kR][2] = {{1.0, 0.0}, {0.0, 1.0}};
      for (int r = 0; r < kR; r++) {
        const double cr = b.corr[t.f * kR + r];
        double v = -0.0;  // s = -rhs with rhs = 0
        if (i == 1) v = dsub(v, ddiv(-cr, dxi));
        else if (b.solid3[ph(F, i - 1, j, k)] != 0) v = dsub(v, ddiv(bg[r][0], dxi));
        if (i == nx) v = dadd(v, ddiv(cr, dxi));
        else if (b.solid3[ph(F, i + 1, j, k)] != 0) v = dadd(v, ddiv(bg[r][0], dxi));
        if (j == 1) v = dsub(v, ddiv(-cr, dyj));
        else if (b.solid3[ph(F, i, j - 1, k)] != 0) v = dsub(v, ddiv(bg[r][1], dyj));
        if (j == ny) v = dadd(v, ddiv(cr, dyj));
        else if (b.solid3[ph(F, i, j + 1, k)] != 0) v = dadd(v, ddiv(bg[r][1], dyj));
        if (k == 1) v = dsub(v, ddiv(-cr, dzk));
        if (k == 2) v = dadd(v, ddiv(cr, dzk));
        s[r] = v;
      }
      if (i > 1 && b.solid3[ph(F, i - 1, j, k)] == 0) d = dadd(d, cw);
      if (i < nx && b.solid3[ph(F, i + 1, j, k)] == 0) d = dadd(d, ce);
      if (j > 1 && b.solid3[ph(F, i, j - 1, k)] == 0) d = dadd(d, cs);
      if (j < ny && b.solid3[ph(F, i, j + 1, k)] == 0) d = dadd(d, cn);
      d = dadd(d, kCz);  // the other z layer of a fluid column is fluid
      wall = 0.0;        // coefficients towards solid neighbours (difference form of the FP32 stencil)
      if (i > 1 && b.solid3[ph(F, i - 1, j, k)] != 0) wall += cw;
      if (i < nx && b.solid3[ph(F, i + 1, j, k)] != 0) wall += ce;
      if (j > 1 && b.solid3[ph(F, i, j - 1, k)] != 0) wall += cs;
      if (j < ny && b.solid3[ph(F, i, j + 1, k)] != 0) wall += cn;
    }
    b.wall32[c] = (float)wall;
    for (int r = 0; r < kR; r++) b.src[r][c] = s[r];
    b.diag[c] = d;
    const double rd = d > 0 ? ddiv(1.0, dmul(dmul(dmul(dxi, dyj), dzk), d)) : 0.0;
    b.rdiag[c] = rd;
    b.diag32[c] = (float)d;
    b.rdiag32[c] = (float)rd;
  }
}

// src + sum c phi_nb - diag phi at (i, j, k) of direction r (reference order).
__device__ __forceinline__ double b2_local_res(const Frame2& F, const Batch2& b, const double* __restrict__ phi,
                                               double src, double dg, double cw, double ce, double cs, double cn,
                                               int i, int j, int k) {
  const long long p = ph(F, i, j, k), px = F.nx + 2, pl = (long long)(F.nx + 2) * (F.ny + 2);
  const double cb = k == 2 ? kCz : 0.0, ct = k == 1 ? kCz : 0.0;
  const long long pb = k == 2 ? p - pl : p, pt = k == 1 ? p + pl : p;
  double t = dadd(src, dmul(cw, phi[p - 1]));
  t = dadd(t, dmul(ce, phi[p + 1]));
  t = dadd(t, dmul(cs, phi[p - px]));
  t = dadd(t, dmul(cn, phi[p + px]));
  t = dadd(t, dmul(cb, phi[pb]));
  t = dadd(t, dmul(ct, phi[pt]));
  return dsub(t, dmul(dg, phi[p]));
}

struct ColCoef {
  double cw, ce, cs, cn;
};
__device__ __forceinline__ ColCoef col_coef(const Frame2& F, const Batch2& b, int i, int j) {
  const double* xc = b.xc + F.ox;
  const double* yc = b.yc + F.oy;
  const double dxi = b.dx[F.ox + i - 1], dyj = b.dy[F.oy + j - 1];
  ColCoef c;
  c.cw = i == 1 ? 0.0 : ddiv(1.0, dmul(dxi, dsub(xc[i], xc[i - 1])));
  c.ce = i == F.nx ? 0.0 : ddiv(1.0, dmul(dxi, dsub(xc[i + 1], xc[i])));
  c.cs = j == 1 ? 0.0 : ddiv(1.0, dmul(dyj, dsub(yc[j], yc[j - 1])));
  c.cn = j == F.ny ? 0.0 : ddiv(1.0, dmul(dyj, dsub(yc[j + 1], yc[j])));
  return c;
}

// ---------------------------------------------------------------- FP64 true residual
// true_residual (src/fpm_stairstep_mpi_3d.f90:297-329) per frame and direction:
// rV = V t on diag > 0 (t = src + sum c phi - diag phi), res = max |t|, and
// the sum and count for the projection; only directions in the set.
__global__ void k_b2_tres(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  const Frame2& F = fr[t.f];
  int set[kR];
  for (int r = 0; r < kR; r++) set[r] = b.in_set[t.f * kR + r];
  if (!set[0] && !set[1]) return;
  double s[3] = {0.0, 0.0, 0.0}, m[2] = {0.0, 0.0};
  if (t.live) {
    const ColCoef cc = col_coef(F, b, t.i, t.j);
    const double vol0 = dmul(dmul(b.dx[F.ox + t.i - 1], b.dy[F.oy + t.j - 1]), 0.5);
    for (int k = 1; k <= 2; k++) {
      const long long c = in(F, t.i, t.j, k);
      const double dg = b.diag[c];
      for (int r = 0; r < kR; r++) {
        if (!set[r]) continue;
        double rv = 0.0;
        if (dg > 0) {
          const double tt = b2_local_res(F, b, b.phi[r], b.src[r][c], dg, cc.cw, cc.ce, cc.cs, cc.cn, t.i, t.j, k);
          m[r] = fmax(m[r], fabs(tt));
          rv = dmul(vol0, tt);
          s[r] += rv;
          if (r == 0) s[2] += 1.0;
        }
        b.r64[r][c] = rv;
      }
    }
  }
  double out[5];
  if (seg_reduce<3, 2>(s, m, F, t.f, b.partials, b.tickets, out, t.tile) && lin_tid() == 0) {
    for (int r = 0; r < kR; r++) {
      if (!set[r]) continue;
      b.res[t.f * kR + r] = out[3 + r];
      b.rmean[t.f * kR + r] = out[2] > 0 ? out[r] / out[2] : 0.0;
    }
  }
}

// ---------------------------------------------------------------- FP32 inner PCG
// Residual replacement (reliable update) for the (frame, direction) pairs in
// the set: r = scale (rV - mean), e = 0, p = rdiag r (pmul == 0) or p *= pmul.
__global__ void k_b2_start(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  const Frame2& F = fr[t.f];
  int set[kR];
  for (int r = 0; r < kR; r++) set[r] = b.in_set[t.f * kR + r];
  if (!set[0] && !set[1]) return;
  double s[kR] = {0.0, 0.0}, m[1] = {0.0};
  F2Pair acc[kR];
  if (t.live) {
    for (int k = 1; k <= 2; k++) {
      const long long c = in(F, t.i, t.j, k), p = ph(F, t.i, t.j, k);
      const float rd = b.rdiag32[c];
      const bool fl = b.diag[c] > 0;
      for (int r = 0; r < kR; r++) {
        if (!set[r]) continue;
        const double rv = fl ? b.r64[r][c] - b.rmean[t.f * kR + r] : 0.0;
        const float rr = (float)(rv * b.scale[t.f * kR + r]);
        const float z = rd * rr;
        const float pm = (float)b.pmul[t.f * kR + r];
        b.r32[r][c] = rr;
        b.p32[r][p] = pm == 0.f ? z : b.p32[r][p] * pm;
        b.e32[r][c] = 0.f;
        acc[r].add_prod(z, rr);
      }
    }
  }
  for (int r = 0; r < kR; r++) s[r] = acc[r].value();
  double out[kR];
  if (seg_reduce<kR, 0>(s, m, F, t.f, b.partials, b.tickets, out, t.tile) && lin_tid() == 0) {
    for (int r = 0; r < kR; r++) {
      if (!set[r]) continue;
      const int q = t.f * kR + r;
      b.rz[q] = out[r];
      b.rz0[q] = out[r];
      b.active[q] = out[r] > 0 ? 1 : 0;
    }
  }
}

__global__ void k_b2_spmv(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  const Frame2& F = fr[t.f];
  int act[kR];
  for (int r = 0; r < kR; r++) act[r] = b.active[t.f * kR + r];
  if (!act[0] && !act[1]) return;
  double s[kR] = {0.0, 0.0}, m[1] = {0.0};
  F2Pair acc[kR];
  if (t.live) {
    // difference form V (sum_nb c (p - p_nb) - wall p) of V (diag p - sum c p_nb)
    const float cw = b.cw32[F.ox + t.i - 1], ce = b.ce32[F.ox + t.i - 1], cs = b.cs32[F.oy + t.j - 1],
                cn = b.cn32[F.oy + t.j - 1], cz = (float)kCz;
    const float vol = (float)b.dx[F.ox + t.i - 1] * (float)b.dy[F.oy + t.j - 1] * 0.5f;
    const long long px = F.nx + 2, pl = (long long)(F.nx + 2) * (F.ny + 2);
    for (int r = 0; r < kR; r++) {
      if (!act[r]) continue;
      const float* pm = b.p32[r];
      const long long p1 = ph(F, t.i, t.j, 1), p2 = p1 + pl;
      const float a1 = pm[p1], a2 = pm[p2];
      for (int k = 1; k <= 2; k++) {
        const long long c = in(F, t.i, t.j, k), p = k == 1 ? p1 : p2;
        const float wl = b.wall32[c];
        const float pc = k == 1 ? a1 : a2, pz = k == 1 ? a2 : a1;
        float q = 0.f;
        if (wl >= 0.f) {
          float tt = -wl * pc;
          tt = fmaf(cw, pc - pm[p - 1], tt);
          tt = fmaf(ce, pc - pm[p + 1], tt);
          tt = fmaf(cs, pc - pm[p - px], tt);
          tt = fmaf(cn, pc - pm[p + px], tt);
          tt = fmaf(cz, pc - pz, tt);
          q = vol * tt;
        }
        b.q32[r][c] = q;
        acc[r].add_prod(pc, q);
      }
    }
  }
  for (int r = 0; r < kR; r++) s[r] = acc[r].value();
  double out[kR];
  if (seg_reduce<kR, 0>(s, m, F, t.f, b.partials, b.tickets, out, t.tile) && lin_tid() == 0) {
    for (int r = 0; r < kR; r++) {
      const int q = t.f * kR + r;
      if (!act[r]) continue;
      if (!(out[r] > 0) || !(b.rz[q] > 0)) {
        b.active[q] = 0;
        b.alpha[q] = 0;
      } else {
        b.alpha[q] = b.rz[q] / out[r];
      }
    }
  }
}

__global__ void k_b2_update(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  const Frame2& F = fr[t.f];
  int act[kR];
  float alpha[kR];
  for (int r = 0; r < kR; r++) {
    act[r] = b.active[t.f * kR + r];
    alpha[r] = (float)b.alpha[t.f * kR + r];
  }
  if (!act[0] && !act[1]) {
    // no iteration for this frame: no direction update either
    if (t.tile == F.tile0 && lin_tid() == 0) b.dir[t.f * kR] = b.dir[t.f * kR + 1] = 0;
    return;
  }
  double s[kR] = {0.0, 0.0}, m[1] = {0.0};
  F2Pair acc[kR];
  if (t.live) {
    for (int k = 1; k <= 2; k++) {
      const long long c = in(F, t.i, t.j, k), p = ph(F, t.i, t.j, k);
      const float rd = b.rdiag32[c];
      for (int r = 0; r < kR; r++) {
        if (!act[r]) continue;
        b.e32[r][c] = fmaf(alpha[r], b.p32[r][p], b.e32[r][c]);
        const float rr = fmaf(-alpha[r], b.q32[r][c], b.r32[r][c]);
        b.r32[r][c] = rr;
        acc[r].add_prod(rd * rr, rr);
      }
    }
  }
  for (int r = 0; r < kR; r++) s[r] = acc[r].value();
  double out[kR];
  if (seg_reduce<kR, 0>(s, m, F, t.f, b.partials, b.tickets, out, t.tile) && lin_tid() == 0) {
    for (int r = 0; r < kR; r++) {
      const int q = t.f * kR + r;
      if (!act[r]) {
        b.dir[q] = 0;
        continue;
      }
      b.iters[q] += 1;
      const double rz_new = out[r];
      if (!(rz_new >= 0)) {
        b.active[q] = 0;
        b.dir[q] = 0;
        continue;
      }
      b.beta[q] = rz_new / b.rz[q];
      b.rz[q] = rz_new;
      b.dir[q] = 1;  // the direction update of this iteration still runs
      if (rz_new <= b.tol2 * b.rz0[q]) b.active[q] = 0;
    }
  }
}

__global__ void k_b2_direction(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  const Frame2& F = fr[t.f];
  int act[kR];
  float beta[kR];
  for (int r = 0; r < kR; r++) {
    act[r] = b.dir[t.f * kR + r];  // set by this iteration's update, even if it stopped the iteration
    beta[r] = (float)b.beta[t.f * kR + r];
  }
  if ((!act[0] && !act[1]) || !t.live) return;
  for (int k = 1; k <= 2; k++) {
    const long long c = in(F, t.i, t.j, k), p = ph(F, t.i, t.j, k);
    const float rd = b.rdiag32[c];
    for (int r = 0; r < kR; r++)
      if (act[r]) b.p32[r][p] = fmaf(rd, b.r32[r][c], beta[r] * b.p32[r][p]);
  }
}

__global__ void k_b2_apply(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  if (!t.live) return;
  const Frame2& F = fr[t.f];
  for (int r = 0; r < kR; r++) {
    const int q = t.f * kR + r;
    if (!b.in_set[q]) continue;
    const double inv = 1.0 / b.scale[q];
    for (int k = 1; k <= 2; k++) b.phi[r][ph(F, t.i, t.j, k)] += (double)b.e32[r][in(F, t.i, t.j, k)] * inv;
  }
}

// Best-iterate bookkeeping: copy phi to phi_best (keep = 1) or back (keep = 2).
__global__ void k_b2_keep(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  if (!t.live) return;
  const Frame2& F = fr[t.f];
  for (int r = 0; r < kR; r++) {
    const int cmd = b.keep[t.f * kR + r];
    if (cmd == 0) continue;
    for (int k = 1; k <= 2; k++) {
      const long long p = ph(F, t.i, t.j, k);
      if (cmd == 1) b.phi_best[r][p] = b.phi[r][p];
      else b.phi[r][p] = b.phi_best[r][p];
    }
  }
}

// ---------------------------------------------------------------- gauge
// src/fpm_stairstep_mpi_3d.f90:170-185 per frame and direction (the
// subtraction only for the directions in the set: the others were solved on
// their own and are gauged already).
__global__ void k_b2_gauge_sum(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  const Frame2& F = fr[t.f];
  double s[3] = {0.0, 0.0, 0.0}, m[1] = {0.0};
  if (t.live) {
    const double dxi = b.dx[F.ox + t.i - 1], dyj = b.dy[F.oy + t.j - 1];
    for (int k = 1; k <= 2; k++) {
      if (b.solid3[ph(F, t.i, t.j, k)] != 0) continue;
      const long long p = ph(F, t.i, t.j, k);
      for (int r = 0; r < kR; r++) s[r] += dmul(dmul(dmul(b.phi[r][p], dxi), dyj), 0.5);
      s[2] += dmul(dmul(dxi, dyj), 0.5);
    }
  }
  double out[3];
  if (seg_reduce<3, 0>(s, m, F, t.f, b.partials, b.tickets, out, t.tile) && lin_tid() == 0)
    for (int r = 0; r < kR; r++) b.rmean[t.f * kR + r] = out[r] / out[2];
}
__global__ void k_b2_gauge_sub(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  if (!t.live) return;
  const Frame2& F = fr[t.f];
  for (int k = 1; k <= 2; k++) {
    const long long p = ph(F, t.i, t.j, k);
    if (b.solid3[p] != 0) continue;
    for (int r = 0; r < kR; r++)
      if (b.in_set[t.f * kR + r]) b.phi[r][p] = dsub(b.phi[r][p], b.rmean[t.f * kR + r]);
  }
}

// ---------------------------------------------------------------- partition
// fpm_partition_terms_2d on layer k = 1 of each direction's phi.
struct Face2 {
  int ii, jj, axis;
  double sgn, hw, len, d, fx, fy;
};
__device__ __forceinline__ Face2 face2(const Frame2& F, const Batch2& b, int i, int j, int f) {
  const double* xf = b.xf + F.ox;
  const double* yf = b.yf + F.oy;
  Face2 g;
  g.ii = i;
  g.jj = j;
  if (f == 1) { g.ii = i + 1; g.axis = 1; g.sgn = 1; }
  else if (f == 2) { g.ii = i - 1; g.axis = 1; g.sgn = -1; }
  else if (f == 3) { g.jj = j + 1; g.axis = 2; g.sgn = 1; }
  else { g.jj = j - 1; g.axis = 2; g.sgn = -1; }
  const double dxi = dsub(xf[i], xf[i - 1]), dyj = dsub(yf[j], yf[j - 1]);
  const double xci = dmul(0.5, dadd(xf[i - 1], xf[i])), ycj = dmul(0.5, dadd(yf[j - 1], yf[j]));
  if (g.axis == 1) {
    g.hw = dmul(0.5, dxi);
    g.len = dyj;
    g.fx = dadd(xci, dmul(g.sgn, g.hw));
    g.fy = ycj;
    g.d = g.hw;
    if (g.ii >= 1 && g.ii <= F.nx) g.d = fabs(dsub(dmul(0.5, dadd(xf[g.ii - 1], xf[g.ii])), xci));
  } else {
    g.hw = dmul(0.5, dyj);
    g.len = dxi;
    g.fx = xci;
    g.fy = dadd(ycj, dmul(g.sgn, g.hw));
    g.d = g.hw;
    if (g.jj >= 1 && g.jj <= F.ny) g.d = fabs(dsub(dmul(0.5, dadd(yf[g.jj - 1], yf[g.jj])), ycj));
  }
  return g;
}

__global__ void k_b2_part1(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  if (!t.live) return;
  const Frame2& F = fr[t.f];
  const int i = t.i, j = t.j;
  const long long c = c2(F, i, j);
  if (b.solid2[c]) {
    b.nxf[c] = 0;
    b.nyf[c] = 0;
    b.omega[c] = 0;
    for (int r = 0; r < kR; r++) {
      b.gpx[r][c] = 0;
      b.gpy[r][c] = 0;
    }
    return;
  }
  const double* kin = b.kin + 6 * t.f;
  double fu[4], fv[4], fp[kR][4];
  const double uc = b.u[c], vc = b.v[c];
  double pc[kR];
  for (int r = 0; r < kR; r++) pc[r] = b.phi[r][ph(F, i, j, 1)];
  for (int f = 1; f <= 4; f++) {
    const Face2 g = face2(F, b, i, j, f);
    if (g.ii < 1 || g.ii > F.nx || g.jj < 1 || g.jj > F.ny) {
      fu[f - 1] = uc;
      fv[f - 1] = vc;
      for (int r = 0; r < kR; r++) fp[r][f - 1] = 0;
    } else {
      const long long n = c2(F, g.ii, g.jj);
      if (b.solid2[n]) {
        fu[f - 1] = dsub(kin[0], dmul(kin[2], g.fy));
        fv[f - 1] = dadd(kin[1], dmul(kin[2], g.fx));
        for (int r = 0; r < kR; r++) fp[r][f - 1] = (g.axis - 1) == r ? 1.0 : 0.0;  // g = e_r
      } else {
        fu[f - 1] = dadd(uc, ddiv(dmul(dsub(b.u[n], uc), g.hw), g.d));
        fv[f - 1] = dadd(vc, ddiv(dmul(dsub(b.v[n], vc), g.hw), g.d));
        for (int r = 0; r < kR; r++)
          fp[r][f - 1] = ddiv(dmul(g.sgn, dsub(b.phi[r][ph(F, g.ii, g.jj, 1)], pc[r])), g.d);
      }
    }
  }
  const double dxi = dsub(b.xf[F.ox + i], b.xf[F.ox + i - 1]), dyj = dsub(b.yf[F.oy + j], b.yf[F.oy + j - 1]);
  b.nxf[c] = dadd(ddiv(dmul(uc, dsub(fu[0], fu[1])), dxi), ddiv(dmul(vc, dsub(fu[2], fu[3])), dyj));
  b.nyf[c] = dadd(ddiv(dmul(uc, dsub(fv[0], fv[1])), dxi), ddiv(dmul(vc, dsub(fv[2], fv[3])), dyj));
  b.omega[c] = dsub(ddiv(dsub(fv[0], fv[1]), dxi), ddiv(dsub(fu[2], fu[3]), dyj));
  for (int r = 0; r < kR; r++) {
    b.gpx[r][c] = dmul(0.5, dadd(fp[r][0], fp[r][1]));
    b.gpy[r][c] = dmul(0.5, dadd(fp[r][2], fp[r][3]));
  }
}

__global__ void k_b2_part2(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b) {
  const TileRef t = tile_ref(fr, tile_frame, b.tiles);
  const Frame2& F = fr[t.f];
  double s[8] = {0, 0, 0, 0, 0, 0, 0, 0}, m[1] = {0.0};  // [r*4 + term]
  const int i = t.i, j = t.j;
  if (t.live) {
    const long long c = c2(F, i, j);
    if (b.solid2[c]) {
      for (int r = 0; r < kR; r++) b.vif[r][c] = 0;
    } else {
      const double* kin = b.kin + 6 * t.f;
      const double k1 = kin[0], k2 = kin[1], k3 = kin[2], k4 = kin[3], k5 = kin[4], k6 = kin[5];
      const double dt = b.dt[t.f];
      const long long L = 2LL * F.nx + 2LL * F.ny;
      const double* ring = b.ring + F.oring;
      const double uc = b.u[c], vc = b.v[c];
      double pc[kR];
      for (int r = 0; r < kR; r++) pc[r] = b.phi[r][ph(F, i, j, 1)];
      double div = 0, lapu = 0, lapv = 0;
      for (int f = 1; f <= 4; f++) {
        const Face2 g = face2(F, b, i, j, f);
        if (g.ii < 1 || g.ii > F.nx || g.jj < 1 || g.jj > F.ny) {
          const double nn = g.axis == 1 ? b.nxf[c] : b.nyf[c];
          div = dadd(div, dmul(dmul(g.sgn, nn), g.len));
          long long mm;
          if (f == 2) mm = j;
          else if (f == 1) mm = (long long)F.ny + j;
          else if (f == 4) mm = 2LL * F.ny + i;
          else mm = 2LL * F.ny + F.nx + i;
          const double dudt = ddiv(dsub(ring[(mm - 1) + L * 2], ring[mm - 1]), dmul(2.0, dt));
          const double dvdt = ddiv(dsub(ring[(mm - 1) + L * 3], ring[(mm - 1) + L]), dmul(2.0, dt));
          const double x = g.axis == 1 ? dadd(dudt, b.nxf[c]) : dadd(dvdt, b.nyf[c]);
          for (int r = 0; r < kR; r++) s[r * 4 + 3] = dadd(s[r * 4 + 3], -dmul(dmul(dmul(g.sgn, x), pc[r]), g.len));
        } else {
          const long long n = c2(F, g.ii, g.jj);
          if (b.solid2[n]) {
            const double ubx = dsub(k1, dmul(k3, g.fy)), uby = dadd(k2, dmul(k3, g.fx));
            const double k33 = dmul(k3, k3);
            const double bax = dsub(dsub(k4, dmul(k6, g.fy)), dmul(k33, g.fx));
            const double bay = dsub(dadd(k5, dmul(k6, g.fx)), dmul(k33, g.fy));
            for (int r = 0; r < kR; r++) {
              const double gax = (g.axis - 1) == r ? 1.0 : 0.0;
              const double phif = dadd(pc[r], dmul(dmul(g.sgn, g.hw), gax));
              s[r * 4] = dadd(s[r * 4], -dmul(dmul(dmul(g.sgn, g.axis == 1 ? bax : bay), phif), g.len));
            }
            const double x = g.axis == 1 ? -dmul(k3, uby) : dmul(k3, ubx);
            div = dadd(div, dmul(dmul(g.sgn, x), g.len));
            lapu = dadd(lapu, dmul(ddiv(dsub(ubx, uc), g.hw), g.len));
            lapv = dadd(lapv, dmul(ddiv(dsub(uby, vc), g.hw), g.len));
          } else {
            const double x = g.axis == 1 ? dadd(b.nxf[c], ddiv(dmul(dsub(b.nxf[n], b.nxf[c]), g.hw), g.d))
                                         : dadd(b.nyf[c], ddiv(dmul(dsub(b.nyf[n], b.nyf[c]), g.hw), g.d));
            div = dadd(div, dmul(dmul(g.sgn, x), g.len));
            lapu = dadd(lapu, dmul(ddiv(dsub(b.u[n], uc), g.d), g.len));
            lapv = dadd(lapv, dmul(ddiv(dsub(b.v[n], vc), g.d), g.len));
          }
        }
      }
      const double dxi = dsub(b.xf[F.ox + i], b.xf[F.ox + i - 1]), dyj = dsub(b.yf[F.oy + j], b.yf[F.oy + j - 1]);
      for (int r = 0; r < kR; r++) {
        b.vif[r][c] = ddiv(dmul(pc[r], div), dmul(dxi, dyj));
        s[r * 4 + 1] = dadd(s[r * 4 + 1], dmul(pc[r], div));
        s[r * 4 + 2] = dadd(s[r * 4 + 2], dmul(b.nu, dadd(dmul(lapu, b.gpx[r][c]), dmul(lapv, b.gpy[r][c]))));
      }
    }
  }
  double out[8];
  if (seg_reduce<8, 0>(s, m, F, t.f, b.partials, b.tickets, out, t.tile) && lin_tid() == 0)
    for (int n = 0; n < 8; n++) b.terms[t.f * 8 + n] = out[n];
}

// ---------------------------------------------------------------- launches
#define B2_LAUNCH(kern)                                                         \
  cudaError_t launch_##kern(const Frame2* fr, const int* tf, int ntiles, const Batch2& b, cudaStream_t st) { \
    kern<<<ntiles, dim3(32, 8), 0, st>>>(fr, tf, b); note_launch();                                          \
    return cudaGetLastError();                                                                               \
  }
B2_LAUNCH(k_b2_compat)
B2_LAUNCH(k_b2_build)
B2_LAUNCH(k_b2_tres)
B2_LAUNCH(k_b2_start)
B2_LAUNCH(k_b2_apply)
B2_LAUNCH(k_b2_keep)
B2_LAUNCH(k_b2_gauge_sum)
B2_LAUNCH(k_b2_gauge_sub)
B2_LAUNCH(k_b2_part1)
B2_LAUNCH(k_b2_part2)

cudaError_t launch_b2_iteration(const Frame2* fr, const int* tf, int ntiles, const Batch2& b, cudaStream_t st) {
  k_b2_spmv<<<ntiles, dim3(32, 8), 0, st>>>(fr, tf, b); note_launch();
  k_b2_update<<<ntiles, dim3(32, 8), 0, st>>>(fr, tf, b); note_launch();
  k_b2_direction<<<ntiles, dim3(32, 8), 0, st>>>(fr, tf, b); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
