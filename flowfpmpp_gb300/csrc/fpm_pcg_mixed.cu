// Mixed-precision, multi-right-hand-side stair-step PCG: the FP32 kernels.
//
// The FP64 side (true residual, projection, max-norm test, phi update) lives
// in the solver driver; these kernels run diagonally preconditioned CG in
// FP32 on A e = scale * r for up to four right-hand sides at once (phi_x,
// phi_y, phi_z share diag, rdiag, the coefficients and the cell volumes).
// Dot products are accumulated per thread as error-free f32 pairs and
// combined across the grid in FP64.
//
// FP32 vectors use the layout of MixedGrid: cell (i, j, k), i in [0, nx+1],
// j in [0, ny+1], k in [1, nz], at 3 + i + px (j + (ny+2)(k-1)) with px a
// multiple of four, so the four cells i = 4g+1 .. 4g+4 of group g start on a
// 16-byte boundary and move as one float4.  Halo and padding entries are zero
// and every kernel maps zero inputs there to zero outputs, so they stay zero.
// A thread owns one group of four cells of one (j) row and marches through a
// chunk of kc planes in k, keeping the planes k-1 and k of the search
// direction in registers (the stencil's z neighbours); x neighbours across
// groups come from the adjacent lane by shuffle.
#include <cstdlib>

#include "fpm_internal.h"

namespace fpm {

// f32 pair accumulator for dot products: a per-thread running sum carried
// with its rounding error (TwoSum), combined across the grid in FP64.
struct F2Acc {
  float s = 0.f, e = 0.f;
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = a * b;
    const float pe = fmaf(a, b, -p);
    const float t = s + p;
    const float bb = t - s;
    e += ((s - (t - bb)) + (p - bb)) + pe;
    s = t;
  }
  __device__ __forceinline__ void add(float p) {  // error-free s + p
    const float t = s + p;
    const float bb = t - s;
    e += (s - (t - bb)) + (p - bb);
    s = t;
  }
  // The four products of one float4 group are summed in FP32 (one rounding
  // each, relative 1e-7 of the group) and the group sum is added error-free.
  __device__ __forceinline__ void add4(const float4& a, const float4& b) {
    add(fmaf(a.w, b.w, fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x))));
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)e; }
};

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ void st4(float* p, const float4& v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 zero4() { return make_float4(0.f, 0.f, 0.f, 0.f); }

// Per-thread position: group g (cells 4g+1 .. 4g+4) of row j, planes k0..k1.
struct MxPos {
  int g, j, k0, k1;
  bool live;
  long long base;  // layout index of cell (4g+1, j, k0)
};
__device__ __forceinline__ MxPos mx_pos(const MixedGrid& G) {
  MxPos t;
  t.g = blockIdx.x * 32 + threadIdx.x;
  t.j = blockIdx.y * 4 + threadIdx.y + 1;
  t.live = t.g < G.ng && t.j <= G.ny;
  t.k0 = blockIdx.z * G.kc + 1;
  t.k1 = min(G.nz, t.k0 + G.kc - 1);
  t.base = 4LL * (t.g + 1) + (long long)G.px * (t.j + (long long)(G.ny + 2) * (t.k0 - 1));
  return t;
}

// FP64 operator arrays (compact (nx, ny, nz)) into the FP32 layout.
__global__ void k_mx_layout(MixedGrid G, const double* __restrict__ a, float* __restrict__ b) {
  const MxPos t = mx_pos(G);
  if (!t.live) return;
  long long base = t.base;
  for (int k = t.k0; k <= t.k1; k++, base += G.plane) {
    float4 v;
    float* vv = &v.x;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int i = 4 * t.g + 1 + c;
      vv[c] = i <= G.nx ? (float)a[(i - 1) + (long long)G.nx * ((t.j - 1) + (long long)G.ny * (k - 1))] : 0.f;
    }
    st4(b + base, v);
  }
}

// wall = sum of the coefficients of the faces towards solid neighbours inside
// the grid (exactly 0 for a cell with only fluid neighbours), -1 in solid
// cells.  With it the stencil is evaluated in difference form,
// V (sum_nb c (p - p_nb) - wall p), which equals V (diag p - sum_nb c p_nb)
// (solid neighbours hold p = 0) but keeps FP32 rounding relative to the
// result instead of to the diagonal term when p is smooth.
__global__ void k_mx_wall(MixedGrid G, Dims d, const int32_t* __restrict__ solid, Coefs cf, float* __restrict__ w) {
  const MxPos t = mx_pos(G);
  if (!t.live) return;
  long long base = t.base;
  for (int k = t.k0; k <= t.k1; k++, base += G.plane) {
    float4 v;
    float* vv = &v.x;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int i = 4 * t.g + 1 + c, j = t.j;
      float x = 0.f;
      if (i <= G.nx) {
        if (solid[d.ph(i, j, k)] != 0) {
          x = -1.f;
        } else {
          double s = 0.0;
          if (solid[d.ph(i - 1, j, k)] != 0) s += cf.cw[i - 1];
          if (solid[d.ph(i + 1, j, k)] != 0) s += cf.ce[i - 1];
          if (solid[d.ph(i, j - 1, k)] != 0) s += cf.cs[j - 1];
          if (solid[d.ph(i, j + 1, k)] != 0) s += cf.cn[j - 1];
          if (k > 1 && solid[d.ph(i, j, k - 1)] != 0) s += cf.cb[k - 1];
          if (k < G.nz && solid[d.ph(i, j, k + 1)] != 0) s += cf.ct[k - 1];
          x = (float)s;
        }
      }
      vv[c] = x;
    }
    st4(w + base, v);
  }
}

// One FP64 x-axis array a(1:n) into the row layout b(3 + i), zero elsewhere.
__global__ void k_mx_row(int n, int len, const double* __restrict__ a, float* __restrict__ b) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < len; m += gridDim.x * blockDim.x) {
    const int i = m - 3;
    b[m] = (i >= 1 && i <= n) ? (float)a[i - 1] : 0.f;
  }
}
__global__ void k_mx_convert(long long n, const double* __restrict__ a, float* __restrict__ b) {
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x)
    b[m] = (float)a[m];
}

// Residual replacement for the right-hand sides in the set: r = scale * rV
// (the projected FP64 true residual, compact layout), e = 0, and either a
// restart from the steepest-descent direction p = rdiag r (pmul == 0) or the
// current direction rescaled to the new residual scale (p *= pmul);
// rz = r.(rdiag r).
__global__ void __launch_bounds__(128) k_mx_start(MixedGrid G, MixedVecs v, DPtr4 rv64, MixedScale sc,
                                                  MixedScalars* S, RedBuf rb) {
  F2Acc acc[kMaxRhs];
  const MxPos t = mx_pos(G);
  if (t.live) {
    long long base = t.base;
    for (int k = t.k0; k <= t.k1; k++, base += G.plane) {
      const float4 rd = ld4(v.rdiag + base);
      const long long c0 = (long long)G.nx * ((t.j - 1) + (long long)G.ny * (k - 1)) + 4 * t.g;
#pragma unroll
      for (int m = 0; m < kMaxRhs; m++) {
        if (!(m < v.nrhs && sc.in_set[m])) continue;
        float4 r;
        float* rr = &r.x;
#pragma unroll
        for (int c = 0; c < 4; c++) rr[c] = 4 * t.g + 1 + c <= G.nx ? (float)(rv64.p[m][c0 + c] * sc.scale[m]) : 0.f;
        const float4 z = make_float4(rd.x * r.x, rd.y * r.y, rd.z * r.z, rd.w * r.w);
        st4(v.r[m] + base, r);
        const float pm = (float)sc.pmul[m];
        float4 p;
        if (pm == 0.f) {
          p = z;
        } else {
          p = ld4(v.p[m] + base);
          p = make_float4(p.x * pm, p.y * pm, p.z * pm, p.w * pm);
        }
        st4(v.p[m] + base, p);
        st4(v.e[m] + base, zero4());
        acc[m].add4(z, r);
      }
    }
  }
  double s[kMaxRhs], mm[1] = {0.0}, out[kMaxRhs];
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) s[m] = acc[m].value();
  if (grid_reduce<kMaxRhs, 0>(s, mm, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      for (int m = 0; m < kMaxRhs; m++) {
        if (!(m < v.nrhs && sc.in_set[m])) continue;
        S->rz[m] = out[m];
        S->rz0[m] = out[m];
        S->active[m] = out[m] > 0 ? 1 : 0;
      }
    }
  }
}

// q = V (sum_nb c (p - p_nb) - wall p) on fluid cells (the difference form of
// V (diag p - sum c p_nb)), pq = p.q, alpha = rz / pq.
template <int NR>
__global__ void __launch_bounds__(128, 4) k_mx_spmv(MixedGrid G, MixedVecs v, MixedScalars* S, RedBuf rb) {
  int act[kMaxRhs];
  bool any = false;
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) {
    act[m] = m < v.nrhs ? S->active[m] : 0;
    any = any || act[m];
  }
  if (!any) return;
  F2Acc acc[NR];
  const MxPos t = mx_pos(G);
  const int lane = threadIdx.x;
  const bool fetch_right = t.live && (lane == 31 || t.g + 1 >= G.ng);
  float4 cw = zero4(), ce = zero4(), dx = zero4();
  float cs = 0.f, cn = 0.f, dy = 0.f;
  if (t.live) {
    const int o = 4 * (t.g + 1);
    cw = ld4(v.cw + o);
    ce = ld4(v.ce + o);
    dx = ld4(v.dx + o);
    cs = v.cs[t.j - 1];
    cn = v.cn[t.j - 1];
    dy = v.dy[t.j - 1];
  }
  const long long px = G.px, pl = G.plane;
  float4 pb[NR], pc[NR];
#pragma unroll
  for (int m = 0; m < NR; m++) {
    pb[m] = pc[m] = zero4();
    if (act[m] && t.live) {
      pc[m] = ld4(v.p[m] + t.base);
      pb[m] = t.k0 > 1 ? ld4(v.p[m] + t.base - pl) : pc[m];
    }
  }
  long long base = t.base;
  for (int k = t.k0; k <= t.k1; k++, base += pl) {
    const float cb = __ldg(v.cb + k - 1), ct = __ldg(v.ct + k - 1), dz = __ldg(v.dz + k - 1);
    // Phase 1: every load of this plane (read-only path, no aliasing with the
    // q stores below), so they are all in flight together.
    float4 dg = make_float4(-1.f, -1.f, -1.f, -1.f), pt[NR], ps[NR], pn[NR];
    float lft[NR], rgt[NR];
    if (t.live) dg = ldg4(v.wall + base);
#pragma unroll
    for (int m = 0; m < NR; m++) {
      pt[m] = pc[m];
      ps[m] = pn[m] = zero4();
      lft[m] = rgt[m] = 0.f;
      if (act[m] && t.live) {
        const float* p = v.p[m];
        if (k < G.nz) pt[m] = ldg4(p + base + pl);
        ps[m] = ldg4(p + base - px);
        pn[m] = ldg4(p + base + px);
        if (lane == 0) lft[m] = __ldg(p + base - 1);
        if (fetch_right) rgt[m] = __ldg(p + base + 4);
      }
    }
    const float4 vol = make_float4(dx.x * dy * dz, dx.y * dy * dz, dx.z * dy * dz, dx.w * dy * dz);
    // Phase 2: x neighbours across lanes, the stencil, stores and dots.
#pragma unroll
    for (int m = 0; m < NR; m++) {
      if (!act[m]) continue;
      float left = __shfl_up_sync(0xffffffffu, pc[m].w, 1);
      float right = __shfl_down_sync(0xffffffffu, pc[m].x, 1);
      if (lane == 0) left = lft[m];
      if (fetch_right) right = rgt[m];
      const float4 c = pc[m], b = pb[m];
      const float pw[4] = {left, c.x, c.y, c.z}, pe[4] = {c.y, c.z, c.w, right};
      const float pcv[4] = {c.x, c.y, c.z, c.w}, psv[4] = {ps[m].x, ps[m].y, ps[m].z, ps[m].w},
                  pnv[4] = {pn[m].x, pn[m].y, pn[m].z, pn[m].w}, pbv[4] = {b.x, b.y, b.z, b.w},
                  ptv[4] = {pt[m].x, pt[m].y, pt[m].z, pt[m].w}, dgv[4] = {dg.x, dg.y, dg.z, dg.w},
                  cwv[4] = {cw.x, cw.y, cw.z, cw.w}, cev[4] = {ce.x, ce.y, ce.z, ce.w},
                  vv[4] = {vol.x, vol.y, vol.z, vol.w};
      float q[4];
#pragma unroll
      for (int n = 0; n < 4; n++) {
        const float x = pcv[n];
        float u = -dgv[n] * x;
        u = fmaf(cwv[n], x - pw[n], u);
        u = fmaf(cev[n], x - pe[n], u);
        u = fmaf(cs, x - psv[n], u);
        u = fmaf(cn, x - pnv[n], u);
        u = fmaf(cb, x - pbv[n], u);
        u = fmaf(ct, x - ptv[n], u);
        q[n] = dgv[n] >= 0.f ? vv[n] * u : 0.f;
      }
      const float4 q4 = make_float4(q[0], q[1], q[2], q[3]);
      if (t.live) {
        st4(v.q[m] + base, q4);
        acc[m].add4(c, q4);
      }
      pb[m] = c;
      pc[m] = pt[m];
    }
  }
  double s[kMaxRhs], mm[1] = {0.0}, out[kMaxRhs];
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) s[m] = m < NR ? acc[m < NR ? m : 0].value() : 0.0;
  if (grid_reduce<kMaxRhs, 0>(s, mm, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      for (int m = 0; m < kMaxRhs; m++) {
        if (!act[m]) continue;
        S->pq[m] = out[m];
        if (!(out[m] > 0) || !(S->rz[m] > 0)) {  // breakdown: stop this right-hand side's inner solve
          S->active[m] = 0;
          S->alpha[m] = 0;
        } else {
          S->alpha[m] = S->rz[m] / out[m];
        }
      }
    }
  }
}

// The same product, one right-hand side at a time: each thread marches its
// planes once per right-hand side, so it holds a third of the state and the
// SM runs twice the warps (the wall and coefficients come from L1 after the
// first pass).
template <int NR>
__global__ void __launch_bounds__(128, 8) k_mx_spmv_seq(MixedGrid G, MixedVecs v, MixedScalars* S, RedBuf rb) {
  int act[kMaxRhs];
  bool any = false;
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) {
    act[m] = m < v.nrhs ? S->active[m] : 0;
    any = any || act[m];
  }
  if (!any) return;
  F2Acc acc[NR];
  const MxPos t = mx_pos(G);
  const int lane = threadIdx.x;
  const bool fetch_right = t.live && (lane == 31 || t.g + 1 >= G.ng);
  const long long px = G.px, pl = G.plane;
#pragma unroll 1
  for (int m = 0; m < NR; m++) {
    if (!act[m]) continue;
    const float* p = v.p[m];
    float4 cw = zero4(), ce = zero4(), dx = zero4(), pb = zero4(), pc = zero4();
    float cs = 0.f, cn = 0.f, dy = 0.f;
    if (t.live) {
      const int o = 4 * (t.g + 1);
      cw = ldg4(v.cw + o);
      ce = ldg4(v.ce + o);
      dx = ldg4(v.dx + o);
      cs = __ldg(v.cs + t.j - 1);
      cn = __ldg(v.cn + t.j - 1);
      dy = __ldg(v.dy + t.j - 1);
      pc = ldg4(p + t.base);
      pb = t.k0 > 1 ? ldg4(p + t.base - pl) : pc;
    }
    long long base = t.base;
    for (int k = t.k0; k <= t.k1; k++, base += pl) {
      const float cb = __ldg(v.cb + k - 1), ct = __ldg(v.ct + k - 1), dz = __ldg(v.dz + k - 1);
      float4 dg = make_float4(-1.f, -1.f, -1.f, -1.f), pt = pc, ps = zero4(), pn = zero4();
      float lft = 0.f, rgt = 0.f;
      if (t.live) {
        dg = ldg4(v.wall + base);
        if (k < G.nz) pt = ldg4(p + base + pl);
        ps = ldg4(p + base - px);
        pn = ldg4(p + base + px);
        if (lane == 0) lft = __ldg(p + base - 1);
        if (fetch_right) rgt = __ldg(p + base + 4);
      }
      float left = __shfl_up_sync(0xffffffffu, pc.w, 1);
      float right = __shfl_down_sync(0xffffffffu, pc.x, 1);
      if (lane == 0) left = lft;
      if (fetch_right) right = rgt;
      const float dyz = dy * dz;
      const float pw[4] = {left, pc.x, pc.y, pc.z}, pe[4] = {pc.y, pc.z, pc.w, right};
      const float pcv[4] = {pc.x, pc.y, pc.z, pc.w}, psv[4] = {ps.x, ps.y, ps.z, ps.w},
                  pnv[4] = {pn.x, pn.y, pn.z, pn.w}, pbv[4] = {pb.x, pb.y, pb.z, pb.w},
                  ptv[4] = {pt.x, pt.y, pt.z, pt.w}, dgv[4] = {dg.x, dg.y, dg.z, dg.w},
                  cwv[4] = {cw.x, cw.y, cw.z, cw.w}, cev[4] = {ce.x, ce.y, ce.z, ce.w},
                  dxv[4] = {dx.x, dx.y, dx.z, dx.w};
      float q[4];
#pragma unroll
      for (int n = 0; n < 4; n++) {
        const float x = pcv[n];
        float u = -dgv[n] * x;
        u = fmaf(cwv[n], x - pw[n], u);
        u = fmaf(cev[n], x - pe[n], u);
        u = fmaf(cs, x - psv[n], u);
        u = fmaf(cn, x - pnv[n], u);
        u = fmaf(cb, x - pbv[n], u);
        u = fmaf(ct, x - ptv[n], u);
        q[n] = dgv[n] >= 0.f ? (dxv[n] * dyz) * u : 0.f;
      }
      const float4 q4 = make_float4(q[0], q[1], q[2], q[3]);
      if (t.live) {
        st4(v.q[m] + base, q4);
        acc[m].add4(pc, q4);
      }
      pb = pc;
      pc = pt;
    }
  }
  double s[kMaxRhs], mm[1] = {0.0}, out[kMaxRhs];
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) s[m] = m < NR ? acc[m < NR ? m : 0].value() : 0.0;
  if (grid_reduce<kMaxRhs, 0>(s, mm, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      for (int m = 0; m < kMaxRhs; m++) {
        if (!act[m]) continue;
        S->pq[m] = out[m];
        if (!(out[m] > 0) || !(S->rz[m] > 0)) {
          S->active[m] = 0;
          S->alpha[m] = 0;
        } else {
          S->alpha[m] = S->rz[m] / out[m];
        }
      }
    }
  }
}

// e += alpha p; r -= alpha q; rz_new = r.(rdiag r); beta = rz_new / rz.
template <int NR>
__global__ void __launch_bounds__(128) k_mx_update(MixedGrid G, MixedVecs v, MixedScalars* S, RedBuf rb) {
  int act[kMaxRhs];
  float alpha[kMaxRhs];
  bool any = false;
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) {
    act[m] = m < v.nrhs ? S->active[m] : 0;
    alpha[m] = (float)S->alpha[m];
    any = any || act[m];
  }
  if (!any) {
    if (lin_bid() == 0 && lin_tid() == 0)
      for (int m = 0; m < kMaxRhs; m++) S->dir[m] = 0;
    return;
  }
  F2Acc acc[NR];
  const MxPos t = mx_pos(G);
  if (t.live) {
    long long base = t.base;
    for (int k = t.k0; k <= t.k1; k++, base += G.plane) {
      const float4 rd = ldg4(v.rdiag + base);
      float4 pp[NR], qq[NR], ee[NR], rr[NR];
#pragma unroll
      for (int m = 0; m < NR; m++) {
        if (!act[m]) continue;
        pp[m] = ldg4(v.p[m] + base);
        qq[m] = ldg4(v.q[m] + base);
        ee[m] = ld4(v.e[m] + base);
        rr[m] = ld4(v.r[m] + base);
      }
#pragma unroll
      for (int m = 0; m < NR; m++) {
        if (!act[m]) continue;
        const float a = alpha[m];
        const float4 p = pp[m], q = qq[m];
        float4 e = ee[m], r = rr[m];
        e = make_float4(fmaf(a, p.x, e.x), fmaf(a, p.y, e.y), fmaf(a, p.z, e.z), fmaf(a, p.w, e.w));
        r = make_float4(fmaf(-a, q.x, r.x), fmaf(-a, q.y, r.y), fmaf(-a, q.z, r.z), fmaf(-a, q.w, r.w));
        st4(v.e[m] + base, e);
        st4(v.r[m] + base, r);
        acc[m].add4(make_float4(rd.x * r.x, rd.y * r.y, rd.z * r.z, rd.w * r.w), r);
      }
    }
  }
  double s[kMaxRhs], mm[1] = {0.0}, out[kMaxRhs];
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) s[m] = m < NR ? acc[m < NR ? m : 0].value() : 0.0;
  if (grid_reduce<kMaxRhs, 0>(s, mm, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      for (int m = 0; m < kMaxRhs; m++) {
        if (!act[m]) {
          S->dir[m] = 0;
          continue;
        }
        const double rz_new = out[m];
        if (!(rz_new >= 0)) {
          S->active[m] = 0;
          S->dir[m] = 0;
          continue;
        }
        S->beta[m] = rz_new / S->rz[m];
        S->rz[m] = rz_new;
        S->dir[m] = 1;  // the direction update of this iteration still runs
        if (rz_new <= S->tol2[m] * S->rz0[m]) S->active[m] = 0;
      }
    }
  }
}

// p = rdiag r + beta p for the right-hand sides still iterating.
template <int NR>
__global__ void __launch_bounds__(128) k_mx_direction(MixedGrid G, MixedVecs v, MixedScalars* S) {
  int act[kMaxRhs];
  float beta[kMaxRhs];
  bool any = false;
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) {
    act[m] = m < v.nrhs ? S->dir[m] : 0;
    beta[m] = (float)S->beta[m];
    any = any || act[m];
  }
  if (!any) return;
  const MxPos t = mx_pos(G);
  if (t.live) {
    long long base = t.base;
    for (int k = t.k0; k <= t.k1; k++, base += G.plane) {
      const float4 rd = ldg4(v.rdiag + base);
      float4 rr[NR], pp[NR];
#pragma unroll
      for (int m = 0; m < NR; m++) {
        if (!act[m]) continue;
        rr[m] = ldg4(v.r[m] + base);
        pp[m] = ld4(v.p[m] + base);
      }
#pragma unroll
      for (int m = 0; m < NR; m++) {
        if (!act[m]) continue;
        const float b = beta[m];
        const float4 r = rr[m], p = pp[m];
        st4(v.p[m] + base, make_float4(fmaf(rd.x, r.x, b * p.x), fmaf(rd.y, r.y, b * p.y),
                                       fmaf(rd.z, r.z, b * p.z), fmaf(rd.w, r.w, b * p.w)));
      }
    }
  }
  if (lin_bid() == 0 && lin_tid() == 0) S->iters += 1;
}

// phi += e / scale (FP64, padded (0:nx+1, 0:ny+1, nz)) for the set.
__global__ void __launch_bounds__(128) k_mx_apply(MixedGrid G, MixedVecs v, DPtr4 phi, MixedScale sc) {
  const MxPos t = mx_pos(G);
  if (!t.live) return;
  long long base = t.base;
  for (int k = t.k0; k <= t.k1; k++, base += G.plane) {
    const long long p0 = 4LL * t.g + 1 + (long long)(G.nx + 2) * (t.j + (long long)(G.ny + 2) * (k - 1));
#pragma unroll
    for (int m = 0; m < kMaxRhs; m++) {
      if (!(m < v.nrhs && sc.in_set[m])) continue;
      const float4 e = ld4(v.e[m] + base);
      const float ev[4] = {e.x, e.y, e.z, e.w};
#pragma unroll
      for (int c = 0; c < 4; c++)
        if (4 * t.g + 1 + c <= G.nx) phi.p[m][p0 + c] += (double)ev[c] / sc.scale[m];
    }
  }
}

static dim3 mx_grid(const MixedGrid& G) {
  return dim3((unsigned)((G.ng + 31) / 32), (unsigned)((G.ny + 3) / 4), (unsigned)((G.nz + G.kc - 1) / G.kc));
}

MixedGrid mixed_grid(int nx, int ny, int nz, int kc) {
  MixedGrid G;
  G.nx = nx;
  G.ny = ny;
  G.nz = nz;
  G.px = ((nx + 5) + 3) / 4 * 4;
  G.ng = (nx + 3) / 4;
  G.kc = kc < 1 ? 1 : kc;
  G.plane = (long long)G.px * (ny + 2);
  G.size = G.plane * nz + G.px;
  const dim3 g = mx_grid(G);
  G.nblocks = (int)(g.x * g.y * g.z);
  return G;
}

cudaError_t launch_mx_layout(const MixedGrid& G, const double* a, float* b, cudaStream_t st) {
  k_mx_layout<<<mx_grid(G), dim3(32, 4), 0, st>>>(G, a, b); note_launch();
  return cudaGetLastError();
}
cudaError_t launch_mx_wall(const MixedGrid& G, const Dims& d, const int32_t* solid, const Coefs& c, float* wall,
                           cudaStream_t st) {
  k_mx_wall<<<mx_grid(G), dim3(32, 4), 0, st>>>(G, d, solid, c, wall); note_launch();
  return cudaGetLastError();
}
cudaError_t launch_mx_row(int n, int len, const double* a, float* b, cudaStream_t st) {
  k_mx_row<<<(len + 255) / 256, 256, 0, st>>>(n, len, a, b); note_launch();
  return cudaGetLastError();
}
cudaError_t launch_mx_convert(const double* a, float* b, long long n, cudaStream_t st) {
  long long nb = (n + 255) / 256;
  if (nb > 152LL * 32) nb = 152LL * 32;
  if (nb < 1) nb = 1;
  k_mx_convert<<<(unsigned)nb, 256, 0, st>>>(n, a, b); note_launch();
  return cudaGetLastError();
}
cudaError_t launch_mx_start(const MixedGrid& G, const MixedVecs& v, const DPtr4& rv64, const MixedScale& sc,
                            MixedScalars* S, const RedBuf& rb, cudaStream_t st) {
  k_mx_start<<<mx_grid(G), dim3(32, 4), 0, st>>>(G, v, rv64, sc, S, rb); note_launch();
  return cudaGetLastError();
}
cudaError_t launch_mx_iteration(const MixedGrid& G, const MixedVecs& v, MixedScalars* S, const RedBuf& rb,
                                cudaStream_t st) {
  const dim3 g = mx_grid(G), b(32, 4);
  static const int seq = [] {
    const char* e = std::getenv("FPM_MIXED_SPMV");
    return (e && e[0] == '1') ? 1 : 0;
  }();
  if (seq) {
    switch (v.nrhs) {
      case 1: k_mx_spmv_seq<1><<<g, b, 0, st>>>(G, v, S, rb); break;
      case 2: k_mx_spmv_seq<2><<<g, b, 0, st>>>(G, v, S, rb); break;
      case 3: k_mx_spmv_seq<3><<<g, b, 0, st>>>(G, v, S, rb); break;
      default: k_mx_spmv_seq<4><<<g, b, 0, st>>>(G, v, S, rb); break;
    }
  } else {
    switch (v.nrhs) {
      case 1: k_mx_spmv<1><<<g, b, 0, st>>>(G, v, S, rb); break;
      case 2: k_mx_spmv<2><<<g, b, 0, st>>>(G, v, S, rb); break;
      case 3: k_mx_spmv<3><<<g, b, 0, st>>>(G, v, S, rb); break;
      default: k_mx_spmv<4><<<g, b, 0, st>>>(G, v, S, rb); break;
    }
  }
  note_launch();
  switch (v.nrhs) {
    case 1: k_mx_update<1><<<g, b, 0, st>>>(G, v, S, rb); k_mx_direction<1><<<g, b, 0, st>>>(G, v, S); break;
    case 2: k_mx_update<2><<<g, b, 0, st>>>(G, v, S, rb); k_mx_direction<2><<<g, b, 0, st>>>(G, v, S); break;
    case 3: k_mx_update<3><<<g, b, 0, st>>>(G, v, S, rb); k_mx_direction<3><<<g, b, 0, st>>>(G, v, S); break;
    default: k_mx_update<4><<<g, b, 0, st>>>(G, v, S, rb); k_mx_direction<4><<<g, b, 0, st>>>(G, v, S); break;
  }
  note_launch();
  note_launch();
  return cudaGetLastError();
}
cudaError_t launch_mx_apply(const MixedGrid& G, const MixedVecs& v, const DPtr4& phi, const MixedScale& sc,
                            cudaStream_t st) {
  k_mx_apply<<<mx_grid(G), dim3(32, 4), 0, st>>>(G, v, phi, sc); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
