// Four-term force partition of a 2-D stair-step body, fpm_partition_terms_2d
// (src/fpm_partition_2d.f90:35-154), as two cell-parallel passes:
//   pass 1: face velocities, (u.grad)u = (nxf, nyf), vorticity, grad(phi);
//   pass 2: divergence of the face-interpolated (u.grad)u flux (F_VIF and its
//           density), the viscous term, F_KINE on body faces and F_BOUND on
//           outer faces, reduced in FP64.
// Per-cell arithmetic is the reference's, separately rounded in its order.
#include "fpm_internal.h"

namespace fpm {

struct FaceGeo {
  int ii, jj, axis;
  double sgn, hw, len, d, fx, fy;
};

// face (src/fpm_partition_2d.f90:113-130); xc/yc/dx/dy from the face arrays.
__device__ __forceinline__ FaceGeo face_geo(const Part2D& p, int i, int j, int f) {
  FaceGeo g;
  g.ii = i;
  g.jj = j;
  if (f == 1) { g.ii = i + 1; g.axis = 1; g.sgn = 1; }
  else if (f == 2) { g.ii = i - 1; g.axis = 1; g.sgn = -1; }
  else if (f == 3) { g.jj = j + 1; g.axis = 2; g.sgn = 1; }
  else { g.jj = j - 1; g.axis = 2; g.sgn = -1; }
  const double dxi = dsub(p.xf[i], p.xf[i - 1]), dyj = dsub(p.yf[j], p.yf[j - 1]);
  const double xci = dmul(0.5, dadd(p.xf[i - 1], p.xf[i])), ycj = dmul(0.5, dadd(p.yf[j - 1], p.yf[j]));
  if (g.axis == 1) {
    g.hw = dmul(0.5, dxi);
    g.len = dyj;
    g.fx = dadd(xci, dmul(g.sgn, g.hw));
    g.fy = ycj;
    g.d = g.hw;
    if (g.ii >= 1 && g.ii <= p.nx) {
      const double xcn = dmul(0.5, dadd(p.xf[g.ii - 1], p.xf[g.ii]));
      g.d = fabs(dsub(xcn, xci));
    }
  } else {
    g.hw = dmul(0.5, dyj);
    g.len = dxi;
    g.fx = xci;
    g.fy = dadd(ycj, dmul(g.sgn, g.hw));
    g.d = g.hw;
    if (g.jj >= 1 && g.jj <= p.ny) {
      const double ycn = dmul(0.5, dadd(p.yf[g.jj - 1], p.yf[g.jj]));
      g.d = fabs(dsub(ycn, ycj));
    }
  }
  return g;
}

__device__ __forceinline__ long long c2(const Part2D& p, int i, int j) {
  return (long long)(i - 1) + (long long)p.nx * (j - 1);
}

__global__ void k_partition_pass1(Part2D p, double* __restrict__ nxf, double* __restrict__ nyf,
                                  double* __restrict__ gpx, double* __restrict__ gpy, double* __restrict__ omega) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  if (i > p.nx || j > p.ny) return;
  const long long c = c2(p, i, j);
  if (p.solid[c]) {
    nxf[c] = 0;
    nyf[c] = 0;
    gpx[c] = 0;
    gpy[c] = 0;
    omega[c] = 0;
    return;
  }
  double fu[4], fv[4], fp[4];
  const double uc = p.u[c], vc = p.v[c], pc = p.phi[c];
  for (int f = 1; f <= 4; f++) {
    const FaceGeo g = face_geo(p, i, j, f);
    if (g.ii < 1 || g.ii > p.nx || g.jj < 1 || g.jj > p.ny) {
      fu[f - 1] = uc;
      fv[f - 1] = vc;
      fp[f - 1] = 0;
    } else {
      const long long n = c2(p, g.ii, g.jj);
      if (p.solid[n]) {
        if (p.slip) {
          fu[f - 1] = uc;
          fv[f - 1] = vc;
        } else {
          fu[f - 1] = dsub(p.k1, dmul(p.k3, g.fy));
          fv[f - 1] = dadd(p.k2, dmul(p.k3, g.fx));
        }
        fp[f - 1] = g.axis == 1 ? p.g0 : p.g1;
      } else {
        fu[f - 1] = dadd(uc, ddiv(dmul(dsub(p.u[n], uc), g.hw), g.d));
        fv[f - 1] = dadd(vc, ddiv(dmul(dsub(p.v[n], vc), g.hw), g.d));
        fp[f - 1] = ddiv(dmul(g.sgn, dsub(p.phi[n], pc)), g.d);
      }
    }
  }
  const double dxi = dsub(p.xf[i], p.xf[i - 1]), dyj = dsub(p.yf[j], p.yf[j - 1]);
  nxf[c] = dadd(ddiv(dmul(uc, dsub(fu[0], fu[1])), dxi), ddiv(dmul(vc, dsub(fu[2], fu[3])), dyj));
  nyf[c] = dadd(ddiv(dmul(uc, dsub(fv[0], fv[1])), dxi), ddiv(dmul(vc, dsub(fv[2], fv[3])), dyj));
  omega[c] = dsub(ddiv(dsub(fv[0], fv[1]), dxi), ddiv(dsub(fu[2], fu[3]), dyj));
  gpx[c] = dmul(0.5, dadd(fp[0], fp[1]));
  gpy[c] = dmul(0.5, dadd(fp[2], fp[3]));
}

__global__ void k_partition_pass2(Part2D p, const double* __restrict__ nxf, const double* __restrict__ nyf,
                                  const double* __restrict__ gpx, const double* __restrict__ gpy,
                                  double* __restrict__ vif, SolveScalars* S, RedBuf rb) {
  double s[4] = {0.0, 0.0, 0.0, 0.0}, m[1] = {0.0};
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const long long L = 2LL * p.nx + 2LL * p.ny;
  if (i <= p.nx && j <= p.ny) {
    const long long c = c2(p, i, j);
    if (p.solid[c]) {
      vif[c] = 0;
    } else {
      double div = 0, lapu = 0, lapv = 0;
      const double uc = p.u[c], vc = p.v[c], pc = p.phi[c];
      for (int f = 1; f <= 4; f++) {
        const FaceGeo g = face_geo(p, i, j, f);
        if (g.ii < 1 || g.ii > p.nx || g.jj < 1 || g.jj > p.ny) {
          const double nn = g.axis == 1 ? nxf[c] : nyf[c];
          div = dadd(div, dmul(dmul(g.sgn, nn), g.len));
          long long mm;
          if (f == 2) mm = j;
          else if (f == 1) mm = (long long)p.ny + j;
          else if (f == 4) mm = 2LL * p.ny + i;
          else mm = 2LL * p.ny + p.nx + i;
          const double dudt = ddiv(dsub(p.ring[(mm - 1) + L * 2], p.ring[(mm - 1)]), dmul(2.0, p.dt));
          const double dvdt = ddiv(dsub(p.ring[(mm - 1) + L * 3], p.ring[(mm - 1) + L]), dmul(2.0, p.dt));
          const double x = g.axis == 1 ? dadd(dudt, nxf[c]) : dadd(dvdt, nyf[c]);
          s[3] = dadd(s[3], -dmul(dmul(dmul(g.sgn, x), pc), g.len));
        } else {
          const long long n = c2(p, g.ii, g.jj);
          if (p.solid[n]) {
            const double ubx = dsub(p.k1, dmul(p.k3, g.fy)), uby = dadd(p.k2, dmul(p.k3, g.fx));
            const double k33 = dmul(p.k3, p.k3);
            const double bax = dsub(dsub(p.k4, dmul(p.k6, g.fy)), dmul(k33, g.fx));
            const double bay = dsub(dadd(p.k5, dmul(p.k6, g.fx)), dmul(k33, g.fy));
            const double phif = dadd(pc, dmul(dmul(g.sgn, g.hw), g.axis == 1 ? p.g0 : p.g1));
            s[0] = dadd(s[0], -dmul(dmul(dmul(g.sgn, g.axis == 1 ? bax : bay), phif), g.len));
            if (p.slip) {
              div = dadd(div, dmul(dmul(g.sgn, g.axis == 1 ? nxf[c] : nyf[c]), g.len));
            } else {
              const double x = g.axis == 1 ? -dmul(p.k3, uby) : dmul(p.k3, ubx);
              div = dadd(div, dmul(dmul(g.sgn, x), g.len));
              lapu = dadd(lapu, dmul(ddiv(dsub(ubx, uc), g.hw), g.len));
              lapv = dadd(lapv, dmul(ddiv(dsub(uby, vc), g.hw), g.len));
            }
          } else {
            const double x = g.axis == 1 ? dadd(nxf[c], ddiv(dmul(dsub(nxf[n], nxf[c]), g.hw), g.d))
                                         : dadd(nyf[c], ddiv(dmul(dsub(nyf[n], nyf[c]), g.hw), g.d));
            div = dadd(div, dmul(dmul(g.sgn, x), g.len));
            lapu = dadd(lapu, dmul(ddiv(dsub(p.u[n], uc), g.d), g.len));
            lapv = dadd(lapv, dmul(ddiv(dsub(p.v[n], vc), g.d), g.len));
          }
        }
      }
      const double dxi = dsub(p.xf[i], p.xf[i - 1]), dyj = dsub(p.yf[j], p.yf[j - 1]);
      vif[c] = ddiv(dmul(pc, div), dmul(dxi, dyj));
      s[1] = dadd(s[1], dmul(pc, div));
      s[2] = dadd(s[2], dmul(p.nu, dadd(dmul(lapu, gpx[c]), dmul(lapv, gpy[c]))));
    }
  }
  double out[4];
  if (grid_reduce<4, 0>(s, m, rb.partials, rb.ticket, out))
    if (lin_tid() == 0)
      for (int n = 0; n < 4; n++) S->red[n] = out[n];
}

cudaError_t launch_partition_2d(const Part2D& p, double* nxf, double* nyf, double* gpx, double* gpy,
                                double* vif_density, double* omega, SolveScalars* S, const RedBuf& rb,
                                cudaStream_t st) {
  dim3 block(32, 8), grid((p.nx + 31) / 32, (p.ny + 7) / 8);
  k_partition_pass1<<<grid, block, 0, st>>>(p, nxf, nyf, gpx, gpy, omega); note_launch();
  k_partition_pass2<<<grid, block, 0, st>>>(p, nxf, nyf, gpx, gpy, vif_density, S, rb); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
