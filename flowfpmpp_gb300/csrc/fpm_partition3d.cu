// Four-term force partition of a 3-D stair-step body.  The reference gives
// the divergence-form partition in 2-D only (fpm_partition_terms_2d,
// src/fpm_partition_2d.f90:35-154); this is the same face-flux scheme on the
// six faces of a cell:
//   pass 1: face velocities (outer: the cell's own; body: rigid-body velocity
//           U_B = V + W x r, or the cell's own with slip; interior: linear
//           interpolation), (u.grad)u = N, vorticity, grad(phi);
//   pass 2: F_VIF = sum phi div(N) with N interpolated to the faces (body
//           faces: W x U_B), F_VIS = nu sum lap(u).grad(phi) (no-slip body
//           flux), F_KINE on body faces with phi extrapolated by the body
//           gradient, F_BOUND on outer faces from Du/Dt = du/dt + N.
// Per-cell arithmetic is separately rounded in the oracle's order.
#include "fpm_internal.h"

namespace fpm {

struct Face3 {
  int ii, jj, kk, axis;
  double sgn, hw, area, d, fx, fy, fz;
};

__device__ __forceinline__ long long c3(const Part3D& p, int i, int j, int k) {
  return (long long)(i - 1) + (long long)p.nx * ((long long)(j - 1) + (long long)p.ny * (k - 1));
}

__device__ __forceinline__ Face3 face3(const Part3D& p, int i, int j, int k, int f) {
  Face3 g;
  g.ii = i;
  g.jj = j;
  g.kk = k;
  g.sgn = (f % 2 == 1) ? 1.0 : -1.0;
  const double dxi = dsub(p.xf[i], p.xf[i - 1]), dyj = dsub(p.yf[j], p.yf[j - 1]), dzk = dsub(p.zf[k], p.zf[k - 1]);
  const double xc = dmul(0.5, dadd(p.xf[i - 1], p.xf[i])), yc = dmul(0.5, dadd(p.yf[j - 1], p.yf[j])),
               zc = dmul(0.5, dadd(p.zf[k - 1], p.zf[k]));
  g.fx = xc;
  g.fy = yc;
  g.fz = zc;
  if (f <= 2) {
    g.axis = 0;
    g.ii = i + (int)g.sgn;
    g.hw = dmul(0.5, dxi);
    g.area = dmul(dyj, dzk);
    g.fx = dadd(xc, dmul(g.sgn, g.hw));
    g.d = g.hw;
    if (g.ii >= 1 && g.ii <= p.nx) g.d = fabs(dsub(dmul(0.5, dadd(p.xf[g.ii - 1], p.xf[g.ii])), xc));
  } else if (f <= 4) {
    g.axis = 1;
    g.jj = j + (int)g.sgn;
    g.hw = dmul(0.5, dyj);
    g.area = dmul(dxi, dzk);
    g.fy = dadd(yc, dmul(g.sgn, g.hw));
    g.d = g.hw;
    if (g.jj >= 1 && g.jj <= p.ny) g.d = fabs(dsub(dmul(0.5, dadd(p.yf[g.jj - 1], p.yf[g.jj])), yc));
  } else {
    g.axis = 2;
    g.kk = k + (int)g.sgn;
    g.hw = dmul(0.5, dzk);
    g.area = dmul(dxi, dyj);
    g.fz = dadd(zc, dmul(g.sgn, g.hw));
    g.d = g.hw;
    if (g.kk >= 1 && g.kk <= p.nz) g.d = fabs(dsub(dmul(0.5, dadd(p.zf[g.kk - 1], p.zf[g.kk])), zc));
  }
  return g;
}

__device__ __forceinline__ bool outer3(const Part3D& p, const Face3& g) {
  return g.ii < 1 || g.ii > p.nx || g.jj < 1 || g.jj > p.ny || g.kk < 1 || g.kk > p.nz;
}

// Rigid-body velocity V + W x r at a face centre.
__device__ __forceinline__ void body_vel(const Part3D& p, const Face3& g, double ub[3]) {
  const double* k = p.kin;
  ub[0] = dadd(k[0], dsub(dmul(k[4], g.fz), dmul(k[5], g.fy)));
  ub[1] = dadd(k[1], dsub(dmul(k[5], g.fx), dmul(k[3], g.fz)));
  ub[2] = dadd(k[2], dsub(dmul(k[3], g.fy), dmul(k[4], g.fx)));
}

#define P3_CELL                                        \
  const int i = blockIdx.x * 32 + threadIdx.x + 1;     \
  const int j = blockIdx.y * 8 + threadIdx.y + 1;      \
  const int k = blockIdx.z + 1;                        \
  const bool live = i <= p.nx && j <= p.ny && k <= p.nz;

__global__ void k_part3_pass1(Part3D p, double* __restrict__ N0, double* __restrict__ N1, double* __restrict__ N2,
                              double* __restrict__ gp0, double* __restrict__ gp1, double* __restrict__ gp2,
                              double* __restrict__ omega) {
  P3_CELL
  if (!live) return;
  const long long c = c3(p, i, j, k), n3 = (long long)p.nx * p.ny * p.nz;
  double* N[3] = {N0, N1, N2};
  double* gp[3] = {gp0, gp1, gp2};
  if (p.solid[c]) {
    for (int a = 0; a < 3; a++) {
      N[a][c] = 0;
      gp[a][c] = 0;
      if (omega) omega[a * n3 + c] = 0;
    }
    return;
  }
  const double* vel[3] = {p.u, p.v, p.w};
  double fv[3][6], fp[6];
  for (int f = 1; f <= 6; f++) {
    const Face3 g = face3(p, i, j, k, f);
    if (outer3(p, g)) {
      for (int a = 0; a < 3; a++) fv[a][f - 1] = vel[a][c];
      fp[f - 1] = 0;
    } else {
      const long long c2 = c3(p, g.ii, g.jj, g.kk);
      if (p.solid[c2]) {
        double ub[3];
        body_vel(p, g, ub);
        for (int a = 0; a < 3; a++) fv[a][f - 1] = p.slip ? vel[a][c] : ub[a];
        fp[f - 1] = p.g[g.axis];
      } else {
        for (int a = 0; a < 3; a++)
          fv[a][f - 1] = dadd(vel[a][c], ddiv(dmul(dsub(vel[a][c2], vel[a][c]), g.hw), g.d));
        fp[f - 1] = ddiv(dmul(g.sgn, dsub(p.phi[c2], p.phi[c])), g.d);
      }
    }
  }
  const double dxi = dsub(p.xf[i], p.xf[i - 1]), dyj = dsub(p.yf[j], p.yf[j - 1]), dzk = dsub(p.zf[k], p.zf[k - 1]);
  for (int a = 0; a < 3; a++)
    N[a][c] = dadd(dadd(ddiv(dmul(p.u[c], dsub(fv[a][0], fv[a][1])), dxi), ddiv(dmul(p.v[c], dsub(fv[a][2], fv[a][3])), dyj)),
                   ddiv(dmul(p.w[c], dsub(fv[a][4], fv[a][5])), dzk));
  if (omega) {
    omega[c] = dsub(ddiv(dsub(fv[2][2], fv[2][3]), dyj), ddiv(dsub(fv[1][4], fv[1][5]), dzk));
    omega[n3 + c] = dsub(ddiv(dsub(fv[0][4], fv[0][5]), dzk), ddiv(dsub(fv[2][0], fv[2][1]), dxi));
    omega[2 * n3 + c] = dsub(ddiv(dsub(fv[1][0], fv[1][1]), dxi), ddiv(dsub(fv[0][2], fv[0][3]), dyj));
  }
  gp0[c] = dmul(0.5, dadd(fp[0], fp[1]));
  gp1[c] = dmul(0.5, dadd(fp[2], fp[3]));
  gp2[c] = dmul(0.5, dadd(fp[4], fp[5]));
}

__global__ void k_part3_pass2(Part3D p, const double* __restrict__ N0, const double* __restrict__ N1,
                              const double* __restrict__ N2, const double* __restrict__ gp0,
                              const double* __restrict__ gp1, const double* __restrict__ gp2,
                              double* __restrict__ vif, SolveScalars* S, RedBuf rb) {
  P3_CELL
  double s[4] = {0.0, 0.0, 0.0, 0.0}, m[1] = {0.0};
  if (live) {
    const long long c = c3(p, i, j, k);
    if (p.solid[c]) {
      vif[c] = 0;
    } else {
      const double* N[3] = {N0, N1, N2};
      const double* vel[3] = {p.u, p.v, p.w};
      const double* kin = p.kin;
      const long long L = 2LL * p.ny * p.nz + 2LL * p.nx * p.nz + 2LL * p.nx * p.ny;
      const double pc = p.phi[c];
      double div = 0, lap[3] = {0, 0, 0};
      for (int f = 1; f <= 6; f++) {
        const Face3 g = face3(p, i, j, k, f);
        const int ax = g.axis;
        if (outer3(p, g)) {
          div = dadd(div, dmul(dmul(g.sgn, N[ax][c]), g.area));
          double dudt = 0;
          if (p.shell) {
            long long mm;
            const long long nyz = (long long)p.ny * p.nz, nxz = (long long)p.nx * p.nz, nxy = (long long)p.nx * p.ny;
            if (f == 2) mm = (j - 1) + (long long)p.ny * (k - 1);
            else if (f == 1) mm = nyz + (j - 1) + (long long)p.ny * (k - 1);
            else if (f == 4) mm = 2 * nyz + (i - 1) + (long long)p.nx * (k - 1);
            else if (f == 3) mm = 2 * nyz + nxz + (i - 1) + (long long)p.nx * (k - 1);
            else if (f == 6) mm = 2 * nyz + 2 * nxz + (i - 1) + (long long)p.nx * (j - 1);
            else mm = 2 * nyz + 2 * nxz + nxy + (i - 1) + (long long)p.nx * (j - 1);
            dudt = ddiv(dsub(p.shell[mm + L * (ax + 3)], p.shell[mm + L * ax]), dmul(2.0, p.dt));
          }
          s[3] = dsub(s[3], dmul(dmul(dmul(g.sgn, dadd(dudt, N[ax][c])), pc), g.area));
        } else {
          const long long c2 = c3(p, g.ii, g.jj, g.kk);
          if (p.solid[c2]) {
            double ub[3];
            body_vel(p, g, ub);
            const double wr[3] = {dsub(dmul(kin[4], g.fz), dmul(kin[5], g.fy)), dsub(dmul(kin[5], g.fx), dmul(kin[3], g.fz)),
                                  dsub(dmul(kin[3], g.fy), dmul(kin[4], g.fx))};
            const double ab[3] = {
                dadd(dadd(kin[6], dsub(dmul(kin[10], g.fz), dmul(kin[11], g.fy))), dsub(dmul(kin[4], wr[2]), dmul(kin[5], wr[1]))),
                dadd(dadd(kin[7], dsub(dmul(kin[11], g.fx), dmul(kin[9], g.fz))), dsub(dmul(kin[5], wr[0]), dmul(kin[3], wr[2]))),
                dadd(dadd(kin[8], dsub(dmul(kin[9], g.fy), dmul(kin[10], g.fx))), dsub(dmul(kin[3], wr[1]), dmul(kin[4], wr[0])))};
            const double phif = dadd(pc, dmul(dmul(g.sgn, g.hw), p.g[ax]));
            s[0] = dsub(s[0], dmul(dmul(dmul(g.sgn, ab[ax]), phif), g.area));
            if (p.slip) {
              div = dadd(div, dmul(dmul(g.sgn, N[ax][c]), g.area));
            } else {
              const double cb[3] = {dsub(dmul(kin[4], ub[2]), dmul(kin[5], ub[1])),
                                    dsub(dmul(kin[5], ub[0]), dmul(kin[3], ub[2])),
                                    dsub(dmul(kin[3], ub[1]), dmul(kin[4], ub[0]))};
              div = dadd(div, dmul(dmul(g.sgn, cb[ax]), g.area));
              for (int a = 0; a < 3; a++) lap[a] = dadd(lap[a], dmul(ddiv(dsub(ub[a], vel[a][c]), g.hw), g.area));
            }
          } else {
            const double x = dadd(N[ax][c], ddiv(dmul(dsub(N[ax][c2], N[ax][c]), g.hw), g.d));
            div = dadd(div, dmul(dmul(g.sgn, x), g.area));
            for (int a = 0; a < 3; a++) lap[a] = dadd(lap[a], dmul(ddiv(dsub(vel[a][c2], vel[a][c]), g.d), g.area));
          }
        }
      }
      const double dxi = dsub(p.xf[i], p.xf[i - 1]), dyj = dsub(p.yf[j], p.yf[j - 1]), dzk = dsub(p.zf[k], p.zf[k - 1]);
      vif[c] = ddiv(dmul(pc, div), dmul(dmul(dxi, dyj), dzk));
      s[1] = dadd(s[1], dmul(pc, div));
      s[2] = dadd(s[2], dmul(p.nu, dadd(dadd(dmul(lap[0], gp0[c]), dmul(lap[1], gp1[c])), dmul(lap[2], gp2[c]))));
    }
  }
  double out[4];
  if (grid_reduce<4, 0>(s, m, rb.partials, rb.ticket, out))
    if (lin_tid() == 0)
      for (int n = 0; n < 4; n++) S->red[n] = out[n];
}

cudaError_t launch_partition_3d(const Part3D& p, double* scratch /* 6 * n3 */, double* vif, double* omega,
                                SolveScalars* S, const RedBuf& rb, cudaStream_t st) {
  dim3 block(32, 8), grid((p.nx + 31) / 32, (p.ny + 7) / 8, p.nz);
  const long long n3 = (long long)p.nx * p.ny * p.nz;
  double *N0 = scratch, *N1 = N0 + n3, *N2 = N1 + n3, *g0 = N2 + n3, *g1 = g0 + n3, *g2 = g1 + n3;
  k_part3_pass1<<<grid, block, 0, st>>>(p, N0, N1, N2, g0, g1, g2, omega); note_launch();
  k_part3_pass2<<<grid, block, 0, st>>>(p, N0, N1, N2, g0, g1, g2, vif, S, rb); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
