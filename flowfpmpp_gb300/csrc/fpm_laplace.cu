// No-body Neumann Poisson solvers and FPM densities of the reference modules
// fpm_laplace_3d (src/fpm_laplace_3d.f90) and fpm_terms_3d (src/fpm_terms_3d.f90).
// Per-cell arithmetic uses separately rounded FP64 operations in the
// reference's order, so every sweep is bit-identical to a serial
// -ffp-contract=off evaluation; only global sums (means, compatibility
// fluxes, integrals) differ in summation order.
#include "fpm_internal.h"

namespace fpm {

// Layouts of this module: phi of the uniform solver is (0:nx+1, 0:ny+1,
// 0:nz+1); the non-uniform solver's phi and every other 3-D array is
// (nx, ny, nz); axes carry no halo (xc(nx), dx(nx)).
struct Dims3 {
  int nx, ny, nz;
  __host__ __device__ __forceinline__ long long g3(int i, int j, int k) const {  // full-halo, 0-based ghosts
    return (long long)i + (long long)(nx + 2) * ((long long)j + (long long)(ny + 2) * (long long)k);
  }
  __host__ __device__ __forceinline__ long long in(int i, int j, int k) const {
    return (long long)(i - 1) + (long long)nx * ((long long)(j - 1) + (long long)ny * (long long)(k - 1));
  }
};

#define LCELL_BEGIN                                        \
  const int i = blockIdx.x * 32 + threadIdx.x + 1;         \
  const int j = blockIdx.y * 8 + threadIdx.y + 1;          \
  const bool inxy = (i <= d.nx) && (j <= d.ny);            \
  for (int k = blockIdx.z + 1; k <= d.nz; k += gridDim.z) { \
    if (inxy) {
#define LCELL_END \
  }               \
  }

static Launch lcells(const Dims3& d) { return cells_launch(Dims{d.nx, d.ny, d.nz}); }

// ---------------------------------------------------------------- compatibility
// enforce_neumann_compatibility_3d (:9-53) and _nonuniform_3d (:150-217).
// Uniform spacing is passed as 1-element "axes" with uniform=1.
struct Spacing {
  const double *dx, *dy, *dz;
  int uniform;
  __device__ __forceinline__ double x(int i) const { return uniform ? dx[0] : dx[i - 1]; }
  __device__ __forceinline__ double y(int j) const { return uniform ? dy[0] : dy[j - 1]; }
  __device__ __forceinline__ double z(int k) const { return uniform ? dz[0] : dz[k - 1]; }
};

__global__ void k_neumann_source(Dims3 d, const double* __restrict__ rhs, Spacing sp, SolveScalars* S, RedBuf rb) {
  double s[1] = {0.0}, m[1] = {0.0};
  LCELL_BEGIN
  s[0] += dmul(dmul(dmul(rhs[d.in(i, j, k)], sp.x(i)), sp.y(j)), sp.z(k));
  LCELL_END
  double out[1];
  if (grid_reduce<1, 0>(s, m, rb.partials, rb.ticket, out))
    if (lin_tid() == 0) S->red[0] = out[0];
}
// Flux through the six outer faces and their area (area only used by the
// non-uniform variant), one thread per face cell of the largest face.
__global__ void k_neumann_flux(Dims3 d, Faces f, Spacing sp, int slot, SolveScalars* S, RedBuf rb) {
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  const long long nxz = (long long)d.nx * d.nz, nyz = (long long)d.ny * d.nz, nxy = (long long)d.nx * d.ny;
  const long long nt = (long long)gridDim.x * blockDim.x;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < nyz + nxz + nxy; n += nt) {
    if (n < nyz) {
      const int j = (int)(n % d.ny) + 1, k = (int)(n / d.ny) + 1;
      s[0] += dmul(dmul(dadd(-f.xlo[n], f.xhi[n]), sp.y(j)), sp.z(k));
      s[1] += dmul(dmul(2.0, sp.y(j)), sp.z(k));
    } else if (n < nyz + nxz) {
      const long long m2 = n - nyz;
      const int i = (int)(m2 % d.nx) + 1, k = (int)(m2 / d.nx) + 1;
      s[0] += dmul(dmul(dadd(-f.ylo[m2], f.yhi[m2]), sp.x(i)), sp.z(k));
      s[1] += dmul(dmul(2.0, sp.x(i)), sp.z(k));
    } else {
      const long long m3 = n - nyz - nxz;
      const int i = (int)(m3 % d.nx) + 1, j = (int)(m3 / d.nx) + 1;
      s[0] += dmul(dmul(dadd(-f.zlo[m3], f.zhi[m3]), sp.x(i)), sp.y(j));
      s[1] += dmul(dmul(2.0, sp.x(i)), sp.y(j));
    }
  }
  double out[2];
  if (grid_reduce<2, 0>(s, m, rb.partials, rb.ticket, out))
    if (lin_tid() == 0) {
      S->red[slot] = out[0];
      S->red[slot + 1] = out[1];
    }
}
__global__ void k_neumann_shift(Dims3 d, Faces f, const double* corr) {
  const double c = *corr;
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n < (long long)d.ny * d.nz) { f.xlo[n] = dsub(f.xlo[n], c); f.xhi[n] = dadd(f.xhi[n], c); }
  if (n < (long long)d.nx * d.nz) { f.ylo[n] = dsub(f.ylo[n], c); f.yhi[n] = dadd(f.yhi[n], c); }
  if (n < (long long)d.nx * d.ny) { f.zlo[n] = dsub(f.zlo[n], c); f.zhi[n] = dadd(f.zhi[n], c); }
}
__global__ void k_neumann_correction(SolveScalars* S, double area_uniform, int uniform) {
  // red[0] source, red[1] flux, red[2] summed area (non-uniform)
  const double area = uniform ? area_uniform : S->red[2];
  S->corr = -(S->red[1] - S->red[0]) / area;
}

cudaError_t launch_neumann_compat(int nx, int ny, int nz, const double* rhs, Faces f, const double* dx,
                                  const double* dy, const double* dz, int uniform, double area_uniform,
                                  SolveScalars* S, const RedBuf& rb, cudaStream_t st) {
  Dims3 d{nx, ny, nz};
  Spacing sp{dx, dy, dz, uniform};
  Launch L = lcells(d);
  k_neumann_source<<<L.grid, L.block, 0, st>>>(d, rhs, sp, S, rb); note_launch();
  k_neumann_flux<<<rb.max_blocks, 256, 0, st>>>(d, f, sp, 1, S, rb); note_launch();
  k_neumann_correction<<<1, 1, 0, st>>>(S, area_uniform, uniform); note_launch();
  long long nmax = (long long)ny * nz;
  if ((long long)nx * nz > nmax) nmax = (long long)nx * nz;
  if ((long long)nx * ny > nmax) nmax = (long long)nx * ny;
  k_neumann_shift<<<(unsigned)((nmax + 255) / 256), 256, 0, st>>>(d, f, &S->corr); note_launch();
  // flux after the shift -> red[3] (red[4] gets an unused area)
  k_neumann_flux<<<rb.max_blocks, 256, 0, st>>>(d, f, sp, 3, S, rb); note_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------- uniform solver
// solve_neumann_poisson_3d sweep (:74-86): undamped Jacobi with clamped
// neighbours; boundary neighbours from the prescribed face derivative.
// cur/nxt are interior arrays (nx,ny,nz): the sweep never reads phi's ghosts.
struct UniCoef {
  double dx, dy, dz, idx2, idy2, idz2, invdiag;
};
__device__ __forceinline__ void uni_neighbours(const Dims3& d, const double* __restrict__ a, const Faces& f,
                                               const UniCoef& u, int i, int j, int k, double& p, double& xm,
                                               double& xp, double& ym, double& yp, double& zm, double& zp) {
  p = a[d.in(i, j, k)];
  xm = a[d.in(i > 1 ? i - 1 : 1, j, k)];
  xp = a[d.in(i < d.nx ? i + 1 : d.nx, j, k)];
  ym = a[d.in(i, j > 1 ? j - 1 : 1, k)];
  yp = a[d.in(i, j < d.ny ? j + 1 : d.ny, k)];
  zm = a[d.in(i, j, k > 1 ? k - 1 : 1)];
  zp = a[d.in(i, j, k < d.nz ? k + 1 : d.nz)];
  const long long xf = (long long)(j - 1) + (long long)d.ny * (k - 1);
  const long long yf = (long long)(i - 1) + (long long)d.nx * (k - 1);
  const long long zf = (long long)(i - 1) + (long long)d.nx * (j - 1);
  if (i == 1) xm = dsub(p, dmul(f.xlo[xf], u.dx));
  if (i == d.nx) xp = dadd(p, dmul(f.xhi[xf], u.dx));
  if (j == 1) ym = dsub(p, dmul(f.ylo[yf], u.dy));
  if (j == d.ny) yp = dadd(p, dmul(f.yhi[yf], u.dy));
  if (k == 1) zm = dsub(p, dmul(f.zlo[zf], u.dz));
  if (k == d.nz) zp = dadd(p, dmul(f.zhi[zf], u.dz));
}
__global__ void k_uniform_sweep(Dims3 d, const double* __restrict__ a, double* __restrict__ b,
                                const double* __restrict__ rhs, Faces f, UniCoef u) {
  LCELL_BEGIN
  double p, xm, xp, ym, yp, zm, zp;
  uni_neighbours(d, a, f, u, i, j, k, p, xm, xp, ym, yp, zm, zp);
  double t = dadd(dadd(dmul(dadd(xm, xp), u.idx2), dmul(dadd(ym, yp), u.idy2)), dmul(dadd(zm, zp), u.idz2));
  b[d.in(i, j, k)] = dmul(dsub(t, rhs[d.in(i, j, k)]), u.invdiag);
  LCELL_END
}
// residual_norm (:109-132).
__global__ void k_uniform_residual(Dims3 d, const double* __restrict__ a, const double* __restrict__ rhs, Faces f,
                                   UniCoef u, SolveScalars* S, RedBuf rb) {
  double s[1] = {0.0}, m[1] = {0.0};
  LCELL_BEGIN
  double p, xm, xp, ym, yp, zm, zp;
  uni_neighbours(d, a, f, u, i, j, k, p, xm, xp, ym, yp, zm, zp);
  const double p2 = dmul(2.0, p);
  double r = dadd(dadd(ddiv(dadd(dsub(xm, p2), xp), dmul(u.dx, u.dx)), ddiv(dadd(dsub(ym, p2), yp), dmul(u.dy, u.dy))),
                  ddiv(dadd(dsub(zm, p2), zp), dmul(u.dz, u.dz)));
  r = dsub(r, rhs[d.in(i, j, k)]);
  m[0] = fmax(m[0], fabs(r));
  LCELL_END
  double out[1];
  if (grid_reduce<0, 1>(s, m, rb.partials, rb.ticket, out))
    if (lin_tid() == 0) S->res = out[0];
}
__global__ void k_uniform_mean(Dims3 d, const double* __restrict__ a, SolveScalars* S, RedBuf rb) {
  double s[1] = {0.0}, m[1] = {0.0};
  LCELL_BEGIN
  s[0] += a[d.in(i, j, k)];
  LCELL_END
  double out[1];
  if (grid_reduce<1, 0>(s, m, rb.partials, rb.ticket, out))
    if (lin_tid() == 0) S->mean = out[0] / (double)((long long)d.nx * d.ny * d.nz);
}
// mean removal, copy into the full-halo phi, then set_ghosts (:134-148).
__global__ void k_uniform_finish(Dims3 d, double* __restrict__ a, double* __restrict__ phi, const SolveScalars* S) {
  const double mean = S->mean;
  LCELL_BEGIN
  const double v = dsub(a[d.in(i, j, k)], mean);
  a[d.in(i, j, k)] = v;
  phi[d.g3(i, j, k)] = v;
  LCELL_END
}
__global__ void k_uniform_ghosts(Dims3 d, double* __restrict__ phi, Faces f, UniCoef u) {
  const long long nyz = (long long)d.ny * d.nz, nxz = (long long)d.nx * d.nz, nxy = (long long)d.nx * d.ny;
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n < nyz) {
    const int j = (int)(n % d.ny) + 1, k = (int)(n / d.ny) + 1;
    phi[d.g3(0, j, k)] = dsub(phi[d.g3(1, j, k)], dmul(f.xlo[n], u.dx));
    phi[d.g3(d.nx + 1, j, k)] = dadd(phi[d.g3(d.nx, j, k)], dmul(f.xhi[n], u.dx));
  }
  if (n < nxz) {
    const int i = (int)(n % d.nx) + 1, k = (int)(n / d.nx) + 1;
    phi[d.g3(i, 0, k)] = dsub(phi[d.g3(i, 1, k)], dmul(f.ylo[n], u.dy));
    phi[d.g3(i, d.ny + 1, k)] = dadd(phi[d.g3(i, d.ny, k)], dmul(f.yhi[n], u.dy));
  }
  if (n < nxy) {
    const int i = (int)(n % d.nx) + 1, j = (int)(n / d.nx) + 1;
    phi[d.g3(i, j, 0)] = dsub(phi[d.g3(i, j, 1)], dmul(f.zlo[n], u.dz));
    phi[d.g3(i, j, d.nz + 1)] = dadd(phi[d.g3(i, j, d.nz)], dmul(f.zhi[n], u.dz));
  }
}
__global__ void k_gather_interior3(Dims3 d, const double* __restrict__ phi, double* __restrict__ a) {
  LCELL_BEGIN
  a[d.in(i, j, k)] = phi[d.g3(i, j, k)];
  LCELL_END
}

// Host driver of solve_neumann_poisson_3d (:55-107): chunks of check_interval
// sweeps, residual after each chunk, then gauge, ghosts and final residual.
// Scalars are read through read_res (a host callback that syncs).
int neumann_uniform_iterate(int nx, int ny, int nz, double* phi, const double* rhs, Faces f, double dx, double dy,
                            double dz, double tol, int max_it, int ci, double* a, double* b, SolveScalars* S,
                            const RedBuf& rb, cudaStream_t st, double (*read_res)(SolveScalars*, cudaStream_t, int),
                            int* iterations, double* final_residual) {
  Dims3 d{nx, ny, nz};
  UniCoef u;
  u.dx = dx;
  u.dy = dy;
  u.dz = dz;
  u.idx2 = 1.0 / (dx * dx);
  u.idy2 = 1.0 / (dy * dy);
  u.idz2 = 1.0 / (dz * dz);
  u.invdiag = 1.0 / (2.0 * (u.idx2 + u.idy2 + u.idz2));
  Launch L = lcells(d);
  k_gather_interior3<<<L.grid, L.block, 0, st>>>(d, phi, a); note_launch();
  double* cur = a;
  double* oth = b;
  int it = 0;
  double fr = HUGE_VAL;
  const int cie = ci < 1 ? 1 : ci;
  while (it < max_it && fr > tol) {
    int nsteps = cie < max_it - it ? cie : max_it - it;
    for (int s = 0; s < nsteps; s++) {
      k_uniform_sweep<<<L.grid, L.block, 0, st>>>(d, cur, oth, rhs, f, u); note_launch();
      double* t = cur;
      cur = oth;
      oth = t;
    }
    it += nsteps;
    k_uniform_residual<<<L.grid, L.block, 0, st>>>(d, cur, rhs, f, u, S, rb); note_launch();
    fr = read_res(S, st, 0);
  }
  k_uniform_mean<<<L.grid, L.block, 0, st>>>(d, cur, S, rb); note_launch();
  k_uniform_finish<<<L.grid, L.block, 0, st>>>(d, cur, phi, S); note_launch();
  long long nmax = (long long)ny * nz;
  if ((long long)nx * nz > nmax) nmax = (long long)nx * nz;
  if ((long long)nx * ny > nmax) nmax = (long long)nx * ny;
  k_uniform_ghosts<<<(unsigned)((nmax + 255) / 256), 256, 0, st>>>(d, phi, f, u); note_launch();
  k_uniform_residual<<<L.grid, L.block, 0, st>>>(d, cur, rhs, f, u, S, rb); note_launch();
  fr = read_res(S, st, 0);
  *iterations = it;
  *final_residual = fr;
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------- non-uniform solver
// 1-D coefficients of solve_neumann_poisson_nonuniform_3d (:239-246):
// aw(i) = 1/(dx(i)(xc(i)-xc(i-1))) for i>1 else 0, ae(i) for i<nx else 0.
__global__ void k_nu_coefs(int nx, int ny, int nz, Axes ax, double* coef) {
  double *aw = coef, *ae = aw + nx, *as = ae + nx, *an = as + ny, *ab = an + ny, *at = ab + nz;
  const int t = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (t <= nx) {
    aw[t - 1] = t > 1 ? ddiv(1.0, dmul(ax.dx[t - 1], dsub(ax.xc[t - 1], ax.xc[t - 2]))) : 0.0;
    ae[t - 1] = t < nx ? ddiv(1.0, dmul(ax.dx[t - 1], dsub(ax.xc[t], ax.xc[t - 1]))) : 0.0;
  }
  if (t <= ny) {
    as[t - 1] = t > 1 ? ddiv(1.0, dmul(ax.dy[t - 1], dsub(ax.yc[t - 1], ax.yc[t - 2]))) : 0.0;
    an[t - 1] = t < ny ? ddiv(1.0, dmul(ax.dy[t - 1], dsub(ax.yc[t], ax.yc[t - 1]))) : 0.0;
  }
  if (t <= nz) {
    ab[t - 1] = t > 1 ? ddiv(1.0, dmul(ax.dz[t - 1], dsub(ax.zc[t - 1], ax.zc[t - 2]))) : 0.0;
    at[t - 1] = t < nz ? ddiv(1.0, dmul(ax.dz[t - 1], dsub(ax.zc[t], ax.zc[t - 1]))) : 0.0;
  }
}
// Weighted 0.2/0.8 Jacobi sweep (:238-264).
__global__ void k_nu_sweep(Dims3 d, const double* __restrict__ a, double* __restrict__ b,
                           const double* __restrict__ rhs, Faces f, Axes ax, const double* __restrict__ coef) {
  const double *aw = coef, *ae = aw + d.nx, *as = ae + d.nx, *an = as + d.ny, *ab = an + d.ny, *at = ab + d.nz;
  LCELL_BEGIN
  const double cw = aw[i - 1], ce = ae[i - 1], cs = as[j - 1], cn = an[j - 1], cb = ab[k - 1], ct = at[k - 1];
  const double diag = dadd(dadd(dadd(dadd(dadd(cw, ce), cs), cn), cb), ct);
  const long long c = d.in(i, j, k);
  double numer = -rhs[c];
  if (i > 1) numer = dadd(numer, dmul(cw, a[c - 1]));
  if (i < d.nx) numer = dadd(numer, dmul(ce, a[c + 1]));
  if (j > 1) numer = dadd(numer, dmul(cs, a[c - d.nx]));
  if (j < d.ny) numer = dadd(numer, dmul(cn, a[c + d.nx]));
  const long long pl = (long long)d.nx * d.ny;
  if (k > 1) numer = dadd(numer, dmul(cb, a[c - pl]));
  if (k < d.nz) numer = dadd(numer, dmul(ct, a[c + pl]));
  const long long xf = (long long)(j - 1) + (long long)d.ny * (k - 1);
  const long long yf = (long long)(i - 1) + (long long)d.nx * (k - 1);
  const long long zf = (long long)(i - 1) + (long long)d.nx * (j - 1);
  if (i == 1) numer = dsub(numer, ddiv(f.xlo[xf], ax.dx[i - 1]));
  if (i == d.nx) numer = dadd(numer, ddiv(f.xhi[xf], ax.dx[i - 1]));
  if (j == 1) numer = dsub(numer, ddiv(f.ylo[yf], ax.dy[j - 1]));
  if (j == d.ny) numer = dadd(numer, ddiv(f.yhi[yf], ax.dy[j - 1]));
  if (k == 1) numer = dsub(numer, ddiv(f.zlo[zf], ax.dz[k - 1]));
  if (k == d.nz) numer = dadd(numer, ddiv(f.zhi[zf], ax.dz[k - 1]));
  b[c] = dadd(dmul(0.2, a[c]), ddiv(dmul(0.8, numer), diag));
  LCELL_END
}
// Face gradients with prescribed boundary values (residual_nonuniform :305-310
// and compute_fpm_terms_nonuniform_3d :379-384).
__device__ __forceinline__ void nu_face_gradients(const Dims3& d, const double* __restrict__ a, const Faces& f,
                                                  const Axes& ax, int i, int j, int k, double g[6]) {
  const long long c = d.in(i, j, k), pl = (long long)d.nx * d.ny;
  const double p = a[c];
  const long long xf = (long long)(j - 1) + (long long)d.ny * (k - 1);
  const long long yf = (long long)(i - 1) + (long long)d.nx * (k - 1);
  const long long zf = (long long)(i - 1) + (long long)d.nx * (j - 1);
  g[0] = i == 1 ? f.xlo[xf] : ddiv(dsub(p, a[c - 1]), dsub(ax.xc[i - 1], ax.xc[i - 2]));
  g[1] = i == d.nx ? f.xhi[xf] : ddiv(dsub(a[c + 1], p), dsub(ax.xc[i], ax.xc[i - 1]));
  g[2] = j == 1 ? f.ylo[yf] : ddiv(dsub(p, a[c - d.nx]), dsub(ax.yc[j - 1], ax.yc[j - 2]));
  g[3] = j == d.ny ? f.yhi[yf] : ddiv(dsub(a[c + d.nx], p), dsub(ax.yc[j], ax.yc[j - 1]));
  g[4] = k == 1 ? f.zlo[zf] : ddiv(dsub(p, a[c - pl]), dsub(ax.zc[k - 1], ax.zc[k - 2]));
  g[5] = k == d.nz ? f.zhi[zf] : ddiv(dsub(a[c + pl], p), dsub(ax.zc[k], ax.zc[k - 1]));
}
__global__ void k_nu_residual(Dims3 d, const double* __restrict__ a, const double* __restrict__ rhs, Faces f, Axes ax,
                              SolveScalars* S, RedBuf rb) {
  double s[1] = {0.0}, m[1] = {0.0};
  LCELL_BEGIN
  double g[6];
  nu_face_gradients(d, a, f, ax, i, j, k, g);
  double r = dadd(dadd(ddiv(dsub(g[1], g[0]), ax.dx[i - 1]), ddiv(dsub(g[3], g[2]), ax.dy[j - 1])),
                  ddiv(dsub(g[5], g[4]), ax.dz[k - 1]));
  r = dsub(r, rhs[d.in(i, j, k)]);
  m[0] = fmax(m[0], fabs(r));
  LCELL_END
  double out[1];
  if (grid_reduce<0, 1>(s, m, rb.partials, rb.ticket, out))
    if (lin_tid() == 0) S->res = out[0];
}
__global__ void k_nu_gauge_sum(Dims3 d, const double* __restrict__ a, Axes ax, SolveScalars* S, RedBuf rb) {
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  LCELL_BEGIN
  const double dxi = ax.dx[i - 1], dyj = ax.dy[j - 1], dzk = ax.dz[k - 1];
  s[0] += dmul(dmul(dmul(a[d.in(i, j, k)], dxi), dyj), dzk);
  s[1] += dmul(dmul(dxi, dyj), dzk);
  LCELL_END
  double out[2];
  if (grid_reduce<2, 0>(s, m, rb.partials, rb.ticket, out))
    if (lin_tid() == 0) S->mean = out[0] / out[1];
}
__global__ void k_sub_mean(long long n, double* __restrict__ a, const SolveScalars* S) {
  const double mean = S->mean;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x)
    a[m] = dsub(a[m], mean);
}

int neumann_nonuniform_iterate(int nx, int ny, int nz, double* phi, const double* rhs, Faces f, const Axes& ax,
                               double tol, int max_it, int ci, double* b, double* coef, SolveScalars* S,
                               const RedBuf& rb, cudaStream_t st,
                               double (*read_res)(SolveScalars*, cudaStream_t, int), int* iterations,
                               double* final_residual) {
  Dims3 d{nx, ny, nz};
  int n1 = nx > ny ? nx : ny;
  if (nz > n1) n1 = nz;
  k_nu_coefs<<<(n1 + 255) / 256, 256, 0, st>>>(nx, ny, nz, ax, coef); note_launch();
  Launch L = lcells(d);
  double* cur = phi;
  double* oth = b;
  int it = 0;
  double fr = HUGE_VAL;
  const int cie = ci < 1 ? 1 : ci;
  while (it < max_it && fr > tol) {
    int nsteps = cie < max_it - it ? cie : max_it - it;
    for (int s = 0; s < nsteps; s++) {
      k_nu_sweep<<<L.grid, L.block, 0, st>>>(d, cur, oth, rhs, f, ax, coef); note_launch();
      double* t = cur;
      cur = oth;
      oth = t;
    }
    it += nsteps;
    k_nu_residual<<<L.grid, L.block, 0, st>>>(d, cur, rhs, f, ax, S, rb); note_launch();
    fr = read_res(S, st, 0);
  }
  const long long n = (long long)nx * ny * nz;
  if (cur != phi) cudaMemcpyAsync(phi, cur, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
  k_nu_gauge_sum<<<L.grid, L.block, 0, st>>>(d, phi, ax, S, rb); note_launch();
  long long nb = (n + 255) / 256;
  if (nb > 152 * 32) nb = 152 * 32;
  k_sub_mean<<<(unsigned)nb, 256, 0, st>>>(n, phi, S); note_launch();
  k_nu_residual<<<L.grid, L.block, 0, st>>>(d, phi, rhs, f, ax, S, rb); note_launch();
  fr = read_res(S, st, 0);
  *iterations = it;
  *final_residual = fr;
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------- fpm_terms_3d
// compute_fpm_terms_uniform_3d (src/fpm_terms_3d.f90:8-37): central
// differences on the full-halo phi; totals with the uniform cell volume.
__global__ void k_terms_uniform(Dims3 d, const double* __restrict__ phi, Flow fl, const int32_t* __restrict__ fluid,
                                double dx, double dy, double dz, TermsOut o, SolveScalars* S, RedBuf rb) {
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  const double volume = dmul(dmul(dx, dy), dz);
  LCELL_BEGIN
  const long long c = d.in(i, j, k);
  const double gx = ddiv(dsub(phi[d.g3(i + 1, j, k)], phi[d.g3(i - 1, j, k)]), dmul(2.0, dx));
  const double gy = ddiv(dsub(phi[d.g3(i, j + 1, k)], phi[d.g3(i, j - 1, k)]), dmul(2.0, dy));
  const double gz = ddiv(dsub(phi[d.g3(i, j, k + 1)], phi[d.g3(i, j, k - 1)]), dmul(2.0, dz));
  o.gx[c] = gx;
  o.gy[c] = gy;
  o.gz[c] = gz;
  const double u = fl.u[c], v = fl.v[c], w = fl.w[c], ox = fl.ox[c], oy = fl.oy[c], oz = fl.oz[c];
  const double cx = dsub(dmul(w, oy), dmul(v, oz));
  const double cy = dsub(dmul(u, oz), dmul(w, ox));
  const double cz = dsub(dmul(v, ox), dmul(u, oy));
  const double mask = (double)fluid[c];
  const double vort = -dmul(mask, dadd(dadd(dmul(cx, gx), dmul(cy, gy)), dmul(cz, gz)));
  const double adv = -dmul(mask, dadd(dadd(dmul(fl.ax[c], gx), dmul(fl.ay[c], gy)), dmul(fl.az[c], gz)));
  o.vortex[c] = vort;
  o.advection[c] = adv;
  s[0] += dmul(volume, vort);
  s[1] += dmul(volume, adv);
  LCELL_END
  double out[2];
  if (grid_reduce<2, 0>(s, m, rb.partials, rb.ticket, out))
    if (lin_tid() == 0) {
      S->red[0] = out[0];
      S->red[1] = out[1];
    }
}
// compute_fpm_terms_nonuniform_3d (src/fpm_terms_3d.f90:39-88).
__global__ void k_terms_nonuniform(Dims3 d, const double* __restrict__ phi, Flow fl, const int32_t* __restrict__ fluid,
                                   Axes ax, Faces f, double b0, double b1, double b2, double b3, double b4, double b5,
                                   TermsOut o, SolveScalars* S, RedBuf rb) {
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  LCELL_BEGIN
  const long long c = d.in(i, j, k);
  double g[6];
  nu_face_gradients(d, phi, f, ax, i, j, k, g);
  const double gx = dmul(0.5, dadd(g[0], g[1]));
  const double gy = dmul(0.5, dadd(g[2], g[3]));
  const double gz = dmul(0.5, dadd(g[4], g[5]));
  o.gx[c] = gx;
  o.gy[c] = gy;
  o.gz[c] = gz;
  const double u = fl.u[c], v = fl.v[c], w = fl.w[c], ox = fl.ox[c], oy = fl.oy[c], oz = fl.oz[c];
  const double cx = dsub(dmul(w, oy), dmul(v, oz));
  const double cy = dsub(dmul(u, oz), dmul(w, ox));
  const double cz = dsub(dmul(v, ox), dmul(u, oy));
  const double mask = (double)fluid[c];
  const double vort = -dmul(mask, dadd(dadd(dmul(cx, gx), dmul(cy, gy)), dmul(cz, gz)));
  const double adv = -dmul(mask, dadd(dadd(dmul(fl.ax[c], gx), dmul(fl.ay[c], gy)), dmul(fl.az[c], gz)));
  o.vortex[c] = vort;
  o.advection[c] = adv;
  const double xci = ax.xc[i - 1], ycj = ax.yc[j - 1], zck = ax.zc[k - 1];
  const double inside = (xci > b0 && xci < b1 && ycj > b2 && ycj < b3 && zck > b4 && zck < b5) ? 1.0 : 0.0;
  const double vol = dmul(dmul(dmul(inside, ax.dx[i - 1]), ax.dy[j - 1]), ax.dz[k - 1]);
  s[0] += dmul(vol, vort);
  s[1] += dmul(vol, adv);
  LCELL_END
  double out[2];
  if (grid_reduce<2, 0>(s, m, rb.partials, rb.ticket, out))
    if (lin_tid() == 0) {
      S->red[0] = out[0];
      S->red[1] = out[1];
    }
}
cudaError_t launch_terms_uniform(int nx, int ny, int nz, const double* phi, const Flow& fl, const int32_t* fluid,
                                 double dx, double dy, double dz, const TermsOut& o, SolveScalars* S,
                                 const RedBuf& rb, cudaStream_t st) {
  Dims3 d{nx, ny, nz};
  Launch L = lcells(d);
  k_terms_uniform<<<L.grid, L.block, 0, st>>>(d, phi, fl, fluid, dx, dy, dz, o, S, rb); note_launch();
  return cudaGetLastError();
}
cudaError_t launch_terms_nonuniform(int nx, int ny, int nz, const double* phi, const Flow& fl, const int32_t* fluid,
                                    const Axes& ax, const Faces& f, const double bounds[6], const TermsOut& o,
                                    SolveScalars* S, const RedBuf& rb, cudaStream_t st) {
  Dims3 d{nx, ny, nz};
  Launch L = lcells(d);
  k_terms_nonuniform<<<L.grid, L.block, 0, st>>>(d, phi, fl, fluid, ax, f, bounds[0], bounds[1], bounds[2],
                                                 bounds[3], bounds[4], bounds[5], o, S, rb); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
