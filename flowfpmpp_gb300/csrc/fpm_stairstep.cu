// Stair-step influence solve: operator build, FP64 weighted Jacobi, FP64 PCG
// with device-resident scalars, true-residual replacement, gauge,
// compatibility, the independent face-gradient residual and the FPM force
// densities.  Each kernel cites the reference routine it implements
// (src/fpm_stairstep_mpi_3d.f90); the per-cell arithmetic uses separately
// rounded FP64 operations in the reference's evaluation order wherever a
// bit-identical per-cell result is wanted (operator build, Jacobi sweep,
// residuals, gauge, densities), and contracted FMAs in the PCG recurrences
// whose global sums differ in order from a serial loop anyway.
#include "fpm_internal.h"

namespace fpm {

Launch cells_launch(const Dims& d, int pad_xy) {
  Launch L;
  L.block = dim3(32, 8, 1);
  int nxl = d.nx + 2 * pad_xy, nyl = d.ny + 2 * pad_xy;
  int gx = (nxl + 31) / 32, gy = (nyl + 7) / 8;
  long long xy = (long long)gx * gy;
  // About 16 blocks of 256 threads per SM over the whole grid.
  long long target = 152LL * 16;
  int gz = (int)((target + xy - 1) / xy);
  if (gz < 1) gz = 1;
  if (gz > d.nz) gz = d.nz;
  L.grid = dim3(gx, gy, gz);
  return L;
}

// src/fpm_stairstep_mpi_3d.f90:499-510 axis_coefficients (both sides physical)
// and the z coefficients of :138-142, into coef = cw, ce | cs, cn | cb, ct.
__global__ void k_axis_coefs(Axes ax, int nx, int ny, int nz, double* coef) {
  double *cw = coef, *ce = cw + nx, *cs = ce + nx, *cn = cs + ny, *cb = cn + ny, *ct = cb + nz;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x + 1; m <= nx; m += gridDim.x * blockDim.x) {
    cw[m - 1] = m == 1 ? 0.0 : ddiv(1.0, dmul(ax.dx[m - 1], dsub(ax.xc[m], ax.xc[m - 1])));
    ce[m - 1] = m == nx ? 0.0 : ddiv(1.0, dmul(ax.dx[m - 1], dsub(ax.xc[m + 1], ax.xc[m])));
  }
  for (int m = blockIdx.x * blockDim.x + threadIdx.x + 1; m <= ny; m += gridDim.x * blockDim.x) {
    cs[m - 1] = m == 1 ? 0.0 : ddiv(1.0, dmul(ax.dy[m - 1], dsub(ax.yc[m], ax.yc[m - 1])));
    cn[m - 1] = m == ny ? 0.0 : ddiv(1.0, dmul(ax.dy[m - 1], dsub(ax.yc[m + 1], ax.yc[m])));
  }
  for (int k = blockIdx.x * blockDim.x + threadIdx.x + 1; k <= nz; k += gridDim.x * blockDim.x) {
    cb[k - 1] = k > 1 ? ddiv(1.0, dmul(ax.dz[k - 1], dsub(ax.zc[k - 1], ax.zc[k - 2]))) : 0.0;
    ct[k - 1] = k < nz ? ddiv(1.0, dmul(ax.dz[k - 1], dsub(ax.zc[k], ax.zc[k - 1]))) : 0.0;
  }
}
cudaError_t launch_axis_coefs(const Axes& ax, int nx, int ny, int nz, double* coef, cudaStream_t st) {
  int n = nx > ny ? nx : ny;
  if (nz > n) n = nz;
  k_axis_coefs<<<(n + 255) / 256, 256, 0, st>>>(ax, nx, ny, nz, coef); note_launch();
  return cudaGetLastError();
}

#define CELL_LOOP_BEGIN                                    \
  const int i = blockIdx.x * 32 + threadIdx.x + 1;         \
  const int j = blockIdx.y * 8 + threadIdx.y + 1;          \
  const bool inxy = (i <= d.nx) && (j <= d.ny);            \
  for (int k = blockIdx.z + 1; k <= d.nz; k += gridDim.z) { \
    if (inxy) {
#define CELL_LOOP_END \
  }                   \
  }

struct Bg {
  double x, y, z;
};

// src/fpm_stairstep_mpi_3d.f90:336-379 build_operator.
__global__ void k_build_operator(Dims d, const double* __restrict__ rhs, const int32_t* __restrict__ solid, Bg bg,
                                 Faces f, Coefs c, Axes ax, int for_pcg, double* __restrict__ src,
                                 double* __restrict__ diag, double* __restrict__ rdiag, SolveScalars* S) {
  int iso = 0;
  CELL_LOOP_BEGIN
  double s = 0, dd = 0;
  const double dxi = ax.dx[i - 1], dyj = ax.dy[j - 1], dzk = ax.dz[k - 1];
  if (solid[d.ph(i, j, k)] == 0) {
    s = -rhs[d.in(i, j, k)];
    if (i == 1) s = dsub(s, ddiv(f.xlo[d.xf(j, k)], dxi));
    else if (solid[d.ph(i - 1, j, k)] != 0) s = dsub(s, ddiv(bg.x, dxi));
    else dd = dadd(dd, c.cw[i - 1]);
    if (i == d.nx) s = dadd(s, ddiv(f.xhi[d.xf(j, k)], dxi));
    else if (solid[d.ph(i + 1, j, k)] != 0) s = dadd(s, ddiv(bg.x, dxi));
    else dd = dadd(dd, c.ce[i - 1]);
    if (j == 1) s = dsub(s, ddiv(f.ylo[d.yf(i, k)], dyj));
    else if (solid[d.ph(i, j - 1, k)] != 0) s = dsub(s, ddiv(bg.y, dyj));
    else dd = dadd(dd, c.cs[j - 1]);
    if (j == d.ny) s = dadd(s, ddiv(f.yhi[d.yf(i, k)], dyj));
    else if (solid[d.ph(i, j + 1, k)] != 0) s = dadd(s, ddiv(bg.y, dyj));
    else dd = dadd(dd, c.cn[j - 1]);
    if (k == 1) s = dsub(s, ddiv(f.zlo[d.zf(i, j)], dzk));
    else if (solid[d.ph(i, j, k - 1)] != 0) s = dsub(s, ddiv(bg.z, dzk));
    else dd = dadd(dd, c.cb[k - 1]);
    if (k == d.nz) s = dadd(s, ddiv(f.zhi[d.zf(i, j)], dzk));
    else if (solid[d.ph(i, j, k + 1)] != 0) s = dadd(s, ddiv(bg.z, dzk));
    else dd = dadd(dd, c.ct[k - 1]);
    if (dd <= 0) iso++;
  }
  const long long cc = d.in(i, j, k);
  src[cc] = s;
  diag[cc] = dd;
  double rd;
  if (dd <= 0) rd = 0;
  else if (for_pcg) rd = ddiv(1.0, dmul(dmul(dmul(dxi, dyj), dzk), dd));
  else rd = ddiv(0.8, dd);
  rdiag[cc] = rd;
  CELL_LOOP_END
  if (iso) atomicAdd(&S->isolated, iso);
}

cudaError_t launch_build_operator(const Dims& d, const double* rhs, const int32_t* solid, const double bg[3],
                                  const Faces& f, const Coefs& c, const Axes& ax, int for_pcg, double* src,
                                  double* diag, double* rdiag, SolveScalars* S, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_build_operator<<<L.grid, L.block, 0, st>>>(d, rhs, solid, Bg{bg[0], bg[1], bg[2]}, f, c, ax, for_pcg, src, diag,
                                               rdiag, S); note_launch();
  return cudaGetLastError();
}

// init loop, src/fpm_stairstep_mpi_3d.f90:152-160: zero phi in solid cells and
// the physical halo, copy phi into next.
__global__ void k_init_fields(Dims d, const int32_t* __restrict__ solid, double* __restrict__ phi,
                              double* __restrict__ next) {
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  if (i > d.nx + 1 || j > d.ny + 1) return;
  for (int k = blockIdx.z + 1; k <= d.nz; k += gridDim.z) {
    const long long p = d.ph(i, j, k);
    double v = phi[p];
    if (solid[p] != 0 || i == 0 || i == d.nx + 1 || j == 0 || j == d.ny + 1) {
      v = 0;
      phi[p] = 0;
    }
    next[p] = v;
  }
}
cudaError_t launch_init_fields(const Dims& d, const int32_t* solid, double* phi, double* next, cudaStream_t st) {
  Launch L = cells_launch(d, 1);
  k_init_fields<<<L.grid, L.block, 0, st>>>(d, solid, phi, next); note_launch();
  return cudaGetLastError();
}

// src/fpm_stairstep_mpi_3d.f90:384-399 jacobi_sweep, bit-identical per cell:
// b = 0.2 a + rdiag (src + cw a_w + ce a_e + cs a_s + cn a_n + cb a_b + ct a_t).
__global__ void k_jacobi_f64(Dims d, const double* __restrict__ a, double* __restrict__ b,
                             const double* __restrict__ src, const double* __restrict__ rdiag, Coefs c) {
  CELL_LOOP_BEGIN
  const int kb = k > 1 ? k - 1 : 1, kt = k < d.nz ? k + 1 : d.nz;
  const long long cc = d.in(i, j, k), p = d.ph(i, j, k);
  double s = dadd(src[cc], dmul(c.cw[i - 1], a[p - 1]));
  s = dadd(s, dmul(c.ce[i - 1], a[p + 1]));
  s = dadd(s, dmul(c.cs[j - 1], a[p - (d.nx + 2)]));
  s = dadd(s, dmul(c.cn[j - 1], a[p + (d.nx + 2)]));
  s = dadd(s, dmul(c.cb[k - 1], a[d.ph(i, j, kb)]));
  s = dadd(s, dmul(c.ct[k - 1], a[d.ph(i, j, kt)]));
  b[p] = dadd(dmul(0.2, a[p]), dmul(rdiag[cc], s));
  CELL_LOOP_END
}
cudaError_t launch_jacobi_f64(const Dims& d, const double* a, double* b, const double* src, const double* rdiag,
                              const Coefs& c, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_jacobi_f64<<<L.grid, L.block, 0, st>>>(d, a, b, src, rdiag, c); note_launch();
  return cudaGetLastError();
}

// The same sweep with fused multiply-adds: FP64 storage and FP64 arithmetic,
// the reference's summation order, one rounding per multiply-add instead of
// two (8 FP64 instructions per cell instead of 15).  On GB300 the FP64 pipe
// (about 0.53 T instructions/s) bounds the sweep, so halving its instruction
// count halves the sweep time; results differ from the separately rounded
// sweep in the last bits only.
__global__ void k_jacobi_f64_fma(Dims d, const double* __restrict__ a, double* __restrict__ b,
                                 const double* __restrict__ src, const double* __restrict__ rdiag, Coefs c) {
  CELL_LOOP_BEGIN
  const int kb = k > 1 ? k - 1 : 1, kt = k < d.nz ? k + 1 : d.nz;
  const long long cc = d.in(i, j, k), p = d.ph(i, j, k);
  double s = __fma_rn(c.cw[i - 1], a[p - 1], src[cc]);
  s = __fma_rn(c.ce[i - 1], a[p + 1], s);
  s = __fma_rn(c.cs[j - 1], a[p - (d.nx + 2)], s);
  s = __fma_rn(c.cn[j - 1], a[p + (d.nx + 2)], s);
  s = __fma_rn(c.cb[k - 1], a[d.ph(i, j, kb)], s);
  s = __fma_rn(c.ct[k - 1], a[d.ph(i, j, kt)], s);
  b[p] = __fma_rn(0.2, a[p], dmul(rdiag[cc], s));
  CELL_LOOP_END
}
cudaError_t launch_jacobi_f64_fma(const Dims& d, const double* a, double* b, const double* src, const double* rdiag,
                                  const Coefs& c, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_jacobi_f64_fma<<<L.grid, L.block, 0, st>>>(d, a, b, src, rdiag, c); note_launch();
  return cudaGetLastError();
}

__global__ void k_copy_interior(Dims d, const double* __restrict__ from, double* __restrict__ to) {
  CELL_LOOP_BEGIN
  const long long p = d.ph(i, j, k);
  to[p] = from[p];
  CELL_LOOP_END
}
cudaError_t launch_copy_interior(const Dims& d, const double* from, double* to, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_copy_interior<<<L.grid, L.block, 0, st>>>(d, from, to); note_launch();
  return cudaGetLastError();
}

// src + sum(c_nb phi_nb) - diag phi, in the reference's order
// (src/fpm_stairstep_mpi_3d.f90:524-526 and :312-313).
__device__ __forceinline__ double local_residual(const Dims& d, const double* __restrict__ phi, double src,
                                                 double dg, const Coefs& c, int i, int j, int k) {
  const int kb = k > 1 ? k - 1 : 1, kt = k < d.nz ? k + 1 : d.nz;
  const long long p = d.ph(i, j, k);
  double t = dadd(src, dmul(c.cw[i - 1], phi[p - 1]));
  t = dadd(t, dmul(c.ce[i - 1], phi[p + 1]));
  t = dadd(t, dmul(c.cs[j - 1], phi[p - (d.nx + 2)]));
  t = dadd(t, dmul(c.cn[j - 1], phi[p + (d.nx + 2)]));
  t = dadd(t, dmul(c.cb[k - 1], phi[d.ph(i, j, kb)]));
  t = dadd(t, dmul(c.ct[k - 1], phi[d.ph(i, j, kt)]));
  return dsub(t, dmul(dg, phi[p]));
}

// src/fpm_stairstep_mpi_3d.f90:514-530 operator_residual -> S->res.
__global__ void k_operator_residual(Dims d, const double* __restrict__ phi, const double* __restrict__ src,
                                    const double* __restrict__ diag, Coefs c, SolveScalars* S, RedBuf rb) {
  double s[1] = {0.0}, m[1] = {0.0};
  CELL_LOOP_BEGIN
  const long long cc = d.in(i, j, k);
  const double dg = diag[cc];
  if (dg > 0) m[0] = fmax(m[0], fabs(local_residual(d, phi, src[cc], dg, c, i, j, k)));
  CELL_LOOP_END
  double out[1];
  if (grid_reduce<0, 1>(s, m, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) S->res = out[0];
  }
}
cudaError_t launch_operator_residual(const Dims& d, const double* phi, const double* src, const double* diag,
                                     const Coefs& c, SolveScalars* S, const RedBuf& rb, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_operator_residual<<<L.grid, L.block, 0, st>>>(d, phi, src, diag, c, S, rb); note_launch();
  return cudaGetLastError();
}

// true_residual, src/fpm_stairstep_mpi_3d.f90:297-329, part 1: res (max norm),
// r = V (src + sum c phi_nb - diag phi) on diag>0, and the sums of r and count.
__global__ void k_true_residual_a(Dims d, const double* __restrict__ phi, const double* __restrict__ src,
                                  const double* __restrict__ diag, double* __restrict__ r, Coefs c, Axes ax,
                                  SolveScalars* S, RedBuf rb) {
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  CELL_LOOP_BEGIN
  const long long cc = d.in(i, j, k);
  const double dg = diag[cc];
  double rv = 0;
  if (dg > 0) {
    const double t = local_residual(d, phi, src[cc], dg, c, i, j, k);
    m[0] = fmax(m[0], fabs(t));
    const double vol = dmul(dmul(ax.dx[i - 1], ax.dy[j - 1]), ax.dz[k - 1]);
    rv = dmul(vol, t);
    s[0] += rv;
    s[1] += 1.0;
  }
  r[cc] = rv;
  CELL_LOOP_END
  double out[3];
  if (grid_reduce<2, 1>(s, m, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      S->red[0] = out[0];
      S->red[1] = out[1];
      S->res = out[2];
    }
  }
}
// part 2: project r by its fluid mean; on reset p = rdiag r; rz = sum rdiag r^2.
__global__ void k_true_residual_b(Dims d, double* __restrict__ r, const double* __restrict__ diag,
                                  const double* __restrict__ rdiag, double* __restrict__ p, int reset,
                                  SolveScalars* S, RedBuf rb) {
  double s[1] = {0.0}, m[1] = {0.0};
  const double shift = S->red[0] / S->red[1];
  CELL_LOOP_BEGIN
  const long long cc = d.in(i, j, k);
  double rv = r[cc];
  if (diag[cc] > 0) {
    rv = rv - shift;
    r[cc] = rv;
  }
  const double rd = rdiag[cc];
  if (reset) p[d.ph(i, j, k)] = rd * rv;
  s[0] += rd * rv * rv;
  CELL_LOOP_END
  double out[1];
  if (grid_reduce<1, 0>(s, m, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      S->rz = out[0];
      S->halt = 0;
    }
  }
}
cudaError_t launch_true_residual(const Dims& d, const double* phi, const double* src, const double* diag,
                                 const double* rdiag, double* r, double* p, const Coefs& c, const Axes& ax, int reset,
                                 SolveScalars* S, const RedBuf& rb, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_true_residual_a<<<L.grid, L.block, 0, st>>>(d, phi, src, diag, r, c, ax, S, rb); note_launch();
  k_true_residual_b<<<L.grid, L.block, 0, st>>>(d, r, diag, rdiag, p, reset, S, rb); note_launch();
  return cudaGetLastError();
}

// pcg_iterate body, src/fpm_stairstep_mpi_3d.f90:245-283, as three kernels
// that read alpha / beta / halt from device memory.
// (1) q = V(diag p - sum c p_nb) on diag>0, pq = p.q; alpha = rz / pq.
__global__ void k_pcg_spmv(Dims d, const double* __restrict__ p, double* __restrict__ q,
                           const double* __restrict__ diag, Coefs c, Axes ax, SolveScalars* S, RedBuf rb) {
  if (S->halt) return;
  double s[1] = {0.0}, m[1] = {0.0};
  CELL_LOOP_BEGIN
  const long long cc = d.in(i, j, k), pp = d.ph(i, j, k);
  const int kb = k > 1 ? k - 1 : 1, kt = k < d.nz ? k + 1 : d.nz;
  const double dg = diag[cc], pc = p[pp];
  double qv = 0;
  if (dg > 0) {
    double t = dg * pc - c.cw[i - 1] * p[pp - 1];
    t = t - c.ce[i - 1] * p[pp + 1];
    t = t - c.cs[j - 1] * p[pp - (d.nx + 2)];
    t = t - c.cn[j - 1] * p[pp + (d.nx + 2)];
    t = t - c.cb[k - 1] * p[d.ph(i, j, kb)];
    t = t - c.ct[k - 1] * p[d.ph(i, j, kt)];
    const double vol = ax.dx[i - 1] * ax.dy[j - 1] * ax.dz[k - 1];
    qv = vol * t;
  }
  q[cc] = qv;
  s[0] += pc * qv;
  CELL_LOOP_END
  double out[1];
  if (grid_reduce<1, 0>(s, m, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      const double pq = out[0], rz = S->rz;
      S->pq = pq;
      if (!(pq > 0) || !(rz > 0)) S->halt = 1;  // negated tests are also true for NaN
      else S->alpha = rz / pq;
    }
  }
}
// (2) phi += alpha p; r -= alpha q; rz_new = sum rdiag r^2; beta = rz_new / rz.
__global__ void k_pcg_update(Dims d, double* __restrict__ phi, const double* __restrict__ p,
                             const double* __restrict__ q, double* __restrict__ r, const double* __restrict__ rdiag,
                             SolveScalars* S, RedBuf rb) {
  if (S->halt) return;
  const double alpha = S->alpha;
  double s[1] = {0.0}, m[1] = {0.0};
  CELL_LOOP_BEGIN
  const long long cc = d.in(i, j, k), pp = d.ph(i, j, k);
  phi[pp] = phi[pp] + alpha * p[pp];
  const double rv = r[cc] - alpha * q[cc];
  r[cc] = rv;
  s[0] += rdiag[cc] * rv * rv;
  CELL_LOOP_END
  double out[1];
  if (grid_reduce<1, 0>(s, m, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      const double rz_new = out[0];
      S->rz_new = rz_new;
      if (!(rz_new >= 0)) S->halt = 2;
      else {
        S->beta = rz_new / S->rz;
        S->rz = rz_new;
      }
    }
  }
}
// (3) p = rdiag r + beta p; count the completed iteration.
__global__ void k_pcg_direction(Dims d, double* __restrict__ p, const double* __restrict__ r,
                                const double* __restrict__ rdiag, SolveScalars* S) {
  if (S->halt) return;
  const double beta = S->beta;
  CELL_LOOP_BEGIN
  const long long cc = d.in(i, j, k), pp = d.ph(i, j, k);
  p[pp] = rdiag[cc] * r[cc] + beta * p[pp];
  CELL_LOOP_END
  if (lin_bid() == 0 && lin_tid() == 0) S->iters += 1;
}
cudaError_t launch_pcg_spmv(const Dims& d, const double* p, double* q, const double* diag, const Coefs& c,
                            const Axes& ax, SolveScalars* S, const RedBuf& rb, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_pcg_spmv<<<L.grid, L.block, 0, st>>>(d, p, q, diag, c, ax, S, rb); note_launch();
  return cudaGetLastError();
}
cudaError_t launch_pcg_iteration(const Dims& d, double* phi, double* p, double* q, double* r, const double* diag,
                                 const double* rdiag, const Coefs& c, const Axes& ax, SolveScalars* S,
                                 const RedBuf& rb, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_pcg_spmv<<<L.grid, L.block, 0, st>>>(d, p, q, diag, c, ax, S, rb); note_launch();
  k_pcg_update<<<L.grid, L.block, 0, st>>>(d, phi, p, q, r, rdiag, S, rb); note_launch();
  k_pcg_direction<<<L.grid, L.block, 0, st>>>(d, p, r, rdiag, S); note_launch();
  return cudaGetLastError();
}

// gauge, src/fpm_stairstep_mpi_3d.f90:170-185: remove the fluid-volume mean.
__global__ void k_gauge_sum(Dims d, const int32_t* __restrict__ solid, const double* __restrict__ phi, Axes ax,
                            SolveScalars* S, RedBuf rb) {
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  CELL_LOOP_BEGIN
  if (solid[d.ph(i, j, k)] == 0) {
    const double dxi = ax.dx[i - 1], dyj = ax.dy[j - 1], dzk = ax.dz[k - 1];
    s[0] += dmul(dmul(dmul(phi[d.ph(i, j, k)], dxi), dyj), dzk);
    s[1] += dmul(dmul(dxi, dyj), dzk);
  }
  CELL_LOOP_END
  double out[2];
  if (grid_reduce<2, 0>(s, m, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) S->mean = out[0] / out[1];
  }
}
__global__ void k_gauge_sub(Dims d, const int32_t* __restrict__ solid, double* __restrict__ phi,
                            const SolveScalars* S) {
  const double mean = S->mean;
  CELL_LOOP_BEGIN
  const long long p = d.ph(i, j, k);
  if (solid[p] == 0) phi[p] = dsub(phi[p], mean);
  CELL_LOOP_END
}
cudaError_t launch_gauge(const Dims& d, const int32_t* solid, double* phi, const Axes& ax, SolveScalars* S,
                         const RedBuf& rb, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_gauge_sum<<<L.grid, L.block, 0, st>>>(d, solid, phi, ax, S, rb); note_launch();
  k_gauge_sub<<<L.grid, L.block, 0, st>>>(d, solid, phi, S); note_launch();
  return cudaGetLastError();
}

// enforce_stairstep_compatibility_3d, src/fpm_stairstep_mpi_3d.f90:41-92.
// Sums: source (fluid rhs V), flux through fluid outer and body faces, and
// outer fluid face area.  phase 0 computes the correction; phase 1 the
// imbalance after the shift.
__global__ void k_compat_sums(Dims d, const double* __restrict__ rhs, const int32_t* __restrict__ solid, Bg bg,
                              Faces f, Axes ax, int phase, SolveScalars* S, RedBuf rb) {
  double s[3] = {0.0, 0.0, 0.0}, m[1] = {0.0};
  CELL_LOOP_BEGIN
  if (solid[d.ph(i, j, k)] == 0) {
    const double dxi = ax.dx[i - 1], dyj = ax.dy[j - 1], dzk = ax.dz[k - 1];
    if (phase == 0) s[0] += dmul(dmul(dmul(rhs[d.in(i, j, k)], dxi), dyj), dzk);
    double flux = 0, area = 0, a = dmul(dyj, dzk);
    if (i == 1) { flux -= f.xlo[d.xf(j, k)] * a; area += a; }
    else if (solid[d.ph(i - 1, j, k)] != 0) flux -= bg.x * a;
    if (i == d.nx) { flux += f.xhi[d.xf(j, k)] * a; area += a; }
    else if (solid[d.ph(i + 1, j, k)] != 0) flux += bg.x * a;
    a = dmul(dxi, dzk);
    if (j == 1) { flux -= f.ylo[d.yf(i, k)] * a; area += a; }
    else if (solid[d.ph(i, j - 1, k)] != 0) flux -= bg.y * a;
    if (j == d.ny) { flux += f.yhi[d.yf(i, k)] * a; area += a; }
    else if (solid[d.ph(i, j + 1, k)] != 0) flux += bg.y * a;
    a = dmul(dxi, dyj);
    if (k == 1) { flux -= f.zlo[d.zf(i, j)] * a; area += a; }
    else if (solid[d.ph(i, j, k - 1)] != 0) flux -= bg.z * a;
    if (k == d.nz) { flux += f.zhi[d.zf(i, j)] * a; area += a; }
    else if (solid[d.ph(i, j, k + 1)] != 0) flux += bg.z * a;
    s[1] += flux;
    s[2] += area;
  }
  CELL_LOOP_END
  double out[3];
  if (grid_reduce<3, 0>(s, m, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      if (phase == 0) {
        S->red[0] = out[0];  // source
        S->red[2] = out[2];  // area
        S->corr = out[2] > 0 ? -(out[1] - out[0]) / out[2] : 0.0;
      } else {
        S->red[1] = out[1] - S->red[0];  // imbalance
      }
    }
  }
}
__global__ void k_shift_faces(Dims d, Faces f, const SolveScalars* S) {
  const double c = S->corr;
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n < (long long)d.ny * d.nz) { f.xlo[n] -= c; f.xhi[n] += c; }
  if (n < (long long)d.nx * d.nz) { f.ylo[n] -= c; f.yhi[n] += c; }
  if (n < (long long)d.nx * d.ny) { f.zlo[n] -= c; f.zhi[n] += c; }
}
cudaError_t launch_compat(const Dims& d, const double* rhs, const int32_t* solid, const double bg[3], Faces f,
                          const Axes& ax, SolveScalars* S, const RedBuf& rb, cudaStream_t st) {
  Launch L = cells_launch(d);
  Bg b{bg[0], bg[1], bg[2]};
  k_compat_sums<<<L.grid, L.block, 0, st>>>(d, rhs, solid, b, f, ax, 0, S, rb); note_launch();
  long long nmax = (long long)d.ny * d.nz;
  if ((long long)d.nx * d.nz > nmax) nmax = (long long)d.nx * d.nz;
  if ((long long)d.nx * d.ny > nmax) nmax = (long long)d.nx * d.ny;
  k_shift_faces<<<(unsigned)((nmax + 255) / 256), 256, 0, st>>>(d, f, S); note_launch();
  k_compat_sums<<<L.grid, L.block, 0, st>>>(d, rhs, solid, b, f, ax, 1, S, rb); note_launch();
  return cudaGetLastError();
}

// face_gradients, src/fpm_stairstep_mpi_3d.f90:472-497.
__device__ __forceinline__ void face_gradients(const Dims& d, const double* __restrict__ phi,
                                               const int32_t* __restrict__ solid, const Bg& bg, const Faces& f,
                                               const Axes& ax, const double* xc, const double* yc, int i, int j,
                                               int k, double g[6]) {
  const long long p = d.ph(i, j, k), px = d.nx + 2, pl = d.plane();
  const double pc = phi[p];
  if (i == 1) g[0] = f.xlo[d.xf(j, k)];
  else if (solid[p - 1] != 0) g[0] = bg.x;
  else g[0] = ddiv(dsub(pc, phi[p - 1]), dsub(xc[i], xc[i - 1]));
  if (i == d.nx) g[1] = f.xhi[d.xf(j, k)];
  else if (solid[p + 1] != 0) g[1] = bg.x;
  else g[1] = ddiv(dsub(phi[p + 1], pc), dsub(xc[i + 1], xc[i]));
  if (j == 1) g[2] = f.ylo[d.yf(i, k)];
  else if (solid[p - px] != 0) g[2] = bg.y;
  else g[2] = ddiv(dsub(pc, phi[p - px]), dsub(yc[j], yc[j - 1]));
  if (j == d.ny) g[3] = f.yhi[d.yf(i, k)];
  else if (solid[p + px] != 0) g[3] = bg.y;
  else g[3] = ddiv(dsub(phi[p + px], pc), dsub(yc[j + 1], yc[j]));
  if (k == 1) g[4] = f.zlo[d.zf(i, j)];
  else if (solid[p - pl] != 0) g[4] = bg.z;
  else g[4] = ddiv(dsub(pc, phi[p - pl]), dsub(ax.zc[k - 1], ax.zc[k - 2]));
  if (k == d.nz) g[5] = f.zhi[d.zf(i, j)];
  else if (solid[p + pl] != 0) g[5] = bg.z;
  else g[5] = ddiv(dsub(phi[p + pl], pc), dsub(ax.zc[k], ax.zc[k - 1]));
}

// a / b from y = RN(1/b), correctly rounded: Markstein's correction step
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990): q0 = RN(a y), the remainder
// r = a - b q0 is exact with one FMA, and RN(q0 + r y) is the IEEE quotient
// when y is the correctly rounded reciprocal and no underflow occurs.  Three
// FP64 instructions instead of a full division; the per-cell parity tests
// compare the densities bit for bit with the oracle's IEEE divisions.
__device__ __forceinline__ double div_rcp(double a, double b, double y) {
  const double q0 = __dmul_rn(a, y);
  const double r = __fma_rn(-b, q0, a);
  return __fma_rn(r, y, q0);
}

// face_gradients with the spacing reciprocals rx[i] = 1 / (xc[i] - xc[i-1]),
// ry[j] likewise, rz[k] = 1 / (zc[k] - zc[k-1]) (zc 0-based).
__device__ __forceinline__ void face_gradients_rcp(const Dims& d, const double* __restrict__ phi,
                                                   const int32_t* __restrict__ solid, const Bg& bg, const Faces& f,
                                                   const Axes& ax, const double* __restrict__ rx,
                                                   const double* __restrict__ ry, const double* __restrict__ rz,
                                                   int i, int j, int k, double g[6]) {
  const long long p = d.ph(i, j, k), px = d.nx + 2, pl = d.plane();
  const double* xc = ax.xc;
  const double* yc = ax.yc;
  const double pc = phi[p];
  if (i == 1) g[0] = f.xlo[d.xf(j, k)];
  else if (solid[p - 1] != 0) g[0] = bg.x;
  else g[0] = div_rcp(dsub(pc, phi[p - 1]), dsub(xc[i], xc[i - 1]), rx[i]);
  if (i == d.nx) g[1] = f.xhi[d.xf(j, k)];
  else if (solid[p + 1] != 0) g[1] = bg.x;
  else g[1] = div_rcp(dsub(phi[p + 1], pc), dsub(xc[i + 1], xc[i]), rx[i + 1]);
  if (j == 1) g[2] = f.ylo[d.yf(i, k)];
  else if (solid[p - px] != 0) g[2] = bg.y;
  else g[2] = div_rcp(dsub(pc, phi[p - px]), dsub(yc[j], yc[j - 1]), ry[j]);
  if (j == d.ny) g[3] = f.yhi[d.yf(i, k)];
  else if (solid[p + px] != 0) g[3] = bg.y;
  else g[3] = div_rcp(dsub(phi[p + px], pc), dsub(yc[j + 1], yc[j]), ry[j + 1]);
  if (k == 1) g[4] = f.zlo[d.zf(i, j)];
  else if (solid[p - pl] != 0) g[4] = bg.z;
  else g[4] = div_rcp(dsub(pc, phi[p - pl]), dsub(ax.zc[k - 1], ax.zc[k - 2]), rz[k - 1]);
  if (k == d.nz) g[5] = f.zhi[d.zf(i, j)];
  else if (solid[p + pl] != 0) g[5] = bg.z;
  else g[5] = div_rcp(dsub(phi[p + pl], pc), dsub(ax.zc[k], ax.zc[k - 1]), rz[k]);
}

// stairstep_residual_3d, src/fpm_stairstep_mpi_3d.f90:403-419 -> S->res.
__global__ void k_face_residual(Dims d, const double* __restrict__ phi, const double* __restrict__ rhs,
                                const int32_t* __restrict__ solid, Bg bg, Faces f, Axes ax, SolveScalars* S,
                                RedBuf rb) {
  double s[1] = {0.0}, m[1] = {0.0};
  CELL_LOOP_BEGIN
  if (solid[d.ph(i, j, k)] == 0) {
    double g[6];
    face_gradients(d, phi, solid, bg, f, ax, ax.xc, ax.yc, i, j, k, g);
    double t = dadd(dadd(ddiv(dsub(g[1], g[0]), ax.dx[i - 1]), ddiv(dsub(g[3], g[2]), ax.dy[j - 1])),
                    ddiv(dsub(g[5], g[4]), ax.dz[k - 1]));
    t = dsub(t, rhs[d.in(i, j, k)]);
    m[0] = fmax(m[0], fabs(t));
  }
  CELL_LOOP_END
  double out[1];
  if (grid_reduce<0, 1>(s, m, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) S->res = out[0];
  }
}
cudaError_t launch_face_residual(const Dims& d, const double* phi, const double* rhs, const int32_t* solid,
                                 const double bg[3], const Faces& f, const Axes& ax, SolveScalars* S,
                                 const RedBuf& rb, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_face_residual<<<L.grid, L.block, 0, st>>>(d, phi, rhs, solid, Bg{bg[0], bg[1], bg[2]}, f, ax, S, rb); note_launch();
  return cudaGetLastError();
}

// compute_stairstep_fpm_terms_3d, src/fpm_stairstep_mpi_3d.f90:426-469:
// cell gradient = mean of the two face gradients, vortex = -(omega x u).grad
// phi, advection = -a.grad phi, and their integrals over cells whose centres
// lie strictly inside bounds -> S->red[0..1].
__global__ void k_terms(Dims d, const double* __restrict__ phi, Flow fl, const int32_t* __restrict__ solid, Bg bg,
                        Axes ax, Faces f, double b0, double b1, double b2, double b3, double b4, double b5,
                        TermsOut o, const double* __restrict__ rx, const double* __restrict__ ry,
                        const double* __restrict__ rz, SolveScalars* S, RedBuf rb) {
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  CELL_LOOP_BEGIN
  const long long cc = d.in(i, j, k);
  double g[6];
  face_gradients_rcp(d, phi, solid, bg, f, ax, rx, ry, rz, i, j, k, g);
  const double mask = solid[d.ph(i, j, k)] == 0 ? 1.0 : 0.0;
  const double hm = dmul(mask, 0.5);
  const double gx = dmul(hm, dadd(g[0], g[1]));
  const double gy = dmul(hm, dadd(g[2], g[3]));
  const double gz = dmul(hm, dadd(g[4], g[5]));
  o.gx[cc] = gx;
  o.gy[cc] = gy;
  o.gz[cc] = gz;
  const double u = fl.u[cc], v = fl.v[cc], w = fl.w[cc], ox = fl.ox[cc], oy = fl.oy[cc], oz = fl.oz[cc];
  const double cx = dsub(dmul(w, oy), dmul(v, oz));
  const double cy = dsub(dmul(u, oz), dmul(w, ox));
  const double cz = dsub(dmul(v, ox), dmul(u, oy));
  const double vort = -dadd(dadd(dmul(cx, gx), dmul(cy, gy)), dmul(cz, gz));
  const double adv = -dadd(dadd(dmul(fl.ax[cc], gx), dmul(fl.ay[cc], gy)), dmul(fl.az[cc], gz));
  o.vortex[cc] = vort;
  o.advection[cc] = adv;
  const double xci = ax.xc[i], ycj = ax.yc[j], zck = ax.zc[k - 1];
  const bool inside = xci > b0 && xci < b1 && ycj > b2 && ycj < b3 && zck > b4 && zck < b5;
  const double vol = inside ? dmul(dmul(ax.dx[i - 1], ax.dy[j - 1]), ax.dz[k - 1]) : 0.0;
  s[0] += dmul(vol, vort);
  s[1] += dmul(vol, adv);
  CELL_LOOP_END
  double out[2];
  if (grid_reduce<2, 0>(s, m, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      S->red[0] = out[0];
      S->red[1] = out[1];
    }
  }
}
// Spacing reciprocals for face_gradients_rcp: rx[i] = 1 / (xc[i] - xc[i-1])
// for i = 1 .. nx+1, ry likewise, rz[k] = 1 / (zc[k] - zc[k-1]) for
// k = 1 .. nz-1 (IEEE divisions; entry 0 unused).
__global__ void k_spacing_rcp(Dims d, Axes ax, double* rx, double* ry, double* rz) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < (d.nx + 2) + (d.ny + 2) + d.nz;
       t += gridDim.x * blockDim.x) {
    if (t < d.nx + 2) {
      rx[t] = t >= 1 ? ddiv(1.0, dsub(ax.xc[t], ax.xc[t - 1])) : 0.0;
    } else if (t < d.nx + 2 + d.ny + 2) {
      const int j = t - (d.nx + 2);
      ry[j] = j >= 1 ? ddiv(1.0, dsub(ax.yc[j], ax.yc[j - 1])) : 0.0;
    } else {
      const int k = t - (d.nx + 2) - (d.ny + 2);
      rz[k] = k >= 1 ? ddiv(1.0, dsub(ax.zc[k], ax.zc[k - 1])) : 0.0;
    }
  }
}

cudaError_t launch_terms(const Dims& d, const double* phi, const Flow& fl, const int32_t* solid, const double bg[3],
                         const Axes& ax, const Faces& f, const double bounds[6], const TermsOut& o, double* rcp,
                         SolveScalars* S, const RedBuf& rb, cudaStream_t st) {
  double* rx = rcp;
  double* ry = rx + (d.nx + 2);
  double* rz = ry + (d.ny + 2);
  const int nr = (d.nx + 2) + (d.ny + 2) + d.nz;
  k_spacing_rcp<<<(nr + 255) / 256, 256, 0, st>>>(d, ax, rx, ry, rz); note_launch();
  Launch L = cells_launch(d);
  k_terms<<<L.grid, L.block, 0, st>>>(d, phi, fl, solid, Bg{bg[0], bg[1], bg[2]}, ax, f, bounds[0], bounds[1],
                                      bounds[2], bounds[3], bounds[4], bounds[5], o, rx, ry, rz, S, rb);
  note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
