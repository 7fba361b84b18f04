// Learned initial guess for the stair-step solve: network inputs from the
// solver's own operator, the network's output scaled by an A-norm projection,
// and the fallback test.
//
// Inputs (voxel order = the solver's compact cell order): fluid flag (diag > 0,
// so isolated or solid cells read as solid), w_min/dx, w_min/dy, w_min/dz
// (w_min = smallest cell width of the grid), and b = V src (the PCG right-hand
// side) divided by max |b|.
//
// The network output y (FP32) is used as phi0 = gamma y_f, y_f = y on fluid
// cells and 0 elsewhere, with gamma = (y_f . b) / (y_f . A y_f): the multiple
// of y_f closest to the solution in the energy norm.  The guess is kept only
// if it is closer to the solution than the caller's phi in the norm CG
// minimises, ||phi - phi*||_A, compared through the energy
// E(phi) = phi.A phi / 2 - phi.b = ||phi - phi*||_A^2 / 2 + const; otherwise
// it is discarded (a fallback) and the solve starts from the caller's phi.
#include "fpm_internal.h"

namespace fpm {

namespace {

__global__ void k_learn_prep(Dims d, const double* __restrict__ src, const double* __restrict__ diag,
                             const double* __restrict__ dx, const double* __restrict__ dy,
                             const double* __restrict__ dz, uint8_t* __restrict__ fluid, float* __restrict__ b,
                             double* partials, unsigned int* ticket, double* bmax) {
  double s[1] = {0.0}, m[1] = {0.0};
  const long long n = d.ncell();
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % d.nx) + 1, j = (int)((c / d.nx) % d.ny) + 1, k = (int)(c / ((long long)d.nx * d.ny)) + 1;
    const bool fl = diag[c] > 0;
    const double v = fl ? dx[i - 1] * dy[j - 1] * dz[k - 1] * src[c] : 0.0;
    fluid[c] = fl ? 1 : 0;
    b[c] = (float)v;
    m[0] = fmax(m[0], fabs(v));
  }
  double out[1];
  if (grid_reduce<0, 1>(s, m, partials, ticket, out) && lin_tid() == 0) *bmax = out[0];
}

__global__ void k_learn_scale(long long n, float* __restrict__ b, const double* __restrict__ bmax) {
  const double m = *bmax;
  const float inv = m > 0 ? (float)(1.0 / m) : 0.f;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
    b[c] *= inv;
}

// One block: w_min over the three axes, then w_min / width per axis.
__global__ void k_learn_metric(int nx, int ny, int nz, const double* __restrict__ dx, const double* __restrict__ dy,
                               const double* __restrict__ dz, float* __restrict__ mx, float* __restrict__ my,
                               float* __restrict__ mz) {
  __shared__ double sh[32];
  double w = 1e300;
  for (int q = threadIdx.x; q < nx + ny + nz; q += blockDim.x) {
    const double x = q < nx ? dx[q] : (q < nx + ny ? dy[q - nx] : dz[q - nx - ny]);
    w = fmin(w, x);
  }
  for (int o = 16; o > 0; o >>= 1) w = fmin(w, __shfl_xor_sync(0xffffffffu, w, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = w;
  __syncthreads();
  if (threadIdx.x < 32) {
    w = threadIdx.x < (blockDim.x + 31) / 32 ? sh[threadIdx.x] : 1e300;
    for (int o = 16; o > 0; o >>= 1) w = fmin(w, __shfl_xor_sync(0xffffffffu, w, o));
    if (threadIdx.x == 0) sh[0] = w;
  }
  __syncthreads();
  w = sh[0];
  for (int q = threadIdx.x; q < nx; q += blockDim.x) mx[q] = (float)(w / dx[q]);
  for (int q = threadIdx.x; q < ny; q += blockDim.x) my[q] = (float)(w / dy[q]);
  for (int q = threadIdx.x; q < nz; q += blockDim.x) mz[q] = (float)(w / dz[q]);
}

// y.b and y.(A y) over fluid cells, A y = V (diag y - sum c y_nb).
__global__ void k_learn_dots(Dims d, const float* __restrict__ y, const double* __restrict__ src,
                             const double* __restrict__ diag, Coefs cf, Axes ax, double* partials,
                             unsigned int* ticket, double* out2) {
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  const long long n = d.ncell();
  auto yv = [&](int i, int j, int k) -> double {
    if (i < 1 || i > d.nx || j < 1 || j > d.ny || k < 1 || k > d.nz) return 0.0;
    const long long c = d.in(i, j, k);
    return diag[c] > 0 ? (double)y[c] : 0.0;
  };
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    if (!(diag[c] > 0)) continue;
    const int i = (int)(c % d.nx) + 1, j = (int)((c / d.nx) % d.ny) + 1, k = (int)(c / ((long long)d.nx * d.ny)) + 1;
    const double vol = ax.dx[i - 1] * ax.dy[j - 1] * ax.dz[k - 1];
    const double yc = y[c];
    const double nb = cf.cw[i - 1] * yv(i - 1, j, k) + cf.ce[i - 1] * yv(i + 1, j, k) + cf.cs[j - 1] * yv(i, j - 1, k) +
                      cf.cn[j - 1] * yv(i, j + 1, k) + cf.cb[k - 1] * yv(i, j, k - 1) + cf.ct[k - 1] * yv(i, j, k + 1);
    s[0] += yc * vol * src[c];
    s[1] += yc * vol * (diag[c] * yc - nb);
  }
  double o[2];
  if (grid_reduce<2, 0>(s, m, partials, ticket, o) && lin_tid() == 0) {
    out2[0] = o[0];
    out2[1] = o[1];
  }
}

// phi(interior) = gamma y on fluid cells, 0 on solid cells (gamma = yb / yAy).
__global__ void k_learn_apply(Dims d, const float* __restrict__ y, const double* __restrict__ diag,
                              const double* __restrict__ dots, double* __restrict__ phi) {
  const double yb = dots[0], yay = dots[1];
  const double g = yay > 0 ? yb / yay : 0.0;
  const long long n = d.ncell();
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % d.nx) + 1, j = (int)((c / d.nx) % d.ny) + 1, k = (int)(c / ((long long)d.nx * d.ny)) + 1;
    phi[d.ph(i, j, k)] = diag[c] > 0 ? g * (double)y[c] : 0.0;
  }
}

// phi.b and phi.(A phi) for a padded FP64 phi (zero in solid cells and the
// physical halo), b = V src, A phi = V (diag phi - sum c phi_nb).
__global__ void k_energy(Dims d, const double* __restrict__ phi, const double* __restrict__ src,
                         const double* __restrict__ diag, Coefs cf, Axes ax, double* partials, unsigned int* ticket,
                         double* out2) {
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  const long long n = d.ncell(), px = d.nx + 2, pl = d.plane();
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    if (!(diag[c] > 0)) continue;
    const int i = (int)(c % d.nx) + 1, j = (int)((c / d.nx) % d.ny) + 1, k = (int)(c / ((long long)d.nx * d.ny)) + 1;
    const long long p = d.ph(i, j, k);
    const double vol = ax.dx[i - 1] * ax.dy[j - 1] * ax.dz[k - 1];
    const double f = phi[p];
    const double nb = cf.cw[i - 1] * phi[p - 1] + cf.ce[i - 1] * phi[p + 1] + cf.cs[j - 1] * phi[p - px] +
                      cf.cn[j - 1] * phi[p + px] + cf.cb[k - 1] * phi[k > 1 ? p - pl : p] +
                      cf.ct[k - 1] * phi[k < d.nz ? p + pl : p];
    s[0] += f * vol * src[c];
    s[1] += f * vol * (diag[c] * f - nb);
  }
  double o[2];
  if (grid_reduce<2, 0>(s, m, partials, ticket, o) && lin_tid() == 0) {
    out2[0] = o[0];
    out2[1] = o[1];
  }
}

// ---------------------------------------------------------------- learned flexible CG
// The network as the preconditioner of a flexible CG (FPM_METHOD_FCG_LEARNED):
// z = M(r) with y = net(fluid, metrics, r / max|r|),
//   z1 = gamma y_f, gamma = (y_f . r) / (y_f . A y_f)   (the multiple of y_f
//        closest to A^-1 r in the energy norm),
//   z  = z1 + rdiag (r - A z1)                           (one diagonal step on
//        what the network left).
// r is the PCG residual in V units (b - A phi with b = V src), so it has the
// units of the network's training input b.

// b = (float) r on fluid cells, 0 elsewhere; *bmax = max |r|.
__global__ void k_fcg_prep(Dims d, const double* __restrict__ r, const double* __restrict__ diag,
                           float* __restrict__ b, double* partials, unsigned int* ticket, double* bmax) {
  double s[1] = {0.0}, m[1] = {0.0};
  const long long n = d.ncell();
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const double v = diag[c] > 0 ? r[c] : 0.0;
    b[c] = (float)v;
    m[0] = fmax(m[0], fabs(v));
  }
  double out[1];
  if (grid_reduce<0, 1>(s, m, partials, ticket, out) && lin_tid() == 0) *bmax = out[0];
}

// ay = A y_f (0 off the fluid), out2 = (y_f . r, y_f . ay).
__global__ void k_fcg_dots(Dims d, const float* __restrict__ y, const double* __restrict__ r,
                           const double* __restrict__ diag, Coefs cf, Axes ax, double* __restrict__ ay,
                           double* partials, unsigned int* ticket, double* out2) {
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  const long long n = d.ncell();
  auto yv = [&](int i, int j, int k) -> double {
    if (i < 1 || i > d.nx || j < 1 || j > d.ny || k < 1 || k > d.nz) return 0.0;
    const long long c = d.in(i, j, k);
    return diag[c] > 0 ? (double)y[c] : 0.0;
  };
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    if (!(diag[c] > 0)) {
      ay[c] = 0.0;
      continue;
    }
    const int i = (int)(c % d.nx) + 1, j = (int)((c / d.nx) % d.ny) + 1, k = (int)(c / ((long long)d.nx * d.ny)) + 1;
    const double vol = ax.dx[i - 1] * ax.dy[j - 1] * ax.dz[k - 1];
    const double yc = y[c];
    const double nb = cf.cw[i - 1] * yv(i - 1, j, k) + cf.ce[i - 1] * yv(i + 1, j, k) + cf.cs[j - 1] * yv(i, j - 1, k) +
                      cf.cn[j - 1] * yv(i, j + 1, k) + cf.cb[k - 1] * yv(i, j, k - 1) + cf.ct[k - 1] * yv(i, j, k + 1);
    const double a = vol * (diag[c] * yc - nb);
    ay[c] = a;
    s[0] += yc * r[c];
    s[1] += yc * a;
  }
  double o[2];
  if (grid_reduce<2, 0>(s, m, partials, ticket, o) && lin_tid() == 0) {
    out2[0] = o[0];
    out2[1] = o[1];
  }
}

// z = gamma y_f + rdiag (r - gamma ay), gamma = dots[0] / dots[1] (0 when the
// network's output has no energy); (zr, zr_prev) = (z . r, z . r_prev).
__global__ void k_fcg_z(Dims d, const float* __restrict__ y, const double* __restrict__ r,
                        const double* __restrict__ rprev, const double* __restrict__ ay,
                        const double* __restrict__ diag, const double* __restrict__ rdiag,
                        const double* __restrict__ dots, double* __restrict__ z, double* partials,
                        unsigned int* ticket, double* out2) {
  const double g = dots[1] > 0 ? dots[0] / dots[1] : 0.0;
  double s[2] = {0.0, 0.0}, m[1] = {0.0};
  const long long n = d.ncell();
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    double zv = 0.0;
    if (diag[c] > 0) zv = g * (double)y[c] + rdiag[c] * (r[c] - g * ay[c]);
    z[c] = zv;
    s[0] += zv * r[c];
    s[1] += zv * rprev[c];
  }
  double o[2];
  if (grid_reduce<2, 0>(s, m, partials, ticket, o) && lin_tid() == 0) {
    out2[0] = o[0];
    out2[1] = o[1];
  }
}

// p = z + beta p (padded p); beta = 0 restarts the direction.
__global__ void k_fcg_direction(Dims d, const double* __restrict__ z, double* __restrict__ p, double beta) {
  const long long n = d.ncell();
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % d.nx) + 1, j = (int)((c / d.nx) % d.ny) + 1, k = (int)(c / ((long long)d.nx * d.ny)) + 1;
    const long long pp = d.ph(i, j, k);
    p[pp] = beta == 0.0 ? z[c] : z[c] + beta * p[pp];
  }
}

// phi += alpha p; r_prev = r; r -= alpha q (alpha from the spmv's scalars).
__global__ void k_fcg_update(Dims d, double* __restrict__ phi, const double* __restrict__ p,
                             const double* __restrict__ q, double* __restrict__ r, double* __restrict__ rprev,
                             const SolveScalars* S) {
  if (S->halt) return;
  const double alpha = S->alpha;
  const long long n = d.ncell();
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % d.nx) + 1, j = (int)((c / d.nx) % d.ny) + 1, k = (int)(c / ((long long)d.nx * d.ny)) + 1;
    const long long pp = d.ph(i, j, k);
    phi[pp] = phi[pp] + alpha * p[pp];
    rprev[c] = r[c];
    r[c] = r[c] - alpha * q[c];
  }
}

unsigned blocks_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 16) b = 152LL * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

cudaError_t launch_learn_inputs(const Dims& d, const double* src, const double* diag, const Axes& ax, uint8_t* fluid,
                                float* mx, float* my, float* mz, float* b, double* bmax, const RedBuf& rb,
                                cudaStream_t st) {
  const unsigned nb = blocks_for(d.ncell());
  if ((int)nb > rb.max_blocks) return cudaErrorInvalidValue;
  k_learn_prep<<<nb, 256, 0, st>>>(d, src, diag, ax.dx, ax.dy, ax.dz, fluid, b, rb.partials, rb.ticket, bmax);
  note_launch();
  k_learn_scale<<<blocks_for(d.ncell()), 256, 0, st>>>(d.ncell(), b, bmax);
  note_launch();
  k_learn_metric<<<1, 256, 0, st>>>(d.nx, d.ny, d.nz, ax.dx, ax.dy, ax.dz, mx, my, mz);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_learn_apply(const Dims& d, const float* y, const double* src, const double* diag, const Coefs& c,
                               const Axes& ax, double* phi, double* dots, const RedBuf& rb, cudaStream_t st) {
  const unsigned nb = blocks_for(d.ncell());
  if ((int)nb > rb.max_blocks) return cudaErrorInvalidValue;
  k_learn_dots<<<nb, 256, 0, st>>>(d, y, src, diag, c, ax, rb.partials, rb.ticket, dots);
  note_launch();
  k_learn_apply<<<blocks_for(d.ncell()), 256, 0, st>>>(d, y, diag, dots, phi);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_fcg_precond(const Dims& d, void* net, const double* r, const double* rprev, const double* diag,
                               const double* rdiag, const Coefs& c, const Axes& ax, const FcgWork& w, double* z,
                               const RedBuf& rb, cudaStream_t st, std::string* err, int* status) {
  const unsigned nb = blocks_for(d.ncell());
  *status = 0;
  if ((int)nb > rb.max_blocks) return cudaErrorInvalidValue;
  k_fcg_prep<<<nb, 256, 0, st>>>(d, r, diag, w.b, rb.partials, rb.ticket, w.sc);
  note_launch();
  k_learn_scale<<<nb, 256, 0, st>>>(d.ncell(), w.b, w.sc);
  note_launch();
  const int rc = net::forward_into(net, d.nx, d.ny, d.nz, w.fluid, w.mx, w.my, w.mz, w.b, w.y, st, err);
  if (rc != 0) {
    *status = rc;
    return cudaSuccess;
  }
  k_fcg_dots<<<nb, 256, 0, st>>>(d, w.y, r, diag, c, ax, w.ay, rb.partials, rb.ticket, w.sc + 2);
  note_launch();
  k_fcg_z<<<nb, 256, 0, st>>>(d, w.y, r, rprev, w.ay, diag, rdiag, w.sc + 2, z, rb.partials, rb.ticket, w.sc + 4);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_fcg_direction(const Dims& d, const double* z, double* p, double beta, cudaStream_t st) {
  k_fcg_direction<<<blocks_for(d.ncell()), 256, 0, st>>>(d, z, p, beta);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_fcg_update(const Dims& d, double* phi, const double* p, const double* q, double* r, double* rprev,
                              const SolveScalars* S, cudaStream_t st) {
  k_fcg_update<<<blocks_for(d.ncell()), 256, 0, st>>>(d, phi, p, q, r, rprev, S);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_energy(const Dims& d, const double* phi, const double* src, const double* diag, const Coefs& c,
                          const Axes& ax, double* out2, const RedBuf& rb, cudaStream_t st) {
  const unsigned nb = blocks_for(d.ncell());
  if ((int)nb > rb.max_blocks) return cudaErrorInvalidValue;
  k_energy<<<nb, 256, 0, st>>>(d, phi, src, diag, c, ax, rb.partials, rb.ticket, out2);
  note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
