// C ABI (include/fpm_capi.h): host-side drivers of the stair-step solve and
// force terms.  The control flow of each solver follows the reference routine
// it replaces; per-iteration scalars stay on the device, so the host only
// synchronises once per convergence check.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/fpm_capi.h"
#include "fpm_internal.h"

namespace fpm {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

struct Error {
  int code;
  std::string msg;
};

#define CUDA_TRY(expr)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (expr);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      throw Error{FPM_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)};             \
  } while (0)

static void require_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n < 1)
    throw Error{FPM_E_NO_DEVICE, std::string("no CUDA device: ") + (e == cudaSuccess ? "count is 0" : cudaGetErrorString(e))};
}

// Stream-ordered scratch allocations, released when the scope ends.
class Scratch {
 public:
  explicit Scratch(cudaStream_t st) : st_(st) {}
  ~Scratch() {
    for (void* p : ptrs_) cudaFreeAsync(p, st_);
  }
  template <class T>
  T* get(size_t n) {
    void* p = nullptr;
    size_t bytes = (n ? n : 1) * sizeof(T);
    CUDA_TRY(cudaMallocAsync(&p, bytes, st_));
    ptrs_.push_back(p);
    return static_cast<T*>(p);
  }
  template <class T>
  T* upload(const T* host, size_t n) {
    T* d = get<T>(n);
    if (n) CUDA_TRY(cudaMemcpyAsync(d, host, n * sizeof(T), cudaMemcpyHostToDevice, st_));
    return d;
  }

 private:
  cudaStream_t st_;
  std::vector<void*> ptrs_;
};

static void download(void* host, const void* dev, size_t bytes, cudaStream_t st) {
  if (bytes) CUDA_TRY(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, st));
}

// Pinned per-thread copy of the device scalars.
static SolveScalars* host_scalars() {
  static thread_local SolveScalars* h = nullptr;
  if (!h) CUDA_TRY(cudaMallocHost(&h, sizeof(SolveScalars)));
  return h;
}
static const SolveScalars& read_scalars(const SolveScalars* S, cudaStream_t st) {
  SolveScalars* h = host_scalars();
  CUDA_TRY(cudaMemcpyAsync(h, S, sizeof(SolveScalars), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return *h;
}

struct Common {
  SolveScalars* S;
  RedBuf rb;
};
static Common make_common(Scratch& A, const Dims& d, cudaStream_t st) {
  Common c;
  c.S = A.get<SolveScalars>(1);
  CUDA_TRY(cudaMemsetAsync(c.S, 0, sizeof(SolveScalars), st));
  Launch L = cells_launch(d);
  int nb = (int)(L.grid.x * L.grid.y * L.grid.z);
  c.rb.max_blocks = nb;
  c.rb.partials = A.get<double>((size_t)4 * nb);
  c.rb.ticket = A.get<unsigned int>(1);
  CUDA_TRY(cudaMemsetAsync(c.rb.ticket, 0, sizeof(unsigned int), st));
  return c;
}

static void check_dims(int nx, int ny, int nz) {
  if (nx < 1 || ny < 1 || nz < 2) throw Error{FPM_E_SIZE, "stair-step solve needs nz>=2 and nonempty ranks"};
  // Cell indices in the launch geometry are 32-bit per axis; sizes are 64-bit.
  if ((long long)nx * ny * nz > (1LL << 40)) throw Error{FPM_E_LIMIT, "grid too large"};
}

struct Trace {
  explicit Trace(const char* name) { nvtxRangePushA(name); }
  ~Trace() { nvtxRangePop(); }
};

// ---------------------------------------------------------------- solve
struct SolveArgs {
  double* phi;
  const double* rhs;
  const int32_t* solid;
  double bg[3];
  Faces f;
  Axes ax;
  int nx, ny, nz;
  double tol;
  int max_sweeps, ci, method;
};

// PCG with the control flow of pcg_iterate (src/fpm_stairstep_mpi_3d.f90:235-293):
// breakdown restarts once from the steepest-descent direction, the recursive
// residual is replaced by the true one at every check, and the iteration stops
// after 50 checks without a 1% improvement.  Iterations between two checks run
// back to back on the device; a breakdown inside a chunk halts the remaining
// kernels of the chunk (device flag) and is handled here at the chunk end.
static double pcg_loop(const SolveArgs& a, const Dims& d, double* p, const double* src, const double* diag,
                       const double* rdiag, const Coefs& c, Scratch& A, Common& cm, int* sweeps, cudaStream_t st) {
  double* r = A.get<double>(d.ncell());
  double* q = A.get<double>(d.ncell());
  CUDA_TRY(launch_true_residual(d, a.phi, src, diag, rdiag, r, p, c, a.ax, 1, cm.S, cm.rb, st));
  double res = read_scalars(cm.S, st).res;
  const int ci = a.ci < 1 ? 1 : a.ci;
  int it = 0, restarts = 0, stalled = 0;
  double best = res;
  int sw = 0;
  while (sw < a.max_sweeps && res > a.tol) {
    int chunk = ci - it % ci;
    if (chunk > a.max_sweeps - sw) chunk = a.max_sweeps - sw;
    CUDA_TRY(cudaMemsetAsync(&cm.S->iters, 0, sizeof(int), st));
    for (int n = 0; n < chunk; n++)
      CUDA_TRY(launch_pcg_iteration(d, a.phi, p, q, r, diag, rdiag, c, a.ax, cm.S, cm.rb, st));
    const SolveScalars& h = read_scalars(cm.S, st);
    const int done = h.iters, halt = h.halt;
    sw += done;
    it += done;
    if (done > 0) restarts = 0;
    if (halt == 1) {
      restarts++;
      if (restarts > 1) break;
      CUDA_TRY(launch_true_residual(d, a.phi, src, diag, rdiag, r, p, c, a.ax, 1, cm.S, cm.rb, st));
      res = read_scalars(cm.S, st).res;
      continue;
    }
    if (halt == 2) break;
    CUDA_TRY(launch_true_residual(d, a.phi, src, diag, rdiag, r, p, c, a.ax, 0, cm.S, cm.rb, st));
    res = read_scalars(cm.S, st).res;
    if (res < 0.99 * best) {
      best = res;
      stalled = 0;
    } else {
      stalled++;
    }
    if (stalled >= 50 || !(res == res)) break;
  }
  *sweeps = sw;
  return res;
}

// jacobi_iterate (src/fpm_stairstep_mpi_3d.f90:200-225): sweeps in chunks of
// check_interval, max-norm residual after each chunk.  The two buffers swap
// roles instead of copying back; every sweep reads the latest iterate, so the
// values are those of the reference's ping-pong with copy.
static void jacobi_loop_f64(const SolveArgs& a, const Dims& d, double* next, const double* src, const double* diag,
                            const double* rdiag, const Coefs& c, Common& cm, int* sweeps, cudaStream_t st) {
  double *cur = a.phi, *oth = next;
  double residual = HUGE_VAL;
  int sw = 0;
  const int ci = a.ci < 1 ? 1 : a.ci;
  while (sw < a.max_sweeps && residual > a.tol) {
    int nsteps = ci < a.max_sweeps - sw ? ci : a.max_sweeps - sw;
    for (int s = 0; s < nsteps; s++) {
      CUDA_TRY(launch_jacobi_f64(d, cur, oth, src, rdiag, c, st));
      std::swap(cur, oth);
    }
    sw += nsteps;
    CUDA_TRY(launch_operator_residual(d, cur, src, diag, c, cm.S, cm.rb, st));
    residual = read_scalars(cm.S, st).res;
  }
  if (cur != a.phi) CUDA_TRY(launch_copy_interior(d, cur, a.phi, st));
  *sweeps = sw;
}

// Same iteration in double-float: phi lives as f32 pairs between checks and
// is written back to FP64 phi for each residual check.
static void jacobi_loop_df(const SolveArgs& a, const Dims& d, double* next, const double* src, const double* diag,
                           const double* rdiag, const double* coef, const Coefs& c, Scratch& A, Common& cm,
                           int* sweeps, cudaStream_t st) {
  (void)next;
  const long long np = d.npad(), nc = d.ncell(), ncoef = 2LL * (d.nx + d.ny + d.nz);
  float2* pa = A.get<float2>(np);
  float2* pb = A.get<float2>(np);
  float2* sdf = A.get<float2>(nc);
  float2* rdf = A.get<float2>(nc);
  float2* cdf = A.get<float2>(ncoef);
  CUDA_TRY(launch_to_df(a.phi, pa, np, st));
  CUDA_TRY(launch_to_df(a.phi, pb, np, st));
  CUDA_TRY(launch_to_df(src, sdf, nc, st));
  CUDA_TRY(launch_to_df(rdiag, rdf, nc, st));
  CUDA_TRY(launch_to_df(coef, cdf, ncoef, st));
  float2 *cur = pa, *oth = pb;
  double residual = HUGE_VAL;
  int sw = 0;
  const int ci = a.ci < 1 ? 1 : a.ci;
  while (sw < a.max_sweeps && residual > a.tol) {
    int nsteps = ci < a.max_sweeps - sw ? ci : a.max_sweeps - sw;
    for (int s = 0; s < nsteps; s++) {
      CUDA_TRY(launch_jacobi_df(d, cur, oth, sdf, rdf, cdf, st));
      std::swap(cur, oth);
    }
    sw += nsteps;
    CUDA_TRY(launch_from_df_interior(d, cur, a.phi, st));
    CUDA_TRY(launch_operator_residual(d, a.phi, src, diag, c, cm.S, cm.rb, st));
    residual = read_scalars(cm.S, st).res;
  }
  *sweeps = sw;
}

// solve_stairstep_poisson_3d (src/fpm_stairstep_mpi_3d.f90:106-330), device arrays.
static void solve_dev(const SolveArgs& a, int* sweeps, double* residual, cudaStream_t st) {
  if (a.method != FPM_METHOD_PCG && a.method != FPM_METHOD_JACOBI && a.method != FPM_METHOD_JACOBI_DF)
    throw Error{FPM_E_METHOD, "stair-step method must be pcg or jacobi"};
  check_dims(a.nx, a.ny, a.nz);
  require_device();
  const Dims d{a.nx, a.ny, a.nz};
  Scratch A(st);
  Common cm = make_common(A, d, st);
  Trace t0("stair-step setup");
  double* coef = A.get<double>(2 * (size_t)(a.nx + a.ny + a.nz));
  CUDA_TRY(launch_axis_coefs(a.ax, a.nx, a.ny, a.nz, coef, st));
  Coefs c{coef, coef + a.nx, coef + 2 * a.nx, coef + 2 * a.nx + a.ny, coef + 2 * a.nx + 2 * a.ny,
          coef + 2 * a.nx + 2 * a.ny + a.nz};
  double* next = A.get<double>(d.npad());
  double* src = A.get<double>(d.ncell());
  double* diag = A.get<double>(d.ncell());
  double* rdiag = A.get<double>(d.ncell());
  const bool use_pcg = a.method == FPM_METHOD_PCG;
  CUDA_TRY(launch_build_operator(d, a.rhs, a.solid, a.bg, a.f, c, a.ax, use_pcg, src, diag, rdiag, cm.S, st));
  if (read_scalars(cm.S, st).isolated > 0) throw Error{FPM_E_ISOLATED, "stair-step fluid cell has no fluid neighbour"};
  CUDA_TRY(launch_init_fields(d, a.solid, a.phi, next, st));
  int sw = 0;
  {
    Trace t1("stair-step iterations");
    if (use_pcg) pcg_loop(a, d, next, src, diag, rdiag, c, A, cm, &sw, st);
    else if (a.method == FPM_METHOD_JACOBI) jacobi_loop_f64(a, d, next, src, diag, rdiag, c, cm, &sw, st);
    else jacobi_loop_df(a, d, next, src, diag, rdiag, coef, c, A, cm, &sw, st);
  }
  Trace t2("stair-step gauge");
  CUDA_TRY(launch_gauge(d, a.solid, a.phi, a.ax, cm.S, cm.rb, st));
  CUDA_TRY(launch_operator_residual(d, a.phi, src, diag, c, cm.S, cm.rb, st));
  *residual = read_scalars(cm.S, st).res;
  *sweeps = sw;
}

static size_t nface_x(int ny, int nz) { return (size_t)ny * nz; }
static size_t nface_y(int nx, int nz) { return (size_t)nx * nz; }
static size_t nface_z(int nx, int ny) { return (size_t)nx * ny; }

template <class F>
static int guarded(F&& f) {
  try {
    f();
    g_last_error.clear();
    return FPM_OK;
  } catch (const Error& e) {
    g_last_error = e.msg;
    return e.code;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return FPM_E_CUDA;
  }
}

}  // namespace fpm

using namespace fpm;

extern "C" {

const char* fpm_last_error(void) { return g_last_error.c_str(); }
int fpm_version(void) { return 100; }

void* fpm_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) return nullptr;
  return p;
}
void fpm_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int fpm_exchange_solid_halo_3d(int32_t* solid, int nx, int ny, int nz) {
  return guarded([&] {
    if (!solid) throw Error{FPM_E_ARG, "null solid"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    const Dims d{nx, ny, nz};
    for (int k = 1; k <= nz; k++)
      for (int j = 0; j <= ny + 1; j++) {
        solid[d.ph(0, j, k)] = 0;
        solid[d.ph(nx + 1, j, k)] = 0;
      }
    for (int k = 1; k <= nz; k++)
      for (int i = 0; i <= nx + 1; i++) {
        solid[d.ph(i, 0, k)] = 0;
        solid[d.ph(i, ny + 1, k)] = 0;
      }
  });
}

int fpm_enforce_stairstep_compatibility_3d_dev(const double* rhs, const int32_t* solid, const double* body_grad,
                                               double* xlo, double* xhi, double* ylo, double* yhi, double* zlo,
                                               double* zhi, const double* dx, const double* dy, const double* dz,
                                               int nx, int ny, int nz, double* correction, double* imbalance,
                                               void* stream) {
  return guarded([&] {
    if (!rhs || !solid || !body_grad || !xlo || !xhi || !ylo || !yhi || !zlo || !zhi || !dx || !dy || !dz ||
        !correction || !imbalance)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = (cudaStream_t)stream;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    Common cm = make_common(A, d, st);
    Axes ax{nullptr, nullptr, nullptr, dx, dy, dz};
    Faces f{xlo, xhi, ylo, yhi, zlo, zhi};
    CUDA_TRY(launch_compat(d, rhs, solid, body_grad, f, ax, cm.S, cm.rb, st));
    const SolveScalars& h = read_scalars(cm.S, st);
    if (!(h.red[2] > 0)) throw Error{FPM_E_NO_OUTER_FACE, "stair-step compatibility needs at least one fluid outer face"};
    *correction = h.corr;
    *imbalance = h.red[1];
  });
}

int fpm_enforce_stairstep_compatibility_3d(const double* rhs, const int32_t* solid, const double* body_grad,
                                           double* xlo, double* xhi, double* ylo, double* yhi, double* zlo,
                                           double* zhi, const double* dx, const double* dy, const double* dz, int nx,
                                           int ny, int nz, double* correction, double* imbalance) {
  return guarded([&] {
    if (!rhs || !solid || !body_grad || !xlo || !xhi || !ylo || !yhi || !zlo || !zhi || !dx || !dy || !dz)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = 0;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    double* drhs = A.upload(rhs, d.ncell());
    int32_t* dsolid = A.upload(solid, d.npad());
    double* f[6];
    double* hf[6] = {xlo, xhi, ylo, yhi, zlo, zhi};
    size_t nf[6] = {nface_x(ny, nz), nface_x(ny, nz), nface_y(nx, nz), nface_y(nx, nz), nface_z(nx, ny),
                    nface_z(nx, ny)};
    for (int m = 0; m < 6; m++) f[m] = A.upload(hf[m], nf[m]);
    double* ddx = A.upload(dx, nx);
    double* ddy = A.upload(dy, ny);
    double* ddz = A.upload(dz, nz);
    int rc = fpm_enforce_stairstep_compatibility_3d_dev(drhs, dsolid, body_grad, f[0], f[1], f[2], f[3], f[4], f[5],
                                                        ddx, ddy, ddz, nx, ny, nz, correction, imbalance, st);
    if (rc != FPM_OK) throw Error{rc, g_last_error};
    for (int m = 0; m < 6; m++) download(hf[m], f[m], nf[m] * sizeof(double), st);
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

int fpm_solve_stairstep_poisson_3d_dev(double* phi, const double* rhs, const int32_t* solid, const double* body_grad,
                                       const double* xlo, const double* xhi, const double* ylo, const double* yhi,
                                       const double* zlo, const double* zhi, const double* xc, const double* yc,
                                       const double* zc, const double* dx, const double* dy, const double* dz, int nx,
                                       int ny, int nz, double tolerance, int max_sweeps, int check_interval,
                                       int method, int* sweeps, double* residual, void* stream) {
  return guarded([&] {
    if (!phi || !rhs || !solid || !body_grad || !xlo || !xhi || !ylo || !yhi || !zlo || !zhi || !xc || !yc || !zc ||
        !dx || !dy || !dz || !sweeps || !residual)
      throw Error{FPM_E_ARG, "null argument"};
    SolveArgs a;
    a.phi = phi;
    a.rhs = rhs;
    a.solid = solid;
    a.bg[0] = body_grad[0];
    a.bg[1] = body_grad[1];
    a.bg[2] = body_grad[2];
    a.f = Faces{const_cast<double*>(xlo), const_cast<double*>(xhi), const_cast<double*>(ylo),
                const_cast<double*>(yhi), const_cast<double*>(zlo), const_cast<double*>(zhi)};
    a.ax = Axes{xc, yc, zc, dx, dy, dz};
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.tol = tolerance;
    a.max_sweeps = max_sweeps;
    a.ci = check_interval;
    a.method = method;
    *sweeps = 0;
    *residual = HUGE_VAL;
    solve_dev(a, sweeps, residual, (cudaStream_t)stream);
  });
}

int fpm_solve_stairstep_poisson_3d(double* phi, const double* rhs, const int32_t* solid, const double* body_grad,
                                   const double* xlo, const double* xhi, const double* ylo, const double* yhi,
                                   const double* zlo, const double* zhi, const double* xc, const double* yc,
                                   const double* zc, const double* dx, const double* dy, const double* dz, int nx,
                                   int ny, int nz, double tolerance, int max_sweeps, int check_interval, int method,
                                   int* sweeps, double* residual) {
  return guarded([&] {
    if (!phi || !rhs || !solid || !body_grad || !xlo || !xhi || !ylo || !yhi || !zlo || !zhi || !xc || !yc || !zc ||
        !dx || !dy || !dz || !sweeps || !residual)
      throw Error{FPM_E_ARG, "null argument"};
    if (method != FPM_METHOD_PCG && method != FPM_METHOD_JACOBI && method != FPM_METHOD_JACOBI_DF)
      throw Error{FPM_E_METHOD, "stair-step method must be pcg or jacobi"};
    check_dims(nx, ny, nz);
    require_device();
    cudaStream_t st = 0;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    double* dphi = A.upload(phi, d.npad());
    const double* drhs = A.upload(rhs, d.ncell());
    const int32_t* dsolid = A.upload(solid, d.npad());
    const double* f[6];
    const double* hf[6] = {xlo, xhi, ylo, yhi, zlo, zhi};
    size_t nf[6] = {nface_x(ny, nz), nface_x(ny, nz), nface_y(nx, nz), nface_y(nx, nz), nface_z(nx, ny),
                    nface_z(nx, ny)};
    for (int m = 0; m < 6; m++) f[m] = A.upload(hf[m], nf[m]);
    const double* dxc = A.upload(xc, nx + 2);
    const double* dyc = A.upload(yc, ny + 2);
    const double* dzc = A.upload(zc, nz);
    const double* ddx = A.upload(dx, nx);
    const double* ddy = A.upload(dy, ny);
    const double* ddz = A.upload(dz, nz);
    int rc = fpm_solve_stairstep_poisson_3d_dev(dphi, drhs, dsolid, body_grad, f[0], f[1], f[2], f[3], f[4], f[5], dxc,
                                                dyc, dzc, ddx, ddy, ddz, nx, ny, nz, tolerance, max_sweeps,
                                                check_interval, method, sweeps, residual, st);
    if (rc != FPM_OK) throw Error{rc, g_last_error};
    download(phi, dphi, d.npad() * sizeof(double), st);
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

int fpm_stairstep_residual_3d(const double* phi, const double* rhs, const int32_t* solid, const double* body_grad,
                              const double* xlo, const double* xhi, const double* ylo, const double* yhi,
                              const double* zlo, const double* zhi, const double* xc, const double* yc,
                              const double* zc, const double* dx, const double* dy, const double* dz, int nx, int ny,
                              int nz, double* value) {
  return guarded([&] {
    if (!phi || !rhs || !solid || !body_grad || !xlo || !xhi || !ylo || !yhi || !zlo || !zhi || !xc || !yc || !zc ||
        !dx || !dy || !dz || !value)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = 0;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    Common cm = make_common(A, d, st);
    const double* dphi = A.upload(phi, d.npad());
    const double* drhs = A.upload(rhs, d.ncell());
    const int32_t* dsolid = A.upload(solid, d.npad());
    double* f[6];
    const double* hf[6] = {xlo, xhi, ylo, yhi, zlo, zhi};
    size_t nf[6] = {nface_x(ny, nz), nface_x(ny, nz), nface_y(nx, nz), nface_y(nx, nz), nface_z(nx, ny),
                    nface_z(nx, ny)};
    for (int m = 0; m < 6; m++) f[m] = A.upload(hf[m], nf[m]);
    Axes ax{A.upload(xc, nx + 2), A.upload(yc, ny + 2), A.upload(zc, nz),
            A.upload(dx, nx),     A.upload(dy, ny),     A.upload(dz, nz)};
    Faces ff{f[0], f[1], f[2], f[3], f[4], f[5]};
    CUDA_TRY(launch_face_residual(d, dphi, drhs, dsolid, body_grad, ff, ax, cm.S, cm.rb, st));
    *value = read_scalars(cm.S, st).res;
  });
}

int fpm_compute_stairstep_fpm_terms_3d_dev(const double* phi, const double* u, const double* v, const double* w,
                                           const double* ox, const double* oy, const double* oz, const double* ax,
                                           const double* ay, const double* az, const int32_t* solid,
                                           const double* body_grad, const double* xc, const double* yc,
                                           const double* zc, const double* dx, const double* dy, const double* dz,
                                           const double* xlo, const double* xhi, const double* ylo,
                                           const double* yhi, const double* zlo, const double* zhi,
                                           const double* bounds, double* gx, double* gy, double* gz, double* vortex,
                                           double* advection, double* totals, int nx, int ny, int nz, void* stream) {
  return guarded([&] {
    if (!phi || !u || !v || !w || !ox || !oy || !oz || !ax || !ay || !az || !solid || !body_grad || !xc || !yc ||
        !zc || !dx || !dy || !dz || !xlo || !xhi || !ylo || !yhi || !zlo || !zhi || !bounds || !gx || !gy || !gz ||
        !vortex || !advection || !totals)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = (cudaStream_t)stream;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    Common cm = make_common(A, d, st);
    Trace t("stair-step FPM terms");
    Flow fl{u, v, w, ox, oy, oz, ax, ay, az};
    Axes axes{xc, yc, zc, dx, dy, dz};
    Faces f{const_cast<double*>(xlo), const_cast<double*>(xhi), const_cast<double*>(ylo),
            const_cast<double*>(yhi), const_cast<double*>(zlo), const_cast<double*>(zhi)};
    TermsOut o{gx, gy, gz, vortex, advection};
    CUDA_TRY(launch_terms(d, phi, fl, solid, body_grad, axes, f, bounds, o, cm.S, cm.rb, st));
    const SolveScalars& h = read_scalars(cm.S, st);
    totals[0] = h.red[0];
    totals[1] = h.red[1];
  });
}

int fpm_compute_stairstep_fpm_terms_3d(const double* phi, const double* u, const double* v, const double* w,
                                       const double* ox, const double* oy, const double* oz, const double* ax,
                                       const double* ay, const double* az, const int32_t* solid,
                                       const double* body_grad, const double* xc, const double* yc, const double* zc,
                                       const double* dx, const double* dy, const double* dz, const double* xlo,
                                       const double* xhi, const double* ylo, const double* yhi, const double* zlo,
                                       const double* zhi, const double* bounds, double* gx, double* gy, double* gz,
                                       double* vortex, double* advection, double* totals, int nx, int ny, int nz) {
  return guarded([&] {
    if (!phi || !u || !v || !w || !ox || !oy || !oz || !ax || !ay || !az || !solid || !body_grad || !xc || !yc ||
        !zc || !dx || !dy || !dz || !xlo || !xhi || !ylo || !yhi || !zlo || !zhi || !bounds || !gx || !gy || !gz ||
        !vortex || !advection || !totals)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = 0;
    const Dims d{nx, ny, nz};
    const size_t nc = d.ncell();
    Scratch A(st);
    const double* in[9] = {u, v, w, ox, oy, oz, ax, ay, az};
    const double* din[9];
    for (int m = 0; m < 9; m++) din[m] = A.upload(in[m], nc);
    const double* hf[6] = {xlo, xhi, ylo, yhi, zlo, zhi};
    size_t nf[6] = {nface_x(ny, nz), nface_x(ny, nz), nface_y(nx, nz), nface_y(nx, nz), nface_z(nx, ny),
                    nface_z(nx, ny)};
    const double* f[6];
    for (int m = 0; m < 6; m++) f[m] = A.upload(hf[m], nf[m]);
    double* out[5];
    for (int m = 0; m < 5; m++) out[m] = A.get<double>(nc);
    int rc = fpm_compute_stairstep_fpm_terms_3d_dev(
        A.upload(phi, d.npad()), din[0], din[1], din[2], din[3], din[4], din[5], din[6], din[7], din[8],
        A.upload(solid, d.npad()), body_grad, A.upload(xc, nx + 2), A.upload(yc, ny + 2), A.upload(zc, nz),
        A.upload(dx, nx), A.upload(dy, ny), A.upload(dz, nz), f[0], f[1], f[2], f[3], f[4], f[5], bounds, out[0],
        out[1], out[2], out[3], out[4], totals, nx, ny, nz, st);
    if (rc != FPM_OK) throw Error{rc, g_last_error};
    double* hout[5] = {gx, gy, gz, vortex, advection};
    for (int m = 0; m < 5; m++) download(hout[m], out[m], nc * sizeof(double), st);
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

static Coefs coef_views(const double* coef, int nx, int ny, int nz) {
  return Coefs{coef, coef + nx, coef + 2 * nx, coef + 2 * nx + ny, coef + 2 * nx + 2 * ny, coef + 2 * nx + 2 * ny + nz};
}

int fpm_stairstep_build_operator_dev(const double* rhs, const int32_t* solid, const double* body_grad,
                                     const double* xlo, const double* xhi, const double* ylo, const double* yhi,
                                     const double* zlo, const double* zhi, const double* xc, const double* yc,
                                     const double* zc, const double* dx, const double* dy, const double* dz, int nx,
                                     int ny, int nz, int for_pcg, double* src, double* diag, double* rdiag,
                                     int* isolated, void* stream) {
  return guarded([&] {
    if (!rhs || !solid || !body_grad || !xlo || !xhi || !ylo || !yhi || !zlo || !zhi || !xc || !yc || !zc || !dx ||
        !dy || !dz || !src || !diag || !rdiag || !isolated)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = (cudaStream_t)stream;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    Common cm = make_common(A, d, st);
    double* coef = A.get<double>(2 * (size_t)(nx + ny + nz));
    Axes ax{xc, yc, zc, dx, dy, dz};
    CUDA_TRY(launch_axis_coefs(ax, nx, ny, nz, coef, st));
    Faces f{const_cast<double*>(xlo), const_cast<double*>(xhi), const_cast<double*>(ylo),
            const_cast<double*>(yhi), const_cast<double*>(zlo), const_cast<double*>(zhi)};
    CUDA_TRY(launch_build_operator(d, rhs, solid, body_grad, f, coef_views(coef, nx, ny, nz), ax, for_pcg, src, diag,
                                   rdiag, cm.S, st));
    *isolated = read_scalars(cm.S, st).isolated;
  });
}

int fpm_stairstep_jacobi_sweeps_dev(double* a, double* b, const double* src, const double* rdiag, const double* xc,
                                    const double* yc, const double* zc, const double* dx, const double* dy,
                                    const double* dz, int nx, int ny, int nz, int nsweeps, int method, void* stream) {
  return guarded([&] {
    if (!a || !b || !src || !rdiag || !xc || !yc || !zc || !dx || !dy || !dz) throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    if (nsweeps < 0) throw Error{FPM_E_ARG, "nsweeps must be >= 0"};
    if (method != FPM_METHOD_JACOBI && method != FPM_METHOD_JACOBI_DF)
      throw Error{FPM_E_METHOD, "sweeps need method jacobi or jacobi_df"};
    require_device();
    cudaStream_t st = (cudaStream_t)stream;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    const long long ncoef = 2LL * (nx + ny + nz);
    double* coef = A.get<double>(ncoef);
    CUDA_TRY(launch_axis_coefs(Axes{xc, yc, zc, dx, dy, dz}, nx, ny, nz, coef, st));
    if (method == FPM_METHOD_JACOBI) {
      Coefs c = coef_views(coef, nx, ny, nz);
      double *cur = a, *oth = b;
      for (int s = 0; s < nsweeps; s++) {
        CUDA_TRY(launch_jacobi_f64(d, cur, oth, src, rdiag, c, st));
        std::swap(cur, oth);
      }
    } else {
      const long long np = d.npad(), nc = d.ncell();
      float2* pa = A.get<float2>(np);
      float2* pb = A.get<float2>(np);
      float2* sdf = A.get<float2>(nc);
      float2* rdf = A.get<float2>(nc);
      float2* cdf = A.get<float2>(ncoef);
      CUDA_TRY(launch_to_df(a, pa, np, st));
      CUDA_TRY(launch_to_df(b, pb, np, st));
      CUDA_TRY(launch_to_df(src, sdf, nc, st));
      CUDA_TRY(launch_to_df(rdiag, rdf, nc, st));
      CUDA_TRY(launch_to_df(coef, cdf, ncoef, st));
      float2 *cur = pa, *oth = pb;
      for (int s = 0; s < nsweeps; s++) {
        CUDA_TRY(launch_jacobi_df(d, cur, oth, sdf, rdf, cdf, st));
        std::swap(cur, oth);
      }
      CUDA_TRY(launch_from_df_interior(d, pa, a, st));
      CUDA_TRY(launch_from_df_interior(d, pb, b, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

int fpm_stairstep_operator_residual_dev(const double* phi, const double* src, const double* diag, const double* xc,
                                        const double* yc, const double* zc, const double* dx, const double* dy,
                                        const double* dz, int nx, int ny, int nz, double* value, void* stream) {
  return guarded([&] {
    if (!phi || !src || !diag || !xc || !yc || !zc || !dx || !dy || !dz || !value)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = (cudaStream_t)stream;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    Common cm = make_common(A, d, st);
    double* coef = A.get<double>(2 * (size_t)(nx + ny + nz));
    CUDA_TRY(launch_axis_coefs(Axes{xc, yc, zc, dx, dy, dz}, nx, ny, nz, coef, st));
    CUDA_TRY(launch_operator_residual(d, phi, src, diag, coef_views(coef, nx, ny, nz), cm.S, cm.rb, st));
    *value = read_scalars(cm.S, st).res;
  });
}

}  // extern "C"
