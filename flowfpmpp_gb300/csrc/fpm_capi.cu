// C ABI (include/fpm_capi.h): host-side drivers of the stair-step solve and
// force terms.  The control flow of each solver follows the reference routine
// it replaces; per-iteration scalars stay on the device, so the host only
// synchronises once per convergence check.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/fpm_capi.h"
#include "fpm_internal.h"

namespace fpm {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

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

// ---------------------------------------------------------------- kernel timing
// Optional CUDA-event timing of the hot loops, on the stream they run on: one
// event pair brackets each run of back-to-back launches of one kernel.
struct KernelTimer {
  std::mutex mu;
  bool on = false;
  struct Pending {
    int id, launches;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  double ms[FPM_TIMER_COUNT] = {0};
  long long launches[FPM_TIMER_COUNT] = {0};
};
static KernelTimer g_timer;

struct TimedRun {
  int id, n;
  cudaStream_t st;
  cudaEvent_t a = nullptr, b = nullptr;
  TimedRun(int id_, int n_, cudaStream_t st_) : id(id_), n(n_), st(st_) {
    bool on;
    {
      std::lock_guard<std::mutex> g(g_timer.mu);
      on = g_timer.on;
    }
    if (on && n > 0) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, st);
    }
  }
  ~TimedRun() {
    if (!a) return;
    cudaEventRecord(b, st);
    std::lock_guard<std::mutex> g(g_timer.mu);
    g_timer.pending.push_back({id, n, a, b});
  }
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
    {
      TimedRun t(FPM_TIMER_PCG_ITER, chunk, st);
      for (int n = 0; n < chunk; n++)
        CUDA_TRY(launch_pcg_iteration(d, a.phi, p, q, r, diag, rdiag, c, a.ax, cm.S, cm.rb, st));
    }
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
    {
      TimedRun t(FPM_TIMER_JACOBI_F64, nsteps, st);
      for (int s = 0; s < nsteps; s++) {
        CUDA_TRY(launch_jacobi_f64(d, cur, oth, src, rdiag, c, st));
        std::swap(cur, oth);
      }
    }
    sw += nsteps;
    CUDA_TRY(launch_operator_residual(d, cur, src, diag, c, cm.S, cm.rb, st));
    residual = read_scalars(cm.S, st).res;
  }
  if (cur != a.phi) CUDA_TRY(launch_copy_interior(d, cur, a.phi, st));
  *sweeps = sw;
}

// ---------------------------------------------------------------- double-float Jacobi plan
struct DfChoice {
  int shape, kchunk;
};
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int>, DfChoice> g_tune_cache;

static int default_kchunk(const Dims& d, int shape) {
  int tx, ty;
  jacobi_df_shape(shape, &tx, &ty);
  const long long tiles = (long long)((d.nx + tx - 1) / tx) * ((d.ny + ty - 1) / ty);
  long long nzc = (152LL * 2 * 4) / tiles;  // about four waves of two CTAs per SM
  if (nzc < 1) nzc = 1;
  if (nzc > d.nz) nzc = d.nz;
  int kc = (int)((d.nz + nzc - 1) / nzc);
  if (kc < 4) kc = d.nz < 4 ? d.nz : 4;
  return kc;
}

static JacobiDfPlan make_df_plan(Scratch& A, const Dims& d) {
  JacobiDfPlan pl;
  std::memset(&pl, 0, sizeof(pl));
  pl.nx = d.nx;
  pl.ny = d.ny;
  pl.nz = d.nz;
  pl.px = ((long long)d.nx + 2 + 1) & ~1LL;
  const size_t nphi = (size_t)pl.px * (d.ny + 2) * d.nz;
  pl.a = A.get<float2>(nphi);
  pl.b = A.get<float2>(nphi);
  pl.sr = A.get<float4>(d.ncell());
  pl.coef = A.get<float2>(2 * (size_t)(d.nx + d.ny + d.nz));
  pl.err = A.get<int>(1);
  pl.shape = 0;
  pl.kchunk = default_kchunk(d, 0);
  return pl;
}

// Picks the tile shape and z-chunk: cached per grid size; otherwise, unless
// FPM_DF_AUTOTUNE=0, times three sweeps a -> b of every candidate (a is left
// unchanged, b is overwritten by the first real sweep anyway).
static void df_choose(JacobiDfPlan& pl, cudaStream_t st) {
  const Dims d{pl.nx, pl.ny, pl.nz};
  const auto key = std::make_tuple(pl.nx, pl.ny, pl.nz);
  // FPM_DF_SHAPE / FPM_DF_KCHUNK pin the choice (tests of every tile shape).
  if (const char* fs = std::getenv("FPM_DF_SHAPE")) {
    pl.shape = std::atoi(fs) % jacobi_df_num_shapes();
    const char* fk = std::getenv("FPM_DF_KCHUNK");
    pl.kchunk = fk ? std::atoi(fk) : default_kchunk(d, pl.shape);
    if (pl.kchunk < 1) pl.kchunk = 1;
    CUDA_TRY(jacobi_df_encode(pl));
    return;
  }
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      pl.shape = it->second.shape;
      pl.kchunk = it->second.kchunk;
      CUDA_TRY(jacobi_df_encode(pl));
      return;
    }
  }
  const char* env = std::getenv("FPM_DF_AUTOTUNE");
  DfChoice best{0, default_kchunk(d, 0)};
  if (!(env && env[0] == '0')) {
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    for (int s = 0; s < jacobi_df_num_shapes(); s++) {
      const int cands[5] = {default_kchunk(d, s), 8, 16, 32, 64};
      for (int c = 0; c < 5; c++) {
        const int kc = cands[c];
        if (kc > d.nz || (c > 0 && kc == cands[0])) continue;
        pl.shape = s;
        pl.kchunk = kc;
        CUDA_TRY(jacobi_df_encode(pl));
        CUDA_TRY(jacobi_df_sweep(pl, pl.a, pl.b, st));
        CUDA_TRY(cudaEventRecord(e0, st));
        for (int r = 0; r < 3; r++) CUDA_TRY(jacobi_df_sweep(pl, pl.a, pl.b, st));
        CUDA_TRY(cudaEventRecord(e1, st));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
          best_ms = ms;
          best = DfChoice{s, kc};
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache[key] = best;
  }
  pl.shape = best.shape;
  pl.kchunk = best.kchunk;
  CUDA_TRY(jacobi_df_encode(pl));
}

static void check_df_err(const JacobiDfPlan& pl, cudaStream_t st) {
  int h = 0;
  CUDA_TRY(cudaMemcpyAsync(&h, pl.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (h) throw Error{FPM_E_TIMEOUT, "double-float Jacobi pipeline wait timed out"};
}

// Same iteration in double-float: phi lives as f32 pairs in the TMA kernel's
// layout between checks and is unpacked to FP64 phi for each residual check.
static void jacobi_loop_df(const SolveArgs& a, const Dims& d, const double* src, const double* diag,
                           const double* rdiag, const double* coef, const Coefs& c, Scratch& A, Common& cm,
                           int* sweeps, cudaStream_t st) {
  JacobiDfPlan pl = make_df_plan(A, d);
  CUDA_TRY(jacobi_df_pack(pl, a.phi, src, rdiag, coef, st));
  df_choose(pl, st);
  float2 *cur = pl.a, *oth = pl.b;
  double residual = HUGE_VAL;
  int sw = 0;
  const int ci = a.ci < 1 ? 1 : a.ci;
  while (sw < a.max_sweeps && residual > a.tol) {
    int nsteps = ci < a.max_sweeps - sw ? ci : a.max_sweeps - sw;
    {
      TimedRun t(FPM_TIMER_JACOBI_DF, nsteps, st);
      for (int s = 0; s < nsteps; s++) {
        CUDA_TRY(jacobi_df_sweep(pl, cur, oth, st));
        std::swap(cur, oth);
      }
    }
    sw += nsteps;
    CUDA_TRY(jacobi_df_unpack(pl, cur, a.phi, st));
    CUDA_TRY(launch_operator_residual(d, a.phi, src, diag, c, cm.S, cm.rb, st));
    residual = read_scalars(cm.S, st).res;
    check_df_err(pl, st);
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
    else jacobi_loop_df(a, d, src, diag, rdiag, coef, c, A, cm, &sw, st);
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

long long fpm_kernel_launches(void) { return g_launches.load(); }

int fpm_timing_enable(int on) {
  std::lock_guard<std::mutex> g(g_timer.mu);
  g_timer.on = on != 0;
  return FPM_OK;
}

int fpm_timing_read(int which, long long* launches, double* total_ms, int reset) {
  return guarded([&] {
    if (which < 0 || which >= FPM_TIMER_COUNT || !launches || !total_ms) throw Error{FPM_E_ARG, "bad timer id"};
    std::lock_guard<std::mutex> g(g_timer.mu);
    for (auto& p : g_timer.pending) {
      CUDA_TRY(cudaEventSynchronize(p.b));
      float ms = 0;
      CUDA_TRY(cudaEventElapsedTime(&ms, p.a, p.b));
      g_timer.ms[p.id] += ms;
      g_timer.launches[p.id] += p.launches;
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    g_timer.pending.clear();
    *launches = g_timer.launches[which];
    *total_ms = g_timer.ms[which];
    if (reset) {
      g_timer.launches[which] = 0;
      g_timer.ms[which] = 0;
    }
  });
}

int fpm_jacobi_df_config(int nx, int ny, int nz, int* tile_x, int* tile_y, int* kchunk) {
  return guarded([&] {
    if (!tile_x || !tile_y || !kchunk) throw Error{FPM_E_ARG, "null argument"};
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune_cache.find(std::make_tuple(nx, ny, nz));
    if (it == g_tune_cache.end()) throw Error{FPM_E_ARG, "no double-float Jacobi run at this size yet"};
    jacobi_df_shape(it->second.shape, tile_x, tile_y);
    *kchunk = it->second.kchunk;
  });
}
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
      TimedRun t(FPM_TIMER_JACOBI_F64, nsweeps, st);
      for (int s = 0; s < nsweeps; s++) {
        CUDA_TRY(launch_jacobi_f64(d, cur, oth, src, rdiag, c, st));
        std::swap(cur, oth);
      }
    } else {
      JacobiDfPlan pl = make_df_plan(A, d);
      CUDA_TRY(jacobi_df_pack(pl, a, src, rdiag, coef, st));
      df_choose(pl, st);
      float2 *cur = pl.a, *oth = pl.b;
      {
        TimedRun t(FPM_TIMER_JACOBI_DF, nsweeps, st);
        for (int s = 0; s < nsweeps; s++) {
          CUDA_TRY(jacobi_df_sweep(pl, cur, oth, st));
          std::swap(cur, oth);
        }
      }
      CUDA_TRY(jacobi_df_unpack(pl, pl.a, a, st));
      CUDA_TRY(jacobi_df_unpack(pl, pl.b, b, st));
      check_df_err(pl, st);
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

static double read_res_cb(SolveScalars* S, cudaStream_t st, int) { return read_scalars(S, st).res; }

static void face_sizes(int nx, int ny, int nz, size_t nf[6]) {
  nf[0] = nf[1] = nface_x(ny, nz);
  nf[2] = nf[3] = nface_y(nx, nz);
  nf[4] = nf[5] = nface_z(nx, ny);
}

// Both Neumann compatibility variants (src/fpm_laplace_3d.f90:9-53, :150-217).
static void neumann_compat_host(const double* rhs, double* const hf[6], const double* dx, const double* dy,
                                const double* dz, int nx, int ny, int nz, int uniform, double* correction,
                                double* imbalance) {
  if (!rhs || !dx || !dy || !dz || !correction || !imbalance) throw Error{FPM_E_ARG, "null argument"};
  for (int m = 0; m < 6; m++)
    if (!hf[m]) throw Error{FPM_E_ARG, "null face array"};
  if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
  require_device();
  cudaStream_t st = 0;
  const Dims d{nx, ny, nz};
  Scratch A(st);
  Common cm = make_common(A, d, st);
  size_t nf[6];
  face_sizes(nx, ny, nz, nf);
  double* f[6];
  for (int m = 0; m < 6; m++) f[m] = A.upload(hf[m], nf[m]);
  const double* drhs = A.upload(rhs, d.ncell());
  const double *ddx, *ddy, *ddz;
  double area = 0;
  if (uniform) {
    ddx = A.upload(dx, 1);
    ddy = A.upload(dy, 1);
    ddz = A.upload(dz, 1);
    area = 2.0 * ((double)(ny * nz) * *dy * *dz + (double)(nx * nz) * *dx * *dz + (double)(nx * ny) * *dx * *dy);
  } else {
    ddx = A.upload(dx, nx);
    ddy = A.upload(dy, ny);
    ddz = A.upload(dz, nz);
  }
  CUDA_TRY(launch_neumann_compat(nx, ny, nz, drhs, Faces{f[0], f[1], f[2], f[3], f[4], f[5]}, ddx, ddy, ddz,
                                 uniform, area, cm.S, cm.rb, st));
  const SolveScalars& h = read_scalars(cm.S, st);
  *correction = h.corr;
  *imbalance = h.red[3] - h.red[0];
  for (int m = 0; m < 6; m++) download(hf[m], f[m], nf[m] * sizeof(double), st);
  CUDA_TRY(cudaStreamSynchronize(st));
}

int fpm_enforce_neumann_compatibility_3d(const double* rhs, double* xlo, double* xhi, double* ylo, double* yhi,
                                         double* zlo, double* zhi, int nx, int ny, int nz, double dx, double dy,
                                         double dz, double* correction, double* imbalance) {
  return guarded([&] {
    double* hf[6] = {xlo, xhi, ylo, yhi, zlo, zhi};
    neumann_compat_host(rhs, hf, &dx, &dy, &dz, nx, ny, nz, 1, correction, imbalance);
  });
}

int fpm_enforce_neumann_compatibility_nonuniform_3d(const double* rhs, double* xlo, double* xhi, double* ylo,
                                                    double* yhi, double* zlo, double* zhi, const double* dx,
                                                    const double* dy, const double* dz, int nx, int ny, int nz,
                                                    double* correction, double* imbalance) {
  return guarded([&] {
    double* hf[6] = {xlo, xhi, ylo, yhi, zlo, zhi};
    neumann_compat_host(rhs, hf, dx, dy, dz, nx, ny, nz, 0, correction, imbalance);
  });
}

int fpm_solve_neumann_poisson_3d(double* phi, const double* rhs, const double* xlo, const double* xhi,
                                 const double* ylo, const double* yhi, const double* zlo, const double* zhi, int nx,
                                 int ny, int nz, double dx, double dy, double dz, double tolerance, int max_iterations,
                                 int check_interval, int* iterations, double* final_residual) {
  return guarded([&] {
    if (!phi || !rhs || !xlo || !xhi || !ylo || !yhi || !zlo || !zhi || !iterations || !final_residual)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = 0;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    Common cm = make_common(A, d, st);
    const size_t nfull = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
    double* dphi = A.upload(phi, nfull);
    const double* drhs = A.upload(rhs, d.ncell());
    size_t nf[6];
    face_sizes(nx, ny, nz, nf);
    const double* hf[6] = {xlo, xhi, ylo, yhi, zlo, zhi};
    double* f[6];
    for (int m = 0; m < 6; m++) f[m] = A.upload(hf[m], nf[m]);
    double* a = A.get<double>(d.ncell());
    double* b = A.get<double>(d.ncell());
    int rc = neumann_uniform_iterate(nx, ny, nz, dphi, drhs, Faces{f[0], f[1], f[2], f[3], f[4], f[5]}, dx, dy, dz,
                                     tolerance, max_iterations, check_interval, a, b, cm.S, cm.rb, st, read_res_cb,
                                     iterations, final_residual);
    if (rc) throw Error{FPM_E_CUDA, cudaGetErrorString((cudaError_t)rc)};
    download(phi, dphi, nfull * sizeof(double), st);
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

int fpm_solve_neumann_poisson_nonuniform_3d(double* phi, const double* rhs, const double* xlo, const double* xhi,
                                            const double* ylo, const double* yhi, const double* zlo,
                                            const double* zhi, const double* xc, const double* yc, const double* zc,
                                            const double* dx, const double* dy, const double* dz, int nx, int ny,
                                            int nz, double tolerance, int max_iterations, int check_interval,
                                            int* iterations, double* final_residual) {
  return guarded([&] {
    if (!phi || !rhs || !xlo || !xhi || !ylo || !yhi || !zlo || !zhi || !xc || !yc || !zc || !dx || !dy || !dz ||
        !iterations || !final_residual)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = 0;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    Common cm = make_common(A, d, st);
    double* dphi = A.upload(phi, d.ncell());
    const double* drhs = A.upload(rhs, d.ncell());
    size_t nf[6];
    face_sizes(nx, ny, nz, nf);
    const double* hf[6] = {xlo, xhi, ylo, yhi, zlo, zhi};
    double* f[6];
    for (int m = 0; m < 6; m++) f[m] = A.upload(hf[m], nf[m]);
    Axes ax{A.upload(xc, nx), A.upload(yc, ny), A.upload(zc, nz), A.upload(dx, nx), A.upload(dy, ny), A.upload(dz, nz)};
    double* b = A.get<double>(d.ncell());
    double* coef = A.get<double>(2 * (size_t)(nx + ny + nz));
    int rc = neumann_nonuniform_iterate(nx, ny, nz, dphi, drhs, Faces{f[0], f[1], f[2], f[3], f[4], f[5]}, ax,
                                        tolerance, max_iterations, check_interval, b, coef, cm.S, cm.rb, st,
                                        read_res_cb, iterations, final_residual);
    if (rc) throw Error{FPM_E_CUDA, cudaGetErrorString((cudaError_t)rc)};
    download(phi, dphi, d.ncell() * sizeof(double), st);
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

int fpm_compute_fpm_terms_uniform_3d(const double* phi, const double* u, const double* v, const double* w,
                                     const double* ox, const double* oy, const double* oz, const double* ax,
                                     const double* ay, const double* az, const int32_t* fluid, double* gx, double* gy,
                                     double* gz, double* vortex, double* advection, double* totals, int nx, int ny,
                                     int nz, double dx, double dy, double dz) {
  return guarded([&] {
    const double* in[9] = {u, v, w, ox, oy, oz, ax, ay, az};
    double* hout[5] = {gx, gy, gz, vortex, advection};
    if (!phi || !fluid || !totals) throw Error{FPM_E_ARG, "null argument"};
    for (int m = 0; m < 9; m++)
      if (!in[m]) throw Error{FPM_E_ARG, "null flow field"};
    for (int m = 0; m < 5; m++)
      if (!hout[m]) throw Error{FPM_E_ARG, "null output"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = 0;
    const Dims d{nx, ny, nz};
    const size_t nc = d.ncell();
    Scratch A(st);
    Common cm = make_common(A, d, st);
    const double* din[9];
    for (int m = 0; m < 9; m++) din[m] = A.upload(in[m], nc);
    double* out[5];
    for (int m = 0; m < 5; m++) out[m] = A.get<double>(nc);
    const double* dphi = A.upload(phi, (size_t)(nx + 2) * (ny + 2) * (nz + 2));
    Flow fl{din[0], din[1], din[2], din[3], din[4], din[5], din[6], din[7], din[8]};
    CUDA_TRY(launch_terms_uniform(nx, ny, nz, dphi, fl, A.upload(fluid, nc), dx, dy, dz,
                                  TermsOut{out[0], out[1], out[2], out[3], out[4]}, cm.S, cm.rb, st));
    const SolveScalars& h = read_scalars(cm.S, st);
    totals[0] = h.red[0];
    totals[1] = h.red[1];
    for (int m = 0; m < 5; m++) download(hout[m], out[m], nc * sizeof(double), st);
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

int fpm_compute_fpm_terms_nonuniform_3d(const double* phi, const double* u, const double* v, const double* w,
                                        const double* ox, const double* oy, const double* oz, const double* ax,
                                        const double* ay, const double* az, const int32_t* fluid, const double* xc,
                                        const double* yc, const double* zc, const double* dx, const double* dy,
                                        const double* dz, const double* xlo, const double* xhi, const double* ylo,
                                        const double* yhi, const double* zlo, const double* zhi,
                                        const double* bounds, double* gx, double* gy, double* gz, double* vortex,
                                        double* advection, double* totals, int nx, int ny, int nz) {
  return guarded([&] {
    const double* in[9] = {u, v, w, ox, oy, oz, ax, ay, az};
    double* hout[5] = {gx, gy, gz, vortex, advection};
    const double* hf[6] = {xlo, xhi, ylo, yhi, zlo, zhi};
    if (!phi || !fluid || !totals || !bounds || !xc || !yc || !zc || !dx || !dy || !dz)
      throw Error{FPM_E_ARG, "null argument"};
    for (int m = 0; m < 9; m++)
      if (!in[m]) throw Error{FPM_E_ARG, "null flow field"};
    for (int m = 0; m < 5; m++)
      if (!hout[m]) throw Error{FPM_E_ARG, "null output"};
    for (int m = 0; m < 6; m++)
      if (!hf[m]) throw Error{FPM_E_ARG, "null face array"};
    if (nx < 2 || ny < 2 || nz < 2)
      throw Error{FPM_E_SIZE, "nonuniform 3-D FPM kernel requires at least two cells per direction"};
    require_device();
    cudaStream_t st = 0;
    const Dims d{nx, ny, nz};
    const size_t nc = d.ncell();
    Scratch A(st);
    Common cm = make_common(A, d, st);
    const double* din[9];
    for (int m = 0; m < 9; m++) din[m] = A.upload(in[m], nc);
    double* out[5];
    for (int m = 0; m < 5; m++) out[m] = A.get<double>(nc);
    size_t nf[6];
    face_sizes(nx, ny, nz, nf);
    double* f[6];
    for (int m = 0; m < 6; m++) f[m] = A.upload(hf[m], nf[m]);
    Axes axes{A.upload(xc, nx), A.upload(yc, ny), A.upload(zc, nz), A.upload(dx, nx), A.upload(dy, ny),
              A.upload(dz, nz)};
    Flow fl{din[0], din[1], din[2], din[3], din[4], din[5], din[6], din[7], din[8]};
    CUDA_TRY(launch_terms_nonuniform(nx, ny, nz, A.upload(phi, nc), fl, A.upload(fluid, nc), axes,
                                     Faces{f[0], f[1], f[2], f[3], f[4], f[5]}, bounds,
                                     TermsOut{out[0], out[1], out[2], out[3], out[4]}, cm.S, cm.rb, st));
    const SolveScalars& h = read_scalars(cm.S, st);
    totals[0] = h.red[0];
    totals[1] = h.red[1];
    for (int m = 0; m < 5; m++) download(hout[m], out[m], nc * sizeof(double), st);
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

int fpm_partition_terms_2d(const double* phi, const double* g, const double* u, const double* v,
                           const uint8_t* solid, const double* xf, const double* yf, const double* kin,
                           const double* ring, double dt, double nu, int nx, int ny, double* terms,
                           double* vif_density, double* omega, int slip_body) {
  return guarded([&] {
    if (!phi || !g || !u || !v || !solid || !xf || !yf || !kin || !ring || !terms || !vif_density || !omega)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = 0;
    Scratch A(st);
    const size_t n2 = (size_t)nx * ny, L = 2 * (size_t)nx + 2 * (size_t)ny;
    Common cm;
    cm.S = A.get<SolveScalars>(1);
    CUDA_TRY(cudaMemsetAsync(cm.S, 0, sizeof(SolveScalars), st));
    const int nb = ((nx + 31) / 32) * ((ny + 7) / 8);
    cm.rb.max_blocks = nb;
    cm.rb.partials = A.get<double>((size_t)4 * nb);
    cm.rb.ticket = A.get<unsigned int>(1);
    CUDA_TRY(cudaMemsetAsync(cm.rb.ticket, 0, sizeof(unsigned int), st));
    Part2D p;
    p.phi = A.upload(phi, n2);
    p.u = A.upload(u, n2);
    p.v = A.upload(v, n2);
    p.xf = A.upload(xf, (size_t)nx + 1);
    p.yf = A.upload(yf, (size_t)ny + 1);
    p.ring = A.upload(ring, 4 * L);
    p.solid = A.upload(solid, n2);
    p.g0 = g[0];
    p.g1 = g[1];
    p.k1 = kin[0];
    p.k2 = kin[1];
    p.k3 = kin[2];
    p.k4 = kin[3];
    p.k5 = kin[4];
    p.k6 = kin[5];
    p.dt = dt;
    p.nu = nu;
    p.nx = nx;
    p.ny = ny;
    p.slip = slip_body ? 1 : 0;
    double* scratch[4];
    for (int m = 0; m < 4; m++) scratch[m] = A.get<double>(n2);
    double* dvif = A.get<double>(n2);
    double* domega = A.get<double>(n2);
    CUDA_TRY(launch_partition_2d(p, scratch[0], scratch[1], scratch[2], scratch[3], dvif, domega, cm.S, cm.rb, st));
    const SolveScalars& h = read_scalars(cm.S, st);
    for (int m = 0; m < 4; m++) terms[m] = h.red[m];
    download(vif_density, dvif, n2 * sizeof(double), st);
    download(omega, domega, n2 * sizeof(double), st);
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

}  // extern "C"
