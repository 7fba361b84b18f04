// C ABI (include/fpm_capi.h): host-side drivers of the stair-step solve and
// force terms.  The control flow of each solver follows the reference routine
// it replaces; per-iteration scalars stay on the device, so the host only
// synchronises once per convergence check.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/fpm_capi.h"
#include "fpm_internal.h"

namespace fpm {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

static std::atomic<long long> g_launches{0};
static thread_local long long t_launches = 0;  // this thread's launches (graph capture accounting)
void note_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  t_launches++;
}
static void note_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

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
    if (on) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, st);
    }
  }
  ~TimedRun() {
    if (!a) return;
    if (n <= 0) {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      return;
    }
    cudaEventRecord(b, st);
    std::lock_guard<std::mutex> g(g_timer.mu);
    g_timer.pending.push_back({id, n, a, b});
  }
};

// ---------------------------------------------------------------- options
// FPM_VERBOSE=1 prints one line per convergence check of every solver loop
// to stderr; FPM_VERBOSE=2 adds the Jacobi autotuner's timings.  FPM_PCG_STALL_CHECKS overrides the number of checks without a
// 1% improvement after which PCG stops (50, src/fpm_stairstep_mpi_3d.f90:288).
static int verbose_level() {
  static int v = -1;
  if (v < 0) {
    const char* e = std::getenv("FPM_VERBOSE");
    v = (e && e[0]) ? std::atoi(e) : 0;
    if (v < 0) v = 0;
  }
  return v;
}
static bool verbose() {
  return verbose_level() >= 1;
}
static int stall_checks() {
  const char* e = std::getenv("FPM_PCG_STALL_CHECKS");
  const int n = e ? std::atoi(e) : 50;
  return n > 0 ? n : 50;
}

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

// ---------------------------------------------------------------- chunk graphs
// The iterations between two convergence checks are replayed as one CUDA
// graph: captured once per solve and chunk length on a private capture stream
// (so the caller's stream may be the legacy default stream), launched on the
// solve's stream.  The kernels read their per-iteration scalars and halt
// flags from device memory, so a replay is exactly the sequence of launches
// it replaces.  FPM_GRAPHS=0 launches the kernels one by one instead.
static bool graphs_enabled() {
  static int v = -1;
  if (v < 0) {
    const char* e = std::getenv("FPM_GRAPHS");
    v = (e && e[0] == '0') ? 0 : 1;
  }
  return v == 1;
}

class ChunkGraphs {
 public:
  ChunkGraphs() = default;
  ~ChunkGraphs() {
    for (auto& kv : exec_) cudaGraphExecDestroy(kv.second.exec);
  }
  // Runs `launch_one(stream)` n times on st, through a cached graph.
  template <class F>
  void run(int n, cudaStream_t st, F&& launch_one) {
    if (n <= 0) return;
    if (!graphs_enabled()) {
      for (int i = 0; i < n; i++) launch_one(st);
      return;
    }
    auto it = exec_.find(n);
    if (it == exec_.end()) {
      cudaStream_t cs = capture_stream();
      const long long before = t_launches;
      CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      try {
        for (int i = 0; i < n; i++) launch_one(cs);
      } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(cs, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      const long long captured = t_launches - before;
      cudaGraph_t g = nullptr;
      CUDA_TRY(cudaStreamEndCapture(cs, &g));
      cudaGraphExec_t x = nullptr;
      const cudaError_t e = cudaGraphInstantiate(&x, g, 0);
      cudaGraphDestroy(g);
      CUDA_TRY(e);
      it = exec_.emplace(n, Entry{x, captured}).first;
      note_launches(-captured);  // counted again below, when they run
    }
    CUDA_TRY(cudaGraphLaunch(it->second.exec, st));
    note_launches(it->second.launches);
  }

 private:
  static cudaStream_t capture_stream() {
    static thread_local cudaStream_t cs = nullptr;
    if (!cs) CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    return cs;
  }
  struct Entry {
    cudaGraphExec_t exec;
    long long launches;  // kernels in the graph (for the launch count)
  };
  std::map<int, Entry> exec_;

 public:
  void clear() {
    for (auto& kv : exec_) cudaGraphExecDestroy(kv.second.exec);
    exec_.clear();
  }
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
  const int max_stalled = stall_checks();
  int it = 0, restarts = 0, stalled = 0;
  double best = res;
  int sw = 0;
  ChunkGraphs graphs;
  while (sw < a.max_sweeps && res > a.tol) {
    int chunk = ci - it % ci;
    if (chunk > a.max_sweeps - sw) chunk = a.max_sweeps - sw;
    CUDA_TRY(cudaMemsetAsync(&cm.S->iters, 0, sizeof(int), st));
    {
      TimedRun t(FPM_TIMER_PCG_ITER, chunk, st);
      graphs.run(chunk, st, [&](cudaStream_t s2) {
        CUDA_TRY(launch_pcg_iteration(d, a.phi, p, q, r, diag, rdiag, c, a.ax, cm.S, cm.rb, s2));
      });
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
    if (verbose()) std::fprintf(stderr, "fpm pcg: iterations %d residual %.3e\n", sw, res);
    if (res < 0.99 * best) {
      best = res;
      stalled = 0;
    } else {
      stalled++;
    }
    if (stalled >= max_stalled || !(res == res)) break;
  }
  *sweeps = sw;
  return res;
}

// jacobi_iterate (src/fpm_stairstep_mpi_3d.f90:200-225): sweeps in chunks of
// check_interval, max-norm residual after each chunk.  The two buffers swap
// roles instead of copying back; every sweep reads the latest iterate, so the
// values are those of the reference's ping-pong with copy.  FPM_METHOD_JACOBI
// sweeps with separately rounded operations, FPM_METHOD_JACOBI_FMA with fused
// multiply-adds.
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
        CUDA_TRY(a.method == FPM_METHOD_JACOBI_FMA ? launch_jacobi_f64_fma(d, cur, oth, src, rdiag, c, st)
                                                   : launch_jacobi_f64(d, cur, oth, src, rdiag, c, st));
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
    int sms = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
    for (int s = 0; s < jacobi_df_num_shapes(); s++) {
      // planes per CTA: the default, fixed lengths, and lengths that make the
      // CTA count a whole number (2..8) of waves at this shape's occupancy
      std::vector<int> cands = {default_kchunk(d, s), 8, 16, 32, 64};
      int tx, ty;
      jacobi_df_shape(s, &tx, &ty);
      const long long tiles = (long long)((d.nx + tx - 1) / tx) * ((d.ny + ty - 1) / ty);
      const long long slots = (long long)sms * jacobi_df_ctas_per_sm(s);
      for (int w = 2; w <= 8; w++) {
        const long long nch = w * slots / tiles;
        if (nch < 1 || nch > d.nz) continue;
        cands.push_back((int)((d.nz + nch - 1) / nch));
      }
      std::sort(cands.begin(), cands.end());
      cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
      for (const int kc : cands) {
        if (kc < 2 || kc > d.nz) continue;
        pl.shape = s;
        pl.kchunk = kc;
        CUDA_TRY(jacobi_df_encode(pl));
        CUDA_TRY(jacobi_df_sweep(pl, pl.a, pl.b, st));
        CUDA_TRY(cudaEventRecord(e0, st));
        for (int r = 0; r < 5; r++) CUDA_TRY(jacobi_df_sweep(pl, pl.a, pl.b, st));
        CUDA_TRY(cudaEventRecord(e1, st));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (verbose_level() >= 2)
          std::fprintf(stderr, "fpm df autotune: shape %d tile %dx%d planes %d: %.1f us per sweep\n", s, tx, ty, kc,
                       200.f * ms);
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

// ---------------------------------------------------------------- triple-float Jacobi plan
static std::map<std::tuple<int, int, int>, DfChoice> g_tf_cache;

static JacobiTfPlan make_tf_plan(Scratch& A, const Dims& d) {
  JacobiTfPlan pl;
  std::memset(&pl, 0, sizeof(pl));
  pl.nx = d.nx;
  pl.ny = d.ny;
  pl.nz = d.nz;
  pl.px = ((long long)d.nx + 2 + 1) & ~1LL;
  const size_t nphi = (size_t)pl.px * (d.ny + 2) * d.nz;
  pl.a = A.get<double>(nphi);
  pl.b = A.get<double>(nphi);
  pl.sr = A.get<double>(2 * (size_t)d.ncell());
  pl.coef = A.get<float4>(2 * (size_t)(d.nx + d.ny + d.nz));
  pl.err = A.get<int>(1);
  pl.shape = 0;
  pl.kchunk = 8;
  return pl;
}

// Tile shape and planes per CTA of the triple-float sweep: cached per grid
// size; otherwise (unless FPM_TF_AUTOTUNE=0) five timed sweeps a -> b of each
// candidate.  FPM_TF_SHAPE / FPM_TF_KCHUNK pin the choice.
static void tf_choose(JacobiTfPlan& pl, cudaStream_t st) {
  const Dims d{pl.nx, pl.ny, pl.nz};
  const auto key = std::make_tuple(pl.nx, pl.ny, pl.nz);
  if (const char* fs = std::getenv("FPM_TF_SHAPE")) {
    pl.shape = std::atoi(fs) % jacobi_tf_num_shapes();
    const char* fk = std::getenv("FPM_TF_KCHUNK");
    pl.kchunk = fk ? std::atoi(fk) : 8;
    if (pl.kchunk < 1) pl.kchunk = 1;
    CUDA_TRY(jacobi_tf_encode(pl));
    return;
  }
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tf_cache.find(key);
    if (it != g_tf_cache.end()) {
      pl.shape = it->second.shape;
      pl.kchunk = it->second.kchunk;
      CUDA_TRY(jacobi_tf_encode(pl));
      return;
    }
  }
  const char* env = std::getenv("FPM_TF_AUTOTUNE");
  DfChoice best{0, std::min(8, d.nz)};
  if (!(env && env[0] == '0')) {
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    for (int s = 0; s < jacobi_tf_num_shapes(); s++) {
      for (const int kc : {4, 8, 16, 32}) {
        if (kc > d.nz && kc != 4) continue;
        pl.shape = s;
        pl.kchunk = std::min(kc, d.nz);
        CUDA_TRY(jacobi_tf_encode(pl));
        CUDA_TRY(jacobi_tf_sweep(pl, pl.a, pl.b, st));
        CUDA_TRY(cudaEventRecord(e0, st));
        for (int r = 0; r < 5; r++) CUDA_TRY(jacobi_tf_sweep(pl, pl.a, pl.b, st));
        CUDA_TRY(cudaEventRecord(e1, st));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (verbose_level() >= 2) {
          int tx, ty;
          jacobi_tf_shape(s, &tx, &ty);
          std::fprintf(stderr, "fpm tf autotune: shape %d tile %dx%d planes %d: %.1f us per sweep\n", s, tx, ty,
                       pl.kchunk, 200.f * ms);
        }
        if (ms < best_ms) {
          best_ms = ms;
          best = DfChoice{s, pl.kchunk};
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tf_cache[key] = best;
  }
  pl.shape = best.shape;
  pl.kchunk = best.kchunk;
  CUDA_TRY(jacobi_tf_encode(pl));
}

// The weighted-Jacobi iteration with FP64 storage and triple-float arithmetic:
// phi lives in the TMA kernel's FP64 layout between checks and is unpacked
// for each residual check.
static void jacobi_loop_tf(const SolveArgs& a, const Dims& d, const double* src, const double* diag,
                           const double* rdiag, const double* coef, const Coefs& c, Scratch& A, Common& cm,
                           int* sweeps, cudaStream_t st) {
  JacobiTfPlan pl = make_tf_plan(A, d);
  CUDA_TRY(jacobi_tf_pack(pl, a.phi, src, rdiag, coef, st));
  tf_choose(pl, st);
  CUDA_TRY(cudaMemsetAsync(pl.err, 0, sizeof(int), st));
  double *cur = pl.a, *oth = pl.b;
  double residual = HUGE_VAL;
  int sw = 0;
  const int ci = a.ci < 1 ? 1 : a.ci;
  while (sw < a.max_sweeps && residual > a.tol) {
    int nsteps = ci < a.max_sweeps - sw ? ci : a.max_sweeps - sw;
    {
      TimedRun t(FPM_TIMER_JACOBI_TF, nsteps, st);
      for (int s = 0; s < nsteps; s++) {
        CUDA_TRY(jacobi_tf_sweep(pl, cur, oth, st));
        std::swap(cur, oth);
      }
    }
    sw += nsteps;
    CUDA_TRY(jacobi_tf_unpack(pl, cur, a.phi, st));
    CUDA_TRY(launch_operator_residual(d, a.phi, src, diag, c, cm.S, cm.rb, st));
    residual = read_scalars(cm.S, st).res;
    int h = 0;
    CUDA_TRY(cudaMemcpyAsync(&h, pl.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (h) throw Error{FPM_E_TIMEOUT, "triple-float Jacobi pipeline wait timed out"};
  }
  *sweeps = sw;
}

// Mixed-precision PCG for 1..4 right-hand sides sharing the operator.
// One FP32 diagonal PCG per right-hand side (batched in the same kernels)
// whose residual is periodically replaced by the FP64 true residual -- the
// reference's true-residual replacement (src/fpm_stairstep_mpi_3d.f90:285-290)
// done as a reliable update: the FP32 correction is added to phi in FP64, the
// projected FP64 residual r = b - A phi becomes the new FP32 residual
// (rescaled to unit max-norm) and the search direction is kept, rescaled, so
// the Krylov process continues instead of restarting.  An update happens
// when the FP32 preconditioned residual norm has dropped by kUpdateDrop since
// the last one, after kUpdateMax iterations, or on a breakdown (then p
// restarts from rdiag r).  Convergence is decided on the FP64 max-norm
// residual at each update, exactly the reference's test; a right-hand side
// also stops after kStallUpdates updates without a 1% improvement (the
// reference's roundoff-floor rule, counted in updates).
// The direction is restarted (p = rdiag r) only after a breakdown or a
// rolled-back update (kBlowup); slow progress keeps it, because a restart
// throws the Krylov space away.  (FPM_MIXED_UPDATE_GAIN = g also restarts
// when an update's residual is not below g times the previous one.)  Every
// right-hand side finishes on its best iterate.
// Tunables of the reliable updates (defaults; FPM_MIXED_UPDATE_DROP,
// FPM_MIXED_UPDATE_MAX and FPM_MIXED_UPDATE_GAIN override them).
static double env_double(const char* name, double dflt) {
  const char* e = std::getenv(name);
  if (!e || !e[0]) return dflt;
  const double v = std::atof(e);
  return v > 0 ? v : dflt;
}
static const double kUpdateDrop = env_double("FPM_MIXED_UPDATE_DROP", 1e-3);
static const double kUpdateGain = env_double("FPM_MIXED_UPDATE_GAIN", 1e300);
static const int kUpdateMax = (int)env_double("FPM_MIXED_UPDATE_MAX", 1000);
constexpr double kBlowup = 4.0;
constexpr int kStallUpdates = 4;
// FP32 stagnation: kSlowUpdates updates in a row that each gain less than
// a factor kSlowGain hand the right-hand side to FP64 PCG from its current
// phi (on strongly stretched grids the FP32 iteration cannot resolve the
// remaining error: its rounding relative to the operator grows with the
// condition number).
constexpr double kSlowGain = 2.0;
constexpr int kSlowUpdates = 2;
// Planes per thread in the FP32 kernels (FPM_MIXED_KCHUNK overrides).
static int mixed_kchunk() {
  static int v = -1;
  if (v < 0) {
    const char* e = std::getenv("FPM_MIXED_KCHUNK");
    v = (e && std::atoi(e) > 0) ? std::atoi(e) : 8;
  }
  return v;
}

static void mixed_solve(const Dims& d, int nrhs, double* const phi[], const double* const src[], const double* diag,
                        const double* rdiag, const int32_t* solid, const Axes& ax, const Coefs& c, double tol,
                        int max_sweeps, int ci, Scratch& A, Common& cm, int* sweeps_out, cudaStream_t st,
                        int* to_fp64 = nullptr) {
  const long long np = d.npad();
  const MixedGrid G = mixed_grid(d.nx, d.ny, d.nz, mixed_kchunk());
  MixedVecs v;
  std::memset(&v, 0, sizeof(v));
  v.nrhs = nrhs;
  auto vec = [&]() {
    float* x = A.get<float>(G.size);
    CUDA_TRY(cudaMemsetAsync(x, 0, G.size * sizeof(float), st));
    return x;
  };
  float* wall32 = vec();
  float* rdiag32 = vec();
  CUDA_TRY(launch_mx_wall(G, d, solid, c, wall32, st));
  CUDA_TRY(launch_mx_layout(G, rdiag, rdiag32, st));
  v.wall = wall32;
  v.rdiag = rdiag32;
  auto row = [&](const double* a) {
    float* x = A.get<float>(G.px);
    CUDA_TRY(launch_mx_row(d.nx, G.px, a, x, st));
    return (const float*)x;
  };
  auto axis = [&](const double* a, int n) {
    float* x = A.get<float>(n);
    CUDA_TRY(launch_mx_convert(a, x, n, st));
    return (const float*)x;
  };
  v.cw = row(c.cw);
  v.ce = row(c.ce);
  v.dx = row(ax.dx);
  v.cs = axis(c.cs, d.ny);
  v.cn = axis(c.cn, d.ny);
  v.dy = axis(ax.dy, d.ny);
  v.cb = axis(c.cb, d.nz);
  v.ct = axis(c.ct, d.nz);
  v.dz = axis(ax.dz, d.nz);
  RedBuf rbm;
  rbm.max_blocks = G.nblocks;
  rbm.partials = A.get<double>((size_t)kMaxRhs * G.nblocks);
  rbm.ticket = A.get<unsigned int>(1);
  CUDA_TRY(cudaMemsetAsync(rbm.ticket, 0, sizeof(unsigned int), st));
  DPtr4 r64{}, phis{};
  double* best_phi[kMaxRhs] = {};
  SolveScalars* S64[kMaxRhs] = {};
  for (int m = 0; m < nrhs; m++) {
    v.p[m] = vec();
    v.q[m] = vec();
    v.r[m] = vec();
    v.e[m] = vec();
    r64.p[m] = A.get<double>(d.ncell());
    phis.p[m] = phi[m];
    best_phi[m] = A.get<double>(np);
    CUDA_TRY(cudaMemcpyAsync(best_phi[m], phi[m], np * sizeof(double), cudaMemcpyDeviceToDevice, st));
    S64[m] = A.get<SolveScalars>(1);
    CUDA_TRY(cudaMemsetAsync(S64[m], 0, sizeof(SolveScalars), st));
  }
  MixedScalars* MS = A.get<MixedScalars>(1);
  {
    // The FP32 iteration of a right-hand side stops itself once its
    // preconditioned residual norm has dropped by kUpdateDrop (tol2 on the
    // squared norm), so it never runs on into the FP32 rounding floor between
    // two host checks.
    MixedScalars h0;
    std::memset(&h0, 0, sizeof(h0));
    for (int m = 0; m < kMaxRhs; m++) h0.tol2[m] = kUpdateDrop * kUpdateDrop;
    CUDA_TRY(cudaMemcpyAsync(MS, &h0, sizeof(MixedScalars), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  }
  auto true_res = [&](int m) {
    CUDA_TRY(launch_true_residual(d, phi[m], src[m], diag, rdiag, r64.p[m], nullptr, c, ax, 0, S64[m], cm.rb, st));
    return read_scalars(S64[m], st).res;
  };
  MixedScalars* hms = nullptr;
  CUDA_TRY(cudaMallocHost(&hms, sizeof(MixedScalars)));
  struct HostFree {
    void* p;
    ~HostFree() { cudaFreeHost(p); }
  } hf{hms};

  double res[kMaxRhs], best[kMaxRhs], prev[kMaxRhs], scale[kMaxRhs];
  int stall[kMaxRhs] = {}, since[kMaxRhs] = {}, done_at[kMaxRhs] = {-1, -1, -1, -1}, slow[kMaxRhs] = {};
  if (to_fp64)
    for (int m = 0; m < nrhs; m++) to_fp64[m] = 0;
  bool live[kMaxRhs] = {};
  MixedScale sc;
  std::memset(&sc, 0, sizeof(sc));
  bool any = false;
  for (int m = 0; m < nrhs; m++) {
    res[m] = best[m] = prev[m] = true_res(m);
    live[m] = res[m] > tol && res[m] == res[m];
    if (!live[m]) done_at[m] = 0;
    scale[m] = res[m] > 0 ? 1.0 / res[m] : 1.0;
    sc.in_set[m] = live[m];
    sc.scale[m] = scale[m];
    sc.pmul[m] = 0.0;
    any = any || live[m];
  }
  if (any) CUDA_TRY(launch_mx_start(G, v, r64, sc, MS, rbm, st));
  const int chunk_len = ci < 1 ? 1 : ci;
  int total = 0;
  ChunkGraphs graphs;
  while (any && total < max_sweeps) {
    int chunk = chunk_len;
    if (chunk > max_sweeps - total) chunk = max_sweeps - total;
    CUDA_TRY(cudaMemsetAsync(&MS->iters, 0, sizeof(int), st));
    {
      TimedRun t(FPM_TIMER_PCG_MIXED_ITER, chunk, st);
      graphs.run(chunk, st, [&](cudaStream_t s2) { CUDA_TRY(launch_mx_iteration(G, v, MS, rbm, s2)); });
    }
    CUDA_TRY(cudaMemcpyAsync(hms, MS, sizeof(MixedScalars), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    total += chunk;
    // Which right-hand sides need a reliable update now?
    std::memset(&sc, 0, sizeof(sc));
    bool upd = false;
    for (int m = 0; m < nrhs; m++) {
      if (!live[m]) continue;
      since[m] += chunk;
      const bool dropped = hms->rz[m] <= kUpdateDrop * kUpdateDrop * hms->rz0[m];
      const bool broke = !hms->active[m] && !dropped;
      if (broke || dropped || since[m] >= kUpdateMax || total >= max_sweeps) {
        sc.in_set[m] = 1;
        sc.scale[m] = scale[m];          // the scale the correction was computed in
        sc.pmul[m] = broke ? 0.0 : 1.0;  // rescaled below
        upd = true;
      }
    }
    if (!upd) continue;
    CUDA_TRY(launch_mx_apply(G, v, phis, sc, st));
    any = false;
    for (int m = 0; m < nrhs; m++) {
      if (sc.in_set[m]) {
        since[m] = 0;
        res[m] = true_res(m);
        if (!(res[m] <= kBlowup * best[m])) {
          // the FP32 correction made things much worse: back to the best
          // iterate and restart the direction there
          CUDA_TRY(cudaMemcpyAsync(phi[m], best_phi[m], np * sizeof(double), cudaMemcpyDeviceToDevice, st));
          res[m] = true_res(m);
          sc.pmul[m] = 0.0;
        }
        stall[m] = res[m] < 0.99 * best[m] ? 0 : stall[m] + 1;
        if (res[m] < best[m]) {
          best[m] = res[m];
          CUDA_TRY(cudaMemcpyAsync(best_phi[m], phi[m], np * sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
        const bool restart = !(res[m] < kUpdateGain * prev[m]);
        slow[m] = res[m] * kSlowGain > prev[m] ? slow[m] + 1 : 0;
        prev[m] = res[m];
        const bool hand_over = to_fp64 && slow[m] >= kSlowUpdates && res[m] > tol;
        if (!(res[m] > tol) || !(res[m] == res[m]) || stall[m] >= kStallUpdates || hand_over) {
          live[m] = false;
          done_at[m] = total;
          if (hand_over) to_fp64[m] = 1;
          sc.in_set[m] = 0;
          if (!(res[m] <= best[m]))  // finish on the best iterate
            CUDA_TRY(cudaMemcpyAsync(phi[m], best_phi[m], np * sizeof(double), cudaMemcpyDeviceToDevice, st));
          // park it: no further iterations for this right-hand side
          const int zero = 0;
          CUDA_TRY(cudaMemcpyAsync(&MS->active[m], &zero, sizeof(int), cudaMemcpyHostToDevice, st));
        } else {
          const double ns = res[m] > 0 ? 1.0 / res[m] : 1.0;
          sc.pmul[m] = (sc.pmul[m] == 0.0 || restart) ? 0.0 : ns / scale[m];
          scale[m] = ns;
          sc.scale[m] = ns;
        }
      }
      any = any || live[m];
    }
    if (verbose())
      std::fprintf(stderr, "fpm pcg_mixed: iterations %d residual %.3e %.3e %.3e\n", total, res[0],
                   nrhs > 1 ? res[1] : 0.0, nrhs > 2 ? res[2] : 0.0);
    bool refresh = false;
    for (int m = 0; m < nrhs; m++) refresh = refresh || sc.in_set[m];
    if (refresh) CUDA_TRY(launch_mx_start(G, v, r64, sc, MS, rbm, st));
  }
  // Fold in any correction still pending (right-hand sides stopped by the cap).
  std::memset(&sc, 0, sizeof(sc));
  bool pend = false;
  for (int m = 0; m < nrhs; m++)
    if (live[m]) {
      sc.in_set[m] = 1;
      sc.scale[m] = scale[m];
      pend = true;
    }
  if (pend) CUDA_TRY(launch_mx_apply(G, v, phis, sc, st));
  for (int m = 0; m < nrhs; m++) sweeps_out[m] = done_at[m] >= 0 ? done_at[m] : total;
}

// FP32 PCG preconditioned by the aggregation multigrid V-cycle of fpm_mg.cu,
// in the same FP64 refinement as mixed_solve: each outer step of a
// right-hand side loads its projected FP64 true residual (scaled to unit
// max-norm), runs PCG until the preconditioned residual norm r.z has dropped
// by mg_drop^2 (or kMgInnerMax iterations), adds the correction to phi in
// FP64 and recomputes the true residual; convergence is the reference's
// max-norm test.  All right-hand sides iterate in the same launches; each
// has its own outer steps.  The host looks at the device scalars after each
// chunk of iterations; a chunk runs until every live right-hand side is
// predicted to have finished its inner solve (its previous inner count + 1;
// for the first inner solve kMgFirstChunk, then doubling), so that on small
// grids (cells x right-hand sides below kMgAdaptCells), where an iteration
// costs little more than its launches, few iterations run after an inner
// solve has converged on the device.  Larger grids run fixed chunks of
// check_interval (at most 50) iterations.
constexpr int kMgInnerMax = 400;
constexpr int kMgFirstChunk = 8;
constexpr double kMgAdaptCells = 4194304.0;
// Residual drop of an inner FP32 solve (FPM_MG_DROP overrides), measured per
// problem class: 1e-4 on small grids (three potentials on 64 x 64 x 32:
// 4.1 ms against 4.9 ms at 5e-5), 5e-5 on large ones (384 x 384 x 192:
// 0.52 s against 0.58 s at 1e-4; 256 x 256 x 128 0.083 against 0.086 s),
// 3e-5 for the batched 2-D frames (0.96 s per batch against 1.04 s).
static double mg_drop(double cells_x_rhs, bool frames) {
  const double e = env_double("FPM_MG_DROP", 0.0);
  if (e > 0.0) return e;
  if (frames) return 3e-5;
  return cells_x_rhs < kMgAdaptCells ? 1e-4 : 5e-5;
}
constexpr int kMgMinChunk = 2;

static void mg_solve(const Dims& d, int nrhs, double* const phi[], const double* const src[], const double* diag,
                     const double* rdiag, const int32_t* solid, const Axes& ax, const Coefs& c, double tol,
                     int max_sweeps, int ci, Scratch& A, Common& cm, int* sweeps_out, cudaStream_t st,
                     int* to_fp64) {
  if (d.ncell() <= 1024) {  // too small for a coarse level: the diagonal preconditioner
    int to64[kMaxRhs] = {};
    mixed_solve(d, nrhs, phi, src, diag, rdiag, solid, ax, c, tol, max_sweeps, ci, A, cm, sweeps_out, st, to64);
    for (int m = 0; m < nrhs; m++) to_fp64[m] = to64[m];
    return;
  }
  Trace tr("multigrid setup");
  MgHierarchy H;
  std::memset(&H, 0, sizeof(H));
  H.nrhs = nrhs;
  // Two cycles on the level-1 problem per level-0 cycle where level 1 is
  // large enough for the extra launches to pay (three potentials on
  // 384 x 384 x 192: 20 % fewer iterations, 12 % less time); small grids are
  // launch-bound and keep the V-cycle.
  const long long n1 = (long long)((d.nx + 1) / 2) * ((d.ny + 1) / 2) * ((d.nz + 1) / 2);
  H.gamma = (int)env_double("FPM_MG_GAMMA", n1 >= 262144 ? 2 : 1);
  H.gamma_depth = (int)env_double("FPM_MG_GAMMA_DEPTH", 1);
  H.omega = (float)env_double("FPM_MG_OMEGA", 0.9);
  H.coarse_sweeps = (int)env_double("FPM_MG_COARSE_SWEEPS", 40);
  H.cscale = (float)env_double("FPM_MG_CSCALE", 1.0);
  // level 0 in the mixed solver's FP32 layout (zero halo), coarse levels
  // compact; the level-0 passes take an even number of planes per chunk (whole
  // aggregates)
  // Planes per CTA: the level-0 passes march kc planes per CTA, so on a small
  // grid a long chunk leaves most SMs idle and the pass waits on one CTA's
  // serial plane loads.  Each chunk length is the largest even value up to its
  // default that still gives at least one CTA per SM (three potentials on a
  // 64 x 64 x 32 sphere grid: TMA chunk 24 -> 6.2 ms, 4 -> 4.3 ms per solve).
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  auto fill_chunk = [&](int kc, long long ctas_per_chunk_row) {
    kc = kc < 2 ? 2 : kc + (kc & 1);
    while (kc > 2 && ctas_per_chunk_row * ((d.nz + kc - 1) / kc) < sms) kc -= 2;
    return kc;
  };
  const bool kc_pinned = std::getenv("FPM_MIXED_KCHUNK") != nullptr;
  int kcm = mixed_kchunk() + (mixed_kchunk() & 1);
  if (!kc_pinned) kcm = fill_chunk(kcm, (long long)((d.nx + 3) / 4 + 31) / 32 * ((d.ny + 3) / 4) * nrhs);
  H.g0 = mixed_grid(d.nx, d.ny, d.nz, kcm);
  // level-0 TMA passes (three potentials on 384 x 384 x 192: 16 -> 0.726 s,
  // 24 -> 0.716 s, 48 -> 0.715 s)
  H.kc0 = (int)env_double("FPM_MG_KCHUNK", 24);
  H.kc0 = H.kc0 < 2 ? 2 : H.kc0 + (H.kc0 & 1);
  if (!std::getenv("FPM_MG_KCHUNK")) H.kc0 = fill_chunk(H.kc0, mg_tma_ctas_per_chunk(H.g0, nrhs));
  H.pxb = (H.g0.px + 15) / 16 * 16;
  auto zeros = [&](long long n) {
    float* x = A.get<float>(n);
    CUDA_TRY(cudaMemsetAsync(x, 0, n * sizeof(float), st));
    return x;
  };
  int nx = d.nx, ny = d.ny, nz = d.nz;
  for (;;) {
    MgLevel& L = H.lv[H.nlev];
    L.nx = nx;
    L.ny = ny;
    L.nz = nz;
    L.zc = std::min(nz, 65535 / kMaxRhs);  // one plane per thread (the most loads in flight) where the grid allows
    if (H.nlev == 0) {
      L.off = 4 + H.g0.px;
      L.sy = H.g0.px;
      L.sz = H.g0.plane;
      L.alloc = H.g0.size;
    } else {  // rows padded to 16 bytes (TMA tiles of level 1)
      L.off = 0;
      L.sy = (nx + 3) / 4 * 4;
      L.sz = L.sy * ny;
      L.alloc = L.sz * nz;
    }
    L.te = zeros(L.alloc);
    L.tn = zeros(L.alloc);
    L.tt = zeros(L.alloc);
    L.dinv = zeros(L.alloc);
    for (int m = 0; m < nrhs && H.nlev > 0; m++) {  // level 0 works on the PCG vectors
      L.t[m] = zeros(L.alloc);
      L.x[m] = zeros(L.alloc);
      L.b[m] = zeros(L.alloc);
    }
    H.nlev++;
    if (L.n() <= 1024 || H.nlev == kMgMaxLevels) break;
    nx = (nx + 1) / 2;
    ny = (ny + 1) / 2;
    nz = (nz + 1) / 2;
  }
  if (H.nlev < 2 || H.lv[H.nlev - 1].n() > 1024)
    throw Error{FPM_E_LIMIT, "grid too small or too large for the multigrid hierarchy"};
  if ((d.ny + 3) / 4 > 65535 || (long long)((d.nz + H.g0.kc - 1) / H.g0.kc) * nrhs > 65535)
    throw Error{FPM_E_LIMIT, "grid too large for the multigrid launch geometry"};
  const long long fb_size = H.pxb * (d.ny + 2) * (long long)d.nz;
  H.fb0 = A.get<uint8_t>(fb_size);
  CUDA_TRY(cudaMemsetAsync(H.fb0, 0, fb_size, st));
  H.aex = zeros(H.g0.px);
  H.dxr = zeros(H.g0.px);
  H.dy = zeros(d.ny);
  H.ayn = zeros(d.ny);
  H.dz = zeros(d.nz);
  H.azt = zeros(d.nz);
  CUDA_TRY(mg_setup(H, d, solid, ax, st));
  const long long n0 = H.lv[0].alloc;
  MgVecs v;
  std::memset(&v, 0, sizeof(v));
  DPtr4 r64{}, phis{};
  SolveScalars* S64[kMaxRhs] = {};
  for (int m = 0; m < nrhs; m++) {
    v.r[m] = zeros(n0);
    v.z[m] = zeros(n0);
    v.p[m] = zeros(n0);
    v.q[m] = zeros(n0);
    v.e[m] = zeros(n0);
    v.r2[m] = zeros(n0);
    v.p2[m] = zeros(n0);
    r64.p[m] = A.get<double>(d.ncell());
    phis.p[m] = phi[m];
    S64[m] = A.get<SolveScalars>(1);
    CUDA_TRY(cudaMemsetAsync(S64[m], 0, sizeof(SolveScalars), st));
  }
  CUDA_TRY(mg_encode(H, v));
  MgRed rb;
  rb.partials = A.get<double>((size_t)mg_red_partials(H));
  rb.tickets = A.get<unsigned int>(kMaxRhs);
  CUDA_TRY(cudaMemsetAsync(rb.tickets, 0, kMaxRhs * sizeof(unsigned int), st));
  rb.err = A.get<int>(1);
  CUDA_TRY(cudaMemsetAsync(rb.err, 0, sizeof(int), st));
  MgScalars* S = A.get<MgScalars>(kMaxRhs);
  CUDA_TRY(cudaMemsetAsync(S, 0, kMaxRhs * sizeof(MgScalars), st));
  MgScalars* hS = nullptr;  // kMaxRhs scalars, then the error flag
  CUDA_TRY(cudaMallocHost(&hS, kMaxRhs * sizeof(MgScalars) + sizeof(int)));
  int* herr = reinterpret_cast<int*>(hS + kMaxRhs);
  struct HostFree {
    void* p;
    ~HostFree() { cudaFreeHost(p); }
  } hf{hS};
  Trace ti("multigrid PCG");
  auto true_res = [&](int m) {
    CUDA_TRY(launch_true_residual(d, phi[m], src[m], diag, rdiag, r64.p[m], nullptr, c, ax, 0, S64[m], cm.rb, st));
    return read_scalars(S64[m], st).res;
  };
  double res[kMaxRhs] = {}, best[kMaxRhs] = {}, scale[kMaxRhs] = {};
  int stall[kMaxRhs] = {}, iters[kMaxRhs] = {};
  int done[kMaxRhs] = {}, est[kMaxRhs] = {};  // inner iterations so far / of the last inner solve
  bool live[kMaxRhs] = {};
  // (Re)start the inner PCG of the right-hand sides in set from their
  // current true residuals: drop by kdrop, or just far enough for the
  // tolerance (with a margin of 30 for the max-norm versus the
  // preconditioned norm).
  const double kdrop = mg_drop((double)d.ncell() * nrhs, false);
  auto start = [&](unsigned set) {
    for (int m = 0; m < nrhs; m++) {
      if (!((set >> m) & 1u)) continue;
      scale[m] = res[m] > 0 ? 1.0 / res[m] : 1.0;
      const double need = tol / (30.0 * res[m]);
      const double drop = need > kdrop ? (need < 0.5 ? need : 0.5) : kdrop;
      MgScalars h0;
      std::memset(&h0, 0, sizeof(h0));
      h0.tol2 = drop * drop;
      h0.active = 1;
      CUDA_TRY(cudaMemcpyAsync(S + m, &h0, sizeof(MgScalars), cudaMemcpyHostToDevice, st));
      done[m] = 0;
    }
    CUDA_TRY(mg_pcg_start(H, r64, scale, set, v, S, rb, st));
  };
  unsigned set = 0;
  for (int m = 0; m < nrhs; m++) {
    res[m] = best[m] = true_res(m);
    live[m] = res[m] > tol && res[m] == res[m];
    if (live[m]) set |= 1u << m;
  }
  if (set) start(set);
  const int chunk_len = ci < 1 ? 1 : (ci > 50 ? 50 : ci);
  int total = 0;
  ChunkGraphs graphs;
  // Adaptive chunks only where an iteration is cheap next to its launches
  // (measured: three potentials on 64 x 64 x 32, 8.1 -> 6.7 ms per solve);
  // on 384 x 384 x 192 fixed chunks are faster (0.665 s vs 0.681 s).
  const bool adapt = (double)d.ncell() * nrhs < kMgAdaptCells;
  while (set && total < max_sweeps) {
    int chunk = adapt ? kMgMinChunk : chunk_len;
    for (int m = 0; m < nrhs && adapt; m++) {
      if (!((set >> m) & 1u)) continue;
      int pred;
      if (est[m] > 0)
        pred = est[m] >= done[m] ? est[m] + 1 - done[m] : est[m] / 8;
      else
        pred = done[m] > kMgFirstChunk ? done[m] : kMgFirstChunk;
      if (pred > chunk) chunk = pred;
    }
    if (chunk > chunk_len) chunk = chunk_len;
    if (chunk > max_sweeps - total) chunk = max_sweeps - total;
    {
      TimedRun t(FPM_TIMER_PCG_MIXED_ITER, chunk, st);
      // one captured iteration, replayed: chunks of any length share it
      for (int i = 0; i < chunk; i++)
        graphs.run(1, st, [&](cudaStream_t s2) { CUDA_TRY(mg_pcg_iteration(H, v, S, rb, s2)); });
    }
    total += chunk;
    CUDA_TRY(cudaMemcpyAsync(hS, S, kMaxRhs * sizeof(MgScalars), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(herr, rb.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (*herr) throw Error{FPM_E_TIMEOUT, "multigrid: a bounded wait for a TMA copy gave up"};
    for (int m = 0; m < nrhs; m++)
      if ((set >> m) & 1u) done[m] = hS[m].iters;
    // Which right-hand sides have finished an outer step?
    unsigned upd = 0;
    for (int m = 0; m < nrhs; m++)
      if (live[m] && (!hS[m].active || hS[m].iters >= kMgInnerMax || total >= max_sweeps)) upd |= 1u << m;
    if (!upd) continue;
    const int zero = 0;
    for (int m = 0; m < nrhs; m++)  // park them until their restart
      if ((upd >> m) & 1u) CUDA_TRY(cudaMemcpyAsync(&S[m].active, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(mg_pcg_apply(H, d, v, S, scale, upd, phis, st));
    unsigned restart = 0;
    for (int m = 0; m < nrhs; m++) {
      if (!((upd >> m) & 1u)) continue;
      const int inner = hS[m].iters;
      iters[m] += inner;
      est[m] = inner;
      const double prev = res[m];
      res[m] = true_res(m);
      if (verbose())
        std::fprintf(stderr, "fpm pcg_mg: rhs %d inner %d total %d residual %.3e\n", m, inner, iters[m], res[m]);
      if (res[m] < 0.99 * best[m]) {
        best[m] = res[m];
        stall[m] = 0;
      } else {
        stall[m]++;
      }
      const bool stop = !(res[m] > tol) || !(res[m] == res[m]) || stall[m] >= kStallUpdates ||
                        (inner == 0 && !(res[m] < prev));  // no progress possible
      if (stop) {
        live[m] = false;
        set &= ~(1u << m);
      } else {
        restart |= 1u << m;
      }
    }
    if (restart && total < max_sweeps) start(restart);
  }
  for (int m = 0; m < nrhs; m++) {
    sweeps_out[m] = iters[m];
    // stopped above the tolerance (FP32 can no longer resolve the error at
    // the FP64 rounding floor of the residual): FP64 PCG finishes
    to_fp64[m] = res[m] > tol ? 1 : 0;
  }
}

// solve_stairstep_poisson_3d (src/fpm_stairstep_mpi_3d.f90:106-330), device
// arrays, for nrhs right-hand sides that share solid and axes.  FP64 methods
// solve them one after the other; FPM_METHOD_PCG_MIXED solves them together.
static bool valid_method(int m) {
  return m == FPM_METHOD_PCG || m == FPM_METHOD_JACOBI || m == FPM_METHOD_JACOBI_DF || m == FPM_METHOD_PCG_MIXED ||
         m == FPM_METHOD_PCG_MG || m == FPM_METHOD_FCG_LEARNED || m == FPM_METHOD_JACOBI_FMA ||
         m == FPM_METHOD_JACOBI_TF;
}

// FPM_METHOD_FCG_LEARNED: FP64 flexible CG (Notay's FCG(1): the Polak-Ribiere
// beta = z_k.(r_k - r_{k-1}) / z_{k-1}.r_{k-1} keeps the method a CG for a
// preconditioner that changes between applications) with z = M(r) the
// network-based preconditioner of launch_fcg_precond.  The true residual
// replaces the recursive one every check_interval iterations, convergence is
// the reference's max-norm test, and the loop stops after the same number of
// checks without a 1 % improvement as the FP64 PCG (the caller then finishes
// with FP64 PCG).  Returns the max-norm residual.
static double fcg_learned_loop(void* net, const SolveArgs& a, const Dims& d, double* p, const double* src,
                               const double* diag, const double* rdiag, const Coefs& c, Scratch& A, Common& cm,
                               int* sweeps, cudaStream_t st) {
  const long long nc = d.ncell();
  double* r = A.get<double>(nc);
  double* q = A.get<double>(nc);
  double* z = A.get<double>(nc);
  double* rprev = A.get<double>(nc);
  CUDA_TRY(cudaMemsetAsync(rprev, 0, nc * sizeof(double), st));
  FcgWork w;
  w.fluid = A.get<uint8_t>(nc);
  w.mx = A.get<float>(d.nx);
  w.my = A.get<float>(d.ny);
  w.mz = A.get<float>(d.nz);
  w.b = A.get<float>(nc);
  w.y = A.get<float>(nc);
  w.ay = A.get<double>(nc);
  w.sc = A.get<double>(8);
  // fluid flags and metric channels (b is refilled from r before every use)
  CUDA_TRY(launch_learn_inputs(d, src, diag, a.ax, w.fluid, w.mx, w.my, w.mz, w.b, w.sc, cm.rb, st));
  CUDA_TRY(launch_true_residual(d, a.phi, src, diag, rdiag, r, p, c, a.ax, 0, cm.S, cm.rb, st));
  double res = read_scalars(cm.S, st).res, best = res;
  const int ci = a.ci < 1 ? 1 : a.ci;
  const int max_stalled = stall_checks();
  int it = 0, stalled = 0, restarts = 0;
  double zr_prev = 0.0;
  bool restart = true;
  double h[2];
  const int zero = 0;
  while (it < a.max_sweeps && res > a.tol) {
    std::string err;
    int status = 0;
    CUDA_TRY(launch_fcg_precond(d, net, r, rprev, diag, rdiag, c, a.ax, w, z, cm.rb, st, &err, &status));
    if (status != FPM_OK) throw Error{status, err};
    CUDA_TRY(cudaMemcpyAsync(h, w.sc + 4, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    const double zr = h[0];
    if (!(zr > 0)) {  // the preconditioned residual lost positivity: restart, give up on the second time
      if (++restarts > 1) break;
      restart = true;
      CUDA_TRY(launch_true_residual(d, a.phi, src, diag, rdiag, r, p, c, a.ax, 0, cm.S, cm.rb, st));
      res = read_scalars(cm.S, st).res;
      continue;
    }
    const double beta = restart || !(zr_prev > 0) ? 0.0 : (zr - h[1]) / zr_prev;
    CUDA_TRY(launch_fcg_direction(d, z, p, beta, st));
    CUDA_TRY(cudaMemcpyAsync(&cm.S->rz, &zr, sizeof(double), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(&cm.S->halt, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(launch_pcg_spmv(d, p, q, diag, c, a.ax, cm.S, cm.rb, st));
    CUDA_TRY(launch_fcg_update(d, a.phi, p, q, r, rprev, cm.S, st));
    zr_prev = zr;
    restart = false;
    it++;
    if (it % ci == 0 || it >= a.max_sweeps) {
      const SolveScalars& hs = read_scalars(cm.S, st);
      if (hs.halt) {  // p.q <= 0: restart from the true residual
        if (++restarts > 1) break;
        restart = true;
      } else {
        restarts = 0;
      }
      CUDA_TRY(launch_true_residual(d, a.phi, src, diag, rdiag, r, p, c, a.ax, 0, cm.S, cm.rb, st));
      res = read_scalars(cm.S, st).res;
      if (verbose()) std::fprintf(stderr, "fpm fcg_learned: iterations %d residual %.3e\n", it, res);
      if (res < 0.99 * best) {
        best = res;
        stalled = 0;
      } else {
        stalled++;
      }
      if (stalled >= max_stalled || !(res == res)) break;
    }
  }
  *sweeps = it;
  return res;
}

// Learned initial guess for every right-hand side (see fpm_learned.cu): the
// network's output, scaled by the A-norm projection, replaces the caller's
// phi unless it is not closer to the solution in the energy norm (the norm CG
// minimises), which counts as a fallback.
static void learned_guess(void* net, const Dims& d, int nrhs, const SolveArgs* args, double* const src[],
                          const double* diag, const double* rdiag, const Coefs& c, Scratch& A, Common& cm,
                          int* fallbacks, cudaStream_t st) {
  Trace tl("learned initial guess");
  const long long nc = d.ncell();
  uint8_t* fluid = A.get<uint8_t>(nc);
  float* mx = A.get<float>(d.nx);
  float* my = A.get<float>(d.ny);
  float* mz = A.get<float>(d.nz);
  float* b = A.get<float>(nc);
  float* y = A.get<float>(nc);
  double* sc = A.get<double>(8);
  double* backup = A.get<double>(d.npad());
  double* r = A.get<double>(nc);
  double h[8];
  for (int m = 0; m < nrhs; m++) {
    const SolveArgs& a = args[m];
    CUDA_TRY(launch_energy(d, a.phi, src[m], diag, c, a.ax, sc + 4, cm.rb, st));
    CUDA_TRY(cudaMemcpyAsync(backup, a.phi, d.npad() * sizeof(double), cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(launch_learn_inputs(d, src[m], diag, a.ax, fluid, mx, my, mz, b, sc + 2, cm.rb, st));
    std::string err;
    const int rc = net::forward_into(net, d.nx, d.ny, d.nz, fluid, mx, my, mz, b, y, st, &err);
    if (rc != FPM_OK) throw Error{rc, err};
    CUDA_TRY(launch_learn_apply(d, y, src[m], diag, c, a.ax, a.phi, sc, cm.rb, st));
    CUDA_TRY(launch_energy(d, a.phi, src[m], diag, c, a.ax, sc + 6, cm.rb, st));
    CUDA_TRY(cudaMemcpyAsync(h, sc, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    const double e_old = 0.5 * h[5] - h[4], e_new = 0.5 * h[7] - h[6];
    const bool fail = !(e_new < e_old);
    if (verbose()) {
      CUDA_TRY(launch_true_residual(d, a.phi, src[m], diag, rdiag, r, nullptr, c, a.ax, 0, cm.S, cm.rb, st));
      const SolveScalars& hs = read_scalars(cm.S, st);
      std::fprintf(stderr, "fpm learned guess: rhs %d energy %.6e -> %.6e, guess residual max %.3e, r.(rdiag r) %.3e%s\n",
                   m, e_old, e_new, hs.res, hs.rz, fail ? " (fallback)" : "");
    }
    if (fail) CUDA_TRY(cudaMemcpyAsync(a.phi, backup, d.npad() * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (fallbacks) fallbacks[m] = fail ? 1 : 0;
  }
}

static void solve_multi_dev(int nrhs, const SolveArgs* args, int* sweeps, double* residual, cudaStream_t st,
                            void* net = nullptr, int* fallbacks = nullptr) {
  const SolveArgs& a0 = args[0];
  if (!valid_method(a0.method)) throw Error{FPM_E_METHOD, "stair-step method must be pcg or jacobi"};
  if (nrhs < 1 || nrhs > kMaxRhs) throw Error{FPM_E_LIMIT, "between 1 and 4 right-hand sides per call"};
  check_dims(a0.nx, a0.ny, a0.nz);
  require_device();
  const Dims d{a0.nx, a0.ny, a0.nz};
  Scratch A(st);
  Common cm = make_common(A, d, st);
  Trace t0("stair-step setup");
  double* coef = A.get<double>(2 * (size_t)(a0.nx + a0.ny + a0.nz));
  CUDA_TRY(launch_axis_coefs(a0.ax, a0.nx, a0.ny, a0.nz, coef, st));
  Coefs c{coef, coef + a0.nx, coef + 2 * a0.nx, coef + 2 * a0.nx + a0.ny, coef + 2 * a0.nx + 2 * a0.ny,
          coef + 2 * a0.nx + 2 * a0.ny + a0.nz};
  double* next = A.get<double>(d.npad());
  double* diag = A.get<double>(d.ncell());
  double* rdiag = A.get<double>(d.ncell());
  const bool for_pcg = a0.method == FPM_METHOD_PCG || a0.method == FPM_METHOD_PCG_MIXED || a0.method == FPM_METHOD_PCG_MG;
  double* src[kMaxRhs] = {};
  for (int m = 0; m < nrhs; m++) {
    src[m] = A.get<double>(d.ncell());
    CUDA_TRY(launch_build_operator(d, args[m].rhs, args[m].solid, args[m].bg, args[m].f, c, args[m].ax, for_pcg,
                                   src[m], diag, rdiag, cm.S, st));
  }
  if (read_scalars(cm.S, st).isolated > 0) throw Error{FPM_E_ISOLATED, "stair-step fluid cell has no fluid neighbour"};
  for (int m = 0; m < nrhs; m++) CUDA_TRY(launch_init_fields(d, args[m].solid, args[m].phi, next, st));
  if (net) learned_guess(net, d, nrhs, args, src, diag, rdiag, c, A, cm, fallbacks, st);
  {
    Trace t1("stair-step iterations");
    // right-hand sides whose FP32 iteration stagnated: FP64 PCG from the
    // current phi (which the reference's PCG takes as its initial guess)
    auto finish_fp64 = [&](const int* to64) {
      for (int m = 0; m < nrhs; m++) {
        if (!to64[m]) continue;
        SolveArgs a = args[m];
        a.method = FPM_METHOD_PCG;
        a.max_sweeps = a0.max_sweeps > sweeps[m] ? a0.max_sweeps - sweeps[m] : 1;
        if (verbose())
          std::fprintf(stderr, "fpm: rhs %d hands over to FP64 PCG after %d FP32 iterations\n", m, sweeps[m]);
        CUDA_TRY(launch_init_fields(d, a.solid, a.phi, next, st));
        CUDA_TRY(cudaMemsetAsync(cm.S, 0, sizeof(SolveScalars), st));
        int extra = 0;
        pcg_loop(a, d, next, src[m], diag, rdiag, c, A, cm, &extra, st);
        sweeps[m] += extra;
      }
    };
    if (a0.method == FPM_METHOD_FCG_LEARNED) {
      if (!net) throw Error{FPM_E_METHOD, "the learned flexible CG needs the network (fpm_solve_stairstep_learned_dev)"};
      int to64[kMaxRhs] = {};
      for (int m = 0; m < nrhs; m++) {
        const SolveArgs& a = args[m];
        CUDA_TRY(launch_init_fields(d, a.solid, a.phi, next, st));
        CUDA_TRY(cudaMemsetAsync(cm.S, 0, sizeof(SolveScalars), st));
        const double res = fcg_learned_loop(net, a, d, next, src[m], diag, rdiag, c, A, cm, &sweeps[m], st);
        to64[m] = res > a.tol ? 1 : 0;
      }
      finish_fp64(to64);
    } else if (a0.method == FPM_METHOD_PCG_MG) {
      double* phis[kMaxRhs] = {};
      for (int m = 0; m < nrhs; m++) phis[m] = args[m].phi;
      int to64[kMaxRhs] = {};
      mg_solve(d, nrhs, phis, src, diag, rdiag, a0.solid, a0.ax, c, a0.tol, a0.max_sweeps, a0.ci, A, cm, sweeps, st,
               to64);
      finish_fp64(to64);
    } else if (a0.method == FPM_METHOD_PCG_MIXED) {
      double* phis[kMaxRhs] = {};
      for (int m = 0; m < nrhs; m++) phis[m] = args[m].phi;
      int to64[kMaxRhs] = {};
      mixed_solve(d, nrhs, phis, src, diag, rdiag, a0.solid, a0.ax, c, a0.tol, a0.max_sweeps, a0.ci, A, cm, sweeps,
                  st, to64);
      finish_fp64(to64);
    } else {
      for (int m = 0; m < nrhs; m++) {
        const SolveArgs& a = args[m];
        if (m > 0) CUDA_TRY(launch_init_fields(d, a.solid, a.phi, next, st));
        CUDA_TRY(cudaMemsetAsync(cm.S, 0, sizeof(SolveScalars), st));
        if (a.method == FPM_METHOD_PCG) pcg_loop(a, d, next, src[m], diag, rdiag, c, A, cm, &sweeps[m], st);
        else if (a.method == FPM_METHOD_JACOBI || a.method == FPM_METHOD_JACOBI_FMA)
          jacobi_loop_f64(a, d, next, src[m], diag, rdiag, c, cm, &sweeps[m], st);
        else if (a.method == FPM_METHOD_JACOBI_TF)
          jacobi_loop_tf(a, d, src[m], diag, rdiag, coef, c, A, cm, &sweeps[m], st);
        else jacobi_loop_df(a, d, src[m], diag, rdiag, coef, c, A, cm, &sweeps[m], st);
      }
    }
  }
  Trace t2("stair-step gauge");
  for (int m = 0; m < nrhs; m++) {
    CUDA_TRY(launch_gauge(d, args[m].solid, args[m].phi, args[m].ax, cm.S, cm.rb, st));
    CUDA_TRY(launch_operator_residual(d, args[m].phi, src[m], diag, c, cm.S, cm.rb, st));
    residual[m] = read_scalars(cm.S, st).res;
  }
}

static void solve_dev(const SolveArgs& a, int* sweeps, double* residual, cudaStream_t st) {
  solve_multi_dev(1, &a, sweeps, residual, st);
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

int fpm_measure_fp64_rate(double* instr_per_s, void* stream) {
  return guarded([&] {
    if (!instr_per_s) throw Error{FPM_E_ARG, "null argument"};
    require_device();
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int blocks = 0, threads = 0;
    fp64_rate_shape(sms, &blocks, &threads);
    Scratch A(st);
    double* out = A.get<double>((size_t)blocks * threads);
    CUDA_TRY(fp64_rate_probe(out, blocks, threads, st, instr_per_s));
  });
}

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
    if (!valid_method(method)) throw Error{FPM_E_METHOD, "stair-step method must be pcg or jacobi"};
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

static void multi_args(int nrhs, double* const* phi, const double* const* rhs, const int32_t* solid,
                       const double* body_grads, const double* const* faces, const double* xc, const double* yc,
                       const double* zc, const double* dx, const double* dy, const double* dz, int nx, int ny,
                       int nz, double tolerance, int max_sweeps, int check_interval, int method, int* sweeps,
                       double* residual, SolveArgs* args) {
  if (!phi || !rhs || !solid || !body_grads || !faces || !xc || !yc || !zc || !dx || !dy || !dz || !sweeps ||
      !residual)
    throw Error{FPM_E_ARG, "null argument"};
  if (nrhs < 1 || nrhs > kMaxRhs) throw Error{FPM_E_LIMIT, "between 1 and 4 right-hand sides per call"};
  for (int m = 0; m < nrhs; m++) {
    SolveArgs& a = args[m];
    if (!phi[m] || !rhs[m]) throw Error{FPM_E_ARG, "null phi or rhs"};
    for (int f = 0; f < 6; f++)
      if (!faces[6 * m + f]) throw Error{FPM_E_ARG, "null face array"};
    a.phi = phi[m];
    a.rhs = rhs[m];
    a.solid = solid;
    for (int q = 0; q < 3; q++) a.bg[q] = body_grads[3 * m + q];
    a.f = Faces{const_cast<double*>(faces[6 * m]), const_cast<double*>(faces[6 * m + 1]),
                const_cast<double*>(faces[6 * m + 2]), const_cast<double*>(faces[6 * m + 3]),
                const_cast<double*>(faces[6 * m + 4]), const_cast<double*>(faces[6 * m + 5])};
    a.ax = Axes{xc, yc, zc, dx, dy, dz};
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.tol = tolerance;
    a.max_sweeps = max_sweeps;
    a.ci = check_interval;
    a.method = method;
    sweeps[m] = 0;
    residual[m] = HUGE_VAL;
  }
}

int fpm_solve_stairstep_multi_dev(int nrhs, double* const* phi, const double* const* rhs, const int32_t* solid,
                                  const double* body_grads, const double* const* faces, const double* xc,
                                  const double* yc, const double* zc, const double* dx, const double* dy,
                                  const double* dz, int nx, int ny, int nz, double tolerance, int max_sweeps,
                                  int check_interval, int method, int* sweeps, double* residual, void* stream) {
  return guarded([&] {
    SolveArgs args[kMaxRhs];
    multi_args(nrhs, phi, rhs, solid, body_grads, faces, xc, yc, zc, dx, dy, dz, nx, ny, nz, tolerance, max_sweeps,
               check_interval, method, sweeps, residual, args);
    solve_multi_dev(nrhs, args, sweeps, residual, (cudaStream_t)stream);
  });
}

int fpm_solve_stairstep_learned_dev(void* net, int nrhs, double* const* phi, const double* const* rhs,
                                    const int32_t* solid, const double* body_grads, const double* const* faces,
                                    const double* xc, const double* yc, const double* zc, const double* dx,
                                    const double* dy, const double* dz, int nx, int ny, int nz, double tolerance,
                                    int max_sweeps, int check_interval, int method, int* sweeps, double* residual,
                                    int* fallbacks, void* stream) {
  return guarded([&] {
    if (!net) throw Error{FPM_E_ARG, "null network handle"};
    SolveArgs args[kMaxRhs];
    multi_args(nrhs, phi, rhs, solid, body_grads, faces, xc, yc, zc, dx, dy, dz, nx, ny, nz, tolerance, max_sweeps,
               check_interval, method, sweeps, residual, args);
    if (fallbacks)
      for (int m = 0; m < nrhs; m++) fallbacks[m] = 0;
    solve_multi_dev(nrhs, args, sweeps, residual, (cudaStream_t)stream, net, fallbacks);
  });
}

int fpm_net_prepare_inputs_dev(const double* src, const double* diag, const double* dx, const double* dy,
                               const double* dz, int nx, int ny, int nz, uint8_t* fluid, float* mx, float* my,
                               float* mz, float* b, void* stream) {
  return guarded([&] {
    if (!src || !diag || !dx || !dy || !dz || !fluid || !mx || !my || !mz || !b) throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = (cudaStream_t)stream;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    Common cm = make_common(A, d, st);
    double* bmax = A.get<double>(1);
    Axes ax{nullptr, nullptr, nullptr, dx, dy, dz};
    CUDA_TRY(launch_learn_inputs(d, src, diag, ax, fluid, mx, my, mz, b, bmax, cm.rb, st));
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
    double* rcp = A.get<double>((long long)(nx + 2) + (ny + 2) + nz);
    CUDA_TRY(launch_terms(d, phi, fl, solid, body_grad, axes, f, bounds, o, rcp, cm.S, cm.rb, st));
    const SolveScalars& h = read_scalars(cm.S, st);
    totals[0] = h.red[0];
    totals[1] = h.red[1];
  });
}

int fpm_compute_stairstep_fpm_terms_3d_multi_dev(int npot, const double* const* phi, const double* u,
                                                 const double* v, const double* w, const double* ox,
                                                 const double* oy, const double* oz, const double* ax,
                                                 const double* ay, const double* az, const int32_t* solid,
                                                 const double* body_grad, const double* xc, const double* yc,
                                                 const double* zc, const double* dx, const double* dy,
                                                 const double* dz, const double* const* faces, const double* bounds,
                                                 double* const* outs, double* totals, int nx, int ny, int nz,
                                                 void* stream) {
  return guarded([&] {
    if (npot < 1 || npot > kMaxRhs) throw Error{FPM_E_ARG, "npot must be 1..4"};
    if (!phi || !u || !v || !w || !ox || !oy || !oz || !ax || !ay || !az || !solid || !body_grad || !xc || !yc ||
        !zc || !dx || !dy || !dz || !faces || !bounds || !outs || !totals)
      throw Error{FPM_E_ARG, "null argument"};
    for (int m = 0; m < npot; m++) {
      if (!phi[m]) throw Error{FPM_E_ARG, "null argument"};
      for (int c = 0; c < 6; c++)
        if (!faces[6 * m + c]) throw Error{FPM_E_ARG, "null argument"};
      for (int c = 0; c < 5; c++)
        if (!outs[5 * m + c]) throw Error{FPM_E_ARG, "null argument"};
    }
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = (cudaStream_t)stream;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    Trace t("stair-step FPM terms");
    Flow fl{u, v, w, ox, oy, oz, ax, ay, az};
    Axes axes{xc, yc, zc, dx, dy, dz};
    Faces f[kMaxRhs];
    for (int m = 0; m < npot; m++)
      f[m] = Faces{const_cast<double*>(faces[6 * m]),     const_cast<double*>(faces[6 * m + 1]),
                   const_cast<double*>(faces[6 * m + 2]), const_cast<double*>(faces[6 * m + 3]),
                   const_cast<double*>(faces[6 * m + 4]), const_cast<double*>(faces[6 * m + 5])};
    const dim3 tg = terms_multi_grid(d);
    const size_t nb = (size_t)tg.x * tg.y * tg.z;
    double* partials = A.get<double>(2 * (size_t)npot * nb);
    unsigned int* ticket = A.get<unsigned int>(1);
    double* dtot = A.get<double>(2 * (size_t)npot);
    void* tables = A.get<unsigned char>(terms_multi_table_bytes(d));
    CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st));
    CUDA_TRY(launch_terms_multi(d, npot, phi, fl, solid, body_grad, axes, f, bounds, outs, tables, partials, ticket,
                                dtot, st));
    CUDA_TRY(cudaMemcpyAsync(totals, dtot, 2 * npot * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
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
    if (method != FPM_METHOD_JACOBI && method != FPM_METHOD_JACOBI_DF && method != FPM_METHOD_JACOBI_FMA &&
        method != FPM_METHOD_JACOBI_TF)
      throw Error{FPM_E_METHOD, "sweeps need method jacobi, jacobi_fma, jacobi_tf or jacobi_df"};
    require_device();
    cudaStream_t st = (cudaStream_t)stream;
    const Dims d{nx, ny, nz};
    Scratch A(st);
    const long long ncoef = 2LL * (nx + ny + nz);
    double* coef = A.get<double>(ncoef);
    CUDA_TRY(launch_axis_coefs(Axes{xc, yc, zc, dx, dy, dz}, nx, ny, nz, coef, st));
    if (method == FPM_METHOD_JACOBI || method == FPM_METHOD_JACOBI_FMA) {
      Coefs c = coef_views(coef, nx, ny, nz);
      double *cur = a, *oth = b;
      TimedRun t(FPM_TIMER_JACOBI_F64, nsweeps, st);
      for (int s = 0; s < nsweeps; s++) {
        CUDA_TRY(method == FPM_METHOD_JACOBI_FMA ? launch_jacobi_f64_fma(d, cur, oth, src, rdiag, c, st)
                                                 : launch_jacobi_f64(d, cur, oth, src, rdiag, c, st));
        std::swap(cur, oth);
      }
    } else if (method == FPM_METHOD_JACOBI_TF) {
      JacobiTfPlan pl = make_tf_plan(A, d);
      CUDA_TRY(jacobi_tf_pack(pl, a, src, rdiag, coef, st));
      tf_choose(pl, st);
      CUDA_TRY(cudaMemsetAsync(pl.err, 0, sizeof(int), st));
      CUDA_TRY(jacobi_tf_pack(pl, a, src, rdiag, coef, st));  // the autotuner overwrote b
      double *cur = pl.a, *oth = pl.b;
      {
        TimedRun t(FPM_TIMER_JACOBI_TF, nsweeps, st);
        for (int s = 0; s < nsweeps; s++) {
          CUDA_TRY(jacobi_tf_sweep(pl, cur, oth, st));
          std::swap(cur, oth);
        }
      }
      CUDA_TRY(jacobi_tf_unpack(pl, pl.a, a, st));
      CUDA_TRY(jacobi_tf_unpack(pl, pl.b, b, st));
      int h = 0;
      CUDA_TRY(cudaMemcpyAsync(&h, pl.err, sizeof(int), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaStreamSynchronize(st));
      if (h) throw Error{FPM_E_TIMEOUT, "triple-float Jacobi pipeline wait timed out"};
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

// ---------------------------------------------------------------- batched 2-D frames
// examples/flapping_foil_fpm.f90:61-81 for every frame of a batch at once:
// phi_x, phi_y (nz = 2, dz = 0.5, zero outer data, compatibility, mixed PCG
// to the tolerance, gauge), then fpm_partition_terms_2d for both directions.
int fpm_partition_frames_2d(int nframes, const int* nx, const int* ny, const double* const* xf,
                            const double* const* yf, const double* const* u, const double* const* v,
                            const uint8_t* const* solid, const double* const* ring, const double* kin,
                            const double* dt, double nu, double tolerance, int max_sweeps, int check_interval,
                            double* terms, int* sweeps, double* residual, double* const* phi_out) {
  return guarded([&] {
    if (nframes < 1) throw Error{FPM_E_SIZE, "no frames"};
    if (!nx || !ny || !xf || !yf || !u || !v || !solid || !ring || !kin || !dt || !terms || !sweeps || !residual)
      throw Error{FPM_E_ARG, "null argument"};
    require_device();
    cudaStream_t st = 0;
    std::vector<Frame2> fr(nframes);
    std::vector<int> tile_frame;
    long long npx = 0, npy = 0, npad = 0, nint = 0, n2 = 0, nring = 0;
    for (int f = 0; f < nframes; f++) {
      if (nx[f] < 1 || ny[f] < 1) throw Error{FPM_E_SIZE, "frame with no cells"};
      if (!xf[f] || !yf[f] || !u[f] || !v[f] || !solid[f] || !ring[f]) throw Error{FPM_E_ARG, "null frame array"};
      Frame2& F = fr[f];
      F.nx = nx[f];
      F.ny = ny[f];
      F.tiles_x = (F.nx + 31) / 32;
      F.tile0 = (int)tile_frame.size();
      F.ntiles = F.tiles_x * ((F.ny + 7) / 8);
      for (int t = 0; t < F.ntiles; t++) tile_frame.push_back(f);
      F.ox = (int)npx;
      F.oy = (int)npy;
      F.opad = npad;
      F.oint = nint;
      F.o2 = n2;
      F.oring = nring;
      npx += F.nx + 2;
      npy += F.ny + 2;
      npad += (long long)(F.nx + 2) * (F.ny + 2) * 2;
      nint += (long long)F.nx * F.ny * 2;
      n2 += (long long)F.nx * F.ny;
      nring += 4LL * (2LL * F.nx + 2LL * F.ny);
    }
    const int ntiles = (int)tile_frame.size();
    // Host staging of the pools (axes as in examples/flapping_foil_fpm.f90:211-213).
    std::vector<double> hxc(npx), hdx(npx), hxf(npx), hyc(npy), hdy(npy), hyf(npy);
    std::vector<int32_t> hs3(npad, 0);
    std::vector<uint8_t> hs2(n2);
    std::vector<double> hu(n2), hv(n2), hring(nring);
    for (int f = 0; f < nframes; f++) {
      const Frame2& F = fr[f];
      for (int i = 0; i <= F.nx; i++) hxf[F.ox + i] = xf[f][i];
      for (int i = 1; i <= F.nx; i++) {
        hdx[F.ox + i - 1] = xf[f][i] - xf[f][i - 1];
        hxc[F.ox + i] = 0.5 * (xf[f][i - 1] + xf[f][i]);
      }
      hxc[F.ox] = hxc[F.ox + 1] - hdx[F.ox];
      hxc[F.ox + F.nx + 1] = hxc[F.ox + F.nx] + hdx[F.ox + F.nx - 1];
      for (int j = 0; j <= F.ny; j++) hyf[F.oy + j] = yf[f][j];
      for (int j = 1; j <= F.ny; j++) {
        hdy[F.oy + j - 1] = yf[f][j] - yf[f][j - 1];
        hyc[F.oy + j] = 0.5 * (yf[f][j - 1] + yf[f][j]);
      }
      hyc[F.oy] = hyc[F.oy + 1] - hdy[F.oy];
      hyc[F.oy + F.ny + 1] = hyc[F.oy + F.ny] + hdy[F.oy + F.ny - 1];
      const long long cells = (long long)F.nx * F.ny;
      for (long long m = 0; m < cells; m++) {
        const int i = (int)(m % F.nx) + 1, j = (int)(m / F.nx) + 1;
        const uint8_t sv = solid[f][m] ? 1 : 0;
        hs2[F.o2 + m] = sv;
        for (int k = 1; k <= 2; k++) hs3[F.opad + i + (long long)(F.nx + 2) * (j + (long long)(F.ny + 2) * (k - 1))] = sv;
      }
      std::memcpy(&hu[F.o2], u[f], cells * sizeof(double));
      std::memcpy(&hv[F.o2], v[f], cells * sizeof(double));
      std::memcpy(&hring[F.oring], ring[f], 4 * (2LL * F.nx + 2LL * F.ny) * sizeof(double));
    }
    Scratch A(st);
    Frame2* dfr = A.upload(fr.data(), fr.size());
    int* dtf = A.upload(tile_frame.data(), tile_frame.size());
    Batch2 b;
    std::memset(&b, 0, sizeof(b));
    std::memset(&b, 0, sizeof(b));
    b.xc = A.upload(hxc.data(), hxc.size());
    b.dx = A.upload(hdx.data(), hdx.size());
    b.xf = A.upload(hxf.data(), hxf.size());
    b.yc = A.upload(hyc.data(), hyc.size());
    b.dy = A.upload(hdy.data(), hdy.size());
    b.yf = A.upload(hyf.data(), hyf.size());
    b.solid3 = A.upload(hs3.data(), hs3.size());
    b.solid2 = A.upload(hs2.data(), hs2.size());
    b.u = A.upload(hu.data(), hu.size());
    b.v = A.upload(hv.data(), hv.size());
    b.ring = A.upload(hring.data(), hring.size());
    b.kin = A.upload(kin, 6 * (size_t)nframes);
    b.dt = A.upload(dt, (size_t)nframes);
    b.nu = nu;
    for (int r = 0; r < 2; r++) {
      b.src[r] = A.get<double>(nint);
      b.phi[r] = A.get<double>(npad);
      CUDA_TRY(cudaMemsetAsync(b.phi[r], 0, npad * sizeof(double), st));
      b.phi_best[r] = A.get<double>(npad);
      CUDA_TRY(cudaMemsetAsync(b.phi_best[r], 0, npad * sizeof(double), st));
      b.r64[r] = A.get<double>(nint);
      b.r32[r] = A.get<float>(nint);
      b.p32[r] = A.get<float>(npad);
      CUDA_TRY(cudaMemsetAsync(b.p32[r], 0, npad * sizeof(float), st));
      b.q32[r] = A.get<float>(nint);
      b.e32[r] = A.get<float>(nint);
      b.gpx[r] = A.get<double>(n2);
      b.gpy[r] = A.get<double>(n2);
      b.vif[r] = A.get<double>(n2);
    }
    b.diag = A.get<double>(nint);
    b.rdiag = A.get<double>(nint);
    b.diag32 = A.get<float>(nint);
    b.rdiag32 = A.get<float>(nint);
    b.wall32 = A.get<float>(nint);
    b.cw32 = A.get<float>(npx);
    b.ce32 = A.get<float>(npx);
    b.cs32 = A.get<float>(npy);
    b.cn32 = A.get<float>(npy);
    b.nxf = A.get<double>(n2);
    b.nyf = A.get<double>(n2);
    b.omega = A.get<double>(n2);
    const size_t nq = 2 * (size_t)nframes;
    b.terms = A.get<double>(8 * (size_t)nframes);
    b.corr = A.get<double>(nq);
    b.res = A.get<double>(nq);
    b.rmean = A.get<double>(nq);
    b.scale = A.get<double>(nq);
    b.rz = A.get<double>(nq);
    b.rz0 = A.get<double>(nq);
    b.alpha = A.get<double>(nq);
    b.beta = A.get<double>(nq);
    b.in_set = A.get<int>(nq);
    b.active = A.get<int>(nq);
    b.iters = A.get<int>(nq);
    CUDA_TRY(cudaMemsetAsync(b.iters, 0, nq * sizeof(int), st));
    CUDA_TRY(cudaMemsetAsync(b.active, 0, nq * sizeof(int), st));
    b.tol2 = kUpdateDrop * kUpdateDrop;  // each (frame, direction) stops its FP32 iteration at the update drop
                                         // (the multigrid method sets its own below)
    b.pmul = A.get<double>(nq);
    b.keep = A.get<int>(nq);
    b.dir = A.get<int>(nq);
    CUDA_TRY(cudaMemsetAsync(b.dir, 0, nq * sizeof(int), st));
    b.partials = A.get<double>(8 * (size_t)ntiles);
    b.tickets = A.get<unsigned int>(nframes);
    CUDA_TRY(cudaMemsetAsync(b.tickets, 0, nframes * sizeof(unsigned int), st));
    b.err = A.get<int>(1);
    CUDA_TRY(cudaMemsetAsync(b.err, 0, sizeof(int), st));

    Trace tr("frames: compatibility and operator");
    CUDA_TRY(launch_k_b2_compat(dfr, dtf, ntiles, b, st));
    CUDA_TRY(launch_k_b2_build(dfr, dtf, ntiles, b, st));
    std::vector<int> set(nq, 1), stall(nq, 0), act(nq);
    std::vector<double> res(nq), scale(nq);
    auto push_set = [&] {
      CUDA_TRY(cudaMemcpyAsync(b.in_set, set.data(), nq * sizeof(int), cudaMemcpyHostToDevice, st));
    };
    auto pull = [&](void* h, const void* d, size_t bytes) {
      CUDA_TRY(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaStreamSynchronize(st));
    };
    push_set();
    CUDA_TRY(launch_k_b2_tres(dfr, dtf, ntiles, b, st));
    pull(res.data(), b.res, nq * sizeof(double));
    int err = 0;
    pull(&err, b.err, sizeof(int));
    if (err == 2) throw Error{FPM_E_NO_OUTER_FACE, "stair-step compatibility needs at least one fluid outer face"};
    // Reliable updates per (frame, direction), as in mixed_solve.
    const int chunk_len = check_interval < 1 ? 1 : check_interval;
    long long total = 0;
    ChunkGraphs graphs;
    // 10 % margin: the final residual pass after the gauge re-evaluates the
    // potentials with a different summation order, which near the FP64 floor
    // can move the max-norm by ~1e-3 relative
    const double target = 0.9 * tolerance;
    std::vector<double> best(res), prev(res), pmul(nq, 0.0), rz(nq), rz0(nq);
    std::vector<int> live(nq), since(nq, 0), keepv(nq, 0), slow(nq, 0), to64(nq, 0), extra_its(nq, 0);
    bool any = false;
    for (size_t q = 0; q < nq; q++) {
      live[q] = res[q] > target && res[q] == res[q];
      set[q] = live[q];
      scale[q] = res[q] > 0 ? 1.0 / res[q] : 1.0;
      any = any || live[q];
    }
    // Frame method: the batched FP32 diagonal PCG above, or (multigrid)
    // every (frame, direction) solved on its own by the multigrid-
    // preconditioned refinement, several at once on worker streams.
    // Frame method: every frame's pair in the same launches with the batched
    // 2-D multigrid preconditioner (default), the same with the diagonal
    // preconditioner (FPM_FRAMES_METHOD=batched), or every pair solved on its
    // own by the multigrid-preconditioned refinement on worker streams
    // (FPM_FRAMES_METHOD=individual).
    const int fmethod = [] {
      const char* e = std::getenv("FPM_FRAMES_METHOD");
      if (e && std::strcmp(e, "batched") == 0) return 0;
      if (e && std::strcmp(e, "individual") == 0) return 1;
      return 2;
    }();
    const int frames_mg = fmethod == 1;
    const bool batched_mg = fmethod == 2;
    int individual_method = batched_mg ? FPM_METHOD_PCG_MG : FPM_METHOD_PCG;
    const double fdrop = mg_drop(0.0, true);
    const double drop2 = batched_mg ? fdrop * fdrop : kUpdateDrop * kUpdateDrop;
    b.tol2 = drop2;
    // the multigrid hierarchy of every frame
    FramesMg M;
    std::memset(&M, 0, sizeof(M));
    std::vector<int> nrestrict_lv(kFmMaxLevels, 0), nall_lv(kFmMaxLevels, 0);
    int nbtiles = 0;
    std::vector<int4> hbt_info;
    if (batched_mg) {
      Trace tm("frames: multigrid set-up");
      std::vector<int> nlev(nframes);
      std::vector<FmLevel> lv((size_t)nframes * kFmMaxLevels, FmLevel{0, 0, 0});
      std::vector<long long> pool(kFmMaxLevels, 0);
      int maxlev = 0;
      for (int f = 0; f < nframes; f++) {
        int nxl = fr[f].nx, nyl = fr[f].ny, l = 0;
        lv[(size_t)f * kFmMaxLevels] = FmLevel{nxl, nyl, fr[f].o2};
        while (l + 1 < kFmMaxLevels && (l < 1 || nxl > kFmCoarseSide || nyl > kFmCoarseSide)) {
          nxl = (nxl + 1) / 2;
          nyl = (nyl + 1) / 2;
          l++;
          lv[(size_t)f * kFmMaxLevels + l] = FmLevel{nxl, nyl, pool[l]};
          pool[l] += (long long)nxl * nyl;
        }
        if (nxl > kFmCoarseSide || nyl > kFmCoarseSide)
          throw Error{FPM_E_LIMIT, "frame too large for the multigrid hierarchy"};
        nlev[f] = l + 1;
        maxlev = std::max(maxlev, l + 1);
      }
      M.nlev = maxlev;
      M.omega = (float)env_double("FPM_FRAMES_OMEGA", 0.9);
      M.coarse_sweeps = (int)env_double("FPM_FRAMES_COARSE_SWEEPS", 60);
      M.cscale = (float)env_double("FPM_FRAMES_CSCALE", 1.0);
      M.lv = A.upload(lv.data(), lv.size());
      M.nlevels = A.upload(nlev.data(), nlev.size());
      for (int l = 1; l < maxlev; l++) {
        // tiles of the frames that have level l: those for which it is not the
        // coarsest first (restriction and prolongation walk that prefix)
        std::vector<FmTile> tl;
        for (int pass = 0; pass < 2; pass++)
          for (int f = 0; f < nframes; f++) {
            if (nlev[f] <= l) continue;
            const bool coarsest = nlev[f] - 1 == l;
            if (coarsest != (pass == 1)) continue;
            const FmLevel& L = lv[(size_t)f * kFmMaxLevels + l];
            for (int j0 = 0; j0 < L.ny; j0 += 8)
              for (int i0 = 0; i0 < L.nx; i0 += 32) tl.push_back(FmTile{f, i0, j0});
            if (pass == 0) nrestrict_lv[l] = (int)tl.size();
          }
        nall_lv[l] = (int)tl.size();
        M.tiles[l] = A.upload(tl.data(), tl.size());
        M.te[l] = A.get<float>(pool[l]);
        M.tn[l] = A.get<float>(pool[l]);
        M.dinv[l] = A.get<float>(pool[l]);
        for (int r = 0; r < 2; r++) {
          M.b[l][r] = A.get<float>(pool[l]);
          M.xa[l][r] = A.get<float>(pool[l]);
          M.xb[l][r] = A.get<float>(pool[l]);
        }
      }
      M.te[0] = A.get<float>(n2);
      M.tn[0] = A.get<float>(n2);
      M.dinv[0] = A.get<float>(n2);
      for (int r = 0; r < 2; r++) {
        M.r[r] = A.get<float>(n2);
        M.z[r] = A.get<float>(n2);
        M.p[r] = A.get<float>(n2);
        M.q[r] = A.get<float>(n2);
        M.e[r] = A.get<float>(n2);
        M.r2[r] = A.get<float>(n2);
        M.p2[r] = A.get<float>(n2);
      }
      // level-0 block tiles (32 x 8 rows cells, rows 2, 4 or 8 per thread) of the stencil passes
      const int brows = (int)env_double("FPM_FRAMES_ROWS", 4);
      M.bt_rows = brows == 2 || brows == 8 ? brows : 4;
      const int bh = 8 * M.bt_rows;
      std::vector<int> bt_frame;
      std::vector<int4> bt_info(nframes);
      for (int f = 0; f < nframes; f++) {
        const int bx = (fr[f].nx + 31) / 32, nbt = bx * ((fr[f].ny + bh - 1) / bh);
        bt_info[f] = make_int4((int)bt_frame.size(), nbt, bx, 0);
        for (int t = 0; t < nbt; t++) bt_frame.push_back(f);
      }
      nbtiles = (int)bt_frame.size();
      M.bt_frame = A.upload(bt_frame.data(), bt_frame.size());
      M.bt_info = A.upload(bt_info.data(), bt_info.size());
      M.bt_list = A.get<int>(nbtiles);
      hbt_info = bt_info;
      CUDA_TRY(fm_setup(dfr, dtf, ntiles, b, M, nall_lv.data(), st));
    }
    if (frames_mg) {
      for (size_t q = 0; q < nq; q++) {
        to64[q] = live[q];
        live[q] = 0;
      }
      any = false;
      individual_method = FPM_METHOD_PCG_MG;
    }
    auto push_start = [&] {
      push_set();
      CUDA_TRY(cudaMemcpyAsync(b.scale, scale.data(), nq * sizeof(double), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(b.pmul, pmul.data(), nq * sizeof(double), cudaMemcpyHostToDevice, st));
      if (batched_mg) CUDA_TRY(fm_start(dfr, dtf, ntiles, nbtiles, b, M, nrestrict_lv.data(), nframes, st));
      else CUDA_TRY(launch_k_b2_start(dfr, dtf, ntiles, b, st));
    };
    if (any) push_start();
    // The iteration kernels run over the tiles of the frames that still have
    // a live direction; the list is compacted whenever frames finish.
    int* dtiles = A.get<int>(ntiles);
    std::vector<int> act_tiles;
    std::vector<char> frame_on(nframes, 0);
    Batch2 bi = b;
    bi.tiles = dtiles;
    int nact = 0, nbact = 0;
    std::vector<int> act_bt;
    auto rebuild_tiles = [&]() {
      bool changed = false;
      for (int f = 0; f < nframes; f++) {
        const char on = (live[2 * f] || live[2 * f + 1]) ? 1 : 0;
        changed = changed || on != frame_on[f];
        frame_on[f] = on;
      }
      if (!changed) return;
      act_tiles.clear();
      for (int f = 0; f < nframes; f++)
        if (frame_on[f])
          for (int t = 0; t < fr[f].ntiles; t++) act_tiles.push_back(fr[f].tile0 + t);
      nact = (int)act_tiles.size();
      if (nact) CUDA_TRY(cudaMemcpyAsync(dtiles, act_tiles.data(), nact * sizeof(int), cudaMemcpyHostToDevice, st));
      if (batched_mg) {
        act_bt.clear();
        for (int f = 0; f < nframes; f++)
          if (frame_on[f])
            for (int t = 0; t < hbt_info[f].y; t++) act_bt.push_back(hbt_info[f].x + t);
        nbact = (int)act_bt.size();
        if (nbact)
          CUDA_TRY(cudaMemcpyAsync(M.bt_list, act_bt.data(), nbact * sizeof(int), cudaMemcpyHostToDevice, st));
      }
      graphs.clear();
    };
    rebuild_tiles();
    // With the batched multigrid, the last pairs (the frames whose aggregates
    // straddle the body converge slowly) leave the batch when at most this
    // fraction of the pairs is still iterating: each is then solved on its
    // own, several at once, instead of the whole batch's launches running
    // for a few frames.
    const double tail = batched_mg ? env_double("FPM_FRAMES_TAIL", 0.2) : 0.0;
    int nlive0 = 0;
    for (size_t q = 0; q < nq; q++) nlive0 += live[q];
    while (any && total < max_sweeps) {
      if (tail > 0) {
        int nlive = 0;
        for (size_t q = 0; q < nq; q++) nlive += live[q];
        if (nlive <= tail * nlive0) break;
      }
      int chunk = chunk_len;
      if (chunk > max_sweeps - total) chunk = (int)(max_sweeps - total);
      {
        TimedRun t(FPM_TIMER_FRAMES_ITER, chunk, st);
        graphs.run(chunk, st, [&](cudaStream_t s2) {
          if (batched_mg) CUDA_TRY(fm_iteration(dfr, nbact, bi, M, nrestrict_lv.data(), nframes, s2));
          else CUDA_TRY(launch_b2_iteration(dfr, dtf, nact, bi, s2));
        });
      }
      total += chunk;
      pull(act.data(), b.active, nq * sizeof(int));
      pull(rz.data(), b.rz, nq * sizeof(double));
      pull(rz0.data(), b.rz0, nq * sizeof(double));
      bool upd = false;
      for (size_t q = 0; q < nq; q++) {
        set[q] = 0;
        if (!live[q]) continue;
        since[q] += chunk;
        const bool dropped = rz[q] <= drop2 * rz0[q];
        const bool broke = !act[q] && !dropped;
        if (broke || dropped || since[q] >= kUpdateMax || total >= max_sweeps) {
          set[q] = 1;
          pmul[q] = broke ? 0.0 : 1.0;
          upd = true;
        }
      }
      if (!upd) continue;
      push_set();  // apply with the scales the corrections were computed in
      if (batched_mg) CUDA_TRY(fm_apply(dfr, dtf, ntiles, b, M, st));
      else CUDA_TRY(launch_k_b2_apply(dfr, dtf, ntiles, b, st));
      CUDA_TRY(launch_k_b2_tres(dfr, dtf, ntiles, b, st));
      pull(res.data(), b.res, nq * sizeof(double));
      {
        // corrections that made things much worse: back to the best iterate,
        // restart the direction there
        bool back = false;
        for (size_t q = 0; q < nq; q++) {
          keepv[q] = 0;
          if (set[q] && !(res[q] <= kBlowup * best[q])) {
            keepv[q] = 2;
            pmul[q] = 0.0;
            back = true;
          }
        }
        if (back) {
          CUDA_TRY(cudaMemcpyAsync(b.keep, keepv.data(), nq * sizeof(int), cudaMemcpyHostToDevice, st));
          CUDA_TRY(launch_k_b2_keep(dfr, dtf, ntiles, b, st));
          CUDA_TRY(launch_k_b2_tres(dfr, dtf, ntiles, b, st));
          pull(res.data(), b.res, nq * sizeof(double));
        }
      }
      any = false;
      bool keep_any = false;
      for (size_t q = 0; q < nq; q++) {
        keepv[q] = 0;
        if (set[q]) {
          since[q] = 0;
          stall[q] = res[q] < 0.99 * best[q] ? 0 : stall[q] + 1;
          if (res[q] < best[q]) {
            best[q] = res[q];
            keepv[q] = 1;
          }
          const bool restart = !(res[q] < kUpdateGain * prev[q]);
          if (verbose_level() >= 2)
            std::fprintf(stderr, "fpm frames: q %zu iterations %lld residual %.3e previous %.3e %s%s\n", q, total,
                         res[q], prev[q], act[q] ? "" : "breakdown ", restart ? "restart" : "keep");
          slow[q] = res[q] * kSlowGain > prev[q] ? slow[q] + 1 : 0;
          prev[q] = res[q];
          const bool hand_over = slow[q] >= kSlowUpdates && res[q] > target;
          if (!(res[q] > target) || !(res[q] == res[q]) || stall[q] >= kStallUpdates || hand_over) {
            live[q] = 0;
            set[q] = 0;
            act[q] = 0;
            if (hand_over) to64[q] = 1;
            if (!(res[q] <= best[q])) keepv[q] = 2;  // finish on the best iterate
          } else {
            const double ns = res[q] > 0 ? 1.0 / res[q] : 1.0;
            pmul[q] = (pmul[q] == 0.0 || restart) ? 0.0 : ns / scale[q];
            scale[q] = ns;
          }
          keep_any = keep_any || keepv[q] != 0;
        }
        any = any || live[q];
      }
      if (keep_any) {
        CUDA_TRY(cudaMemcpyAsync(b.keep, keepv.data(), nq * sizeof(int), cudaMemcpyHostToDevice, st));
        CUDA_TRY(launch_k_b2_keep(dfr, dtf, ntiles, b, st));
      }
      CUDA_TRY(cudaMemcpyAsync(b.active, act.data(), nq * sizeof(int), cudaMemcpyHostToDevice, st));
      rebuild_tiles();
      bool refresh = false;
      for (size_t q = 0; q < nq; q++) refresh = refresh || set[q];
      if (refresh) push_start();
      if (verbose()) {
        int nlive = 0;
        double worst = 0;
        for (size_t q = 0; q < nq; q++) {
          nlive += live[q];
          if (live[q] && res[q] > worst) worst = res[q];
        }
        std::fprintf(stderr, "fpm frames: iterations %lld live %d worst live residual %.3e\n", total, nlive, worst);
      }
    }
    // fold in corrections still pending (stopped by the iteration cap)
    bool pend = false;
    for (size_t q = 0; q < nq; q++) {
      set[q] = live[q];
      pend = pend || live[q];
    }
    if (pend) {
      push_set();
      if (batched_mg) CUDA_TRY(fm_apply(dfr, dtf, ntiles, b, M, st));
      else CUDA_TRY(launch_k_b2_apply(dfr, dtf, ntiles, b, st));
      // the batch's tail: solved on its own from the current phi
      if (batched_mg)
        for (size_t q = 0; q < nq; q++)
          if (live[q]) to64[q] = 1;
    }
    // (frame, direction) pairs solved on their own: with the multigrid frame
    // method all of them; otherwise those whose FP32 iteration stagnated
    // (FP64 PCG from their current phi).  Each is the reference's 3-D solve of
    // that frame with nz = 2 and the outer face data of its compatibility
    // correction.
    {
      bool any64 = false;
      for (size_t q = 0; q < nq; q++) any64 = any64 || to64[q];
      if (any64) {
        Trace t64("frames: individual solves");
        std::vector<double> hcorr(nq);
        pull(hcorr.data(), b.corr, nq * sizeof(double));
        const double zc2[2] = {0.25, 0.75}, dz2[2] = {0.5, 0.5};
        double* dzc = A.upload(zc2, 2);
        double* ddz = A.upload(dz2, 2);
        // jobs[job_first[n] .. job_first[n + 1]) are the directions of one
        // frame, solved together (they share the solid flags and the axes)
        std::vector<SolveArgs> jobs;
        std::vector<size_t> job_q, job_first;
        for (int f = 0; f < nframes; f++) {
          if (to64[2 * (size_t)f] || to64[2 * (size_t)f + 1]) job_first.push_back(jobs.size());
          for (int r = 0; r < 2; r++) {
            const size_t q = 2 * (size_t)f + r;
            if (!to64[q]) continue;
            const Frame2& F = fr[f];
            const int fnx = F.nx, fny = F.ny;
            const double cr = hcorr[q];
            std::vector<double> xl((size_t)fny * 2, -cr), xh((size_t)fny * 2, cr), yl((size_t)fnx * 2, -cr),
                yh((size_t)fnx * 2, cr), zl((size_t)fnx * fny, -cr), zh((size_t)fnx * fny, cr);
            SolveArgs a;
            a.phi = b.phi[r] + F.opad;
            double* zero_rhs = A.get<double>((size_t)fnx * fny * 2);
            CUDA_TRY(cudaMemsetAsync(zero_rhs, 0, (size_t)fnx * fny * 2 * sizeof(double), st));
            a.rhs = zero_rhs;
            a.solid = b.solid3 + F.opad;
            a.bg[0] = r == 0 ? 1.0 : 0.0;
            a.bg[1] = r == 1 ? 1.0 : 0.0;
            a.bg[2] = 0.0;
            a.f = Faces{A.upload(xl.data(), xl.size()), A.upload(xh.data(), xh.size()), A.upload(yl.data(), yl.size()),
                        A.upload(yh.data(), yh.size()), A.upload(zl.data(), zl.size()), A.upload(zh.data(), zh.size())};
            a.ax = Axes{b.xc + F.ox, b.yc + F.oy, dzc, b.dx + F.ox, b.dy + F.oy, ddz};
            a.nx = fnx;
            a.ny = fny;
            a.nz = 2;
            // 10 % margin: the batch's own residual pass re-evaluates these
            // potentials with a different summation order, which near the FP64
            // floor can move the max-norm by ~1e-3 relative
            a.tol = 0.9 * tolerance;
            a.max_sweeps = max_sweeps;
            a.ci = check_interval;
            a.method = individual_method;
            jobs.push_back(a);
            job_q.push_back(q);
          }
        }
        job_first.push_back(jobs.size());
        const size_t ngroups = job_first.size() - 1;
        CUDA_TRY(cudaStreamSynchronize(st));
        // The frames are small next to the GPU, so several of them are solved
        // at once: host worker threads, one stream each.
        int dev = 0;
        CUDA_TRY(cudaGetDevice(&dev));
        const int nworkers = (int)std::min<size_t>(ngroups, (size_t)env_double("FPM_FRAMES_WORKERS", 12));
        std::vector<int> sws(jobs.size(), 0);
        std::vector<double> rrs(jobs.size(), 0.0);
        std::vector<std::string> errs(nworkers);
        std::vector<int> codes(nworkers, FPM_OK);
        std::atomic<size_t> next_job{0};
        std::vector<std::thread> pool;
        for (int w = 0; w < nworkers; w++) {
          pool.emplace_back([&, w] {
            cudaStream_t ws = nullptr;
            try {
              CUDA_TRY(cudaSetDevice(dev));
              CUDA_TRY(cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking));
              for (size_t n = next_job++; n < ngroups; n = next_job++) {
                const size_t j = job_first[n];
                solve_multi_dev((int)(job_first[n + 1] - j), &jobs[j], &sws[j], &rrs[j], ws);
              }
            } catch (const Error& e) {
              codes[w] = e.code;
              errs[w] = e.msg;
            }
            if (ws) cudaStreamDestroy(ws);
          });
        }
        for (auto& t : pool) t.join();
        for (int w = 0; w < nworkers; w++)
          if (codes[w] != FPM_OK) throw Error{codes[w], errs[w]};
        for (size_t j = 0; j < jobs.size(); j++) {
          extra_its[job_q[j]] = sws[j];
          if (verbose())
            std::fprintf(stderr, "fpm frames: frame %zu direction %zu solved alone: %d iterations, residual %.3e\n",
                         job_q[j] / 2, job_q[j] % 2, sws[j], rrs[j]);
        }
      }
    }
    Trace tg("frames: gauge and partition");
    for (size_t q = 0; q < nq; q++) set[q] = to64[q] ? 0 : 1;  // individually solved ones are gauged
    push_set();
    CUDA_TRY(launch_k_b2_gauge_sum(dfr, dtf, ntiles, b, st));
    CUDA_TRY(launch_k_b2_gauge_sub(dfr, dtf, ntiles, b, st));
    std::fill(set.begin(), set.end(), 1);
    push_set();
    CUDA_TRY(launch_k_b2_tres(dfr, dtf, ntiles, b, st));
    CUDA_TRY(launch_k_b2_part1(dfr, dtf, ntiles, b, st));
    CUDA_TRY(launch_k_b2_part2(dfr, dtf, ntiles, b, st));
    pull(residual, b.res, nq * sizeof(double));
    pull(sweeps, b.iters, nq * sizeof(int));
    for (size_t q = 0; q < nq; q++) sweeps[q] += extra_its[q];
    pull(terms, b.terms, 8 * (size_t)nframes * sizeof(double));
    if (phi_out) {
      for (int f = 0; f < nframes; f++) {
        if (!phi_out[f]) continue;
        const Frame2& F = fr[f];
        // layer k = 1 of each direction, (nx, ny) column-major, direction-major
        for (int r = 0; r < 2; r++)
          CUDA_TRY(cudaMemcpy2DAsync(phi_out[f] + (size_t)r * F.nx * F.ny, F.nx * sizeof(double),
                                     b.phi[r] + F.opad + 1 + (F.nx + 2), (F.nx + 2) * sizeof(double),
                                     F.nx * sizeof(double), F.ny, cudaMemcpyDeviceToHost, st));
      }
      CUDA_TRY(cudaStreamSynchronize(st));
    }
  });
}

int fpm_stairstep_operator_residual_noalloc_dev(const double* phi, const double* src, const double* diag,
                                                const double* xc, const double* yc, const double* zc,
                                                const double* dx, const double* dy, const double* dz, int nx, int ny,
                                                int nz, double* value, void* stream) {
  return guarded([&] {
    if (!phi || !src || !diag || !xc || !yc || !zc || !dx || !dy || !dz || !value)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    std::string msg;
    const int rc = operator_residual_noalloc(phi, src, diag, Axes{xc, yc, zc, dx, dy, dz}, nx, ny, nz, value,
                                             (cudaStream_t)stream, &msg);
    if (rc != FPM_OK) throw Error{rc, msg};
  });
}

int fpm_partition_terms_3d(const double* phi, const double* g, const double* u, const double* v, const double* w,
                           const uint8_t* solid, const double* xf, const double* yf, const double* zf,
                           const double* kin, const double* shell, double dt, double nu, int nx, int ny, int nz,
                           double* terms, double* vif_density, double* omega, int slip_body) {
  return guarded([&] {
    if (!phi || !g || !u || !v || !w || !solid || !xf || !yf || !zf || !kin || !terms || !vif_density)
      throw Error{FPM_E_ARG, "null argument"};
    if (nx < 1 || ny < 1 || nz < 1) throw Error{FPM_E_SIZE, "empty grid"};
    require_device();
    cudaStream_t st = 0;
    Scratch A(st);
    const size_t n3 = (size_t)nx * ny * nz;
    const size_t L = 2 * (size_t)ny * nz + 2 * (size_t)nx * nz + 2 * (size_t)nx * ny;
    Common cm;
    cm.S = A.get<SolveScalars>(1);
    CUDA_TRY(cudaMemsetAsync(cm.S, 0, sizeof(SolveScalars), st));
    const int nb = ((nx + 31) / 32) * ((ny + 7) / 8) * nz;
    cm.rb.max_blocks = nb;
    cm.rb.partials = A.get<double>((size_t)4 * nb);
    cm.rb.ticket = A.get<unsigned int>(1);
    CUDA_TRY(cudaMemsetAsync(cm.rb.ticket, 0, sizeof(unsigned int), st));
    Part3D p;
    p.phi = A.upload(phi, n3);
    p.u = A.upload(u, n3);
    p.v = A.upload(v, n3);
    p.w = A.upload(w, n3);
    p.solid = A.upload(solid, n3);
    p.xf = A.upload(xf, (size_t)nx + 1);
    p.yf = A.upload(yf, (size_t)ny + 1);
    p.zf = A.upload(zf, (size_t)nz + 1);
    p.kin = A.upload(kin, 12);
    p.shell = shell ? A.upload(shell, 6 * L) : nullptr;
    for (int a = 0; a < 3; a++) p.g[a] = g[a];
    p.dt = dt;
    p.nu = nu;
    p.nx = nx;
    p.ny = ny;
    p.nz = nz;
    p.slip = slip_body ? 1 : 0;
    double* scratch = A.get<double>(6 * n3);
    double* dvif = A.get<double>(n3);
    double* domega = omega ? A.get<double>(3 * n3) : nullptr;
    CUDA_TRY(launch_partition_3d(p, scratch, dvif, domega, cm.S, cm.rb, st));
    const SolveScalars& h = read_scalars(cm.S, st);
    for (int m = 0; m < 4; m++) terms[m] = h.red[m];
    download(vif_density, dvif, n3 * sizeof(double), st);
    if (omega) download(omega, domega, 3 * n3 * sizeof(double), st);
    CUDA_TRY(cudaStreamSynchronize(st));
  });
}

}  // extern "C"
