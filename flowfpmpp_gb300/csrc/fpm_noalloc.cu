// Allocation-free variant of the max-norm operator residual
// (operator_residual, src/fpm_stairstep_mpi_3d.f90:514-530).
//
// Some callers cannot allocate device memory while they run: a solver that
// owns a fixed memory pool, a caller inside a region where cudaMalloc would
// synchronise the device or is forbidden by its allocator policy, or an
// embedding that must not grow the process's GPU footprint after start-up.
// This entry point takes only the caller's inputs and output and keeps its
// scratch (the 1-D stencil coefficients, per-block partial maxima, a
// completion counter) in one file-scope __device__ array of fixed size.
//
// Limits and sharing: nx + ny + nz <= kNoAllocMaxAxes, and every call on a
// device uses the same array (it keeps the last call's contents), so calls
// whose work overlaps on the GPU -- on different streams or host threads --
// race on it and must be serialised by the caller.  The counter that must
// start at zero is cleared by every call.  Every GPU that loads the library
// holds the array until the process exits.
#include <cstddef>
#include <mutex>

#include "fpm_internal.h"

namespace fpm {

constexpr int kNoAllocMaxAxes = 12288;  // nx + ny + nz
constexpr int kNoAllocBlocks = 1024;    // fixed reduction grid

struct NoAllocScratch {
  double coef[2 * kNoAllocMaxAxes];    // cw, ce | cs, cn | cb, ct
  double partials[kNoAllocBlocks];     // per-block maxima
  double result;
  unsigned int ticket;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Same arithmetic as k_operator_residual, over a fixed 1-D grid that strides
// through every interior cell, with the scratch passed in as a pointer.
__global__ void k_operator_residual_fixed(Dims d, const double* __restrict__ phi, const double* __restrict__ src,
                                          const double* __restrict__ diag, NoAllocScratch* sc) {
  const double* cw = sc->coef;
  const double* ce = cw + d.nx;
  const double* cs = ce + d.nx;
  const double* cn = cs + d.ny;
  const double* cb = cn + d.ny;
  const double* ct = cb + d.nz;
  const long long n = d.ncell();
  double m = 0.0;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const double dg = diag[c];
    if (!(dg > 0)) continue;
    const int i = (int)(c % d.nx) + 1;
    const long long r = c / d.nx;
    const int j = (int)(r % d.ny) + 1, k = (int)(r / d.ny) + 1;
    const int kb = k > 1 ? k - 1 : 1, kt = k < d.nz ? k + 1 : d.nz;
    const long long p = d.ph(i, j, k);
    double t = dadd(src[c], dmul(cw[i - 1], phi[p - 1]));
    t = dadd(t, dmul(ce[i - 1], phi[p + 1]));
    t = dadd(t, dmul(cs[j - 1], phi[p - (d.nx + 2)]));
    t = dadd(t, dmul(cn[j - 1], phi[p + (d.nx + 2)]));
    t = dadd(t, dmul(cb[k - 1], phi[d.ph(i, j, kb)]));
    t = dadd(t, dmul(ct[k - 1], phi[d.ph(i, j, kt)]));
    t = dsub(t, dmul(dg, phi[p]));
    m = fmax(m, fabs(t));
  }
  double s[1] = {0.0}, mm[1] = {m}, out[1];
  if (grid_reduce<0, 1>(s, mm, sc->partials, &sc->ticket, out) && lin_tid() == 0) sc->result = out[0];
}

// Device address of the scratch array, looked up once per device (with that
// device current) and cached.
static NoAllocScratch* noalloc_scratch(int device, cudaError_t* err) {
  static std::mutex mu;
  static NoAllocScratch* addr[64] = {};
  std::lock_guard<std::mutex> g(mu);
  *err = cudaSuccess;
  if (device < 0 || device >= 64) {
    *err = cudaErrorInvalidDevice;
    return nullptr;
  }
  if (!addr[device]) {
    void* p = nullptr;
    *err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (*err != cudaSuccess) return nullptr;
    addr[device] = static_cast<NoAllocScratch*>(p);
  }
  return addr[device];
}

int operator_residual_noalloc(const double* phi, const double* src, const double* diag, const Axes& ax, int nx, int ny,
                              int nz, double* value, cudaStream_t st, std::string* msg) {
  if ((long long)nx + ny + nz > kNoAllocMaxAxes) {
    *msg = "nx + ny + nz exceeds the allocation-free limit of " + std::to_string(kNoAllocMaxAxes);
    return 8;  // FPM_E_LIMIT
  }
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  NoAllocScratch* sc = e == cudaSuccess ? noalloc_scratch(device, &e) : nullptr;
  if (e != cudaSuccess) {
    *msg = std::string("scratch set-up: ") + cudaGetErrorString(e);
    return 6;  // FPM_E_CUDA
  }
  const Dims d{nx, ny, nz};
  // Device addresses of the members (no host dereference of sc).
  char* base = reinterpret_cast<char*>(sc);
  double* coef = reinterpret_cast<double*>(base + offsetof(NoAllocScratch, coef));
  unsigned int* ticket = reinterpret_cast<unsigned int*>(base + offsetof(NoAllocScratch, ticket));
  double* result = reinterpret_cast<double*>(base + offsetof(NoAllocScratch, result));
  e = cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st);
  if (e == cudaSuccess) e = launch_axis_coefs(ax, nx, ny, nz, coef, st);
  if (e == cudaSuccess) {
    long long nb = (d.ncell() + 255) / 256;
    if (nb > kNoAllocBlocks) nb = kNoAllocBlocks;
    k_operator_residual_fixed<<<(unsigned)nb, 256, 0, st>>>(d, phi, src, diag, sc); note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(value, result, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    *msg = cudaGetErrorString(e);
    return 6;
  }
  return 0;
}

}  // namespace fpm
