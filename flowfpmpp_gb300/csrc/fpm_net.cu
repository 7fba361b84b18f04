// Learned initial guess / preconditioner: a small 3-D convolutional
// encoder-decoder trained and run with this library's own kernels.
//
// Network (4 levels, 16-64 channels, 3x3x3 convolutions, BF16 activations
// and weights on the tensor cores, FP32 accumulation, FP32 master weights,
// gradients and Adam state):
//
//   x0  (L0, 16 ch: fluid mask, w0/dx, w0/dy, w0/dz, right-hand side, 11 zero)
//   a0 = relu(conv0(x0))                     16   L0
//   a1 = relu(conv1(pool(a0)))               32   L1 = L0 / 2
//   a2 = relu(conv2(pool(a1)))               48   L2
//   a3 = relu(conv3(pool(a2)))               64   L3
//   d2 = relu(conv4(a2 ++ up(a3)))           48   L2   (112 input channels)
//   d1 = relu(conv5(a1 ++ up(d2)))           32   L1   (80)
//   d0 = relu(conv6(a0 ++ up(d1)))           16   L0   (48)
//   y  = conv7(d0), channel 0                 1   L0   (16 computed, FP32)
//
// pool = 2x2x2 average, up = nearest neighbour, ++ = channel concatenation
// (fused into the convolution's loads).  The loss is free of scale and
// offset, 1 - cos^2 of the angle between y and the target potential over the
// fluid cells after removing their fluid means, because the solver only uses
// y up to a scale (the best multiple of y is taken by an A-norm projection)
// and a constant (the operator's null space).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fpm_capi.h"
#include "fpm_internal.h"
#include "fpm_net.h"

namespace fpm {
namespace net {

namespace {

struct NetError {
  int code;
  std::string msg;
};

#define NET_TRY(expr)                                                                           \
  do {                                                                                          \
    cudaError_t e_ = (expr);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      throw NetError{FPM_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)};          \
  } while (0)

// The tcgen05 convolution's bounded waits: a timeout is reported as an error
// (its outputs are invalid) instead of a hang.
void check_tc(cudaStream_t st) {
  int flag = 0;
  NET_TRY(conv_tc_error(st, &flag));
  if (flag) throw NetError{FPM_E_TIMEOUT, "tensor-core convolution: a bounded wait gave up"};
}

template <class F>
int net_guard(F&& f) {
  try {
    f();
    set_error("");
    return FPM_OK;
  } catch (const NetError& e) {
    set_error(e.msg);
    return e.code;
  }
}

using bf16 = __nv_bfloat16;

// ---------------------------------------------------------------- small kernels
__global__ void k_input(int nx, int ny, int nz, const uint8_t* __restrict__ fluid, const float* __restrict__ mx,
                        const float* __restrict__ my, const float* __restrict__ mz, const float* __restrict__ rhs,
                        bf16* __restrict__ x0) {
  const long long n = (long long)nx * ny * nz;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long long)nx * ny));
    const float f = fluid[v] ? 1.f : 0.f;
    const float c[8] = {f, mx[i], my[j], mz[k], f * rhs[v], 0.f, 0.f, 0.f};
    uint4 lo, hi;
    __nv_bfloat162* pl = reinterpret_cast<__nv_bfloat162*>(&lo);
#pragma unroll
    for (int q = 0; q < 4; q++) pl[q] = __floats2bfloat162_rn(c[2 * q], c[2 * q + 1]);
    hi = make_uint4(0, 0, 0, 0);
    uint4* dst = reinterpret_cast<uint4*>(x0 + v * 16);
    dst[0] = lo;
    dst[1] = hi;
  }
}

// 2x2x2 average: fine (nx, ny, nz) -> coarse, C channels.
__global__ void k_pool(int nx, int ny, int nz, int C, const bf16* __restrict__ in, bf16* __restrict__ out) {
  const int hx = nx >> 1, hy = ny >> 1, hz = nz >> 1;
  const long long n = (long long)hx * hy * hz * (C / 2);
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x) {
    const int c2 = (int)(m % (C / 2));
    const long long vc = m / (C / 2);
    const int i = (int)(vc % hx), j = (int)((vc / hx) % hy), k = (int)(vc / ((long long)hx * hy));
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int o = 0; o < 8; o++) {
      const long long vf = (2 * i + (o & 1)) + (long long)nx * ((2 * j + ((o >> 1) & 1)) + (long long)ny * (2 * k + (o >> 2)));
      const float2 x = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(in + vf * C + 2 * c2));
      s0 += x.x;
      s1 += x.y;
    }
    *reinterpret_cast<__nv_bfloat162*>(out + vc * C + 2 * c2) = __floats2bfloat162_rn(s0 * 0.125f, s1 * 0.125f);
  }
}

// gfine[v][c] += gcoarse[parent(v)][c] / 8.
__global__ void k_pool_bwd(int nx, int ny, int nz, int C, const float* __restrict__ gc, float* __restrict__ gf) {
  const long long n = (long long)nx * ny * nz * C;
  const int hx = nx >> 1, hy = ny >> 1;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(m % C);
    const long long v = m / C;
    const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long long)nx * ny));
    const long long vc = (i >> 1) + (long long)hx * ((j >> 1) + (long long)hy * (k >> 1));
    gf[m] += 0.125f * gc[vc * C + c];
  }
}

// dy = g where y > 0 (ReLU adjoint), as BF16.
__global__ void k_relu_bwd(long long n, const float* __restrict__ g, const bf16* __restrict__ y, bf16* __restrict__ dy) {
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x)
    dy[m] = __float2bfloat16_rn(__bfloat162float(y[m]) > 0.f ? g[m] : 0.f);
}

// Head adjoint: channel 0 carries the loss gradient, channels 1..15 zero.
__global__ void k_head_bwd(long long nvox, const float* __restrict__ g, bf16* __restrict__ dy) {
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x) {
    uint4 lo = make_uint4(0, 0, 0, 0), hi = make_uint4(0, 0, 0, 0);
    reinterpret_cast<bf16*>(&lo)[0] = __float2bfloat16_rn(g[v]);
    uint4* d = reinterpret_cast<uint4*>(dy + v * 16);
    d[0] = lo;
    d[1] = hi;
  }
}

// db[c] += sum_v dy[v][c]  (C <= 64).
__global__ void k_bias_grad(long long nvox, int C, const bf16* __restrict__ dy, float* __restrict__ db) {
  __shared__ float sh[64];
  for (int c = threadIdx.x; c < C; c += blockDim.x) sh[c] = 0.f;
  __syncthreads();
  float acc = 0.f;
  const int c = threadIdx.x % C;
  const int lanes = blockDim.x / C;  // blockDim.x is a multiple of C
  const int r = threadIdx.x / C;
  for (long long v = (long long)blockIdx.x * lanes + r; v < nvox; v += (long long)gridDim.x * lanes)
    acc += __bfloat162float(dy[v * C + c]);
  if (threadIdx.x < lanes * C) atomicAdd(&sh[c], acc);
  __syncthreads();
  for (int q = threadIdx.x; q < C; q += blockDim.x) atomicAdd(&db[q], sh[q]);
}

// Loss sums over fluid cells: n, sum y, sum t, yy, yt, tt (FP64,
// deterministic grid reduction).
__global__ void k_loss_sums(long long nvox, const float* __restrict__ y, int ystride, const float* __restrict__ t,
                            const uint8_t* __restrict__ fluid, double* partials, unsigned int* ticket,
                            double* out) {
  double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, m[1] = {0.0};
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x) {
    if (!fluid[v]) continue;
    const double a = y[v * ystride], b = t[v];
    s[0] += 1.0;
    s[1] += a;
    s[2] += b;
    s[3] += a * a;
    s[4] += a * b;
    s[5] += b * b;
  }
  double o[6];
  if (grid_reduce<6, 0>(s, m, partials, ticket, o) && lin_tid() == 0) {
    const double n = o[0] > 0 ? o[0] : 1.0, my = o[1] / n, mt = o[2] / n;
    out[0] = o[3] - n * my * my;  // centred yy, yt, tt
    out[1] = o[4] - n * my * mt;
    out[2] = o[5] - n * mt * mt;
    out[3] = my;
    out[4] = mt;
  }
}

// dL/dy for L = 1 - yt^2 / (yy tt) of the fluid-mean-free y and t.
__global__ void k_loss_grad(long long nvox, const float* __restrict__ y, int ystride, const float* __restrict__ t,
                            const uint8_t* __restrict__ fluid, const double* __restrict__ sums, float* __restrict__ g) {
  const double yy = sums[0], yt = sums[1], tt = sums[2], my = sums[3], mt = sums[4];
  const double ok = (yy > 0 && tt > 0) ? 1.0 : 0.0;
  const double ca = ok * (-2.0 * yt / (yy * tt)), cb = ok * (2.0 * yt * yt / (yy * yy * tt));
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x)
    g[v] = fluid[v] ? (float)(ca * (t[v] - mt) + cb * (y[v * ystride] - my)) : 0.f;
}

__global__ void k_adam(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const float gg = g[q];
    const float a = b1 * m1[q] + (1.f - b1) * gg;
    const float b = b2 * m2[q] + (1.f - b2) * gg * gg;
    m1[q] = a;
    m2[q] = b;
    w[q] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
  }
}

// FP32 master weights [27][cout][cin] -> BF16 forward layout [cin/16][27][cout][16]
// and backward-data layout (flipped taps, transposed) [cout/16][27][cin][16].
__global__ void k_pack(int cin, int cout, const float* __restrict__ w, bf16* __restrict__ wf, bf16* __restrict__ wt) {
  const long long n = 27LL * cout * cin;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(q % cin), co = (int)((q / cin) % cout), t = (int)(q / ((long long)cin * cout));
    const bf16 x = __float2bfloat16_rn(w[q]);
    wf[(((long long)(ci / 16) * 27 + t) * cout + co) * 16 + (ci % 16)] = x;
    if (wt) wt[(((long long)(co / 16) * 27 + (26 - t)) * cin + ci) * 16 + (co % 16)] = x;
  }
}

inline unsigned nblk(long long n, int per = 256) {
  long long b = (n + per - 1) / per;
  if (b > 152LL * 64) b = 152LL * 64;
  return (unsigned)(b < 1 ? 1 : b);
}

// ---------------------------------------------------------------- network
struct Layer {
  int cin, ca, cout, level, relu;
  float *w, *b, *gw, *gb, *m1w, *m2w, *m1b, *m2b;
  bf16 *wf, *wt;
  long long nw() const { return 27LL * cout * cin; }
};

constexpr int kLayers = 8;
// cin, ca (channels from the same-resolution input), cout, level, relu
constexpr int kSpec[kLayers][5] = {{16, 16, 16, 0, 1},  {16, 16, 32, 1, 1},  {32, 32, 48, 2, 1},
                                   {48, 48, 64, 3, 1},  {112, 48, 48, 2, 1}, {80, 32, 32, 1, 1},
                                   {48, 16, 16, 0, 1},  {16, 16, 16, 0, 0}};

struct Acts {
  int nx = 0, ny = 0, nz = 0;
  bool grads = false;
  std::vector<void*> owned;
  bf16 *x0 = nullptr, *a0 = nullptr, *p1 = nullptr, *a1 = nullptr, *p2 = nullptr, *a2 = nullptr, *p3 = nullptr,
       *a3 = nullptr, *d2 = nullptr, *d1 = nullptr, *d0 = nullptr, *dy = nullptr;
  float* y = nullptr;
  // gradients (FP32)
  float *gy = nullptr, *g_d0 = nullptr, *g_a0 = nullptr, *g_d1 = nullptr, *g_a1 = nullptr, *g_d2 = nullptr,
        *g_a2 = nullptr, *g_a3 = nullptr, *g_p1 = nullptr, *g_p2 = nullptr, *g_p3 = nullptr;
  double* sums = nullptr;
  double* partials = nullptr;
  unsigned int* ticket = nullptr;
};

struct Net {
  Layer L[kLayers];
  std::vector<void*> owned;
  Acts A;
  long long step = 0;

  long long vox(int level) const {
    return (long long)(A.nx >> level) * (A.ny >> level) * (A.nz >> level);
  }
  template <class T>
  T* alloc(std::vector<void*>& list, long long n) {
    void* p = nullptr;
    NET_TRY(cudaMalloc(&p, (size_t)(n > 0 ? n : 1) * sizeof(T)));
    list.push_back(p);
    return static_cast<T*>(p);
  }
  void free_acts() {
    for (void* p : A.owned) cudaFree(p);
    A = Acts();
  }
  ~Net() {
    free_acts();
    for (void* p : owned) cudaFree(p);
  }

  void ensure(int nx, int ny, int nz, bool grads) {
    if (A.nx == nx && A.ny == ny && A.nz == nz && (A.grads || !grads)) return;
    free_acts();
    A.nx = nx;
    A.ny = ny;
    A.nz = nz;
    A.grads = grads;
    auto& o = A.owned;
    const long long v0 = vox(0), v1 = vox(1), v2 = vox(2), v3 = vox(3);
    A.x0 = alloc<bf16>(o, v0 * 16);
    A.a0 = alloc<bf16>(o, v0 * 16);
    A.p1 = alloc<bf16>(o, v1 * 16);
    A.a1 = alloc<bf16>(o, v1 * 32);
    A.p2 = alloc<bf16>(o, v2 * 32);
    A.a2 = alloc<bf16>(o, v2 * 48);
    A.p3 = alloc<bf16>(o, v3 * 48);
    A.a3 = alloc<bf16>(o, v3 * 64);
    A.d2 = alloc<bf16>(o, v2 * 48);
    A.d1 = alloc<bf16>(o, v1 * 32);
    A.d0 = alloc<bf16>(o, v0 * 16);
    A.y = alloc<float>(o, v0 * 16);
    A.sums = alloc<double>(o, 8);
    const long long nb = nblk(v0);
    A.partials = alloc<double>(o, 8 * nb);
    A.ticket = alloc<unsigned int>(o, 1);
    NET_TRY(cudaMemset(A.ticket, 0, sizeof(unsigned int)));
    if (grads) {
      A.dy = alloc<bf16>(o, v0 * 16 > v1 * 32 ? v0 * 16 : v1 * 32);
      A.gy = alloc<float>(o, v0);
      A.g_d0 = alloc<float>(o, v0 * 16);
      A.g_a0 = alloc<float>(o, v0 * 16);
      A.g_d1 = alloc<float>(o, v1 * 32);
      A.g_a1 = alloc<float>(o, v1 * 32);
      A.g_d2 = alloc<float>(o, v2 * 48);
      A.g_a2 = alloc<float>(o, v2 * 48);
      A.g_a3 = alloc<float>(o, v3 * 64);
      A.g_p1 = alloc<float>(o, v1 * 16);
      A.g_p2 = alloc<float>(o, v2 * 32);
      A.g_p3 = alloc<float>(o, v3 * 48);
    }
  }

  void init(unsigned long long seed) {
    uint64_t s = seed ? seed : 0x9e3779b97f4a7c15ULL;
    auto next = [&]() {
      s += 0x9e3779b97f4a7c15ULL;
      uint64_t z = s;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
      return z ^ (z >> 31);
    };
    auto unif = [&]() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
    for (int l = 0; l < kLayers; l++) {
      Layer& y = L[l];
      y.cin = kSpec[l][0];
      y.ca = kSpec[l][1];
      y.cout = kSpec[l][2];
      y.level = kSpec[l][3];
      y.relu = kSpec[l][4];
      const long long nw = y.nw();
      y.w = alloc<float>(owned, nw);
      y.b = alloc<float>(owned, y.cout);
      y.gw = alloc<float>(owned, nw);
      y.gb = alloc<float>(owned, y.cout);
      y.m1w = alloc<float>(owned, nw);
      y.m2w = alloc<float>(owned, nw);
      y.m1b = alloc<float>(owned, y.cout);
      y.m2b = alloc<float>(owned, y.cout);
      y.wf = alloc<bf16>(owned, nw);
      y.wt = alloc<bf16>(owned, nw);
      // He-normal over the real fan-in (the input layer has 5 live channels);
      // the head keeps only output channel 0.
      const int live_in = l == 0 ? 5 : y.cin;
      const double sd = std::sqrt(2.0 / (27.0 * live_in)) * (y.relu ? 1.0 : 0.5);
      std::vector<float> hw((size_t)nw, 0.f), hb((size_t)y.cout, 0.f);
      for (long long q = 0; q < nw; q++) {
        const int ci = (int)(q % y.cin), co = (int)((q / y.cin) % y.cout);
        const double u1 = unif(), u2 = unif();
        const double gauss = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        const bool live = (l != 0 || ci < 5) && (l != kLayers - 1 || co == 0);
        hw[(size_t)q] = live ? (float)(sd * gauss) : 0.f;
      }
      NET_TRY(cudaMemcpy(y.w, hw.data(), nw * sizeof(float), cudaMemcpyHostToDevice));
      NET_TRY(cudaMemcpy(y.b, hb.data(), y.cout * sizeof(float), cudaMemcpyHostToDevice));
      NET_TRY(cudaMemset(y.m1w, 0, nw * sizeof(float)));
      NET_TRY(cudaMemset(y.m2w, 0, nw * sizeof(float)));
      NET_TRY(cudaMemset(y.m1b, 0, y.cout * sizeof(float)));
      NET_TRY(cudaMemset(y.m2b, 0, y.cout * sizeof(float)));
    }
    pack(0);
    NET_TRY(cudaDeviceSynchronize());
  }

  void pack(cudaStream_t st) {
    for (int l = 0; l < kLayers; l++) {
      k_pack<<<nblk(L[l].nw()), 256, 0, st>>>(L[l].cin, L[l].cout, L[l].w, L[l].wf, L[l].wt);
      note_launch();
    }
    NET_TRY(cudaGetLastError());
  }

  ConvArgs conv_args(int l, const bf16* a, const bf16* b) const {
    const Layer& y = L[l];
    ConvArgs c;
    std::memset(&c, 0, sizeof(c));
    c.nx = A.nx >> y.level;
    c.ny = A.ny >> y.level;
    c.nz = A.nz >> y.level;
    c.ca = y.ca;
    c.cb = y.cin - y.ca;
    c.cin = y.cin;
    c.a = a;
    c.b = b;
    c.w = y.wf;
    c.bias = y.b;
    c.relu = y.relu;
    return c;
  }
  void conv_fwd(int l, const bf16* a, const bf16* b, bf16* out, cudaStream_t st) {
    ConvArgs c = conv_args(l, a, b);
    c.mode = kConvBf16;
    c.y = out;
    NET_TRY(launch_conv(c, L[l].cout, st));
  }
  void pool(int level_fine, int C, const bf16* in, bf16* out, cudaStream_t st) {
    const int nx = A.nx >> level_fine, ny = A.ny >> level_fine, nz = A.nz >> level_fine;
    k_pool<<<nblk(vox(level_fine + 1) * C / 2), 256, 0, st>>>(nx, ny, nz, C, in, out);
    note_launch();
    NET_TRY(cudaGetLastError());
  }

  void forward(const uint8_t* fluid, const float* mx, const float* my, const float* mz, const float* rhs,
               cudaStream_t st) {
    k_input<<<nblk(vox(0)), 256, 0, st>>>(A.nx, A.ny, A.nz, fluid, mx, my, mz, rhs, A.x0);
    note_launch();
    NET_TRY(cudaGetLastError());
    conv_fwd(0, A.x0, nullptr, A.a0, st);
    pool(0, 16, A.a0, A.p1, st);
    conv_fwd(1, A.p1, nullptr, A.a1, st);
    pool(1, 32, A.a1, A.p2, st);
    conv_fwd(2, A.p2, nullptr, A.a2, st);
    pool(2, 48, A.a2, A.p3, st);
    conv_fwd(3, A.p3, nullptr, A.a3, st);
    conv_fwd(4, A.a2, A.a3, A.d2, st);
    conv_fwd(5, A.a1, A.d2, A.d1, st);
    conv_fwd(6, A.a0, A.d1, A.d0, st);
    ConvArgs c = conv_args(7, A.d0, nullptr);
    c.mode = kConvF32;
    c.yf = A.y;
    NET_TRY(launch_conv(c, 16, st));
  }

  double loss(const uint8_t* fluid, const float* target, bool grad, cudaStream_t st) {
    const long long n = vox(0);
    const unsigned nb = nblk(n);
    k_loss_sums<<<nb, 256, 0, st>>>(n, A.y, 16, target, fluid, A.partials, A.ticket, A.sums);
    note_launch();
    if (grad) {
      k_loss_grad<<<nblk(n), 256, 0, st>>>(n, A.y, 16, target, fluid, A.sums, A.gy);
      note_launch();
    }
    NET_TRY(cudaGetLastError());
    double h[3];
    NET_TRY(cudaMemcpyAsync(h, A.sums, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    NET_TRY(cudaStreamSynchronize(st));
    return (h[0] > 0 && h[2] > 0) ? 1.0 - h[1] * h[1] / (h[0] * h[2]) : 1.0;
  }

  // Weight, bias and input gradients of layer l given its output adjoint dy
  // (BF16, cout channels, already through the ReLU adjoint).
  void layer_bwd(int l, const bf16* in_a, const bf16* in_b, float* g_a, float* g_b, cudaStream_t st) {
    const Layer& y = L[l];
    ConvArgs c = conv_args(l, in_a, in_b);
    WgradArgs w;
    w.conv = c;
    w.dy = A.dy;
    w.dw = y.gw;
    const long long nvox = vox(y.level);
    const long long tiles = (long long)((c.nx + 31) / 32) * ((c.ny + 3) / 4) * c.nz;
    // enough CTAs to fill the GPU, few enough that the atomic flush stays small
    long long per = tiles * (y.cin / 16) * 3 / (152 * 8);
    w.tiles_per_cta = (int)(per < 1 ? 1 : (per > 64 ? 64 : per));
    NET_TRY(launch_conv_wgrad(w, y.cout, st));
    k_bias_grad<<<nblk(nvox, 1024), 256, 0, st>>>(nvox, y.cout, A.dy, y.gb);
    note_launch();
    NET_TRY(cudaGetLastError());
    if (!g_a) return;
    // backward data: the adjoint convolution (flipped taps, transposed
    // channels) of dy, split into the two inputs' gradients
    ConvArgs b;
    std::memset(&b, 0, sizeof(b));
    b.nx = c.nx;
    b.ny = c.ny;
    b.nz = c.nz;
    b.ca = y.cout;
    b.cb = 0;
    b.cin = y.cout;
    b.a = A.dy;
    b.w = y.wt;
    b.mode = kConvGrad;
    b.csplit = y.ca;
    b.ga = g_a;
    b.gb = g_b;
    NET_TRY(launch_conv(b, y.cin, st));
  }
  void relu_bwd(int level, int C, const float* g, const bf16* y, cudaStream_t st) {
    const long long n = vox(level) * C;
    k_relu_bwd<<<nblk(n), 256, 0, st>>>(n, g, y, A.dy);
    note_launch();
    NET_TRY(cudaGetLastError());
  }
  void pool_bwd(int level_fine, int C, const float* gc, float* gf, cudaStream_t st) {
    const long long n = vox(level_fine) * C;
    k_pool_bwd<<<nblk(n), 256, 0, st>>>(A.nx >> level_fine, A.ny >> level_fine, A.nz >> level_fine, C, gc, gf);
    note_launch();
    NET_TRY(cudaGetLastError());
  }

  void backward(cudaStream_t st) {
    for (int l = 0; l < kLayers; l++) {
      NET_TRY(cudaMemsetAsync(L[l].gw, 0, L[l].nw() * sizeof(float), st));
      NET_TRY(cudaMemsetAsync(L[l].gb, 0, L[l].cout * sizeof(float), st));
    }
    const long long v0 = vox(0), v1 = vox(1), v2 = vox(2), v3 = vox(3);
    struct Z {
      float* p;
      long long n;
    } zs[] = {{A.g_d0, v0 * 16}, {A.g_a0, v0 * 16}, {A.g_d1, v1 * 32}, {A.g_a1, v1 * 32}, {A.g_d2, v2 * 48},
              {A.g_a2, v2 * 48}, {A.g_a3, v3 * 64}, {A.g_p1, v1 * 16}, {A.g_p2, v2 * 32}, {A.g_p3, v3 * 48}};
    for (const Z& z : zs) NET_TRY(cudaMemsetAsync(z.p, 0, z.n * sizeof(float), st));
    k_head_bwd<<<nblk(v0), 256, 0, st>>>(v0, A.gy, A.dy);
    note_launch();
    layer_bwd(7, A.d0, nullptr, A.g_d0, nullptr, st);
    relu_bwd(0, 16, A.g_d0, A.d0, st);
    layer_bwd(6, A.a0, A.d1, A.g_a0, A.g_d1, st);
    relu_bwd(1, 32, A.g_d1, A.d1, st);
    layer_bwd(5, A.a1, A.d2, A.g_a1, A.g_d2, st);
    relu_bwd(2, 48, A.g_d2, A.d2, st);
    layer_bwd(4, A.a2, A.a3, A.g_a2, A.g_a3, st);
    relu_bwd(3, 64, A.g_a3, A.a3, st);
    layer_bwd(3, A.p3, nullptr, A.g_p3, nullptr, st);
    pool_bwd(2, 48, A.g_p3, A.g_a2, st);
    relu_bwd(2, 48, A.g_a2, A.a2, st);
    layer_bwd(2, A.p2, nullptr, A.g_p2, nullptr, st);
    pool_bwd(1, 32, A.g_p2, A.g_a1, st);
    relu_bwd(1, 32, A.g_a1, A.a1, st);
    layer_bwd(1, A.p1, nullptr, A.g_p1, nullptr, st);
    pool_bwd(0, 16, A.g_p1, A.g_a0, st);
    relu_bwd(0, 16, A.g_a0, A.a0, st);
    layer_bwd(0, A.x0, nullptr, nullptr, nullptr, st);
  }

  void adam(float lr, cudaStream_t st) {
    step++;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - (float)std::pow(b1, (double)step), c2 = 1.f - (float)std::pow(b2, (double)step);
    for (int l = 0; l < kLayers; l++) {
      k_adam<<<nblk(L[l].nw()), 256, 0, st>>>(L[l].nw(), L[l].w, L[l].gw, L[l].m1w, L[l].m2w, lr, b1, b2, eps, c1, c2);
      note_launch();
      k_adam<<<1, 64, 0, st>>>(L[l].cout, L[l].b, L[l].gb, L[l].m1b, L[l].m2b, lr, b1, b2, eps, c1, c2);
      note_launch();
    }
    NET_TRY(cudaGetLastError());
    pack(st);
  }

  long long param_count() const {
    long long n = 0;
    for (int l = 0; l < kLayers; l++) n += L[l].nw() + L[l].cout;
    return n;
  }
  // Flattened [layer][w (27 cout cin) | b (cout)] copies between host and device.
  void copy_params(float* host, bool to_host, bool grads) {
    long long o = 0;
    for (int l = 0; l < kLayers; l++) {
      float* w = grads ? L[l].gw : L[l].w;
      float* b = grads ? L[l].gb : L[l].b;
      if (to_host) {
        NET_TRY(cudaMemcpy(host + o, w, L[l].nw() * sizeof(float), cudaMemcpyDeviceToHost));
        NET_TRY(cudaMemcpy(host + o + L[l].nw(), b, L[l].cout * sizeof(float), cudaMemcpyDeviceToHost));
      } else {
        NET_TRY(cudaMemcpy(w, host + o, L[l].nw() * sizeof(float), cudaMemcpyHostToDevice));
        NET_TRY(cudaMemcpy(b, host + o + L[l].nw(), L[l].cout * sizeof(float), cudaMemcpyHostToDevice));
      }
      o += L[l].nw() + L[l].cout;
    }
    if (!to_host && !grads) {
      pack(0);
      NET_TRY(cudaDeviceSynchronize());
    }
  }
};

void check_grid(int nx, int ny, int nz) {
  if (nx < 8 || ny < 8 || nz < 8 || nx % 8 || ny % 8 || nz % 8)
    throw NetError{FPM_E_SIZE, "the network needs nx, ny, nz multiples of 8 (three 2x poolings)"};
}

}  // namespace

int forward_into(void* net, int nx, int ny, int nz, const uint8_t* fluid, const float* mx, const float* my,
                 const float* mz, const float* rhs, float* out, cudaStream_t st, std::string* err) {
  try {
    Net* p = static_cast<Net*>(net);
    if (!p) throw NetError{FPM_E_ARG, "null network handle"};
    check_grid(nx, ny, nz);
    p->ensure(nx, ny, nz, false);
    p->forward(fluid, mx, my, mz, rhs, st);
    const long long n = (long long)nx * ny * nz;
    NET_TRY(cudaMemcpy2DAsync(out, sizeof(float), p->A.y, 16 * sizeof(float), sizeof(float), (size_t)n,
                              cudaMemcpyDeviceToDevice, st));
    return FPM_OK;
  } catch (const NetError& e) {
    if (err) *err = e.msg;
    return e.code;
  }
}

// Used by the learned solver driver.
void* net_create(unsigned long long seed) {
  Net* n = new Net();
  try {
    n->init(seed);
  } catch (...) {
    delete n;
    throw;
  }
  return n;
}

}  // namespace net
}  // namespace fpm

using fpm::net::Net;
using fpm::net::NetError;
using fpm::net::net_guard;
using fpm::net::check_tc;

extern "C" {

int fpm_net_create(unsigned long long seed, void** net) {
  return net_guard([&] {
    if (!net) throw NetError{FPM_E_ARG, "null handle pointer"};
    *net = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) throw NetError{FPM_E_NO_DEVICE, "no CUDA device"};
    *net = fpm::net::net_create(seed);
  });
}

int fpm_net_destroy(void* net) {
  return net_guard([&] { delete static_cast<Net*>(net); });
}

long long fpm_net_param_count(void* net) { return net ? static_cast<Net*>(net)->param_count() : 0; }

int fpm_net_get_params(void* net, float* host, long long n) {
  return net_guard([&] {
    Net* p = static_cast<Net*>(net);
    if (!p || !host || n != p->param_count()) throw NetError{FPM_E_ARG, "parameter buffer size mismatch"};
    p->copy_params(host, true, false);
  });
}

int fpm_net_set_params(void* net, const float* host, long long n) {
  return net_guard([&] {
    Net* p = static_cast<Net*>(net);
    if (!p || !host || n != p->param_count()) throw NetError{FPM_E_ARG, "parameter buffer size mismatch"};
    p->copy_params(const_cast<float*>(host), false, false);
  });
}

int fpm_net_get_grads(void* net, float* host, long long n) {
  return net_guard([&] {
    Net* p = static_cast<Net*>(net);
    if (!p || !host || n != p->param_count()) throw NetError{FPM_E_ARG, "parameter buffer size mismatch"};
    p->copy_params(host, true, true);
  });
}

int fpm_net_forward_dev(void* net, int nx, int ny, int nz, const uint8_t* fluid, const float* mx, const float* my,
                        const float* mz, const float* rhs, float* out, void* stream) {
  return net_guard([&] {
    Net* p = static_cast<Net*>(net);
    if (!p || !fluid || !mx || !my || !mz || !rhs || !out) throw NetError{FPM_E_ARG, "null argument"};
    fpm::net::check_grid(nx, ny, nz);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    p->ensure(nx, ny, nz, false);
    p->forward(fluid, mx, my, mz, rhs, st);
    const long long n = (long long)nx * ny * nz;
    NET_TRY(cudaMemcpy2DAsync(out, sizeof(float), p->A.y, 16 * sizeof(float), sizeof(float), (size_t)n,
                              cudaMemcpyDeviceToDevice, st));
    NET_TRY(cudaStreamSynchronize(st));
    check_tc(st);
  });
}

int fpm_net_backward_dev(void* net, int nx, int ny, int nz, const uint8_t* fluid, const float* mx, const float* my,
                         const float* mz, const float* rhs, const float* target, double* loss, void* stream) {
  return net_guard([&] {
    Net* p = static_cast<Net*>(net);
    if (!p || !fluid || !mx || !my || !mz || !rhs || !target) throw NetError{FPM_E_ARG, "null argument"};
    fpm::net::check_grid(nx, ny, nz);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    p->ensure(nx, ny, nz, true);
    p->forward(fluid, mx, my, mz, rhs, st);
    const double l = p->loss(fluid, target, true, st);
    p->backward(st);
    NET_TRY(cudaStreamSynchronize(st));
    check_tc(st);
    if (loss) *loss = l;
  });
}

int fpm_net_train_step_dev(void* net, int nx, int ny, int nz, const uint8_t* fluid, const float* mx,
                           const float* my, const float* mz, const float* rhs, const float* target, float lr,
                           double* loss, void* stream) {
  return net_guard([&] {
    Net* p = static_cast<Net*>(net);
    if (!p || !fluid || !mx || !my || !mz || !rhs || !target) throw NetError{FPM_E_ARG, "null argument"};
    if (!(lr > 0)) throw NetError{FPM_E_ARG, "learning rate must be positive"};
    fpm::net::check_grid(nx, ny, nz);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    p->ensure(nx, ny, nz, true);
    p->forward(fluid, mx, my, mz, rhs, st);
    const double l = p->loss(fluid, target, true, st);
    p->backward(st);
    p->adam(lr, st);
    NET_TRY(cudaStreamSynchronize(st));
    check_tc(st);
    if (loss) *loss = l;
  });
}

}  // extern "C"
