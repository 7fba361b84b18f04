// Learned initial guess / preconditioner: kernel argument blocks shared by
// fpm_net_kernels.cu (convolutions) and fpm_net.cu (the rest of the network).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace fpm {
namespace net {

enum ConvMode { kConvBf16 = 0, kConvF32 = 1, kConvGrad = 2 };

// One 3x3x3 convolution (zero padding) at resolution (nx, ny, nz).  Input
// channels [0, ca) come from `a` (same resolution, ca channels per voxel),
// [ca, cin) from `b` at half resolution (cb = cin - ca channels per voxel,
// nearest-neighbour upsampling).  Weights: [cin/16][27][cout][16] BF16, tap
// t = (dk+1)*9 + (dj+1)*3 + (di+1).
//   kConvBf16: y = relu?(conv + bias), BF16, cout channels per voxel.
//   kConvF32:  yf = conv + bias, FP32.
//   kConvGrad: the backward-data pass of a forward layer whose input was
//              (A: csplit channels, B: cout - csplit channels at half
//              resolution): ga += conv[:, :csplit] (same resolution) and
//              gb += the 2x2x2 sum of conv[:, csplit:] (atomics).
struct ConvArgs {
  int nx, ny, nz;
  int ca, cb, cin;
  const __nv_bfloat16* a;
  const __nv_bfloat16* b;
  const __nv_bfloat16* w;
  const float* bias;
  int mode, relu, csplit;
  __nv_bfloat16* y;
  float* yf;
  float* ga;
  float* gb;
};

// dW[t][co][ci] += sum over voxels of dy[v][co] * in[v + t][ci]; `conv`
// describes the forward layer's input exactly as in ConvArgs (a, b, ca, cb,
// cin); dw is FP32 [27][cout][cin].
struct WgradArgs {
  ConvArgs conv;
  const __nv_bfloat16* dy;
  float* dw;
  int tiles_per_cta;
};

cudaError_t launch_conv(const ConvArgs& a, int cout, cudaStream_t st);
cudaError_t launch_conv_wgrad(const WgradArgs& w, int cout, cudaStream_t st);
// Reads and clears the timeout flag of the tcgen05 convolution (nonzero: a
// bounded wait for its tensor-core work gave up and the output is invalid).
cudaError_t conv_tc_error(cudaStream_t st, int* flag);

}  // namespace net
}  // namespace fpm
