// Internal host-side declarations shared by the kernel files and the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "fpm_common.cuh"

namespace fpm {

// Device-resident scalars of one solve.  The iteration kernels read and write
// these directly, so a PCG chunk runs without any host round trip.
struct SolveScalars {
  double rz, pq, alpha, beta, rz_new;  // PCG recurrences
  double red[4];                       // generic reduction outputs
  double res;                          // max-norm residual of L(phi)-f
  double mean;                         // gauge mean
  double corr;                         // compatibility correction
  int halt;                            // 0 running, 1 breakdown (pq or rz), 2 rz_new invalid
  int iters;                           // PCG iterations completed since the host last cleared it
  int isolated;                        // fluid cells without a fluid neighbour
  int pad;
};

// Stair-step operator coefficients (1-D, device): cw, ce (nx) | cs, cn (ny) | cb, ct (nz).
struct Coefs {
  const double *cw, *ce, *cs, *cn, *cb, *ct;
};
struct Axes {
  const double *xc, *yc, *zc, *dx, *dy, *dz;
};
struct Faces {
  double *xlo, *xhi, *ylo, *yhi, *zlo, *zhi;
};

// Scratch for the deterministic grid reductions.
struct RedBuf {
  double* partials;      // >= 4 * max blocks doubles
  unsigned int* ticket;  // one counter, zero between launches
  int max_blocks;
};

struct Launch {
  dim3 grid, block;
};
// (32 x 8)-thread blocks over the interior x-y plane, grid.z strides over k.
Launch cells_launch(const Dims& d, int pad_xy = 0);

// ---- stair-step kernels (fpm_stairstep.cu) -------------------------------
cudaError_t launch_axis_coefs(const Axes& ax, int nx, int ny, int nz, double* coef /* 2nx+2ny+2nz */,
                              cudaStream_t st);
cudaError_t launch_build_operator(const Dims& d, const double* rhs, const int32_t* solid, const double bg[3],
                                  const Faces& f, const Coefs& c, const Axes& ax, int for_pcg, double* src,
                                  double* diag, double* rdiag, SolveScalars* S, cudaStream_t st);
cudaError_t launch_init_fields(const Dims& d, const int32_t* solid, double* phi, double* next, cudaStream_t st);
cudaError_t launch_jacobi_f64(const Dims& d, const double* a, double* b, const double* src, const double* rdiag,
                              const Coefs& c, cudaStream_t st);
cudaError_t launch_copy_interior(const Dims& d, const double* from, double* to, cudaStream_t st);
cudaError_t launch_operator_residual(const Dims& d, const double* phi, const double* src, const double* diag,
                                     const Coefs& c, SolveScalars* S, const RedBuf& rb, cudaStream_t st);
cudaError_t launch_true_residual(const Dims& d, const double* phi, const double* src, const double* diag,
                                 const double* rdiag, double* r, double* p, const Coefs& c, const Axes& ax, int reset,
                                 SolveScalars* S, const RedBuf& rb, cudaStream_t st);
cudaError_t launch_pcg_iteration(const Dims& d, double* phi, double* p, double* q, double* r, const double* diag,
                                 const double* rdiag, const Coefs& c, const Axes& ax, SolveScalars* S,
                                 const RedBuf& rb, cudaStream_t st);
cudaError_t launch_gauge(const Dims& d, const int32_t* solid, double* phi, const Axes& ax, SolveScalars* S,
                         const RedBuf& rb, cudaStream_t st);
cudaError_t launch_compat(const Dims& d, const double* rhs, const int32_t* solid, const double bg[3], Faces f,
                          const Axes& ax, SolveScalars* S, const RedBuf& rb, cudaStream_t st);
cudaError_t launch_face_residual(const Dims& d, const double* phi, const double* rhs, const int32_t* solid,
                                 const double bg[3], const Faces& f, const Axes& ax, SolveScalars* S,
                                 const RedBuf& rb, cudaStream_t st);
struct Flow {
  const double *u, *v, *w, *ox, *oy, *oz, *ax, *ay, *az;
};
struct TermsOut {
  double *gx, *gy, *gz, *vortex, *advection;
};
cudaError_t launch_terms(const Dims& d, const double* phi, const Flow& fl, const int32_t* solid, const double bg[3],
                         const Axes& ax, const Faces& f, const double bounds[6], const TermsOut& o, SolveScalars* S,
                         const RedBuf& rb, cudaStream_t st);

// Double-float fast Jacobi (fpm_stairstep_df.cu).
cudaError_t launch_to_df(const double* x, float2* y, long long n, cudaStream_t st);
cudaError_t launch_from_df_interior(const Dims& d, const float2* x, double* y, cudaStream_t st);
cudaError_t launch_jacobi_df(const Dims& d, const float2* a, float2* b, const float2* src, const float2* rdiag,
                             const float2* coef_df, cudaStream_t st);

// ---- error reporting (fpm_capi.cu) ----------------------------------------
void set_error(const std::string& msg);

}  // namespace fpm
