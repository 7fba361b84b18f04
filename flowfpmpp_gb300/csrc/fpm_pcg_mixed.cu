// Mixed-precision, multi-right-hand-side stair-step PCG.
//
// Outer loop (FP64): the true residual r = V(src + sum c phi_nb - diag phi),
// projected by its fluid mean as in true_residual
// (src/fpm_stairstep_mpi_3d.f90:297-329), and the max-norm of L(phi)-f that
// decides convergence exactly as the reference does.
// Inner loop (FP32): diagonally preconditioned CG on A e = r/|res| for every
// right-hand side at once (phi_x, phi_y, phi_z share diag, rdiag, the
// coefficients and the cell volumes), FP32 stencil, preconditioner and
// direction updates, dot products accumulated per thread as error-free f32
// pairs and combined across the grid in FP64.  Each right-hand side stops its
// inner iteration when its preconditioned residual norm drops by kInnerDrop;
// the correction is then added to phi in FP64 and the outer loop repeats.
#include "fpm_internal.h"

namespace fpm {

// Error-free f32 pair accumulator for dot products.
struct F2Acc {
  float s = 0.f, e = 0.f;
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = a * b;
    const float pe = fmaf(a, b, -p);
    const float t = s + p;
    const float bb = t - s;
    e += ((s - (t - bb)) + (p - bb)) + pe;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)e; }
};

#define MX_CELL_BEGIN                                      \
  const int i = blockIdx.x * 32 + threadIdx.x + 1;         \
  const int j = blockIdx.y * 8 + threadIdx.y + 1;          \
  const bool inxy = (i <= d.nx) && (j <= d.ny);            \
  for (int k = blockIdx.z + 1; k <= d.nz; k += gridDim.z) { \
    if (inxy) {
#define MX_CELL_END \
  }                 \
  }

__global__ void k_mx_convert(long long n, const double* __restrict__ a, float* __restrict__ b) {
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x)
    b[m] = (float)a[m];
}

// Residual replacement for the right-hand sides in the set: r = scale * rV
// (the projected FP64 true residual), e = 0, and either a restart from the
// steepest-descent direction p = rdiag r (pmul == 0) or the current direction
// rescaled to the new residual scale (p *= pmul); rz = r.(rdiag r).
__global__ void k_mx_start(Dims d, MixedVecs v, DPtr4 rv64, MixedScale sc,
                           MixedScalars* S, RedBuf rb) {
  double s[kMaxRhs] = {0.0, 0.0, 0.0, 0.0}, mm[1] = {0.0};
  F2Acc acc[kMaxRhs];
  MX_CELL_BEGIN
  const long long c = d.in(i, j, k), p = d.ph(i, j, k);
  const float rd = v.rdiag[c];
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) {
    if (m < v.nrhs && sc.in_set[m]) {
      const float r = (float)(rv64.p[m][c] * sc.scale[m]);
      const float z = rd * r;
      v.r[m][c] = r;
      const float pm = (float)sc.pmul[m];
      v.p[m][p] = pm == 0.f ? z : v.p[m][p] * pm;
      v.e[m][c] = 0.f;
      acc[m].add_prod(z, r);
    }
  }
  MX_CELL_END
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) s[m] = acc[m].value();
  double out[kMaxRhs];
  if (grid_reduce<kMaxRhs, 0>(s, mm, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      for (int m = 0; m < kMaxRhs; m++) {
        if (!(m < v.nrhs && sc.in_set[m])) continue;
        S->rz[m] = out[m];
        S->rz0[m] = out[m];
        S->active[m] = out[m] > 0 ? 1 : 0;
      }
    }
  }
}

// q = V (diag p - sum c p_nb) on diag > 0, pq = p.q, alpha = rz / pq.
__global__ void k_mx_spmv(Dims d, MixedVecs v, MixedScalars* S, RedBuf rb) {
  int act[kMaxRhs];
  bool any = false;
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) {
    act[m] = m < v.nrhs ? S->active[m] : 0;
    any = any || act[m];
  }
  if (!any) return;
  double s[kMaxRhs] = {0.0, 0.0, 0.0, 0.0}, mm[1] = {0.0};
  F2Acc acc[kMaxRhs];
  const long long px = d.nx + 2, pl = d.plane();
  MX_CELL_BEGIN
  const long long c = d.in(i, j, k), p = d.ph(i, j, k);
  const float dg = v.diag[c];
  const float cw = v.coef[i - 1], ce = v.coef[d.nx + i - 1], cs = v.coef[2 * d.nx + j - 1],
              cn = v.coef[2 * d.nx + d.ny + j - 1], cb = v.coef[2 * d.nx + 2 * d.ny + k - 1],
              ct = v.coef[2 * d.nx + 2 * d.ny + d.nz + k - 1];
  const float vol = v.dx[i - 1] * v.dy[j - 1] * v.dz[k - 1];
  const long long pb = k > 1 ? p - pl : p, pt = k < d.nz ? p + pl : p;
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) {
    if (act[m]) {
      const float* pm = v.p[m];
      const float pc = pm[p];
      float q = 0.f;
      if (dg > 0.f) {
        float t = dg * pc;
        t = fmaf(-cw, pm[p - 1], t);
        t = fmaf(-ce, pm[p + 1], t);
        t = fmaf(-cs, pm[p - px], t);
        t = fmaf(-cn, pm[p + px], t);
        t = fmaf(-cb, pm[pb], t);
        t = fmaf(-ct, pm[pt], t);
        q = vol * t;
      }
      v.q[m][c] = q;
      acc[m].add_prod(pc, q);
    }
  }
  MX_CELL_END
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) s[m] = acc[m].value();
  double out[kMaxRhs];
  if (grid_reduce<kMaxRhs, 0>(s, mm, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      for (int m = 0; m < kMaxRhs; m++) {
        if (!act[m]) continue;
        S->pq[m] = out[m];
        if (!(out[m] > 0) || !(S->rz[m] > 0)) {  // breakdown: stop this right-hand side's inner solve
          S->active[m] = 0;
          S->alpha[m] = 0;
        } else {
          S->alpha[m] = S->rz[m] / out[m];
        }
      }
    }
  }
}

// e += alpha p; r -= alpha q; rz_new = r.(rdiag r); beta = rz_new / rz.
__global__ void k_mx_update(Dims d, MixedVecs v, MixedScalars* S, RedBuf rb) {
  int act[kMaxRhs];
  float alpha[kMaxRhs];
  bool any = false;
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) {
    act[m] = m < v.nrhs ? S->active[m] : 0;
    alpha[m] = (float)S->alpha[m];
    any = any || act[m];
  }
  if (!any) return;
  double s[kMaxRhs] = {0.0, 0.0, 0.0, 0.0}, mm[1] = {0.0};
  F2Acc acc[kMaxRhs];
  MX_CELL_BEGIN
  const long long c = d.in(i, j, k), p = d.ph(i, j, k);
  const float rd = v.rdiag[c];
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) {
    if (act[m]) {
      v.e[m][c] = fmaf(alpha[m], v.p[m][p], v.e[m][c]);
      const float r = fmaf(-alpha[m], v.q[m][c], v.r[m][c]);
      v.r[m][c] = r;
      acc[m].add_prod(rd * r, r);
    }
  }
  MX_CELL_END
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) s[m] = acc[m].value();
  double out[kMaxRhs];
  if (grid_reduce<kMaxRhs, 0>(s, mm, rb.partials, rb.ticket, out)) {
    if (lin_tid() == 0) {
      for (int m = 0; m < kMaxRhs; m++) {
        if (!act[m]) continue;
        const double rz_new = out[m];
        if (!(rz_new >= 0)) {
          S->active[m] = 0;
          continue;
        }
        S->beta[m] = rz_new / S->rz[m];
        S->rz[m] = rz_new;
        if (rz_new <= S->tol2[m] * S->rz0[m]) S->active[m] = 0;
      }
    }
  }
}

// p = rdiag r + beta p for the right-hand sides still iterating.
__global__ void k_mx_direction(Dims d, MixedVecs v, MixedScalars* S) {
  int act[kMaxRhs];
  float beta[kMaxRhs];
  bool any = false;
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++) {
    act[m] = m < v.nrhs ? S->active[m] : 0;
    beta[m] = (float)S->beta[m];
    any = any || act[m];
  }
  if (!any) return;
  MX_CELL_BEGIN
  const long long c = d.in(i, j, k), p = d.ph(i, j, k);
  const float rd = v.rdiag[c];
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++)
    if (act[m]) v.p[m][p] = fmaf(rd, v.r[m][c], beta[m] * v.p[m][p]);
  MX_CELL_END
  if (lin_bid() == 0 && lin_tid() == 0) S->iters += 1;
}

// phi += e / scale (FP64) for the right-hand sides of this outer step.
__global__ void k_mx_apply(Dims d, MixedVecs v, DPtr4 phi, MixedScale sc) {
  MX_CELL_BEGIN
  const long long c = d.in(i, j, k), p = d.ph(i, j, k);
#pragma unroll
  for (int m = 0; m < kMaxRhs; m++)
    if (m < v.nrhs && sc.in_set[m]) phi.p[m][p] += (double)v.e[m][c] / sc.scale[m];
  MX_CELL_END
}

cudaError_t launch_mx_convert(const double* a, float* b, long long n, cudaStream_t st) {
  long long nb = (n + 255) / 256;
  if (nb > 152LL * 32) nb = 152LL * 32;
  if (nb < 1) nb = 1;
  k_mx_convert<<<(unsigned)nb, 256, 0, st>>>(n, a, b); note_launch();
  return cudaGetLastError();
}
cudaError_t launch_mx_start(const Dims& d, const MixedVecs& v, const DPtr4& rv64, const MixedScale& sc,
                            MixedScalars* S, const RedBuf& rb, cudaStream_t st) {
  Launch L = cells_launch(d);
  k_mx_start<<<L.grid, L.block, 0, st>>>(d, v, rv64, sc, S, rb); note_launch();
  return cudaGetLastError();
}
cudaError_t launch_mx_iteration(const Dims& d, const MixedVecs& v, MixedScalars* S, const RedBuf& rb,
                                cudaStream_t st) {
  Launch L = cells_launch(d);
  k_mx_spmv<<<L.grid, L.block, 0, st>>>(d, v, S, rb); note_launch();
  k_mx_update<<<L.grid, L.block, 0, st>>>(d, v, S, rb); note_launch();
  k_mx_direction<<<L.grid, L.block, 0, st>>>(d, v, S); note_launch();
  return cudaGetLastError();
}
cudaError_t launch_mx_apply(const Dims& d, const MixedVecs& v, const DPtr4& phi, const MixedScale& sc,
                            cudaStream_t st) {
  Launch L = cells_launch(d);
  k_mx_apply<<<L.grid, L.block, 0, st>>>(d, v, phi, sc); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
