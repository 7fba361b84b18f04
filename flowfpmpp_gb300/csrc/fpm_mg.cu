// Aggregation multigrid V-cycle as the preconditioner of the FP32 PCG inside
// the FP64 refinement (FPM_METHOD_PCG_MG).
//
// Every level stores the operator as face transmissibilities: Te, Tn, Tt for
// the east, north and top face of each cell (0 on physical boundaries and on
// faces that touch a solid or empty cell), with
//   (A x)_c = sum over the six faces f of c of T_f (x_c - x_nb(f)),
// which on level 0 is exactly the stair-step PCG operator
// V (diag x - sum c x_nb) of src/fpm_stairstep_mpi_3d.f90:336-379 (east face
// of cell i: V_i ce_i = dy dz / (xc_{i+1} - xc_i), symmetric).  Level l+1
// aggregates 2 x 2 x 2 cells of level l; its operator is the Galerkin product
// P^T A P with piecewise-constant P, which keeps the 7-point form: a coarse
// face carries the sum of the fine faces between the two aggregates.  The
// V-cycle is symmetric (weighted Jacobi pre- and post-smoothing, restriction
// = P^T, a fixed number of Jacobi sweeps on the coarsest level), so it is a
// valid preconditioner for CG.
//
// Vectors are FP32 in the compact cell order (x fastest) of each level.
#include "fpm_internal.h"

namespace fpm {

namespace {

__device__ __forceinline__ long long ix(const MgLevel& L, int i, int j, int k) {
  return i + (long long)L.nx * (j + (long long)L.ny * k);
}

#define MG_CELLS(L)                                                                       \
  for (int k = blockIdx.z; k < (L).nz; k += gridDim.z)                                    \
    for (int j = blockIdx.y * blockDim.y + threadIdx.y; j < (L).ny; j += gridDim.y * blockDim.y) \
      for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (L).nx; i += gridDim.x * blockDim.x)

// Level 0 from the solid flags (padded (0:nx+1, 0:ny+1, nz)) and the axes.
__global__ void k_mg_level0(MgLevel L, Dims d, const int32_t* __restrict__ solid, Axes ax) {
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    const bool fl = solid[d.ph(i + 1, j + 1, k + 1)] == 0;
    double te = 0.0, tn = 0.0, tt = 0.0;
    if (fl && i + 1 < L.nx && solid[d.ph(i + 2, j + 1, k + 1)] == 0)
      te = ax.dy[j] * ax.dz[k] / (ax.xc[i + 2] - ax.xc[i + 1]);
    if (fl && j + 1 < L.ny && solid[d.ph(i + 1, j + 2, k + 1)] == 0)
      tn = ax.dx[i] * ax.dz[k] / (ax.yc[j + 2] - ax.yc[j + 1]);
    if (fl && k + 1 < L.nz && solid[d.ph(i + 1, j + 1, k + 2)] == 0)
      tt = ax.dx[i] * ax.dy[j] / (ax.zc[k + 1] - ax.zc[k]);
    L.te[c] = (float)te;
    L.tn[c] = (float)tn;
    L.tt[c] = (float)tt;
  }
}

// Coarse faces: the sum of the fine faces on the aggregate's east / north /
// top boundary (none when that boundary is the domain's).
__global__ void k_mg_coarsen(MgLevel F, MgLevel C) {
  MG_CELLS(C) {
    float te = 0.f, tn = 0.f, tt = 0.f;
    const int fi = 2 * i, fj = 2 * j, fk = 2 * k;
    for (int b = 0; b < 2; b++)
      for (int a = 0; a < 2; a++) {
        // east boundary: fine cells (2i+1, fj+a, fk+b)
        if (fi + 1 < F.nx && fj + a < F.ny && fk + b < F.nz) te += F.te[ix(F, fi + 1, fj + a, fk + b)];
        if (fj + 1 < F.ny && fi + a < F.nx && fk + b < F.nz) tn += F.tn[ix(F, fi + a, fj + 1, fk + b)];
        if (fk + 1 < F.nz && fi + a < F.nx && fj + b < F.ny) tt += F.tt[ix(F, fi + a, fj + b, fk + 1)];
      }
    const long long c = ix(C, i, j, k);
    C.te[c] = i + 1 < C.nx ? te : 0.f;
    C.tn[c] = j + 1 < C.ny ? tn : 0.f;
    C.tt[c] = k + 1 < C.nz ? tt : 0.f;
  }
}

__device__ __forceinline__ float face_sum(const MgLevel& L, int i, int j, int k, long long c) {
  float d = L.te[c] + L.tn[c] + L.tt[c];
  if (i > 0) d += L.te[c - 1];
  if (j > 0) d += L.tn[c - L.nx];
  if (k > 0) d += L.tt[c - (long long)L.nx * L.ny];
  return d;
}

__global__ void k_mg_dinv(MgLevel L) {
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    const float d = face_sum(L, i, j, k, c);
    L.dinv[c] = d > 0.f ? 1.f / d : 0.f;
  }
}

// (A x)_c in face form.
__device__ __forceinline__ float apply_a(const MgLevel& L, const float* __restrict__ x, int i, int j, int k,
                                        long long c) {
  const long long pl = (long long)L.nx * L.ny;
  const float xc = x[c];
  float u = 0.f;
  if (i + 1 < L.nx) u = fmaf(L.te[c], xc - x[c + 1], u);
  if (i > 0) u = fmaf(L.te[c - 1], xc - x[c - 1], u);
  if (j + 1 < L.ny) u = fmaf(L.tn[c], xc - x[c + L.nx], u);
  if (j > 0) u = fmaf(L.tn[c - L.nx], xc - x[c - L.nx], u);
  if (k + 1 < L.nz) u = fmaf(L.tt[c], xc - x[c + pl], u);
  if (k > 0) u = fmaf(L.tt[c - pl], xc - x[c - pl], u);
  return u;
}

// xo = (first ? 0 : x) + omega dinv (b - A x)   (first: x is taken as 0)
__global__ void k_mg_smooth(MgLevel L, const float* __restrict__ x, const float* __restrict__ b,
                            float* __restrict__ xo, float omega, int first) {
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    const float w = omega * L.dinv[c];
    xo[c] = first ? w * b[c] : fmaf(w, b[c] - apply_a(L, x, i, j, k, c), x[c]);
  }
}

// r = b - A x
__global__ void k_mg_residual(MgLevel L, const float* __restrict__ x, const float* __restrict__ b,
                              float* __restrict__ r) {
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    r[c] = b[c] - apply_a(L, x, i, j, k, c);
  }
}

// bc = sum of the fine residuals of each aggregate
__global__ void k_mg_restrict(MgLevel F, MgLevel C, const float* __restrict__ rf, float* __restrict__ bc) {
  MG_CELLS(C) {
    float s = 0.f;
    for (int o = 0; o < 8; o++) {
      const int fi = 2 * i + (o & 1), fj = 2 * j + ((o >> 1) & 1), fk = 2 * k + (o >> 2);
      if (fi < F.nx && fj < F.ny && fk < F.nz) s += rf[ix(F, fi, fj, fk)];
    }
    bc[ix(C, i, j, k)] = s;
  }
}

// xf += xc(parent)
__global__ void k_mg_prolong(MgLevel F, MgLevel C, const float* __restrict__ xc, float* __restrict__ xf) {
  MG_CELLS(F) { xf[ix(F, i, j, k)] += xc[ix(C, i >> 1, j >> 1, k >> 1)]; }
}

// Coarsest level: nsweeps weighted Jacobi sweeps from 0 in one block
// (the level has at most 1024 cells); ping-pong in global scratch.
__global__ void k_mg_coarse(MgLevel L, const float* __restrict__ b, float* __restrict__ x, float* __restrict__ tmp,
                            float omega, int nsweeps) {
  const int n = (int)L.n();
  for (int c = threadIdx.x; c < n; c += blockDim.x) x[c] = omega * L.dinv[c] * b[c];
  __syncthreads();
  float* a = x;
  float* o = tmp;
  for (int s = 1; s < nsweeps; s++) {
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      const int i = c % L.nx, j = (c / L.nx) % L.ny, k = c / (L.nx * L.ny);
      o[c] = fmaf(omega * L.dinv[c], b[c] - apply_a(L, a, i, j, k, c), a[c]);
    }
    __syncthreads();
    float* t = a;
    a = o;
    o = t;
  }
  if (a != x) {
    for (int c = threadIdx.x; c < n; c += blockDim.x) x[c] = a[c];
  }
}

dim3 mg_grid(const MgLevel& L) {
  const int gx = (L.nx + 31) / 32, gy = (L.ny + 7) / 8;
  long long gz = (152LL * 16 + (long long)gx * gy - 1) / ((long long)gx * gy);
  if (gz > L.nz) gz = L.nz;
  if (gz < 1) gz = 1;
  return dim3(gx, gy, (unsigned)gz);
}

}  // namespace

cudaError_t mg_setup(MgHierarchy& H, const Dims& d, const int32_t* solid, const Axes& ax, cudaStream_t st) {
  const dim3 blk(32, 8);
  k_mg_level0<<<mg_grid(H.lv[0]), blk, 0, st>>>(H.lv[0], d, solid, ax);
  note_launch();
  for (int l = 0; l + 1 < H.nlev; l++) {
    k_mg_coarsen<<<mg_grid(H.lv[l + 1]), blk, 0, st>>>(H.lv[l], H.lv[l + 1]);
    note_launch();
  }
  for (int l = 0; l < H.nlev; l++) {
    k_mg_dinv<<<mg_grid(H.lv[l]), blk, 0, st>>>(H.lv[l]);
    note_launch();
  }
  return cudaGetLastError();
}

// x = V-cycle(b) on level l.  Smoothing alternates between x and the level's
// scratch t; the first write goes to t, and 2 nu - 1 sweeps later the result
// is in x.
static cudaError_t vcycle(const MgHierarchy& H, int l, const float* b, float* x, cudaStream_t st) {
  const MgLevel& L = H.lv[l];
  const dim3 blk(32, 8), g = mg_grid(L);
  if (l == H.nlev - 1) {
    k_mg_coarse<<<1, 1024, 0, st>>>(L, b, x, L.t, H.omega, H.coarse_sweeps);
    note_launch();
    return cudaGetLastError();
  }
  float* cur = L.t;
  float* oth = x;
  k_mg_smooth<<<g, blk, 0, st>>>(L, cur, b, cur, H.omega, 1);
  note_launch();
  for (int s = 1; s < H.nu; s++) {
    k_mg_smooth<<<g, blk, 0, st>>>(L, cur, b, oth, H.omega, 0);
    note_launch();
    float* t = cur;
    cur = oth;
    oth = t;
  }
  k_mg_residual<<<g, blk, 0, st>>>(L, cur, b, L.r);
  note_launch();
  const MgLevel& C = H.lv[l + 1];
  k_mg_restrict<<<mg_grid(C), blk, 0, st>>>(L, C, L.r, C.b);
  note_launch();
  cudaError_t e = vcycle(H, l + 1, C.b, C.x, st);
  if (e != cudaSuccess) return e;
  k_mg_prolong<<<g, blk, 0, st>>>(L, C, C.x, cur);
  note_launch();
  for (int s = 0; s < H.nu; s++) {
    k_mg_smooth<<<g, blk, 0, st>>>(L, cur, b, oth, H.omega, 0);
    note_launch();
    float* t = cur;
    cur = oth;
    oth = t;
  }
  return cudaGetLastError();
}

cudaError_t mg_vcycle(const MgHierarchy& H, const float* r, float* z, cudaStream_t st) { return vcycle(H, 0, r, z, st); }

// ---------------------------------------------------------------- PCG pieces (level-0 layout)
namespace {

// q = A p, pq = p.q, alpha = rz / pq
__global__ void k_mgp_spmv(MgLevel L, const float* __restrict__ p, float* __restrict__ q, MgScalars* S, RedBuf rb) {
  if (!S->active) return;
  double s[1] = {0.0}, m[1] = {0.0};
  float acc = 0.f, err = 0.f;
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    const float v = apply_a(L, p, i, j, k, c);
    q[c] = v;
    const float prod = p[c] * v;
    const float t = acc + prod, bb = t - acc;
    err += (acc - (t - bb)) + (prod - bb);
    acc = t;
  }
  s[0] = (double)acc + (double)err;
  double out[1];
  if (grid_reduce<1, 0>(s, m, rb.partials, rb.ticket, out) && lin_tid() == 0) {
    S->pq = out[0];
    if (!(out[0] > 0) || !(S->rz > 0)) {
      S->active = 0;
      S->alpha = 0;
    } else {
      S->alpha = S->rz / out[0];
    }
  }
}

// e += alpha p; r -= alpha q
__global__ void k_mgp_update(MgLevel L, const float* __restrict__ p, const float* __restrict__ q, float* __restrict__ e,
                             float* __restrict__ r, const MgScalars* S) {
  if (!S->active) return;
  const float a = (float)S->alpha;
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    e[c] = fmaf(a, p[c], e[c]);
    r[c] = fmaf(-a, q[c], r[c]);
  }
}

// rz_new = r.z; beta; stop at the drop
__global__ void k_mgp_rz(MgLevel L, const float* __restrict__ r, const float* __restrict__ z, MgScalars* S, RedBuf rb,
                         int start) {
  if (!start && !S->active) return;
  double s[1] = {0.0}, m[1] = {0.0};
  float acc = 0.f, err = 0.f;
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    const float prod = r[c] * z[c];
    const float t = acc + prod, bb = t - acc;
    err += (acc - (t - bb)) + (prod - bb);
    acc = t;
  }
  s[0] = (double)acc + (double)err;
  double out[1];
  if (grid_reduce<1, 0>(s, m, rb.partials, rb.ticket, out) && lin_tid() == 0) {
    const double rz = out[0];
    if (start) {
      S->rz = rz;
      S->rz0 = rz;
      S->beta = 0.0;
      S->active = rz > 0 ? 1 : 0;
      S->dir = S->active;
      return;
    }
    S->iters += 1;
    if (!(rz >= 0)) {
      S->active = 0;
      S->dir = 0;
      return;
    }
    S->beta = rz / S->rz;
    S->rz = rz;
    S->dir = 1;
    if (rz <= S->tol2 * S->rz0) S->active = 0;
  }
}

// p = z + beta p  (start: p = z)
__global__ void k_mgp_direction(MgLevel L, const float* __restrict__ z, float* __restrict__ p, const MgScalars* S,
                                int start) {
  if (!start && !S->dir) return;
  const float b = start ? 0.f : (float)S->beta;
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    p[c] = start ? z[c] : fmaf(b, p[c], z[c]);
  }
}

// r32 = scale * rV (compact FP64 projected residual) on fluid cells, e = 0
__global__ void k_mgp_load(MgLevel L, const double* __restrict__ rv, double scale, float* __restrict__ r,
                           float* __restrict__ e) {
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    r[c] = L.dinv[c] > 0.f ? (float)(rv[c] * scale) : 0.f;
    e[c] = 0.f;
  }
}

// phi(padded) += e / scale on fluid cells
__global__ void k_mgp_apply(MgLevel L, Dims d, const float* __restrict__ e, double scale, double* __restrict__ phi) {
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    if (L.dinv[c] > 0.f) phi[d.ph(i + 1, j + 1, k + 1)] += (double)e[c] / scale;
  }
}

}  // namespace

cudaError_t mg_pcg_start(const MgHierarchy& H, const double* rv, double scale, MgVecs& v, MgScalars* S, const RedBuf& rb,
                         cudaStream_t st) {
  const MgLevel& L = H.lv[0];
  const dim3 blk(32, 8), g = mg_grid(L);
  k_mgp_load<<<g, blk, 0, st>>>(L, rv, scale, v.r, v.e);
  note_launch();
  cudaError_t e = mg_vcycle(H, v.r, v.z, st);
  if (e != cudaSuccess) return e;
  k_mgp_rz<<<g, blk, 0, st>>>(L, v.r, v.z, S, rb, 1);
  note_launch();
  k_mgp_direction<<<g, blk, 0, st>>>(L, v.z, v.p, S, 1);
  note_launch();
  return cudaGetLastError();
}

cudaError_t mg_pcg_iteration(const MgHierarchy& H, MgVecs& v, MgScalars* S, const RedBuf& rb, cudaStream_t st) {
  const MgLevel& L = H.lv[0];
  const dim3 blk(32, 8), g = mg_grid(L);
  k_mgp_spmv<<<g, blk, 0, st>>>(L, v.p, v.q, S, rb);
  note_launch();
  k_mgp_update<<<g, blk, 0, st>>>(L, v.p, v.q, v.e, v.r, S);
  note_launch();
  cudaError_t e = mg_vcycle(H, v.r, v.z, st);
  if (e != cudaSuccess) return e;
  k_mgp_rz<<<g, blk, 0, st>>>(L, v.r, v.z, S, rb, 0);
  note_launch();
  k_mgp_direction<<<g, blk, 0, st>>>(L, v.z, v.p, S, 0);
  note_launch();
  return cudaGetLastError();
}

cudaError_t mg_pcg_apply(const MgHierarchy& H, const Dims& d, const MgVecs& v, double scale, double* phi,
                         cudaStream_t st) {
  const MgLevel& L = H.lv[0];
  k_mgp_apply<<<mg_grid(L), dim3(32, 8), 0, st>>>(L, d, v.e, scale, phi);
  note_launch();
  return cudaGetLastError();
}

int mg_grid_blocks(const MgLevel& L) {
  const dim3 g = mg_grid(L);
  return (int)(g.x * g.y * g.z);
}

}  // namespace fpm
