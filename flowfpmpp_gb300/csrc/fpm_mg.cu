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
// Level 0 uses the FP32 layout of the mixed solver (16-byte aligned rows,
// zero x-y halo, see MixedGrid): its three stencil passes stream planes
// through shared memory with TMA and also carry the PCG vector updates (no
// pointwise pass).  The coarse levels are compact (x fastest, rows padded to
// 16 bytes) and take four cells per thread (float4).  All right-hand sides
// share each launch.
#include "fpm_internal.h"
#include "fpm_tma.cuh"

namespace fpm {

namespace {

__device__ __forceinline__ long long ix(const MgLevel& L, int i, int j, int k) {
  return L.off + i + L.sy * j + L.sz * k;
}

// Grids of the one-thread-per-cell kernels: (x, y) tiles and L.zc strided
// chunks of planes per right-hand side; blockIdx.z = chunk + zc * rhs.
#define MG_RHS(L) const int mrhs = (int)blockIdx.z / (L).zc
#define MG_SKIP(m) \
  if (!(((mask >> (m)) & 1u) && S[m].active)) return

// Pointers of one vector per right-hand side.
struct Vec4 {
  float* p[kMaxRhs];
};
// p[m] of a kernel-parameter pointer table, selected with constant indices
// (a dynamic index would copy the table to local memory in every thread).
template <class T>
__device__ __forceinline__ T pick(T const (&p)[kMaxRhs], int m) {
  static_assert(kMaxRhs == 4, "pick covers four right-hand sides");
  return m == 0 ? p[0] : (m == 1 ? p[1] : (m == 2 ? p[2] : p[3]));
}
#define MG_CELLS(L)                                                                       \
  for (int k = (int)blockIdx.z % (L).zc; k < (L).nz; k += (L).zc)                         \
    for (int j = blockIdx.y * blockDim.y + threadIdx.y; j < (L).ny; j += gridDim.y * blockDim.y) \
      for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (L).nx; i += gridDim.x * blockDim.x)

// Level 0 from the solid flags (padded (0:nx+1, 0:ny+1, nz)) and the axes;
// also the open-face bits of the float4 kernels (row pitch pxb).
__global__ void k_mg_level0(MgLevel L, Dims d, const int32_t* __restrict__ solid, Axes ax, uint8_t* __restrict__ fb,
                            long long pxb) {
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
    fb[4 + i + pxb * ((j + 1) + (long long)(L.ny + 2) * k)] =
        (uint8_t)((te > 0.0 ? 1 : 0) | (tn > 0.0 ? 2 : 0) | (tt > 0.0 ? 4 : 0));
  }
}

// 1-D FP32 factors of the level-0 faces (see MgHierarchy).
__global__ void k_mg_axes0(MixedGrid G, Axes ax, float* aex, float* dxr, float* dy, float* ayn, float* dz, float* azt) {
  const int n = max(G.px, max(G.ny, G.nz));
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    if (m < G.px) {
      const int i = m - 3;  // 1-based cell
      aex[m] = (i >= 1 && i + 1 <= G.nx) ? (float)(1.0 / (ax.xc[i + 1] - ax.xc[i])) : 0.f;
      dxr[m] = (i >= 1 && i <= G.nx) ? (float)ax.dx[i - 1] : 0.f;
    }
    if (m < G.ny) {
      dy[m] = (float)ax.dy[m];
      ayn[m] = m + 1 < G.ny ? (float)(1.0 / (ax.yc[m + 2] - ax.yc[m + 1])) : 0.f;
    }
    if (m < G.nz) {
      dz[m] = (float)ax.dz[m];
      azt[m] = m + 1 < G.nz ? (float)(1.0 / (ax.zc[m + 1] - ax.zc[m])) : 0.f;
    }
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
  if (j > 0) d += L.tn[c - L.sy];
  if (k > 0) d += L.tt[c - L.sz];
  return d;
}

// dinv = scale / diag (level 0: scale = omega, the smoothing weight folded in)
__global__ void k_mg_dinv(MgLevel L, float scale) {
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    const float d = face_sum(L, i, j, k, c);
    L.dinv[c] = d > 0.f ? scale / d : 0.f;
  }
}

// Coarsest level (at most 1024 cells): nsweeps weighted Jacobi sweeps from 0
// in one block per right-hand side, with the level's operator, right-hand side
// and iterate in shared memory (compact there, x fastest).
__global__ void __launch_bounds__(1024) k_mg_coarse(MgLevel L, Vec4 bv, Vec4 xv, float omega, int nsweeps,
                                                    const MgScalars* S, unsigned mask) {
  const int mrhs = blockIdx.x;
  MG_SKIP(mrhs);
  const float* __restrict__ b = pick(bv.p, mrhs);
  float* __restrict__ x = pick(xv.p, mrhs);
  __shared__ float te[1024], tn[1024], tt[1024], wd[1024], bb[1024], xa[1024], xb[1024];
  const int n = (int)L.n();
  const int c = threadIdx.x;
  const int sy = L.nx, sz = L.nx * L.ny;  // shared-memory strides
  int i = 0, j = 0, k = 0;
  long long gc = 0;
  if (c < n) {
    i = c % L.nx;
    j = (c / L.nx) % L.ny;
    k = c / (L.nx * L.ny);
    gc = ix(L, i, j, k);
    te[c] = L.te[gc];
    tn[c] = L.tn[gc];
    tt[c] = L.tt[gc];
    wd[c] = omega * L.dinv[gc];
    bb[c] = b[gc];
    xa[c] = wd[c] * bb[c];
  }
  __syncthreads();
  float* a = xa;
  float* o = xb;
  for (int s = 1; s < nsweeps; s++) {
    if (c < n) {
      const float xc = a[c];
      float u = 0.f;
      if (i + 1 < L.nx) u = fmaf(te[c], xc - a[c + 1], u);
      if (i > 0) u = fmaf(te[c - 1], xc - a[c - 1], u);
      if (j + 1 < L.ny) u = fmaf(tn[c], xc - a[c + sy], u);
      if (j > 0) u = fmaf(tn[c - sy], xc - a[c - sy], u);
      if (k + 1 < L.nz) u = fmaf(tt[c], xc - a[c + sz], u);
      if (k > 0) u = fmaf(tt[c - sz], xc - a[c - sz], u);
      o[c] = fmaf(wd[c], bb[c] - u, xc);
    }
    __syncthreads();
    float* t = a;
    a = o;
    o = t;
  }
  if (c < n) x[gc] = a[c];
}

dim3 mg_grid(const MgLevel& L) { return dim3((L.nx + 31) / 32, (L.ny + 7) / 8, (unsigned)L.zc); }
dim3 rhs_grid(const MgLevel& L, int nrhs) { return dim3((L.nx + 31) / 32, (L.ny + 7) / 8, (unsigned)(L.zc * nrhs)); }
Vec4 vec4(float* const (&p)[kMaxRhs]) {
  Vec4 v;
  for (int m = 0; m < kMaxRhs; m++) v.p[m] = p[m];
  return v;
}

}  // namespace

cudaError_t mg_setup(MgHierarchy& H, const Dims& d, const int32_t* solid, const Axes& ax, cudaStream_t st) {
  const dim3 blk(32, 8);
  k_mg_level0<<<mg_grid(H.lv[0]), blk, 0, st>>>(H.lv[0], d, solid, ax, H.fb0, H.pxb);
  note_launch();
  k_mg_axes0<<<8, 256, 0, st>>>(H.g0, ax, H.aex, H.dxr, H.dy, H.ayn, H.dz, H.azt);
  note_launch();
  for (int l = 0; l + 1 < H.nlev; l++) {
    k_mg_coarsen<<<mg_grid(H.lv[l + 1]), blk, 0, st>>>(H.lv[l], H.lv[l + 1]);
    note_launch();
  }
  for (int l = 0; l < H.nlev; l++) {
    k_mg_dinv<<<mg_grid(H.lv[l]), blk, 0, st>>>(H.lv[l], l == 0 ? H.omega : 1.f);
    note_launch();
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------- level 0: float4 kernels
namespace {

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ void st4(float* p, const float4& v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 zero4() { return make_float4(0.f, 0.f, 0.f, 0.f); }
__device__ __forceinline__ float el(const float4& v, int n) { return n == 0 ? v.x : (n == 1 ? v.y : (n == 2 ? v.z : v.w)); }

// f32 running sum with its rounding error (TwoSum)
struct Acc2 {
  float s = 0.f, e = 0.f;
  __device__ __forceinline__ void add(float p) {
    const float t = s + p, bb = t - s;
    e += (s - (t - bb)) + (p - bb);
    s = t;
  }
  __device__ __forceinline__ void add4(const float4& a, const float4& b) {
    add(fmaf(a.w, b.w, fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x))));
  }
};

// Thread position on level 0: group g (cells 4g .. 4g+3, 0-based) of row j
// (1-based), planes k0..k1 (1-based), as in the mixed solver's kernels.
// blockIdx.z = chunk of kc planes + zc x right-hand side m.
struct P0 {
  int g, j, k0, k1, m, zc;
  bool live;
  long long base;
};

// Sum of s over the blocks of right-hand side m (the zc chunks of its
// blockIdx.z range); true in the last of them, with *out set in thread 0.
__device__ bool rhs_reduce(double s, int m, int zc, const MgRed& rb, double* out) {
  __shared__ bool am_last;
  double a[1] = {s}, mm[1] = {0.0};
  block_reduce<1, 0>(a, mm);
  const int nb = (int)(gridDim.x * gridDim.y) * zc;
  const int bid = (int)blockIdx.x + (int)gridDim.x * ((int)blockIdx.y + (int)gridDim.y * ((int)blockIdx.z - m * zc));
  double* part = rb.partials + (size_t)m * nb;
  const int tid = lin_tid();
  if (tid == 0) {
    part[bid] = a[0];
    __threadfence();
    am_last = atomicAdd(rb.tickets + m, 1u) == (unsigned int)nb - 1;
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  a[0] = 0.0;
  for (int b = tid; b < nb; b += lin_nthreads()) a[0] += __ldcg(part + b);
  block_reduce<1, 0>(a, mm);
  if (tid == 0) {
    *out = a[0];
    rb.tickets[m] = 0u;
    __threadfence();
  }
  __syncthreads();
  return true;
}

// Level-0 faces rebuilt from the open-face bits and the 1-D factors.
struct Ops0 {
  const float *aex, *dxr, *dy, *ayn, *dz, *azt;
};
struct Row0 {  // per-thread constants of a group's row
  float4 aex, dx;
  float dy, ayn, ayn_s, aex_w;
};
__device__ __forceinline__ Row0 row0(const Ops0& O, const P0& t) {
  Row0 r;
  r.aex = r.dx = zero4();
  r.dy = r.ayn = r.ayn_s = r.aex_w = 0.f;
  if (t.live) {
    const int o = 4 * (t.g + 1);
    r.aex = ld4(O.aex + o);
    r.dx = ld4(O.dxr + o);
    r.dy = __ldg(O.dy + t.j - 1);
    r.ayn = __ldg(O.ayn + t.j - 1);
    r.ayn_s = t.j > 1 ? __ldg(O.ayn + t.j - 2) : 0.f;
    r.aex_w = __ldg(O.aex + o - 1);
  }
  return r;
}
// Faces of a group's cells in pairs (cells 0,1 and 2,3), from the open-face
// bits of the group (f), of the row below (fs) and of the west cell (fw), one
// byte per cell; the FP32x2 instructions of sm_100+ give the same per-lane
// rounding as the scalar ones.
__device__ __forceinline__ float2 lo2(const float4& v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4& v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 dif2(float2 a, float2 b) {  // a - b (fma with -1 rounds like the subtraction)
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ float2 sel2(uint32_t p0, uint32_t p1, float2 v) {
  return make_float2(p0 ? v.x : 0.f, p1 ? v.y : 0.f);
}
struct Faces2 {
  float2 te[2], tn[2], tns[2], tt[2];
  float te_w;
};
__device__ __forceinline__ Faces2 faces2(const Row0& R, float dz, float azt, uint32_t f, uint32_t fs, uint32_t fw) {
  const float ex = R.dy * dz, ny = dz * R.ayn, nys = dz * R.ayn_s, tz = R.dy * azt;
  Faces2 F;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const float2 ax = h ? hi2(R.aex) : lo2(R.aex), dx = h ? hi2(R.dx) : lo2(R.dx);
    const uint32_t b0 = f >> (16 * h), b1 = f >> (16 * h + 8), s0 = fs >> (16 * h), s1 = fs >> (16 * h + 8);
    F.te[h] = sel2(b0 & 1u, b1 & 1u, __fmul2_rn(ax, dup2(ex)));
    F.tn[h] = sel2(b0 & 2u, b1 & 2u, __fmul2_rn(dx, dup2(ny)));
    F.tns[h] = sel2(s0 & 2u, s1 & 2u, __fmul2_rn(dx, dup2(nys)));
    F.tt[h] = sel2(b0 & 4u, b1 & 4u, __fmul2_rn(dx, dup2(tz)));
  }
  F.te_w = (fw & 1u) ? R.aex_w * ex : 0.f;
  return F;
}
// Top faces of the plane below (bits fb, its z factor aztb): the bottom faces
// of a chunk's first plane; later planes carry them over.
__device__ __forceinline__ void bottom2(const Row0& R, float aztb, uint32_t fb, float2 (&ttb)[2]) {
  const float tzb = R.dy * aztb;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const float2 dx = h ? hi2(R.dx) : lo2(R.dx);
    ttb[h] = sel2((fb >> (16 * h)) & 4u, (fb >> (16 * h + 8)) & 4u, __fmul2_rn(dx, dup2(tzb)));
  }
}
// u = (A v) for the four cells of a group: per cell
//   te (x - xe) + tw (x - xw) + tn (x - xn) + ts (x - xs) + tt (x - xt) + tb (x - xb)
// summed in that order (mul, then fma).
__device__ __forceinline__ float4 face_apply2(const float4& c, float left, float right, const float4& s,
                                              const float4& n, const float4& b, const float4& t, const Faces2& F,
                                              const float2 (&ttb)[2]) {
  const float2 x[2] = {lo2(c), hi2(c)};
  const float2 mid = make_float2(c.y, c.z);
  const float2 xe[2] = {mid, make_float2(c.w, right)};
  const float2 xw[2] = {make_float2(left, c.x), mid};
  const float2 tw[2] = {make_float2(F.te_w, F.te[0].x), make_float2(F.te[0].y, F.te[1].x)};
  const float2 xn[2] = {lo2(n), hi2(n)}, xs[2] = {lo2(s), hi2(s)}, xt[2] = {lo2(t), hi2(t)}, xb[2] = {lo2(b), hi2(b)};
  float2 u[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    float2 v = __fmul2_rn(F.te[h], dif2(x[h], xe[h]));
    v = __ffma2_rn(tw[h], dif2(x[h], xw[h]), v);
    v = __ffma2_rn(F.tn[h], dif2(x[h], xn[h]), v);
    v = __ffma2_rn(F.tns[h], dif2(x[h], xs[h]), v);
    v = __ffma2_rn(F.tt[h], dif2(x[h], xt[h]), v);
    v = __ffma2_rn(ttb[h], dif2(x[h], xb[h]), v);
    u[h] = v;
  }
  return make_float4(u[0].x, u[0].y, u[1].x, u[1].y);
}

// ---------------------------------------------------------------- float4 kernels of the V-cycle
// Every level's rows start on 16 bytes (level 0: off = 4 + px, levels >= 1:
// off = 0; sy a multiple of 4), so a thread takes the four cells 4g .. 4g+3
// of a row on one plane.  Faces outside the grid and at padding cells are
// zero, so neighbours outside the grid read as zero; outputs at padding
// cells are written as zero.
#define MG4_CELLS(L)                                                                        \
  for (int k = (int)blockIdx.z % (L).zc; k < (L).nz; k += (L).zc)                           \
    for (int j = blockIdx.y * blockDim.y + threadIdx.y; j < (L).ny; j += gridDim.y * blockDim.y) \
      for (int g = blockIdx.x * blockDim.x + threadIdx.x; 4 * g < (L).nx; g += gridDim.x * blockDim.x)

struct X4 {  // a group's values and its neighbours' (s, n: rows j -+ 1; b, t: planes k -+ 1; l, r: x)
  float4 c, s, n, b, t;
  float l, r;
};
__device__ __forceinline__ X4 load_x4(const MgLevel& L, const float* __restrict__ x, int g, int j, int k,
                                      long long c) {
  X4 v;
  v.c = ld4(x + c);
  v.s = j > 0 ? ld4(x + c - L.sy) : zero4();
  v.n = j + 1 < L.ny ? ld4(x + c + L.sy) : zero4();
  v.b = k > 0 ? ld4(x + c - L.sz) : zero4();
  v.t = k + 1 < L.nz ? ld4(x + c + L.sz) : zero4();
  v.l = g > 0 ? __ldg(x + c - 1) : 0.f;
  v.r = 4 * g + 4 < L.nx ? __ldg(x + c + 4) : 0.f;
  return v;
}
// The first smoothing sweep from zero, t = omega dinv b, at the group and
// its neighbours (the layout of load_x4), for passes that rebuild t instead
// of reading it.
__device__ __forceinline__ X4 load_t4(const MgLevel& L, const float* __restrict__ b, float omega, int g, int j,
                                      int k, long long c) {
  auto t4 = [&](long long o) {
    const float4 bb = ld4(b + o), dv = ld4(L.dinv + o);
    return make_float4(omega * dv.x * bb.x, omega * dv.y * bb.y, omega * dv.z * bb.z, omega * dv.w * bb.w);
  };
  auto t1 = [&](long long o) { return omega * __ldg(L.dinv + o) * __ldg(b + o); };
  X4 v;
  v.c = t4(c);
  v.s = j > 0 ? t4(c - L.sy) : zero4();
  v.n = j + 1 < L.ny ? t4(c + L.sy) : zero4();
  v.b = k > 0 ? t4(c - L.sz) : zero4();
  v.t = k + 1 < L.nz ? t4(c + L.sz) : zero4();
  v.l = g > 0 ? t1(c - 1) : 0.f;
  v.r = 4 * g + 4 < L.nx ? t1(c + 4) : 0.f;
  return v;
}

// A x for the group from its faces (stored transmissibilities).
__device__ __forceinline__ float4 apply4(const MgLevel& L, const X4& X, int g, int j, int k, long long c) {
  const float4 te = ld4(L.te + c), tn = ld4(L.tn + c), tt = ld4(L.tt + c);
  const float4 tns = j > 0 ? ld4(L.tn + c - L.sy) : zero4();
  const float4 ttb4 = k > 0 ? ld4(L.tt + c - L.sz) : zero4();
  Faces2 F;
  F.te[0] = lo2(te);
  F.te[1] = hi2(te);
  F.tn[0] = lo2(tn);
  F.tn[1] = hi2(tn);
  F.tns[0] = lo2(tns);
  F.tns[1] = hi2(tns);
  F.tt[0] = lo2(tt);
  F.tt[1] = hi2(tt);
  F.te_w = g > 0 ? __ldg(L.te + c - 1) : 0.f;
  const float2 ttb[2] = {lo2(ttb4), hi2(ttb4)};
  return face_apply2(X.c, X.l, X.r, X.s, X.n, X.b, X.t, F, ttb);
}
// out = y + omega dinv (b - u) per cell, zero at padding cells (i >= nx)
__device__ __forceinline__ float4 smooth_out(const MgLevel& L, int g, const float4& y, const float4& dv,
                                             const float4& bb, const float4& u, float omega) {
  float o[4];
#pragma unroll
  for (int q = 0; q < 4; q++)
    o[q] = 4 * g + q < L.nx ? fmaf(omega * el(dv, q), el(bb, q) - el(u, q), el(y, q)) : 0.f;
  return make_float4(o[0], o[1], o[2], o[3]);
}

// xo = x + omega dinv (b - A x): the smoothing sweep of a warm cycle (cold
// cycles fold their sweep from zero into the next two passes)
__global__ void __launch_bounds__(256) k_mg_smooth4(MgLevel L, Vec4 xv, Vec4 bv, Vec4 xov, float omega,
                                                    const MgScalars* S, unsigned mask) {
  MG_RHS(L);
  MG_SKIP(mrhs);
  const float* __restrict__ x = pick(xv.p, mrhs);
  const float* __restrict__ b = pick(bv.p, mrhs);
  float* __restrict__ xo = pick(xov.p, mrhs);
  MG4_CELLS(L) {
    const long long c = ix(L, 4 * g, j, k);
    const float4 dv = ld4(L.dinv + c), bb = ld4(b + c);
    const X4 X = load_x4(L, x, g, j, k, c);
    st4(xo + c, smooth_out(L, g, X.c, dv, bb, apply4(L, X, g, j, k, c), omega));
  }
}

// bc = scale x restriction of b - A x: a thread takes two coarse cells
// (cg: 2cg, 2cg+1), i.e. fine group cg on the aggregate's two rows and two
// planes.  first: x is the first smoothing sweep from zero, rebuilt as
// omega dinv b.  scale > 1 over-corrects with the coarse solution (the
// cycle stays linear and symmetric).
template <bool FIRST>
__global__ void __launch_bounds__(256, 4) k_mg_resrestrict4(MgLevel F, MgLevel C, Vec4 xv, Vec4 bv, Vec4 bcv,
                                                         float scale, const MgScalars* S, unsigned mask,
                                                         float omega) {
  MG_RHS(C);
  MG_SKIP(mrhs);
  const float* __restrict__ x = pick(xv.p, mrhs);
  const float* __restrict__ b = pick(bv.p, mrhs);
  float* __restrict__ bc = pick(bcv.p, mrhs);
  for (int ck = (int)blockIdx.z % C.zc; ck < C.nz; ck += C.zc)
    for (int cj = blockIdx.y * blockDim.y + threadIdx.y; cj < C.ny; cj += gridDim.y * blockDim.y)
      for (int cg = blockIdx.x * blockDim.x + threadIdx.x; 2 * cg < C.nx; cg += gridDim.x * blockDim.x) {
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int o = 0; o < 4; o++) {
          const int j = 2 * cj + (o & 1), k = 2 * ck + (o >> 1);
          if (j < F.ny && k < F.nz) {
            const long long c = ix(F, 4 * cg, j, k);
            const X4 X = FIRST ? load_t4(F, b, omega, cg, j, k, c) : load_x4(F, x, cg, j, k, c);
            const float4 u = apply4(F, X, cg, j, k, c), bb = ld4(b + c);
            s0 += (bb.x - u.x) + (bb.y - u.y);
            s1 += (bb.z - u.z) + (bb.w - u.w);
          }
        }
        float* o = bc + ix(C, 2 * cg, cj, ck);
        o[0] = scale * s0;
        if (2 * cg + 1 < C.nx) o[1] = scale * s1;
      }
}

// xo = y + omega dinv (b - A y) with y = x + P xc (the prolonged correction is
// added on the fly, also at the neighbours): prolongation and the first
// post-smoothing sweep in one pass (first: x rebuilt as omega dinv b, as in
// k_mg_resrestrict4).  Fine cells 4g .. 4g+3 have the coarse
// parents 2g, 2g, 2g+1, 2g+1 (a float2 of the coarse row: 2g is even and
// the row starts on 16 bytes).
template <bool FIRST>
__global__ void __launch_bounds__(256, 4) k_mg_prolong_smooth4(MgLevel F, MgLevel C, Vec4 xv, Vec4 xcv, Vec4 bv,
                                                            Vec4 xov, float omega, const MgScalars* S,
                                                            unsigned mask) {
  MG_RHS(F);
  MG_SKIP(mrhs);
  const float* __restrict__ x = pick(xv.p, mrhs);
  const float* __restrict__ xc = pick(xcv.p, mrhs);
  const float* __restrict__ b = pick(bv.p, mrhs);
  float* __restrict__ xo = pick(xov.p, mrhs);
  auto par = [&](int g, int j, int k) {  // parents of fine group g on row j, plane k
    const float2 p = __ldg(reinterpret_cast<const float2*>(xc + ix(C, 2 * g, j >> 1, k >> 1)));
    return make_float4(p.x, p.x, p.y, p.y);
  };
  auto add = [](float4& a, const float4& v) {
    a.x += v.x;
    a.y += v.y;
    a.z += v.z;
    a.w += v.w;
  };
  MG4_CELLS(F) {
    const long long c = ix(F, 4 * g, j, k);
    X4 X = FIRST ? load_t4(F, b, omega, g, j, k, c) : load_x4(F, x, g, j, k, c);
    add(X.c, par(g, j, k));
    if (j > 0) add(X.s, par(g, j - 1, k));
    if (j + 1 < F.ny) add(X.n, par(g, j + 1, k));
    if (k > 0) add(X.b, par(g, j, k - 1));
    if (k + 1 < F.nz) add(X.t, par(g, j, k + 1));
    if (g > 0) X.l += __ldg(xc + ix(C, 2 * g - 1, j >> 1, k >> 1));
    if (4 * g + 4 < F.nx) X.r += __ldg(xc + ix(C, 2 * g + 2, j >> 1, k >> 1));
    const float4 dv = ld4(F.dinv + c), bb = ld4(b + c);
    st4(xo + c, smooth_out(F, g, X.c, dv, bb, apply4(F, X, g, j, k, c), omega));
  }
}

dim3 grid4(const MgLevel& L, int nrhs) {
  return dim3((unsigned)(((L.nx + 3) / 4 + 31) / 32), (unsigned)((L.ny + 7) / 8), (unsigned)(L.zc * nrhs));
}
dim3 grid4r(const MgLevel& C, int nrhs) {  // k_mg_resrestrict4: two coarse cells per thread
  return dim3((unsigned)(((C.nx + 1) / 2 + 31) / 32), (unsigned)((C.ny + 7) / 8), (unsigned)(C.zc * nrhs));
}

}  // namespace

// Cycles on the level-(l+1) problem asked for by level l: gamma on the first
// gamma_depth levels (W-like there), one below; the coarsest level is solved
// (from zero) once.
static int coarse_cycles(const MgHierarchy& H, int l) {
  if (l + 1 == H.nlev - 1) return 1;
  return l < H.gamma_depth ? H.gamma : 1;
}

// x = cycle(b) on level l >= 1 for every right-hand side at once, from x = 0,
// or from the current x when warm (one smoothing sweep each way; the
// prolongation + post-smoothing pass writes x).
static cudaError_t vcycle(const MgHierarchy& H, int l, const MgScalars* S, unsigned mask, cudaStream_t st,
                          bool warm = false) {
  const MgLevel& L = H.lv[l];
  const dim3 blk(32, 8), g = grid4(L, H.nrhs);
  const Vec4 b = vec4(L.b), x = vec4(L.x), t = vec4(L.t);
  if (l == H.nlev - 1) {
    k_mg_coarse<<<H.nrhs, 1024, 0, st>>>(L, b, x, H.omega, H.coarse_sweeps, S, mask);
    note_launch();
    return cudaGetLastError();
  }
  // cold cycles rebuild the first sweep (t = omega dinv b) inside the next
  // two passes; warm ones smooth from x into t
  if (warm) {
    k_mg_smooth4<<<g, blk, 0, st>>>(L, x, b, t, H.omega, S, mask);
    note_launch();
  }
  const MgLevel& C = H.lv[l + 1];
  if (warm)
    k_mg_resrestrict4<false><<<grid4r(C, H.nrhs), blk, 0, st>>>(L, C, t, b, vec4(C.b), H.cscale, S, mask, H.omega);
  else
    k_mg_resrestrict4<true><<<grid4r(C, H.nrhs), blk, 0, st>>>(L, C, t, b, vec4(C.b), H.cscale, S, mask, H.omega);
  note_launch();
  for (int c = 0; c < coarse_cycles(H, l); c++) {
    cudaError_t e = vcycle(H, l + 1, S, mask, st, c > 0);
    if (e != cudaSuccess) return e;
  }
  if (warm)
    k_mg_prolong_smooth4<false><<<g, blk, 0, st>>>(L, C, t, vec4(C.x), b, x, H.omega, S, mask);
  else
    k_mg_prolong_smooth4<true><<<g, blk, 0, st>>>(L, C, t, vec4(C.x), b, x, H.omega, S, mask);
  note_launch();
  return cudaGetLastError();
}

namespace {

// Level-0 stencil passes, streamed through shared memory by TMA.  Level 0's
// dinv holds omega D^-1 (wd below).  Each pass loads two operand fields with
// their x-y halo and turns them into the stencil operand in shared memory
// when a plane lands:
//   kSpmv      p = z + beta p_old (the direction update); q = A p, p.q and
//              alpha = rz / pq; writes p and q, and adds the previous
//              iteration's alpha p_old to e (so e lags one step: the apply
//              pass adds the last alpha p)
//   kResidual  r = r_old - alpha q (the PCG residual update; not at a start),
//              written out; t = wd r (the first pre-smoothing sweep from
//              zero); b1 = cscale x P^T (r - A t), the residual restricted to
//              level 1 on the fly (an aggregate's two planes summed in
//              registers, its two rows through shared memory; chunks hold
//              whole aggregates)
//   kSmooth    y = wd r + P x1 (the pre-smoothed iterate plus the prolonged
//              level-1 correction, the level-1 tile of each plane's parents
//              streamed alongside); z = y + wd (r - A y), r.z and the PCG
//              scalar updates (start: rz = rz0, beta = 0 and p = 0; otherwise
//              beta and the stop test)
// r and p have two buffers each: kSpmv reads p from buffer (iters & 1) and
// writes buffer (iters & 1) ^ 1, kResidual does the same for r, and kSmooth
// (which counts the iteration) reads the new r, so no pass writes a field
// that another CTA of the same pass reads as a halo.
// A CTA owns kTX x kTY cells of a plane (a warp per row, four cells per
// thread) and marches through kc0 planes.  Thread 0 keeps a 4-deep ring of
// planes (both operand tiles, the open-face bits, the level-1 tile) in flight
// with cp.async.bulk.tensor, completion on mbarriers; every thread reads its
// seven neighbours from shared memory, so the DRAM stream never waits on a
// dependent load.  Each
// thread transforms its own four cells of a landed plane (keeping their raw
// values for the plane's own step) and threads 0 .. 83 the 84 float4 of the
// halo, one step ahead of the plane's use as the top neighbour.  (Transforming
// two steps ahead saves a barrier per plane but shortens the TMA prefetch
// distance; measured slower.)
//
// TMA boxes (x coordinates in elements of the MixedGrid row, cell i at 3 + i):
//   operands (kTX + 8) x (kTY + 2) floats from (kTX bx, kTY by): cells
//            kTX bx - 3 .. kTX bx + kTX + 4, so the tile's cells and both
//            x neighbours; the x start is a multiple of 4 (16 bytes)
//   bits     (kTX + 16) x (kTY + 2) bytes from the same corner (x a multiple
//            of 16 bytes; the bits' row pitch pxb is a multiple of 16)
//   q        (kResidual) the operand box of q
//   x1       kCW x kCH floats of level 1 (rows padded to 16 bytes) from
//            (kTX bx / 2 - 4, kTY by / 2 - 1, parent plane): the parents of
//            the operand tile's cells
// Rows and planes outside the grid (plane 0 and nz + 1) read as zero, where
// the open-face bits are zero as well; halo cells may pick up a level-1
// value, which only ever meets a zero face.
enum { kSpmv = 0, kResidual = 1, kSmooth = 2 };
constexpr int kTX = 128, kTY = 8, kTThreads = (kTX / 4) * kTY;
constexpr int kPW = kTX + 8, kPWB = kTX + 16, kPH = kTY + 2;
constexpr int kQ = kPW / 4, kHalo4 = 2 * kQ + 2 * kTY;  // float4 per tile row; halo float4 per plane
constexpr int kCW = kTX / 2 + 8, kCH = kTY / 2 + 2;     // level-1 tile: columns -4 .. kTX/2+3, rows -1 .. kTY/2
constexpr uint32_t kXBytes = kPW * kPH * 4, kBBytes = kPWB * kPH, kX1Bytes = kCW * kCH * 4;
constexpr uint32_t kXStage = (kXBytes + 127) / 128 * 128, kBStage = (kBBytes + 127) / 128 * 128,
                   kX1Stage = (kX1Bytes + 127) / 128 * 128;
constexpr int kXSt = 4;  // planes k-1 .. k+1 in use, k+2 in flight
static_assert(kTX % 16 == 0 && kTY % 2 == 0, "tile: bits box start and row pairs");
static_assert((kPW * 4) % 16 == 0 && kPWB % 16 == 0, "TMA box rows are whole 16-byte units");
static_assert((kCW * 4) % 16 == 0, "level-1 box rows are whole 16-byte units");
static_assert(kPW % 4 == 0 && 2 * (kQ - 1) + 3 < kCW, "prolongation: float4 rows, parents inside the tile");
static_assert(kHalo4 <= kTThreads, "one halo float4 per thread at most");

// One ring stage: operand A, operand B, bits, and the level-1 tile (kSmooth)
// or q (kResidual).
__host__ __device__ constexpr uint32_t tma_stage(int mode) {
  return 2 * kXStage + kBStage + (mode == kSmooth ? kX1Stage : mode == kResidual ? kXStage : 0u);
}
__host__ __device__ constexpr uint32_t tma_smem(int mode) { return kXSt * tma_stage(mode) + 8 * kXSt; }

template <int MODE>
__global__ void __launch_bounds__(kTThreads, 3)
    k_mg0_tma(const __grid_constant__ MgMaps M, MixedGrid G, int kc, MgLevel L, MgLevel C, Ops0 O, MgVecs v,
              float cscale, MgScalars* S, MgRed rb, unsigned mask, int start) {
  const int zc = (G.nz + kc - 1) / kc;
  const int m = (int)blockIdx.z / zc;
  MG_SKIP(m);
  if (*reinterpret_cast<volatile int*>(rb.err)) return;  // an earlier wait gave up: the solve is abandoned
  const int k0 = ((int)blockIdx.z - m * zc) * kc + 1;
  const int k1 = min(G.nz, k0 + kc - 1);
  constexpr uint32_t kStage = tma_stage(MODE);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kXSt * kStage);
  const uint32_t s_base = tma::smem_u32(smem), bar_base = tma::smem_u32(bars);
  const int tid = threadIdx.x, q = tid & 31, ty = tid >> 5;
  const int x0 = kTX * (int)blockIdx.x, y0 = kTY * (int)blockIdx.y;
  P0 t;
  t.g = x0 / 4 + q;
  t.j = y0 + ty + 1;
  t.live = t.g < G.ng && t.j <= G.ny;
  auto sel = [m](const CUtensorMap* a) { return m == 0 ? a : m == 1 ? a + 1 : m == 2 ? a + 2 : a + 3; };
  // buffers: par = current r / p (kSmooth reads the r that kResidual wrote)
  const int par = S[m].iters & 1;
  const int rpar = MODE == kSmooth && !start ? par ^ 1 : par;
  // operand A: z (kSpmv) or r; operand B: p (kSpmv) or wd; kResidual: q
  const CUtensorMap* ma = MODE == kSpmv ? sel(M.z) : (rpar ? sel(M.r2) : sel(M.r));
  const CUtensorMap* mb = MODE == kSpmv ? (par ? sel(M.p2) : sel(M.p)) : &M.dinv;
  const CUtensorMap* m1 = MODE == kSmooth ? sel(M.x1) : sel(M.q);
  const bool with_q = MODE == kResidual && !start;
  const float beta = MODE == kSpmv ? (float)S[m].beta : 0.f;
  // kSpmv: the previous alpha (for e += alpha p_old); kResidual: this one
  const float alpha = MODE == kSmooth ? 0.f : (float)S[m].alpha;
  if (tid == 0) {
    for (int s = 0; s < kXSt; s++) tma::mbar_init(bar_base + 8 * s, 1);
    tma::mbar_init_fence();
  }
  __syncthreads();
  // Plane p (p = k0 - 1 .. k1 + 1) goes to ring slot (p - (k0 - 1)) % kXSt;
  // the n-th use of a slot completes its barrier's phase n.
  auto issue = [&](int p) {
    const int s = (p - (k0 - 1)) % kXSt;
    const uint32_t bar = bar_base + 8 * s, dst = s_base + s * kStage;
    tma::mbar_expect_tx(bar, 2 * kXBytes + kBBytes + (MODE == kSmooth ? kX1Bytes : with_q ? kXBytes : 0u));
    tma::load_3d(dst, ma, x0, y0, p - 1, bar);
    tma::load_3d(dst + kXStage, mb, x0, y0, p - 1, bar);
    tma::load_3d(dst + 2 * kXStage, &M.fb, x0, y0, p - 1, bar);
    if (MODE == kSmooth) tma::load_3d(dst + 2 * kXStage + kBStage, m1, x0 / 2 - 4, y0 / 2 - 1, (p - 1) >> 1, bar);
    if (with_q) tma::load_3d(dst + 2 * kXStage + kBStage, m1, x0, y0, p - 1, bar);
  };
  auto ready = [&](int p) {
    const int u = p - (k0 - 1);
    return tma::mbar_wait(bar_base + 8 * (u % kXSt), (uint32_t)((u / kXSt) & 1));
  };
  // The stencil operand of plane p: kResidual keeps it in B's place, the
  // others in A's.
  auto operand = [&](int p) {
    return reinterpret_cast<float*>(smem + ((p - (k0 - 1)) % kXSt) * kStage + (MODE == kResidual ? kXStage : 0));
  };
  const int oc = (ty + 1) * kPW + 4 + 4 * q;  // this thread's four cells in a tile plane
  // Turn plane p into the stencil operand; own_a / own_b: the raw A and B
  // values of this thread's cells.
  auto transform = [&](int p, float4& own_a, float4& own_b) {
    unsigned char* st = smem + ((p - (k0 - 1)) % kXSt) * kStage;
    float* A = reinterpret_cast<float*>(st);
    float* B = reinterpret_cast<float*>(st + kXStage);
    const float* X1 = reinterpret_cast<const float*>(st + 2 * kXStage + kBStage);  // kSmooth: level 1; kResidual: q
    auto one = [&](int e, int r, int a4, float4& ra, float4& rb4) {  // float4 e = (row r, column 4 a4)
      ra = *reinterpret_cast<const float4*>(A + e);
      rb4 = *reinterpret_cast<const float4*>(B + e);
      if (MODE == kResidual && with_q) {  // r = r_old - alpha q, kept as this cell's raw value
        const float4 qq = *reinterpret_cast<const float4*>(X1 + e);
        ra = make_float4(fmaf(-alpha, qq.x, ra.x), fmaf(-alpha, qq.y, ra.y), fmaf(-alpha, qq.z, ra.z),
                         fmaf(-alpha, qq.w, ra.w));
      }
      const float2 a0 = lo2(ra), a1 = hi2(ra), b0 = lo2(rb4), b1 = hi2(rb4);
      float2 r0, r1;
      if (MODE == kSpmv) {  // p = z + beta p_old
        r0 = __ffma2_rn(dup2(beta), b0, a0);
        r1 = __ffma2_rn(dup2(beta), b1, a1);
      } else if (MODE == kResidual) {  // t = wd r
        r0 = __fmul2_rn(b0, a0);
        r1 = __fmul2_rn(b1, a1);
      } else {  // y = wd r + parent (columns 4a4, 4a4+1 -> 2a4+2; 4a4+2, 4a4+3 -> 2a4+3)
        const float2 c = *reinterpret_cast<const float2*>(X1 + (((r - 1) >> 1) + 1) * kCW + 2 * a4 + 2);
        r0 = __ffma2_rn(b0, a0, dup2(c.x));
        r1 = __ffma2_rn(b1, a1, dup2(c.y));
      }
      *reinterpret_cast<float4*>((MODE == kResidual ? B : A) + e) = make_float4(r0.x, r0.y, r1.x, r1.y);
    };
    one(oc, ty + 1, q + 1, own_a, own_b);
    if (tid < kHalo4) {
      int r, a4;
      if (tid < kQ) {
        r = 0;
        a4 = tid;
      } else if (tid < 2 * kQ) {
        r = kPH - 1;
        a4 = tid - kQ;
      } else {
        r = 1 + ((tid - 2 * kQ) >> 1);
        a4 = ((tid - 2 * kQ) & 1) ? kQ - 1 : 0;
      }
      float4 da, db;
      one(r * kPW + 4 * a4, r, a4, da, db);
    }
  };
  int next = k0 - 1;
  if (tid == 0)
    for (; next <= k0 + kXSt - 2 && next <= k1 + 1; next++) issue(next);

  float* __restrict__ out = MODE == kSpmv ? v.q[m] : (MODE == kResidual ? C.b[m] : v.z[m]);
  // kSpmv: the new p; kResidual: the new r; kSmooth (start): p = 0
  float* __restrict__ out2 = MODE == kSpmv ? (par ? v.p[m] : v.p2[m])
                                           : MODE == kResidual ? (par ? v.r[m] : v.r2[m]) : (par ? v.p2[m] : v.p[m]);
  // kResidual: the odd rows' aggregate sums, double-buffered by aggregate
  // plane (with an odd nz the last two planes complete aggregates in
  // consecutive steps)
  __shared__ float2 pair_sum[2][kTY / 2][32];
  float2 agg = make_float2(0.f, 0.f);  // kResidual: this row's sums of the group's two aggregates
  const int i0 = 4 * t.g;              // first cell of the group (0-based)
  const int cb = (ty + 1) * kPWB + 4 + 4 * q;
  const Row0 R = row0(O, t);
  Acc2 acc;
  float2 ttb[2];  // bottom faces of the current plane: the previous plane's top faces
  // raw A / B values of this thread's cells: plane k (cur), k + 1 (nxt)
  float4 cur_a = zero4(), cur_b = zero4(), nxt_a = zero4(), nxt_b = zero4();
  bool ok = ready(k0 - 1) && ready(k0);
  if (ok) {
    transform(k0 - 1, nxt_a, nxt_b);
    transform(k0, cur_a, cur_b);
  }
  {
    const uint8_t* Bb = smem + 2 * kXStage;  // bits of plane k0 - 1 (slot 0)
    bottom2(R, k0 > 1 ? __ldg(O.azt + k0 - 2) : 0.f, ok ? *reinterpret_cast<const uint32_t*>(Bb + cb) : 0u, ttb);
  }
  int kfail = k0;
  bool failed = false;
  // kSpmv: e of this thread's cells, loaded one plane ahead
  const long long base0 = 4LL * (t.g + 1) + (long long)G.px * (t.j + (long long)(G.ny + 2) * (k0 - 1));
  float4 e_nxt = zero4();
  if (MODE == kSpmv && t.live) e_nxt = ld4(v.e[m] + base0);
  for (int k = k0; k <= k1; k++) {
    float4 e_cur = e_nxt;
    if (MODE == kSpmv && t.live && k < k1) e_nxt = ld4(v.e[m] + base0 + (long long)G.plane * (k + 1 - k0));
    ok = ok && ready(k + 1);
    if (ok) transform(k + 1, nxt_a, nxt_b);
    __syncthreads();
    const bool pair_done = MODE == kResidual && (((k - 1) & 1) || k == G.nz);
    if (ok && t.live) {
      const float* X0 = operand(k - 1);
      const float* X1p = operand(k);
      const float* X2 = operand(k + 1);
      const float4 pc = *reinterpret_cast<const float4*>(X1p + oc);
      // (x neighbours from the adjacent lanes by shuffles measured slower)
      const float left = X1p[oc - 1], right = X1p[oc + 4];
      const uint8_t* B1 = smem + ((k - (k0 - 1)) % kXSt) * kStage + 2 * kXStage;
      const float4 pb = *reinterpret_cast<const float4*>(X0 + oc);
      const float4 pt = *reinterpret_cast<const float4*>(X2 + oc);
      const float4 ps = *reinterpret_cast<const float4*>(X1p + oc - kPW);
      const float4 pn = *reinterpret_cast<const float4*>(X1p + oc + kPW);
      const uint32_t f4 = *reinterpret_cast<const uint32_t*>(B1 + cb);
      const uint32_t fs4 = *reinterpret_cast<const uint32_t*>(B1 + cb - kPWB);
      const Faces2 Fc = faces2(R, __ldg(O.dz + k - 1), __ldg(O.azt + k - 1), f4, fs4, B1[cb - 1]);
      const float4 uu = face_apply2(pc, left, right, ps, pn, pb, pt, Fc, ttb);
      ttb[0] = Fc.tt[0];
      ttb[1] = Fc.tt[1];
      const long long base = 4LL * (t.g + 1) + (long long)G.px * (t.j + (long long)(G.ny + 2) * (k - 1));
      if (MODE == kSpmv) {
        st4(out + base, uu);
        acc.add4(pc, uu);
        st4(out2 + base, pc);  // the new direction (pc is this thread's p = z + beta p_old)
        const float4 &ee = e_cur, &po = cur_b;
        st4(v.e[m] + base, make_float4(fmaf(alpha, po.x, ee.x), fmaf(alpha, po.y, ee.y), fmaf(alpha, po.z, ee.z),
                                       fmaf(alpha, po.w, ee.w)));
      } else if (MODE == kResidual) {
        const float4& rr = cur_a;
        agg.x += (rr.x - uu.x) + (rr.y - uu.y);
        agg.y += (rr.z - uu.z) + (rr.w - uu.w);
        if (with_q) st4(out2 + base, rr);
      } else {
        const float4 &rr = cur_a, &wd = cur_b;
        float zz[4];
#pragma unroll
        for (int n = 0; n < 4; n++)
          zz[n] = i0 + n < L.nx ? fmaf(el(wd, n), el(rr, n) - el(uu, n), el(pc, n)) : 0.f;
        const float4 z4 = make_float4(zz[0], zz[1], zz[2], zz[3]);
        st4(out + base, z4);
        if (start) st4(out2 + base, zero4());  // the first direction is z itself
        acc.add4(rr, z4);
      }
    }
    // rows 2c and 2c+1 (0-based) of an aggregate are warps ty = 2h and 2h+1
    if (pair_done && (ty & 1)) pair_sum[((k - 1) >> 1) & 1][ty >> 1][q] = agg;
    if (__syncthreads_or(!ok)) {  // also: every thread is done with plane k - 1's slot
      failed = true;
      kfail = k;
      break;
    }
    if (pair_done) {
      if (!(ty & 1) && t.live) {
        const float2 o = pair_sum[((k - 1) >> 1) & 1][ty >> 1][q];
        const int ci = 2 * t.g, cj = (t.j - 1) >> 1, ck = (k - 1) >> 1;
        float* bc = out + ix(C, ci, cj, ck);
        bc[0] = cscale * (agg.x + o.x);
        if (ci + 1 < C.nx) bc[1] = cscale * (agg.y + o.y);
      }
      agg = make_float2(0.f, 0.f);
    }
    cur_a = nxt_a;
    cur_b = nxt_b;
    if (tid == 0 && next <= k1 + 1) issue(next++);
  }
  if (failed && tid == 0) {
    atomicExch(rb.err, 1);
    for (int p = kfail - 1; p < next; p++) ready(p);  // drain the copies still in flight (bounded)
  }
  if (MODE == kResidual) return;
  // every block of the right-hand side takes part, also after a failure
  double out_sum = 0.0;
  if (!rhs_reduce((double)acc.s + (double)acc.e, m, zc, rb, &out_sum) || tid != 0) return;
  MgScalars& Q = S[m];
  if (MODE == kSpmv) {
    Q.pq = out_sum;
    if (!(out_sum > 0) || !(Q.rz > 0)) {
      Q.active = 0;
      Q.alpha = 0;
    } else {
      Q.alpha = Q.rz / out_sum;
    }
    return;
  }
  const double rz = out_sum;
  if (start) {
    Q.rz = rz;
    Q.rz0 = rz;
    Q.beta = 0.0;
    Q.active = rz > 0 ? 1 : 0;
    return;
  }
  Q.iters += 1;
  if (!(rz >= 0)) {
    Q.active = 0;
    return;
  }
  Q.beta = rz / Q.rz;
  Q.rz = rz;
  if (rz <= Q.tol2 * Q.rz0) Q.active = 0;
}

struct Scale4 {
  double s[kMaxRhs];
};

// r = scale * rV (compact FP64 projected residual) on fluid cells, e = 0
__global__ void k_mgp_load(MgLevel L, DPtr4 rv, Scale4 sc, unsigned mask, MgVecs v) {
  MG_RHS(L);
  if (!((mask >> mrhs) & 1u)) return;
  const double* __restrict__ rm = pick(rv.p, mrhs);
  const double scale = pick(sc.s, mrhs);
  float* __restrict__ r = pick(v.r, mrhs);
  float* __restrict__ e = pick(v.e, mrhs);
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    const long long cc = i + (long long)L.nx * (j + (long long)L.ny * k);
    r[c] = L.dinv[c] > 0.f ? (float)(rm[cc] * scale) : 0.f;
    e[c] = 0.f;
  }
}

// phi(padded) += (e + alpha p) / scale on fluid cells: the correction with
// the last iteration's alpha p, which the spmv pass adds to e only in the
// iteration after (alpha is zero after a breakdown)
__global__ void k_mgp_apply(MgLevel L, Dims d, MgVecs v, const MgScalars* S, Scale4 sc, unsigned mask,
                            DPtr4 phiv) {
  MG_RHS(L);
  if (!((mask >> mrhs) & 1u)) return;
  const float* __restrict__ e = pick(v.e, mrhs);
  const float a = (float)S[mrhs].alpha;
  const float* __restrict__ p = (S[mrhs].iters & 1) ? pick(v.p2, mrhs) : pick(v.p, mrhs);
  const double scale = pick(sc.s, mrhs);
  double* __restrict__ phi = pick(phiv.p, mrhs);
  MG_CELLS(L) {
    const long long c = ix(L, i, j, k);
    if (L.dinv[c] > 0.f) {
      const float ec = a != 0.f ? fmaf(a, p[c], e[c]) : e[c];
      phi[d.ph(i + 1, j + 1, k + 1)] += (double)ec / scale;
    }
  }
}

Ops0 ops0(const MgHierarchy& H) {
  Ops0 O;
  O.aex = H.aex;
  O.dxr = H.dxr;
  O.dy = H.dy;
  O.ayn = H.ayn;
  O.dz = H.dz;
  O.azt = H.azt;
  return O;
}

dim3 tma_grid(const MgHierarchy& H) {
  return dim3((unsigned)((H.g0.ng + kTX / 4 - 1) / (kTX / 4)), (unsigned)((H.g0.ny + kTY - 1) / kTY),
              (unsigned)(((H.g0.nz + H.kc0 - 1) / H.kc0) * H.nrhs));
}

Scale4 scale4(const double* s, unsigned mask) {
  Scale4 r;
  for (int m = 0; m < kMaxRhs; m++) r.s[m] = ((mask >> m) & 1u) ? s[m] : 1.0;
  return r;
}

}  // namespace

// CTAs of one z-chunk of the level-0 TMA passes (all right-hand sides).
long long mg_tma_ctas_per_chunk(const MixedGrid& G, int nrhs) {
  return (long long)((G.ng + kTX / 4 - 1) / (kTX / 4)) * ((G.ny + kTY - 1) / kTY) * nrhs;
}

// Level-0 V-cycle tail shared by start and iteration: the residual of the
// first smoothing sweep restricted to level 1, the coarse cycle, and the
// post-smoothing + r.z pass.
static cudaError_t level0_tail(const MgHierarchy& H, MgVecs& v, MgScalars* S, const MgRed& rb, unsigned mask,
                               int start, cudaStream_t st) {
  const MgLevel& L = H.lv[0];
  const MgLevel& C = H.lv[1];
  const dim3 gt = tma_grid(H);
  k_mg0_tma<kResidual><<<gt, kTThreads, tma_smem(kResidual), st>>>(H.maps, H.g0, H.kc0, L, C, ops0(H), v, H.cscale,
                                                                   S, rb, mask, start);
  note_launch();
  for (int cy = 0; cy < coarse_cycles(H, 0); cy++) {
    cudaError_t e = vcycle(H, 1, S, mask, st, cy > 0);
    if (e != cudaSuccess) return e;
  }
  k_mg0_tma<kSmooth><<<gt, kTThreads, tma_smem(kSmooth), st>>>(H.maps, H.g0, H.kc0, L, C, ops0(H), v, H.cscale, S,
                                                                 rb, mask, start);
  note_launch();
  return cudaGetLastError();
}

cudaError_t mg_pcg_start(const MgHierarchy& H, const DPtr4& rv, const double* scale, unsigned mask, MgVecs& v,
                         MgScalars* S, const MgRed& rb, cudaStream_t st) {
  const MgLevel& L = H.lv[0];
  k_mgp_load<<<rhs_grid(L, H.nrhs), dim3(32, 8), 0, st>>>(L, rv, scale4(scale, mask), mask, v);
  note_launch();
  return level0_tail(H, v, S, rb, mask, 1, st);
}

// One PCG iteration: direction + q = A p, the PCG update, the V-cycle.
cudaError_t mg_pcg_iteration(const MgHierarchy& H, MgVecs& v, MgScalars* S, const MgRed& rb, cudaStream_t st) {
  const MgLevel& L = H.lv[0];
  const unsigned all = (1u << H.nrhs) - 1u;
  k_mg0_tma<kSpmv><<<tma_grid(H), kTThreads, tma_smem(kSpmv), st>>>(H.maps, H.g0, H.kc0, L, H.lv[1], ops0(H), v,
                                                                     H.cscale, S, rb, all, 0);
  note_launch();
  return level0_tail(H, v, S, rb, all, 0, st);
}

cudaError_t mg_pcg_apply(const MgHierarchy& H, const Dims& d, const MgVecs& v, const MgScalars* S,
                         const double* scale, unsigned mask, const DPtr4& phi, cudaStream_t st) {
  const MgLevel& L = H.lv[0];
  k_mgp_apply<<<rhs_grid(L, H.nrhs), dim3(32, 8), 0, st>>>(L, d, v, S, scale4(scale, mask), mask, phi);
  note_launch();
  return cudaGetLastError();
}

long long mg_red_partials(const MgHierarchy& H) {
  const dim3 g = tma_grid(H);  // z covers all right-hand sides: blocks per right-hand side x kMaxRhs
  return (long long)kMaxRhs * g.x * g.y * (g.z / H.nrhs);
}

cudaError_t mg_encode(MgHierarchy& H, const MgVecs& v) {
  const MixedGrid& G = H.g0;
  const uint64_t rows = (uint64_t)G.ny + 2, pitch = 4ULL * G.px;
  auto f32 = [&](CUtensorMap* map, float* base, uint32_t b0, uint32_t b1) {
    return tma_encode_3d(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, base, G.px, rows, G.nz, pitch, pitch * rows, b0, b1);
  };
  bool ok = true;
  for (int m = 0; m < H.nrhs; m++) {
    ok = ok && f32(&H.maps.z[m], v.z[m], kPW, kPH) && f32(&H.maps.p[m], v.p[m], kPW, kPH) &&
         f32(&H.maps.r[m], v.r[m], kPW, kPH) && f32(&H.maps.q[m], v.q[m], kPW, kPH) &&
         f32(&H.maps.p2[m], v.p2[m], kPW, kPH) && f32(&H.maps.r2[m], v.r2[m], kPW, kPH);
  }
  const MgLevel& L1 = H.lv[1];
  for (int m = 0; m < H.nrhs; m++)
    ok = ok && tma_encode_3d(&H.maps.x1[m], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, L1.x[m], (uint64_t)L1.sy,
                             (uint64_t)L1.ny, (uint64_t)L1.nz, 4ULL * L1.sy, 4ULL * L1.sz, kCW, kCH);
  ok = ok && f32(&H.maps.dinv, H.lv[0].dinv, kPW, kPH) &&
       tma_encode_3d(&H.maps.fb, CU_TENSOR_MAP_DATA_TYPE_UINT8, H.fb0, (uint64_t)H.pxb, rows, G.nz, (uint64_t)H.pxb,
                     (uint64_t)H.pxb * rows, kPWB, kPH);
  if (!ok) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_mg0_tma<kResidual>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)tma_smem(kResidual));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mg0_tma<kSmooth>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tma_smem(kSmooth));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mg0_tma<kSpmv>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tma_smem(kSpmv));
  return e;
}

}  // namespace fpm
