// Batched 2-D multigrid for the uneven frames of fpm_partition_frames_2d:
// the preconditioner of the frames' FP32 PCG inside the FP64 refinement,
// for every frame and both directions in the same launches.
//
// A frame is the reference's 2-D usage of the 3-D solver (nz = 2, dz = 0.5,
// zero z data; examples/flapping_foil_fpm.f90:61-81).  Its right-hand side is
// the same in both layers and both layers carry the same solid flags, so the
// solution is the same in both layers (the z coupling cancels): the FP32
// inner solve runs on one layer with the per-layer operator
//   (A x)_c = sum over the four x-y faces f of T_f (x_c - x_nb(f)),
//   T_east(i, j) = dz dy_j / (xc_{i+1} - xc_i), T_north likewise,
// zero towards solid cells and on the outer boundary (src/fpm_stairstep_mpi_3d.f90:336-379
// with V = dx dy dz folded in), and the correction is added to both layers.
//
// Levels: level l+1 aggregates 2 x 2 cells of level l (Galerkin product with
// piecewise-constant prolongation: a coarse face is the sum of the fine faces
// between two aggregates), down to at most 32 x 32 cells per frame (at least
// one coarsening), where one CTA per frame runs weighted-Jacobi sweeps out
// of shared memory.  The cycle is a symmetric V-cycle (one weighted-Jacobi
// sweep before and after each coarse correction, the pre-smoothing from zero
// folded into the residual), so it is a valid PCG preconditioner.
//
// Every kernel walks a tile list (32 x 8 cells of one frame at one level);
// frames that have finished (per frame and direction flags) return at once,
// and the per-frame reductions are segmented (last tile of a frame combines
// the frame's partials in tile order), so results do not depend on timing.
#include "fpm_internal.h"

namespace fpm {

namespace {

constexpr int kR = 2;  // directions per frame

__device__ __forceinline__ bool on(const Batch2& b, int f, int r, int mode) {
  const int q = f * kR + r;
  return mode ? b.in_set[q] != 0 : b.active[q] != 0;
}

// f32 sum with its rounding error (TwoSum), for the dot products
struct Sum2 {
  float s = 0.f, e = 0.f;
  __device__ __forceinline__ void add_prod(float a, float c) {
    const float p = a * c;
    const float pe = fmaf(a, c, -p);
    const float t = s + p;
    const float bb = t - s;
    e += ((s - (t - bb)) + (p - bb)) + pe;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)e; }
};

// Segmented sum of kR values over the level-0 tiles of frame f (tile ids
// tile0 .. tile0 + ntiles - 1); true in the last tile of the frame to finish,
// with out[] = the frame's sums combined in tile order.
__device__ bool fm_seg_sum(double (&s)[kR], int f, int tile, int tile0, int ntiles, double* partials,
                           unsigned int* tickets, double (&out)[kR]) {
  __shared__ bool am_last;
  double m[1] = {0.0};
  block_reduce<kR, 0>(s, m);
  const int tid = lin_tid();
  if (tid == 0) {
    for (int n = 0; n < kR; n++) partials[(size_t)tile * kR + n] = s[n];
    __threadfence();
    const unsigned int t = atomicAdd(&tickets[f], 1u);
    am_last = (t == (unsigned int)ntiles - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double as[kR] = {0.0, 0.0}, am[1] = {0.0};
  for (int bl = tid; bl < ntiles; bl += lin_nthreads())
    for (int n = 0; n < kR; n++) as[n] += __ldcg(partials + (size_t)(tile0 + bl) * kR + n);
  block_reduce<kR, 0>(as, am);
  if (tid == 0) {
    for (int n = 0; n < kR; n++) out[n] = as[n];
    tickets[f] = 0u;
    __threadfence();
  }
  __syncthreads();
  return true;
}

// Level-0 tile of this block: frame, 0-based cell, live flag.
struct T0 {
  int tile, f, i, j;
  bool live;
};
__device__ __forceinline__ T0 t0_ref(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame,
                                     const int* __restrict__ tiles) {
  T0 t;
  t.tile = tiles ? tiles[blockIdx.x] : (int)blockIdx.x;
  t.f = tile_frame[t.tile];
  const Frame2& F = fr[t.f];
  const int idx = t.tile - F.tile0;
  t.i = (idx % F.tiles_x) * 32 + threadIdx.x;
  t.j = (idx / F.tiles_x) * 8 + threadIdx.y;
  t.live = t.i < F.nx && t.j < F.ny;
  return t;
}

// Coarse-level tile of this block.
struct TL {
  int f, i, j;
  FmLevel L;
  bool live;
};
__device__ __forceinline__ TL tl_ref(const FramesMg& M, int l) {
  const FmTile tt = M.tiles[l][blockIdx.x];
  TL t;
  t.f = tt.f;
  t.L = M.lv[(size_t)tt.f * kFmMaxLevels + l];
  t.i = tt.i0 + threadIdx.x;
  t.j = tt.j0 + threadIdx.y;
  t.live = t.i < t.L.nx && t.j < t.L.ny;
  return t;
}

// A x at (i, j) of a level for operand values xc (this cell) and its four
// neighbours (zero faces make out-of-grid neighbours irrelevant).
__device__ __forceinline__ float apply4(float xc, float xw, float xe, float xs, float xn, float tw, float te, float ts,
                                        float tn) {
  float a = te * (xc - xe);
  a = fmaf(tw, xc - xw, a);
  a = fmaf(tn, xc - xn, a);
  a = fmaf(ts, xc - xs, a);
  return a;
}

}  // namespace

// ---------------------------------------------------------------- set-up
// Level-0 faces of every frame from its axes and solid flags (one layer,
// dz = 0.5 folded in).
__global__ void k_fm_faces0(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b, FramesMg M) {
  const T0 t = t0_ref(fr, tile_frame, nullptr);
  if (!t.live) return;
  const Frame2& F = fr[t.f];
  const int i = t.i, j = t.j;
  const long long c = F.o2 + i + (long long)F.nx * j;
  const uint8_t* s2 = b.solid2 + F.o2;
  const bool fl = s2[i + (long long)F.nx * j] == 0;
  double te = 0.0, tn = 0.0;
  if (fl && i + 1 < F.nx && s2[i + 1 + (long long)F.nx * j] == 0)
    te = 0.5 * b.dy[F.oy + j] / (b.xc[F.ox + i + 2] - b.xc[F.ox + i + 1]);
  if (fl && j + 1 < F.ny && s2[i + (long long)F.nx * (j + 1)] == 0)
    tn = 0.5 * b.dx[F.ox + i] / (b.yc[F.oy + j + 2] - b.yc[F.oy + j + 1]);
  M.te[0][c] = (float)te;
  M.tn[0][c] = (float)tn;
}

// Coarse faces of level l+1 from level l.
__global__ void k_fm_coarsen(FramesMg M, int l) {
  const TL t = tl_ref(M, l + 1);
  if (!t.live) return;
  const FmLevel Fl = M.lv[(size_t)t.f * kFmMaxLevels + l];
  const int fi = 2 * t.i, fj = 2 * t.j;
  const float* te = M.te[l] + Fl.off;
  const float* tn = M.tn[l] + Fl.off;
  float e = 0.f, n = 0.f;
  if (fi + 1 < Fl.nx) {
    e = te[fi + 1 + (long long)Fl.nx * fj];
    if (fj + 1 < Fl.ny) e += te[fi + 1 + (long long)Fl.nx * (fj + 1)];
  }
  if (fj + 1 < Fl.ny) {
    n = tn[fi + (long long)Fl.nx * (fj + 1)];
    if (fi + 1 < Fl.nx) n += tn[fi + 1 + (long long)Fl.nx * (fj + 1)];
  }
  const long long c = t.L.off + t.i + (long long)t.L.nx * t.j;
  M.te[l + 1][c] = t.i + 1 < t.L.nx ? e : 0.f;
  M.tn[l + 1][c] = t.j + 1 < t.L.ny ? n : 0.f;
}

// dinv = omega / (sum of the four faces) on level l (0 for cells without a
// fluid face).  Level 0 walks the frames' tile list, other levels theirs.
__global__ void k_fm_dinv(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, FramesMg M, int l) {
  FmLevel L;
  int i, j;
  if (l == 0) {
    const T0 t = t0_ref(fr, tile_frame, nullptr);
    if (!t.live) return;
    const Frame2& F = fr[t.f];
    L = FmLevel{F.nx, F.ny, F.o2};
    i = t.i;
    j = t.j;
  } else {
    const TL t = tl_ref(M, l);
    if (!t.live) return;
    L = t.L;
    i = t.i;
    j = t.j;
  }
  const long long c = L.off + i + (long long)L.nx * j;
  const float* te = M.te[l];
  const float* tn = M.tn[l];
  float d = te[c] + tn[c];
  if (i > 0) d += te[c - 1];
  if (j > 0) d += tn[c - L.nx];
  M.dinv[l][c] = d > 0.f ? M.omega / d : 0.f;
}

// ---------------------------------------------------------------- the V-cycle
// Residual of the first smoothing sweep from zero, restricted: on level l,
// t = dinv b (stored as xa on levels >= 1), res = b - A t, and
// b_{l+1} = sum of res over each 2 x 2 aggregate.  Level 0's b is r.
__global__ void __launch_bounds__(256) k_fm_restrict(const Frame2* __restrict__ fr,
                                                     const int* __restrict__ tile_frame, Batch2 b, FramesMg M, int l,
                                                     int mode) {
  __shared__ float res_s[kR][8][33];
  int f, i, j;
  FmLevel L;
  bool live;
  if (l == 0) {
    const T0 t = t0_ref(fr, tile_frame, b.tiles);
    const Frame2& F = fr[t.f];
    f = t.f;
    i = t.i;
    j = t.j;
    live = t.live;
    L = FmLevel{F.nx, F.ny, F.o2};
  } else {
    const TL t = tl_ref(M, l);
    f = t.f;
    i = t.i;
    j = t.j;
    live = t.live;
    L = t.L;
  }
  bool act[kR];
  for (int r = 0; r < kR; r++) act[r] = on(b, f, r, mode);
  if (!act[0] && !act[1]) return;
  const float* te = M.te[l] + L.off;
  const float* tn = M.tn[l] + L.off;
  const float* dv = M.dinv[l] + L.off;
  const long long c = i + (long long)L.nx * j;
  for (int r = 0; r < kR; r++) {
    float res = 0.f;
    if (live && act[r]) {
      const float* bb = (l == 0 ? M.r[r] : M.b[l][r]) + L.off;
      const float tc = dv[c] * bb[c];
      const float tw = i > 0 ? dv[c - 1] * bb[c - 1] : 0.f;
      const float tE = i + 1 < L.nx ? dv[c + 1] * bb[c + 1] : 0.f;
      const float ts = j > 0 ? dv[c - L.nx] * bb[c - L.nx] : 0.f;
      const float tN = j + 1 < L.ny ? dv[c + L.nx] * bb[c + L.nx] : 0.f;
      const float a = apply4(tc, tw, tE, ts, tN, i > 0 ? te[c - 1] : 0.f, te[c], j > 0 ? tn[c - L.nx] : 0.f, tn[c]);
      res = bb[c] - a;
      if (l > 0) M.xa[l][r][L.off + c] = tc;
    }
    res_s[r][threadIdx.y][threadIdx.x] = res;
  }
  __syncthreads();
  if ((threadIdx.x & 1) || (threadIdx.y & 1) || !live) return;
  const FmLevel C = M.lv[(size_t)f * kFmMaxLevels + l + 1];
  const int ci = i >> 1, cj = j >> 1;
  const int x = threadIdx.x, y = threadIdx.y;
  for (int r = 0; r < kR; r++) {
    if (!act[r]) continue;
    const float s = (res_s[r][y][x] + res_s[r][y][x + 1]) + (res_s[r][y + 1][x] + res_s[r][y + 1][x + 1]);
    M.b[l + 1][r][C.off + ci + (long long)C.nx * cj] = s;
  }
}

// Coarsest level of every frame (at most kFmMaxCoarse cells): nsweeps
// weighted-Jacobi sweeps from zero out of shared memory, one CTA per frame;
// the result goes to xb (the input of the next finer prolongation).
__global__ void __launch_bounds__(kFmMaxCoarse) k_fm_coarse(Batch2 b, FramesMg M, int nsweeps, int mode) {
  __shared__ float x_s[2][kFmMaxCoarse];
  __shared__ float te_s[kFmMaxCoarse], tn_s[kFmMaxCoarse], dv_s[kFmMaxCoarse], b_s[kFmMaxCoarse];
  const int f = blockIdx.x;
  const int lc = M.nlevels[f] - 1;
  const FmLevel L = M.lv[(size_t)f * kFmMaxLevels + lc];
  const int n = L.nx * L.ny, c = threadIdx.x;
  if (c < n) {
    te_s[c] = M.te[lc][L.off + c];
    tn_s[c] = M.tn[lc][L.off + c];
    dv_s[c] = M.dinv[lc][L.off + c];
  }
  const int i = c % L.nx, j = c / L.nx;
  for (int r = 0; r < kR; r++) {
    if (!on(b, f, r, mode)) continue;  // uniform over the block
    __syncthreads();
    if (c < n) {
      b_s[c] = M.b[lc][r][L.off + c];
      x_s[0][c] = 0.f;
    }
    __syncthreads();
    int cur = 0;
    for (int s = 0; s < nsweeps; s++) {
      if (c < n) {
        const float* x = x_s[cur];
        const float xc = x[c];
        const float a = apply4(xc, i > 0 ? x[c - 1] : 0.f, i + 1 < L.nx ? x[c + 1] : 0.f, j > 0 ? x[c - L.nx] : 0.f,
                               j + 1 < L.ny ? x[c + L.nx] : 0.f, i > 0 ? te_s[c - 1] : 0.f, te_s[c],
                               j > 0 ? tn_s[c - L.nx] : 0.f, tn_s[c]);
        x_s[cur ^ 1][c] = fmaf(dv_s[c], b_s[c] - a, xc);
      }
      cur ^= 1;
      __syncthreads();
    }
    if (c < n) M.xb[lc][r][L.off + c] = x_s[cur][c];
  }
}

// Prolongation and post-smoothing on level l >= 1: y = xa + cscale P xb_{l+1},
// xb = y + dinv (b - A y) (y at the neighbours rebuilt the same way).
__global__ void __launch_bounds__(256) k_fm_prolong(Batch2 b, FramesMg M, int l, int mode) {
  const TL t = tl_ref(M, l);
  bool act[kR];
  for (int r = 0; r < kR; r++) act[r] = on(b, t.f, r, mode);
  if ((!act[0] && !act[1]) || !t.live) return;
  const FmLevel& L = t.L;
  const FmLevel C = M.lv[(size_t)t.f * kFmMaxLevels + l + 1];
  const int i = t.i, j = t.j;
  const long long c = i + (long long)L.nx * j;
  const float* te = M.te[l] + L.off;
  const float* tn = M.tn[l] + L.off;
  const float* dv = M.dinv[l] + L.off;
  for (int r = 0; r < kR; r++) {
    if (!act[r]) continue;
    const float* xa = M.xa[l][r] + L.off;
    const float* xc1 = M.xb[l + 1][r] + C.off;
    const float cs = M.cscale;
    auto y = [&](int ii, int jj) {
      return fmaf(cs, xc1[(ii >> 1) + (long long)C.nx * (jj >> 1)], xa[ii + (long long)L.nx * jj]);
    };
    const float yc = y(i, j);
    const float a = apply4(yc, i > 0 ? y(i - 1, j) : 0.f, i + 1 < L.nx ? y(i + 1, j) : 0.f, j > 0 ? y(i, j - 1) : 0.f,
                           j + 1 < L.ny ? y(i, j + 1) : 0.f, i > 0 ? te[c - 1] : 0.f, te[c], j > 0 ? tn[c - L.nx] : 0.f,
                           tn[c]);
    M.xb[l][r][L.off + c] = fmaf(dv[c], M.b[l][r][L.off + c] - a, yc);
  }
}

// Level 0: y = dinv r + P xb_1, z = y + dinv (r - A y); r.z per frame and
// direction.  Start mode (the pairs in the set): rz0 = rz, beta = 0, the
// pair is active if rz > 0.  Iteration mode (the active pairs): the PCG
// scalar update of the reference's pcg_iterate with this preconditioner --
// beta = rz_new / rz, the direction update enabled, and the pair stops when
// rz has dropped by the inner tolerance.
__global__ void __launch_bounds__(256) k_fm_final0(const Frame2* __restrict__ fr,
                                                   const int* __restrict__ tile_frame, Batch2 b, FramesMg M,
                                                   int mode) {
  const T0 t = t0_ref(fr, tile_frame, b.tiles);
  const Frame2& F = fr[t.f];
  bool act[kR];
  for (int r = 0; r < kR; r++) act[r] = on(b, t.f, r, mode);
  if (!act[0] && !act[1]) {
    if (!mode && t.tile == F.tile0 && lin_tid() == 0) b.dir[t.f * kR] = b.dir[t.f * kR + 1] = 0;
    return;
  }
  const FmLevel C = M.lv[(size_t)t.f * kFmMaxLevels + 1];
  double s[kR] = {0.0, 0.0};
  Sum2 acc[kR];
  if (t.live) {
    const int i = t.i, j = t.j, nx = F.nx, ny = F.ny;
    const long long c = F.o2 + i + (long long)nx * j;
    const float* te = M.te[0];
    const float* tn = M.tn[0];
    const float* dv = M.dinv[0];
    for (int r = 0; r < kR; r++) {
      if (!act[r]) continue;
      const float* rr = M.r[r];
      const float* xc1 = M.xb[1][r] + C.off;
      const float cs = M.cscale;
      auto y = [&](int ii, int jj) {
        const long long cc = F.o2 + ii + (long long)nx * jj;
        return fmaf(dv[cc], rr[cc], cs * xc1[(ii >> 1) + (long long)C.nx * (jj >> 1)]);
      };
      const float yc = y(i, j);
      const float a = apply4(yc, i > 0 ? y(i - 1, j) : 0.f, i + 1 < nx ? y(i + 1, j) : 0.f, j > 0 ? y(i, j - 1) : 0.f,
                             j + 1 < ny ? y(i, j + 1) : 0.f, i > 0 ? te[c - 1] : 0.f, te[c],
                             j > 0 ? tn[c - nx] : 0.f, tn[c]);
      // cells without a fluid face (solid) keep z = 0, so p, e and phi stay
      // zero there as the reference's operator requires
      const float z = dv[c] > 0.f ? fmaf(dv[c], rr[c] - a, yc) : 0.f;
      M.z[r][c] = z;
      acc[r].add_prod(z, rr[c]);
    }
  }
  for (int r = 0; r < kR; r++) s[r] = acc[r].value();
  double out[kR];
  if (fm_seg_sum(s, t.f, t.tile, F.tile0, F.ntiles, b.partials, b.tickets, out) && lin_tid() == 0) {
    for (int r = 0; r < kR; r++) {
      const int q = t.f * kR + r;
      if (!act[r]) {
        if (!mode) b.dir[q] = 0;
        continue;
      }
      const double rz = out[r];
      if (mode) {
        b.rz[q] = rz;
        b.rz0[q] = rz;
        b.beta[q] = 0.0;
        b.active[q] = rz > 0 ? 1 : 0;
        b.dir[q] = 1;
        continue;
      }
      b.iters[q] += 1;
      if (!(rz >= 0)) {
        b.active[q] = 0;
        b.dir[q] = 0;
        continue;
      }
      b.beta[q] = rz / b.rz[q];
      b.rz[q] = rz;
      b.dir[q] = 1;
      if (rz <= b.tol2 * b.rz0[q]) b.active[q] = 0;
    }
  }
}

// p = z + beta p for the pairs whose last scalar update asked for it (in
// start mode only the pairs in the set: the others are mid-iteration).
__global__ void k_fm_direction(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b,
                               FramesMg M, int mode) {
  const T0 t = t0_ref(fr, tile_frame, b.tiles);
  if (!t.live) return;
  const Frame2& F = fr[t.f];
  const long long c = F.o2 + t.i + (long long)F.nx * t.j;
  for (int r = 0; r < kR; r++) {
    const int q = t.f * kR + r;
    if (!b.dir[q] || (mode && !b.in_set[q])) continue;
    M.p[r][c] = fmaf((float)b.beta[q], M.p[r][c], M.z[r][c]);
  }
}

// q = A p, p.q per frame and direction, alpha = rz / pq (a breakdown stops the pair).
__global__ void __launch_bounds__(256) k_fm_spmv(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame,
                                                 Batch2 b, FramesMg M) {
  const T0 t = t0_ref(fr, tile_frame, b.tiles);
  const Frame2& F = fr[t.f];
  bool act[kR];
  for (int r = 0; r < kR; r++) act[r] = on(b, t.f, r, 0);
  if (!act[0] && !act[1]) return;
  double s[kR] = {0.0, 0.0};
  Sum2 acc[kR];
  if (t.live) {
    const int i = t.i, j = t.j, nx = F.nx, ny = F.ny;
    const long long c = F.o2 + i + (long long)nx * j;
    const float* te = M.te[0];
    const float* tn = M.tn[0];
    for (int r = 0; r < kR; r++) {
      if (!act[r]) continue;
      const float* p = M.p[r];
      const float pc = p[c];
      const float q = apply4(pc, i > 0 ? p[c - 1] : 0.f, i + 1 < nx ? p[c + 1] : 0.f, j > 0 ? p[c - nx] : 0.f,
                             j + 1 < ny ? p[c + nx] : 0.f, i > 0 ? te[c - 1] : 0.f, te[c], j > 0 ? tn[c - nx] : 0.f,
                             tn[c]);
      M.q[r][c] = q;
      acc[r].add_prod(pc, q);
    }
  }
  for (int r = 0; r < kR; r++) s[r] = acc[r].value();
  double out[kR];
  if (fm_seg_sum(s, t.f, t.tile, F.tile0, F.ntiles, b.partials, b.tickets, out) && lin_tid() == 0) {
    for (int r = 0; r < kR; r++) {
      const int q = t.f * kR + r;
      if (!act[r]) continue;
      if (!(out[r] > 0) || !(b.rz[q] > 0)) {
        b.active[q] = 0;
        b.alpha[q] = 0;
      } else {
        b.alpha[q] = b.rz[q] / out[r];
      }
    }
  }
}

// e += alpha p, r -= alpha q.
__global__ void k_fm_update(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b, FramesMg M) {
  const T0 t = t0_ref(fr, tile_frame, b.tiles);
  if (!t.live) return;
  const Frame2& F = fr[t.f];
  const long long c = F.o2 + t.i + (long long)F.nx * t.j;
  for (int r = 0; r < kR; r++) {
    const int q = t.f * kR + r;
    if (!b.active[q]) continue;
    const float a = (float)b.alpha[q];
    M.e[r][c] = fmaf(a, M.p[r][c], M.e[r][c]);
    M.r[r][c] = fmaf(-a, M.q[r][c], M.r[r][c]);
  }
}

// Start of an inner solve for the pairs in the set: r = scale (rV - mean) of
// layer 1 on fluid cells (the layers are equal), e = 0, p = 0.
__global__ void k_fm_load(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b, FramesMg M) {
  const T0 t = t0_ref(fr, tile_frame, nullptr);
  if (!t.live) return;
  const Frame2& F = fr[t.f];
  const long long c = F.o2 + t.i + (long long)F.nx * t.j;
  const long long c3 = F.oint + t.i + (long long)F.nx * t.j;  // layer 1 of the 3-D interior fields
  const bool fl = b.diag[c3] > 0;
  for (int r = 0; r < kR; r++) {
    const int q = t.f * kR + r;
    if (!b.in_set[q]) continue;
    M.r[r][c] = fl ? (float)((b.r64[r][c3] - b.rmean[q]) * b.scale[q]) : 0.f;
    M.e[r][c] = 0.f;
    M.p[r][c] = 0.f;
  }
}

// phi += e / scale in both layers on fluid cells, for the pairs in the set.
__global__ void k_fm_apply(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b, FramesMg M) {
  const T0 t = t0_ref(fr, tile_frame, nullptr);
  if (!t.live) return;
  const Frame2& F = fr[t.f];
  const long long c = F.o2 + t.i + (long long)F.nx * t.j;
  const long long pl = (long long)(F.nx + 2) * (F.ny + 2);
  const long long p1 = F.opad + (t.i + 1) + (long long)(F.nx + 2) * (t.j + 1);
  if (!(b.diag[F.oint + t.i + (long long)F.nx * t.j] > 0)) return;  // fluid cells only
  for (int r = 0; r < kR; r++) {
    const int q = t.f * kR + r;
    if (!b.in_set[q]) continue;
    const double d = (double)M.e[r][c] / b.scale[q];
    b.phi[r][p1] += d;
    b.phi[r][p1 + pl] += d;
  }
}

// ---------------------------------------------------------------- launches
cudaError_t fm_setup(const Frame2* fr, const int* tf, int ntiles, const Batch2& b, const FramesMg& M,
                     const int* ntiles_lv, cudaStream_t st) {
  const dim3 blk(32, 8);
  k_fm_faces0<<<ntiles, blk, 0, st>>>(fr, tf, b, M); note_launch();
  for (int l = 0; l + 1 < M.nlev; l++) {
    k_fm_coarsen<<<ntiles_lv[l + 1], blk, 0, st>>>(M, l); note_launch();
  }
  k_fm_dinv<<<ntiles, blk, 0, st>>>(fr, tf, M, 0); note_launch();
  for (int l = 1; l < M.nlev; l++) {
    k_fm_dinv<<<ntiles_lv[l], blk, 0, st>>>(fr, tf, M, l); note_launch();
  }
  return cudaGetLastError();
}

// The preconditioner z = M r for the pairs selected by mode, ending in
// k_fm_final0 (which also updates the PCG scalars).  nact: level-0 blocks
// (the compacted tile list in b.tiles when b.tiles is set); ntiles_lv[l]:
// tiles of the frames whose level l is not their coarsest (level l's list).
static cudaError_t fm_cycle(const Frame2* fr, const int* tf, int nact, const Batch2& b, const FramesMg& M,
                            const int* nrestrict_lv, int nframes, int mode, cudaStream_t st) {
  const dim3 blk(32, 8);
  k_fm_restrict<<<nact, blk, 0, st>>>(fr, tf, b, M, 0, mode); note_launch();
  for (int l = 1; l + 1 < M.nlev; l++) {
    if (nrestrict_lv[l] == 0) break;
    k_fm_restrict<<<nrestrict_lv[l], blk, 0, st>>>(fr, tf, b, M, l, mode); note_launch();
  }
  k_fm_coarse<<<nframes, kFmMaxCoarse, 0, st>>>(b, M, M.coarse_sweeps, mode); note_launch();
  for (int l = M.nlev - 2; l >= 1; l--) {
    if (nrestrict_lv[l] == 0) continue;
    k_fm_prolong<<<nrestrict_lv[l], blk, 0, st>>>(b, M, l, mode); note_launch();
  }
  k_fm_final0<<<nact, blk, 0, st>>>(fr, tf, b, M, mode); note_launch();
  return cudaGetLastError();
}

cudaError_t fm_start(const Frame2* fr, const int* tf, int ntiles, const Batch2& b, const FramesMg& M,
                     const int* nrestrict_lv, int nframes, cudaStream_t st) {
  const dim3 blk(32, 8);
  Batch2 b0 = b;
  b0.tiles = nullptr;  // all level-0 tiles
  k_fm_load<<<ntiles, blk, 0, st>>>(fr, tf, b0, M); note_launch();
  cudaError_t e = fm_cycle(fr, tf, ntiles, b0, M, nrestrict_lv, nframes, 1, st);
  if (e != cudaSuccess) return e;
  k_fm_direction<<<ntiles, blk, 0, st>>>(fr, tf, b0, M, 1); note_launch();
  return cudaGetLastError();
}

cudaError_t fm_iteration(const Frame2* fr, const int* tf, int nact, const Batch2& b, const FramesMg& M,
                         const int* nrestrict_lv, int nframes, cudaStream_t st) {
  const dim3 blk(32, 8);
  k_fm_spmv<<<nact, blk, 0, st>>>(fr, tf, b, M); note_launch();
  k_fm_update<<<nact, blk, 0, st>>>(fr, tf, b, M); note_launch();
  cudaError_t e = fm_cycle(fr, tf, nact, b, M, nrestrict_lv, nframes, 0, st);
  if (e != cudaSuccess) return e;
  k_fm_direction<<<nact, blk, 0, st>>>(fr, tf, b, M, 0); note_launch();
  return cudaGetLastError();
}

cudaError_t fm_apply(const Frame2* fr, const int* tf, int ntiles, const Batch2& b, const FramesMg& M,
                     cudaStream_t st) {
  k_fm_apply<<<ntiles, dim3(32, 8), 0, st>>>(fr, tf, b, M); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
