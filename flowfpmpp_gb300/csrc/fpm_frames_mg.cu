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
// frames that have finished (per frame and direction flags) return at once.
// The level-0 stencil passes stage their operand with its one-cell halo in
// shared memory (a 34 x 10 tile per direction) and carry the PCG vector
// updates, so an iteration has no pointwise pass: the spmv pass forms
// p = z + beta p_old, writes it and adds the previous alpha p_old to e (e lags
// one step; the apply pass adds the last alpha p), the restriction pass forms
// r = r_old - alpha q and writes it.  r and p have two buffers each, chosen by
// the parity of the (frame, direction)'s iteration count, so no pass
// overwrites a value another CTA reads as a halo.  The dot products go to one
// partial per tile; a finalize kernel per frame and direction combines them in
// tile order (one warp, fixed order) and updates the PCG scalars, so results
// do not depend on timing.
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

// Level-0 stencil passes work on block tiles (a thread owns column x and
// rows y, y + 8, ...) with the operand and its one-cell halo in shared memory:
// cell (i0 - 1 + x, j0 - 1 + y) of the frame at [y][x]; the first HALO threads
// fill the halo.
// A block tile is 32 cells wide and 8 ROWS high (ROWS = 2, 4 or 8 rows per
// thread; FPM_FRAMES_ROWS, default 4).
constexpr int kBW = 32, kBWH = kBW + 2;
template <int ROWS>
struct BT {
  static constexpr int H = 8 * ROWS, HH = H + 2, HALO = 2 * kBWH + 2 * H;
  static_assert(HALO <= 256, "one halo slot per thread");
};
template <int ROWS>
__device__ __forceinline__ void bhalo_pos(int tid, int& x, int& y) {
  if (tid < kBWH) {
    x = tid;
    y = 0;
  } else if (tid < 2 * kBWH) {
    x = tid - kBWH;
    y = BT<ROWS>::HH - 1;
  } else {
    const int k = tid - 2 * kBWH;
    y = 1 + (k >> 1);
    x = (k & 1) ? kBWH - 1 : 0;
  }
}

// Per-tile partial of a level-0 dot product (block sum; thread 0 stores it).
__device__ __forceinline__ void tile_partial(double (&s)[kR], int tile, double* partials) {
  double m[1] = {0.0};
  block_reduce<kR, 0>(s, m);
  if (lin_tid() == 0)
    for (int n = 0; n < kR; n++) partials[(size_t)tile * kR + n] = s[n];
}

// Sum of direction r's block-tile partials of frame f in tile order (one warp).
__device__ __forceinline__ double frame_sum(const int4 bi, int r, const double* partials) {
  double s = 0.0;
  for (int t = (int)threadIdx.x; t < bi.y; t += 32) s += __ldcg(partials + (size_t)(bi.x + t) * kR + r);
  return warp_sum(s);
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
// Residual of the first smoothing sweep from zero, restricted: on level
// l >= 1, t = dinv b (stored as xa), res = b - A t, and b_{l+1} = sum of res
// over each 2 x 2 aggregate (level 0: k_fm_restrict0).
__global__ void __launch_bounds__(256) k_fm_restrict(const Frame2* __restrict__ fr,
                                                     const int* __restrict__ tile_frame, Batch2 b, FramesMg M, int l,
                                                     int mode) {
  __shared__ float res_s[kR][8][33];
  const TL t = tl_ref(M, l);
  const int f = t.f, i = t.i, j = t.j;
  const bool live = t.live;
  const FmLevel L = t.L;
  bool act[kR];
  for (int r = 0; r < kR; r++) act[r] = on(b, f, r, mode);
  if (!act[0] && !act[1]) return;
  const float* __restrict__ te = M.te[l] + L.off;
  const float* __restrict__ tn = M.tn[l] + L.off;
  const float* __restrict__ dv = M.dinv[l] + L.off;
  const long long c = i + (long long)L.nx * j;
  // every load of both directions first (the cell, its four neighbours, the faces)
  const bool w = i > 0, e = i + 1 < L.nx, so = j > 0, no = j + 1 < L.ny;
  float fw = 0.f, fe = 0.f, fs = 0.f, fn = 0.f, d[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, v[kR][5];
  if (live) {
    fw = w ? te[c - 1] : 0.f;
    fe = te[c];
    fs = so ? tn[c - L.nx] : 0.f;
    fn = tn[c];
    d[0] = dv[c];
    d[1] = w ? dv[c - 1] : 0.f;
    d[2] = e ? dv[c + 1] : 0.f;
    d[3] = so ? dv[c - L.nx] : 0.f;
    d[4] = no ? dv[c + L.nx] : 0.f;
  }
  for (int r = 0; r < kR; r++) {
    const float* __restrict__ bb = M.b[l][r] + L.off;
    const bool ld = live && act[r];
    v[r][0] = ld ? bb[c] : 0.f;
    v[r][1] = ld && w ? bb[c - 1] : 0.f;
    v[r][2] = ld && e ? bb[c + 1] : 0.f;
    v[r][3] = ld && so ? bb[c - L.nx] : 0.f;
    v[r][4] = ld && no ? bb[c + L.nx] : 0.f;
  }
  for (int r = 0; r < kR; r++) {
    float res = 0.f;
    if (live && act[r]) {
      const float tc = d[0] * v[r][0];
      const float tw = w ? d[1] * v[r][1] : 0.f;
      const float tE = e ? d[2] * v[r][2] : 0.f;
      const float ts = so ? d[3] * v[r][3] : 0.f;
      const float tN = no ? d[4] * v[r][4] : 0.f;
      const float a = apply4(tc, tw, tE, ts, tN, fw, fe, fs, fn);
      res = v[r][0] - a;
      M.xa[l][r][L.off + c] = tc;
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
  const float* __restrict__ te = M.te[l] + L.off;
  const float* __restrict__ tn = M.tn[l] + L.off;
  const float* __restrict__ dv = M.dinv[l] + L.off;
  const bool w = i > 0, e = i + 1 < L.nx, so = j > 0, no = j + 1 < L.ny;
  // every load of both directions first
  const float fw = w ? te[c - 1] : 0.f, fe = te[c], fs = so ? tn[c - L.nx] : 0.f, fn = tn[c], dc = dv[c];
  const float cs = M.cscale;
  float yv[kR][5], bc[kR];
  for (int r = 0; r < kR; r++) {
    const float* __restrict__ xa = M.xa[l][r] + L.off;
    const float* __restrict__ xc1 = M.xb[l + 1][r] + C.off;
    auto y = [&](int ii, int jj) {
      return fmaf(cs, xc1[(ii >> 1) + (long long)C.nx * (jj >> 1)], xa[ii + (long long)L.nx * jj]);
    };
    const bool ld = act[r];
    yv[r][0] = ld ? y(i, j) : 0.f;
    yv[r][1] = ld && w ? y(i - 1, j) : 0.f;
    yv[r][2] = ld && e ? y(i + 1, j) : 0.f;
    yv[r][3] = ld && so ? y(i, j - 1) : 0.f;
    yv[r][4] = ld && no ? y(i, j + 1) : 0.f;
    bc[r] = ld ? M.b[l][r][L.off + c] : 0.f;
  }
  for (int r = 0; r < kR; r++) {
    if (!act[r]) continue;
    const float a = apply4(yv[r][0], yv[r][1], yv[r][2], yv[r][3], yv[r][4], fw, fe, fs, fn);
    M.xb[l][r][L.off + c] = fmaf(dc, bc[r] - a, yv[r][0]);
  }
}

// ---------------------------------------------------------------- level 0
// The current r / p buffer of (frame f, direction r) and the other one.
__device__ __forceinline__ int fm_par(const Batch2& b, int f, int r) { return b.iters[f * kR + r] & 1; }

// Level-0 block tile of this block.
struct B0 {
  int tile, f, nx, ny, i0, j0, hx, hy;
  long long o2;
  bool halo;
};
template <int ROWS>
__device__ __forceinline__ B0 b0_ref(const Frame2* __restrict__ fr, const FramesMg& M, const int* __restrict__ list) {
  B0 h;
  h.tile = list ? list[blockIdx.x] : (int)blockIdx.x;
  h.f = M.bt_frame[h.tile];
  const int4 bi = M.bt_info[h.f];
  const Frame2& F = fr[h.f];
  h.nx = F.nx;
  h.ny = F.ny;
  h.o2 = F.o2;
  const int idx = h.tile - bi.x;
  h.i0 = (idx % bi.z) * kBW;
  h.j0 = (idx / bi.z) * BT<ROWS>::H;
  const int tid = lin_tid();
  h.halo = tid < BT<ROWS>::HALO;
  h.hx = h.hy = 0;
  if (h.halo) bhalo_pos<ROWS>(tid, h.hx, h.hy);
  return h;
}
// Frame cell of row k of this thread (-1 outside the frame), and of its halo slot.
__device__ __forceinline__ long long own_cell(const B0& h, int k) {
  const int i = h.i0 + (int)threadIdx.x, j = h.j0 + (int)threadIdx.y + 8 * k;
  return (i < h.nx && j < h.ny) ? h.o2 + i + (long long)h.nx * j : -1;
}
__device__ __forceinline__ long long halo_cell(const B0& h) {
  const int i = h.i0 - 1 + h.hx, j = h.j0 - 1 + h.hy;
  return (i >= 0 && i < h.nx && j >= 0 && j < h.ny) ? h.o2 + i + (long long)h.nx * j : -1;
}
// Faces of an own cell: west, east, south, north.
__device__ __forceinline__ float4 faces_of(const B0& h, const FramesMg& M, long long c, int k) {
  const int i = h.i0 + (int)threadIdx.x, j = h.j0 + (int)threadIdx.y + 8 * k;
  return make_float4(i > 0 ? M.te[0][c - 1] : 0.f, M.te[0][c], j > 0 ? M.tn[0][c - h.nx] : 0.f, M.tn[0][c]);
}
// A x at smem cell (x, y) of a haloed tile.
template <int HH>
__device__ __forceinline__ float apply_s(const float (&v)[HH][kBWH], int x, int y, float4 t) {
  return apply4(v[y][x], v[y][x - 1], v[y][x + 1], v[y - 1][x], v[y + 1][x], t.x, t.y, t.z, t.w);
}

// q = A p with p = z + beta p_old formed on the fly (the direction update;
// beta = 0 and p_old = 0 after a start); writes p and q, e += alpha_prev
// p_old; p.q per block tile.  The active pairs only.
template <int ROWS>
__global__ void __launch_bounds__(256) k_fm_spmv(const Frame2* __restrict__ fr, Batch2 b, FramesMg M) {
  using T = BT<ROWS>;
  __shared__ float ps[kR][T::HH][kBWH];
  const B0 h = b0_ref<ROWS>(fr, M, M.bt_list);
  const int f = h.f;
  bool act[kR];
  for (int r = 0; r < kR; r++) act[r] = b.active[f * kR + r] != 0;
  if (!act[0] && !act[1]) return;
  const int x = threadIdx.x + 1;
  for (int r = 0; r < kR; r++) {
    if (!act[r]) continue;
    const int q = f * kR + r, par = fm_par(b, f, r);
    const float beta = (float)b.beta[q], aprev = (float)b.alpha[q];
    const float* __restrict__ pold = par ? M.p2[r] : M.p[r];
    float* __restrict__ pnew = par ? M.p[r] : M.p2[r];
    const float* __restrict__ z = M.z[r];
    float* __restrict__ e = M.e[r];
    // all loads of the pass first (own rows and the halo slot), then the stores
    long long cc[ROWS];
    float po[ROWS], zz[ROWS], ee[ROWS];
#pragma unroll
    for (int k = 0; k < ROWS; k++) {
      cc[k] = own_cell(h, k);
      po[k] = cc[k] >= 0 ? pold[cc[k]] : 0.f;
      zz[k] = cc[k] >= 0 ? z[cc[k]] : 0.f;
      ee[k] = cc[k] >= 0 ? e[cc[k]] : 0.f;
    }
    const long long ch = h.halo ? halo_cell(h) : -1;
    const float hp = ch >= 0 ? pold[ch] : 0.f, hz = ch >= 0 ? z[ch] : 0.f;
#pragma unroll
    for (int k = 0; k < ROWS; k++) {
      const float pn = fmaf(beta, po[k], zz[k]);
      if (cc[k] >= 0) {
        pnew[cc[k]] = pn;
        e[cc[k]] = fmaf(aprev, po[k], ee[k]);
      }
      ps[r][threadIdx.y + 1 + 8 * k][x] = cc[k] >= 0 ? pn : 0.f;
    }
    if (h.halo) ps[r][h.hy][h.hx] = ch >= 0 ? fmaf(beta, hp, hz) : 0.f;
  }
  __syncthreads();
  Sum2 acc[kR];
#pragma unroll
  for (int k = 0; k < ROWS; k++) {
    const long long c = own_cell(h, k);
    if (c < 0) continue;
    const float4 t = faces_of(h, M, c, k);
    const int y = threadIdx.y + 1 + 8 * k;
    for (int r = 0; r < kR; r++) {
      if (!act[r]) continue;
      const float pc = ps[r][y][x];
      const float qv = apply_s(ps[r], x, y, t);
      M.q[r][c] = qv;
      acc[r].add_prod(pc, qv);
    }
  }
  double s[kR];
  for (int r = 0; r < kR; r++) s[r] = acc[r].value();
  tile_partial(s, h.tile, b.partials);
}

// alpha = rz / p.q per active pair (a breakdown stops the pair).  One warp
// per direction, one block per frame.
__global__ void k_fm_fin_spmv(FramesMg M, Batch2 b) {
  const int f = blockIdx.x, r = threadIdx.y, q = f * kR + r;
  if (!b.active[q]) return;
  const double pq = frame_sum(M.bt_info[f], r, b.partials);
  if (threadIdx.x != 0) return;
  if (!(pq > 0) || !(b.rz[q] > 0)) {
    b.active[q] = 0;
    b.alpha[q] = 0;
  } else {
    b.alpha[q] = b.rz[q] / pq;
  }
}

// Level-0 restriction: r = r_old - alpha q (iteration mode; written to the
// other r buffer), t = dinv r (the first smoothing sweep from zero),
// b_1 = sum over each 2 x 2 aggregate of r - A t.
template <int ROWS>
__global__ void __launch_bounds__(256) k_fm_restrict0(const Frame2* __restrict__ fr, Batch2 b, FramesMg M,
                                                      const int* __restrict__ list, int mode) {
  using T = BT<ROWS>;
  __shared__ float ts_s[kR][T::HH][kBWH];
  __shared__ float res_s[kR][T::H][kBW + 1];
  const B0 h = b0_ref<ROWS>(fr, M, list);
  const int f = h.f;
  bool act[kR];
  for (int r = 0; r < kR; r++) act[r] = on(b, f, r, mode);
  if (!act[0] && !act[1]) return;
  const float* __restrict__ dv = M.dinv[0];
  const int x = threadIdx.x + 1;
  float4 fc[ROWS];  // faces of the own rows, loaded with the operands
#pragma unroll
  for (int k = 0; k < ROWS; k++) {
    const long long c = own_cell(h, k);
    fc[k] = c >= 0 ? faces_of(h, M, c, k) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  float rown[kR][ROWS];
  for (int r = 0; r < kR; r++) {
    if (!act[r]) continue;
    const int par = fm_par(b, f, r);
    const float alpha = mode ? 0.f : (float)b.alpha[f * kR + r];
    const float* __restrict__ rold = par ? M.r2[r] : M.r[r];
    float* __restrict__ rnew = par ? M.r[r] : M.r2[r];
    const float* __restrict__ qv = M.q[r];
    // all loads of the pass first (own rows and the halo slot), then the stores
    long long cc[ROWS];
    float ro[ROWS], qq[ROWS], dd[ROWS];
#pragma unroll
    for (int k = 0; k < ROWS; k++) {
      cc[k] = own_cell(h, k);
      ro[k] = cc[k] >= 0 ? rold[cc[k]] : 0.f;
      qq[k] = cc[k] >= 0 && !mode ? qv[cc[k]] : 0.f;
      dd[k] = cc[k] >= 0 ? dv[cc[k]] : 0.f;
    }
    const long long ch = h.halo ? halo_cell(h) : -1;
    const float hr = ch >= 0 ? rold[ch] : 0.f, hq = ch >= 0 && !mode ? qv[ch] : 0.f, hd = ch >= 0 ? dv[ch] : 0.f;
#pragma unroll
    for (int k = 0; k < ROWS; k++) {
      const float rn = mode ? ro[k] : fmaf(-alpha, qq[k], ro[k]);
      if (cc[k] >= 0 && !mode) rnew[cc[k]] = rn;
      rown[r][k] = cc[k] >= 0 ? rn : 0.f;
      ts_s[r][threadIdx.y + 1 + 8 * k][x] = cc[k] >= 0 ? dd[k] * rn : 0.f;
    }
    if (h.halo) ts_s[r][h.hy][h.hx] = ch >= 0 ? hd * (mode ? hr : fmaf(-alpha, hq, hr)) : 0.f;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < ROWS; k++) {
    const long long c = own_cell(h, k);
    const int y = threadIdx.y + 1 + 8 * k;
    const float4 t = fc[k];
    for (int r = 0; r < kR; r++) {
      float res = 0.f;
      if (c >= 0 && act[r]) res = rown[r][k] - apply_s(ts_s[r], x, y, t);
      res_s[r][y - 1][threadIdx.x] = res;
    }
  }
  __syncthreads();
  // the 2 x 2 aggregates of the tile, one per thread at a time
  const FmLevel C = M.lv[(size_t)f * kFmMaxLevels + 1];
  for (int ag = lin_tid(); ag < 16 * (T::H / 2); ag += 256) {
    const int ax = ag & 15, ay = ag >> 4;
    const int i = h.i0 + 2 * ax, j = h.j0 + 2 * ay;
    if (i >= h.nx || j >= h.ny) continue;
    for (int r = 0; r < kR; r++) {
      if (!act[r]) continue;
      const float sm = (res_s[r][2 * ay][2 * ax] + res_s[r][2 * ay][2 * ax + 1]) +
                       (res_s[r][2 * ay + 1][2 * ax] + res_s[r][2 * ay + 1][2 * ax + 1]);
      M.b[1][r][C.off + (i >> 1) + (long long)C.nx * (j >> 1)] = sm;
    }
  }
}

// Level 0: y = dinv r + P xb_1, z = y + dinv (r - A y); r.z per block tile.
// The pairs selected by mode (start: those in the set, reading the r that the
// load pass wrote; iteration: the active ones, reading the r of the
// restriction).
template <int ROWS>
__global__ void __launch_bounds__(256) k_fm_final0(const Frame2* __restrict__ fr, Batch2 b, FramesMg M,
                                                   const int* __restrict__ list, int mode) {
  using T = BT<ROWS>;
  __shared__ float ys[kR][T::HH][kBWH];
  const B0 h = b0_ref<ROWS>(fr, M, list);
  const int f = h.f;
  bool act[kR];
  for (int r = 0; r < kR; r++) act[r] = on(b, f, r, mode);
  if (!act[0] && !act[1]) return;
  const FmLevel C = M.lv[(size_t)f * kFmMaxLevels + 1];
  const float* __restrict__ dv = M.dinv[0];
  const float cs = M.cscale;
  const int x = threadIdx.x + 1;
  float4 fc[ROWS];  // faces of the own rows, loaded with the operands
#pragma unroll
  for (int k = 0; k < ROWS; k++) {
    const long long c = own_cell(h, k);
    fc[k] = c >= 0 ? faces_of(h, M, c, k) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  float rown[kR][ROWS], dvc[ROWS];
#pragma unroll
  for (int k = 0; k < ROWS; k++) {
    const long long c = own_cell(h, k);
    dvc[k] = c >= 0 ? dv[c] : 0.f;
  }
  for (int r = 0; r < kR; r++) {
    if (!act[r]) continue;
    const int par = fm_par(b, f, r) ^ (mode ? 0 : 1);
    const float* __restrict__ rr = par ? M.r2[r] : M.r[r];
    const float* __restrict__ xc1 = M.xb[1][r] + C.off;
    auto parent = [&](int i, int j) { return cs * xc1[(i >> 1) + (long long)C.nx * (j >> 1)]; };
    // all loads of the pass first (own rows and the halo slot), then the stores
    float pa[ROWS];
#pragma unroll
    for (int k = 0; k < ROWS; k++) {
      const long long c = own_cell(h, k);
      rown[r][k] = c >= 0 ? rr[c] : 0.f;
      pa[k] = c >= 0 ? parent(h.i0 + (int)threadIdx.x, h.j0 + (int)threadIdx.y + 8 * k) : 0.f;
    }
    const long long ch = h.halo ? halo_cell(h) : -1;
    const float hr = ch >= 0 ? rr[ch] : 0.f, hd = ch >= 0 ? dv[ch] : 0.f;
    const float hpa = ch >= 0 ? parent(h.i0 - 1 + h.hx, h.j0 - 1 + h.hy) : 0.f;
#pragma unroll
    for (int k = 0; k < ROWS; k++)
      ys[r][threadIdx.y + 1 + 8 * k][x] = own_cell(h, k) >= 0 ? fmaf(dvc[k], rown[r][k], pa[k]) : 0.f;
    if (h.halo) ys[r][h.hy][h.hx] = ch >= 0 ? fmaf(hd, hr, hpa) : 0.f;
  }
  __syncthreads();
  Sum2 acc[kR];
#pragma unroll
  for (int k = 0; k < ROWS; k++) {
    const long long c = own_cell(h, k);
    if (c < 0) continue;
    const float4 t = fc[k];
    const int y = threadIdx.y + 1 + 8 * k;
    for (int r = 0; r < kR; r++) {
      if (!act[r]) continue;
      const float yc = ys[r][y][x];
      const float a = apply_s(ys[r], x, y, t);
      // cells without a fluid face (solid) keep z = 0, so p, e and phi stay
      // zero there as the reference's operator requires
      const float zv = dvc[k] > 0.f ? fmaf(dvc[k], rown[r][k] - a, yc) : 0.f;
      M.z[r][c] = zv;
      acc[r].add_prod(zv, rown[r][k]);
    }
  }
  double s[kR];
  for (int r = 0; r < kR; r++) s[r] = acc[r].value();
  tile_partial(s, h.tile, b.partials);
}

// The PCG scalars after the preconditioner: start mode (the pairs in the set):
// rz0 = rz, beta = 0, the pair is active if rz > 0.  Iteration mode (the
// active pairs): the scalar update of the reference's pcg_iterate with this
// preconditioner -- beta = rz_new / rz, and the pair stops when rz has
// dropped by the inner tolerance.
__global__ void k_fm_fin_final(FramesMg M, Batch2 b, int mode) {
  const int f = blockIdx.x, r = threadIdx.y, q = f * kR + r;
  if (!on(b, f, r, mode)) return;
  const double rz = frame_sum(M.bt_info[f], r, b.partials);
  if (threadIdx.x != 0) return;
  if (mode) {
    b.rz[q] = rz;
    b.rz0[q] = rz;
    b.beta[q] = 0.0;
    b.active[q] = rz > 0 ? 1 : 0;
    return;
  }
  b.iters[q] += 1;
  if (!(rz >= 0)) {
    b.active[q] = 0;
    return;
  }
  b.beta[q] = rz / b.rz[q];
  b.rz[q] = rz;
  if (rz <= b.tol2 * b.rz0[q]) b.active[q] = 0;
}

// Start of an inner solve for the pairs in the set: r = scale (rV - mean) of
// layer 1 on fluid cells (the layers are equal), e = 0, p = 0 (the current
// buffers), alpha = 0 (nothing pending for e).
__global__ void k_fm_load(const Frame2* __restrict__ fr, const int* __restrict__ tile_frame, Batch2 b, FramesMg M) {
  const T0 t = t0_ref(fr, tile_frame, nullptr);
  const Frame2& F = fr[t.f];
  if (t.tile == F.tile0 && lin_tid() < kR && b.in_set[t.f * kR + lin_tid()]) b.alpha[t.f * kR + lin_tid()] = 0.0;
  if (!t.live) return;
  const long long c = F.o2 + t.i + (long long)F.nx * t.j;
  const long long c3 = F.oint + t.i + (long long)F.nx * t.j;  // layer 1 of the 3-D interior fields
  const bool fl = b.diag[c3] > 0;
  for (int r = 0; r < kR; r++) {
    const int q = t.f * kR + r;
    if (!b.in_set[q]) continue;
    const int par = fm_par(b, t.f, r);
    (par ? M.r2[r] : M.r[r])[c] = fl ? (float)((b.r64[r][c3] - b.rmean[q]) * b.scale[q]) : 0.f;
    M.e[r][c] = 0.f;
    (par ? M.p2[r] : M.p[r])[c] = 0.f;
  }
}

// phi += (e + alpha p) / scale in both layers on fluid cells, for the pairs in
// the set: the correction with the last iteration's alpha p, which the spmv
// pass adds to e only in the iteration after (alpha is zero after a
// breakdown and after a load).
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
    const float a = (float)b.alpha[q];
    const float* __restrict__ p = fm_par(b, t.f, r) ? M.p2[r] : M.p[r];
    const float ec = a != 0.f ? fmaf(a, p[c], M.e[r][c]) : M.e[r][c];
    const double d = (double)ec / b.scale[q];
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
// k_fm_final0 and the scalar update.  Level 0: nblocks block tiles of list
// (NULL: all); nrestrict_lv[l]: tiles of the frames whose level l is not their
// coarsest (level l's list).
template <int ROWS>
static cudaError_t fm_cycle(const Frame2* fr, int nblocks, const int* list, const Batch2& b, const FramesMg& M,
                            const int* nrestrict_lv, int nframes, int mode, cudaStream_t st) {
  const dim3 blk(32, 8);
  k_fm_restrict0<ROWS><<<nblocks, blk, 0, st>>>(fr, b, M, list, mode); note_launch();
  for (int l = 1; l + 1 < M.nlev; l++) {
    if (nrestrict_lv[l] == 0) break;
    k_fm_restrict<<<nrestrict_lv[l], blk, 0, st>>>(fr, nullptr, b, M, l, mode); note_launch();
  }
  k_fm_coarse<<<nframes, kFmMaxCoarse, 0, st>>>(b, M, M.coarse_sweeps, mode); note_launch();
  for (int l = M.nlev - 2; l >= 1; l--) {
    if (nrestrict_lv[l] == 0) continue;
    k_fm_prolong<<<nrestrict_lv[l], blk, 0, st>>>(b, M, l, mode); note_launch();
  }
  k_fm_final0<ROWS><<<nblocks, blk, 0, st>>>(fr, b, M, list, mode); note_launch();
  k_fm_fin_final<<<nframes, dim3(32, kR), 0, st>>>(M, b, mode); note_launch();
  return cudaGetLastError();
}

cudaError_t fm_start(const Frame2* fr, const int* tf, int ntiles, int nbtiles, const Batch2& b, const FramesMg& M,
                     const int* nrestrict_lv, int nframes, cudaStream_t st) {
  Batch2 b0 = b;
  b0.tiles = nullptr;  // all 32 x 8 tiles
  k_fm_load<<<ntiles, dim3(32, 8), 0, st>>>(fr, tf, b0, M); note_launch();
  switch (M.bt_rows) {
    case 2: return fm_cycle<2>(fr, nbtiles, nullptr, b0, M, nrestrict_lv, nframes, 1, st);
    case 8: return fm_cycle<8>(fr, nbtiles, nullptr, b0, M, nrestrict_lv, nframes, 1, st);
    default: return fm_cycle<4>(fr, nbtiles, nullptr, b0, M, nrestrict_lv, nframes, 1, st);
  }
}

cudaError_t fm_iteration(const Frame2* fr, int nbact, const Batch2& b, const FramesMg& M, const int* nrestrict_lv,
                         int nframes, cudaStream_t st) {
  switch (M.bt_rows) {
    case 2: k_fm_spmv<2><<<nbact, dim3(32, 8), 0, st>>>(fr, b, M); break;
    case 8: k_fm_spmv<8><<<nbact, dim3(32, 8), 0, st>>>(fr, b, M); break;
    default: k_fm_spmv<4><<<nbact, dim3(32, 8), 0, st>>>(fr, b, M); break;
  }
  note_launch();
  k_fm_fin_spmv<<<nframes, dim3(32, kR), 0, st>>>(M, b); note_launch();
  switch (M.bt_rows) {
    case 2: return fm_cycle<2>(fr, nbact, M.bt_list, b, M, nrestrict_lv, nframes, 0, st);
    case 8: return fm_cycle<8>(fr, nbact, M.bt_list, b, M, nrestrict_lv, nframes, 0, st);
    default: return fm_cycle<4>(fr, nbact, M.bt_list, b, M, nrestrict_lv, nframes, 0, st);
  }
}

cudaError_t fm_apply(const Frame2* fr, const int* tf, int ntiles, const Batch2& b, const FramesMg& M,
                     cudaStream_t st) {
  k_fm_apply<<<ntiles, dim3(32, 8), 0, st>>>(fr, tf, b, M); note_launch();
  return cudaGetLastError();
}

}  // namespace fpm
