// Internal host-side declarations shared by the kernel files and the C ABI.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "fpm_common.cuh"

namespace fpm {

// Device-resident scalars of one solve.  The iteration kernels read and write
// these directly, so a PCG chunk runs without any host round trip.
struct SolveScalars {
  double rz, pq, alpha, beta, rz_new;  // PCG recurrences
  double red[6];                       // generic reduction outputs
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
cudaError_t launch_jacobi_f64_fma(const Dims& d, const double* a, double* b, const double* src, const double* rdiag,
                                  const Coefs& c, cudaStream_t st);
void fp64_rate_shape(int sms, int* blocks, int* threads);
cudaError_t fp64_rate_probe(double* out, int blocks, int threads, cudaStream_t st, double* instr_per_s);
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
// Force densities of np <= kMaxRhs potentials in one pass (fpm_terms_multi.cu):
// phi[m], faces[m], bg[3m..3m+2] per potential; outs[5m..5m+4] = gx, gy, gz,
// vortex, advection; totals[2m], totals[2m+1] = the two integrals.  tables
// holds terms_multi_table_bytes(d); partials 2 np x (blocks of cells_launch).
cudaError_t launch_terms_multi(const Dims& d, int np, const double* const* phi, const Flow& fl,
                               const int32_t* solid, const double* bg, const Axes& ax, const Faces* faces,
                               const double bounds[6], double* const* outs, void* tables, double* partials,
                               unsigned int* ticket, double* totals, cudaStream_t st);
size_t terms_multi_table_bytes(const Dims& d);
dim3 terms_multi_grid(const Dims& d);  // partials: 2 np x its block count
// rcp: scratch for (nx+2) + (ny+2) + nz spacing reciprocals.
cudaError_t launch_terms(const Dims& d, const double* phi, const Flow& fl, const int32_t* solid, const double bg[3],
                         const Axes& ax, const Faces& f, const double bounds[6], const TermsOut& o, double* rcp,
                         SolveScalars* S, const RedBuf& rb, cudaStream_t st);

// FP64 -> double-float conversion (fpm_stairstep_df.cu).
cudaError_t launch_to_df(const double* x, float2* y, long long n, cudaStream_t st);

// TMA-streamed double-float Jacobi (fpm_jacobi_tma.cu).
struct JacobiDfPlan {
  int nx, ny, nz;
  long long px;      // x pitch (elements) of the internal phi layout, even
  int kchunk;        // planes per CTA along z
  int shape;         // index into the tile-shape table
  float2 *a, *b;     // internal phi buffers, px * (ny+2) * nz
  float4* sr;        // (src, rdiag) as double-float, nx * ny * nz
  float2* coef;      // cw, ce, cs, cn, cb, ct as double-float
  int* err;          // set to 1 if a pipeline wait timed out
  CUtensorMap tm_a, tm_b, tm_sr;
};
int jacobi_df_num_shapes();
int jacobi_df_ctas_per_sm(int shape);
cudaError_t jacobi_df_pack(JacobiDfPlan& pl, const double* phi, const double* src, const double* rdiag,
                           const double* coef64, cudaStream_t st);
cudaError_t jacobi_df_encode(JacobiDfPlan& pl);
void jacobi_df_shape(int shape, int* tx, int* ty);
cudaError_t jacobi_df_sweep(const JacobiDfPlan& pl, const float2* src_phi, float2* dst_phi, cudaStream_t st);
cudaError_t jacobi_df_unpack(const JacobiDfPlan& pl, const float2* cur, double* phi, cudaStream_t st);

// TMA-streamed Jacobi with FP64 storage and triple-float arithmetic
// (fpm_jacobi_tf.cu); the same pipeline as the double-float plan.
struct JacobiTfPlan {
  int nx, ny, nz;
  long long px;      // x pitch (elements) of the internal phi layout, even
  int kchunk;        // planes per CTA along z
  int shape;         // index into the tile-shape table
  double *a, *b;     // internal phi buffers, px * (ny+2) * nz
  double* sr;        // (src, rdiag) pairs, 2 * nx * ny * nz
  float4* coef;      // cw, ce, cs, cn, cb, ct as three FP32 limbs
  float4 point2;     // 0.2 as three FP32 limbs
  int* err;          // set to 1 if a pipeline wait timed out
  CUtensorMap tm_a, tm_b, tm_sr;
};
int jacobi_tf_num_shapes();
void jacobi_tf_shape(int shape, int* tx, int* ty);
cudaError_t jacobi_tf_pack(JacobiTfPlan& pl, const double* phi, const double* src, const double* rdiag,
                           const double* coef64, cudaStream_t st);
cudaError_t jacobi_tf_encode(JacobiTfPlan& pl);
cudaError_t jacobi_tf_sweep(const JacobiTfPlan& pl, const double* src_phi, double* dst_phi, cudaStream_t st);
cudaError_t jacobi_tf_unpack(const JacobiTfPlan& pl, const double* cur, double* phi, cudaStream_t st);

// Mixed-precision multi-right-hand-side PCG (fpm_pcg_mixed.cu).
constexpr int kMaxRhs = 4;
// FP32 vector layout: cell (i, j, k), i in [0, nx+1], j in [0, ny+1], k in
// [1, nz], at 3 + i + px (j + (ny + 2)(k - 1)), px a multiple of 4; groups of
// four cells along x are 16-byte aligned.
struct MixedGrid {
  int nx, ny, nz, px, ng, kc, nblocks;
  long long plane, size;
};
MixedGrid mixed_grid(int nx, int ny, int nz, int kc);
struct MixedVecs {
  int nrhs;
  const float *wall, *rdiag;         // FP32 operator, MixedGrid layout: wall = sum of the
                                     // coefficients towards solid neighbours (-1 in solid cells)
  const float *cw, *ce, *dx;         // x-axis: row layout (index 3 + i)
  const float *cs, *cn, *dy;         // y-axis: index j - 1
  const float *cb, *ct, *dz;         // z-axis: index k - 1
  float *p[kMaxRhs], *q[kMaxRhs], *r[kMaxRhs], *e[kMaxRhs];
};
struct MixedScale {
  double scale[kMaxRhs];
  double pmul[kMaxRhs];  // 0: restart p from rdiag r; else rescale p by pmul
  int in_set[kMaxRhs];
};
struct MixedScalars {
  double rz[kMaxRhs], rz0[kMaxRhs], pq[kMaxRhs], alpha[kMaxRhs], beta[kMaxRhs], tol2[kMaxRhs];
  int active[kMaxRhs];
  int dir[kMaxRhs];  // the update computed beta: the direction update runs (even if it stopped the iteration)
  int iters;
  int pad[3];
};
struct DPtr4 {
  double* p[kMaxRhs];
};
cudaError_t launch_mx_layout(const MixedGrid& G, const double* a, float* b, cudaStream_t st);
cudaError_t launch_mx_wall(const MixedGrid& G, const Dims& d, const int32_t* solid, const Coefs& c, float* wall,
                           cudaStream_t st);
cudaError_t launch_mx_row(int n, int len, const double* a, float* b, cudaStream_t st);
cudaError_t launch_mx_convert(const double* a, float* b, long long n, cudaStream_t st);
cudaError_t launch_mx_start(const MixedGrid& G, const MixedVecs& v, const DPtr4& rv64, const MixedScale& sc,
                            MixedScalars* S, const RedBuf& rb, cudaStream_t st);
cudaError_t launch_mx_iteration(const MixedGrid& G, const MixedVecs& v, MixedScalars* S, const RedBuf& rb,
                                cudaStream_t st);
cudaError_t launch_mx_apply(const MixedGrid& G, const MixedVecs& v, const DPtr4& phi, const MixedScale& sc,
                            cudaStream_t st);

// Batched uneven 2-D frames (fpm_frames2d.cu).
struct Frame2 {
  int nx, ny;           // cells; nz = 2 (dz = 0.5)
  int tile0, ntiles;    // range in the tile list (32 x 8 columns)
  int tiles_x;          // tiles along x
  int ox, oy;           // offsets into the x / y axis pools (stride >= n+2 per frame)
  long long opad;       // offset of padded 3-D fields, (nx+2)(ny+2)*2 per frame
  long long oint;       // offset of interior 3-D fields, nx*ny*2 per frame
  long long o2;         // offset of 2-D fields, nx*ny per frame
  long long oring;      // offset of the outer ring, (2nx+2ny)*4 per frame
};
struct Batch2 {
  // inputs
  const double *xc, *yc, *dx, *dy, *xf, *yf;  // axis pools: xc(0:nx+1), dx(1:nx), xf(0:nx) at ox
  const int32_t* solid3;                      // padded, both layers
  const uint8_t* solid2;                      // (nx, ny)
  const double *u, *v, *ring, *kin, *dt;
  double nu;
  // operator and solution (two directions)
  double *src[2], *diag, *rdiag, *phi[2], *phi_best[2], *r64[2];
  float *diag32, *rdiag32, *r32[2], *p32[2], *q32[2], *e32[2];
  float *wall32;                      // per cell: sum of coefficients towards solid neighbours, -1 in solid
  float *cw32, *ce32, *cs32, *cn32;   // FP32 axis coefficients (x pools at ox + i - 1, y pools at oy + j - 1)
  // partition
  double *nxf, *nyf, *omega, *gpx[2], *gpy[2], *vif[2], *terms;
  // per (frame, direction) scalars, index 2*f + r
  double *corr, *res, *rmean, *scale, *pmul, *rz, *rz0, *alpha, *beta;
  int *in_set, *active, *iters;
  int* dir;   // per (frame, direction): the update computed beta, so the direction update runs
  int* keep;  // per (frame, direction): 1 = save phi as the best iterate, 2 = restore it
  double tol2;
  double* partials;       // ntiles * 8
  unsigned int* tickets;  // one per frame
  const int* tiles;       // compacted list of tile ids launched (NULL: block = tile)
  int* err;
};
#define B2_DECL(kern) \
  cudaError_t launch_##kern(const Frame2* fr, const int* tf, int ntiles, const Batch2& b, cudaStream_t st);
B2_DECL(k_b2_compat)
B2_DECL(k_b2_build)
B2_DECL(k_b2_tres)
B2_DECL(k_b2_start)
B2_DECL(k_b2_apply)
B2_DECL(k_b2_keep)
B2_DECL(k_b2_gauge_sum)
B2_DECL(k_b2_gauge_sub)
B2_DECL(k_b2_part1)
B2_DECL(k_b2_part2)
cudaError_t launch_b2_iteration(const Frame2* fr, const int* tf, int ntiles, const Batch2& b, cudaStream_t st);

// Batched 2-D multigrid preconditioner of the frames (fpm_frames_mg.cu).
constexpr int kFmMaxLevels = 12;
constexpr int kFmMaxCoarse = 1024;  // threads of the coarsest-level kernel (cells of a 32 x 32 level)
constexpr int kFmCoarseSide = 8;    // a frame's coarsest level has at most this many cells per side
struct FmLevel {
  int nx, ny;
  long long off;  // offset of the frame's level in the level's pools (level 0: Frame2::o2)
};
struct FmTile {
  int f, i0, j0;  // frame and 0-based origin of a 32 x 8 tile
};
struct FramesMg {
  int nlev;                              // levels of the deepest frame
  const FmLevel* lv;                     // [frame * kFmMaxLevels + level]
  const int* nlevels;                    // levels per frame (>= 2; the last one is the coarsest)
  const FmTile* tiles[kFmMaxLevels];     // level >= 1: frames whose level is not their coarsest first
  float *te[kFmMaxLevels], *tn[kFmMaxLevels], *dinv[kFmMaxLevels];  // faces east / north, omega / diag
  float *b[kFmMaxLevels][2], *xa[kFmMaxLevels][2], *xb[kFmMaxLevels][2];  // levels >= 1, per direction
  float *r[2], *z[2], *p[2], *q[2], *e[2];  // level 0 (2-D frame layout), per direction
  float *r2[2], *p2[2];  // second r and p buffers (the current one: iterations & 1)
  // level-0 blocks of the stencil passes: 32 x (8 bt_rows) cells of one frame
  const int* bt_frame;   // frame of each block tile
  const int4* bt_info;   // per frame: first block tile, block tiles, block tiles along x
  int* bt_list;          // the block tiles of the frames still iterating (compacted by the host)
  int bt_rows;           // rows per thread of a block tile: 2, 4 or 8 (32 x 8 bt_rows cells)
  float omega;
  float cscale;  // scale of the prolonged coarse correction (the cycle stays symmetric)
  int coarse_sweeps;
};
cudaError_t fm_setup(const Frame2* fr, const int* tf, int ntiles, const Batch2& b, const FramesMg& M,
                     const int* ntiles_lv, cudaStream_t st);
// fm_start: every block tile and the 32 x 8 load tiles (ntiles, nbtiles);
// fm_iteration: the nbact block tiles of M.bt_list.
cudaError_t fm_start(const Frame2* fr, const int* tf, int ntiles, int nbtiles, const Batch2& b, const FramesMg& M,
                     const int* nrestrict_lv, int nframes, cudaStream_t st);
cudaError_t fm_iteration(const Frame2* fr, int nbact, const Batch2& b, const FramesMg& M, const int* nrestrict_lv,
                         int nframes, cudaStream_t st);
cudaError_t fm_apply(const Frame2* fr, const int* tf, int ntiles, const Batch2& b, const FramesMg& M,
                     cudaStream_t st);

// ---- no-body Neumann solvers and densities (fpm_laplace.cu) --------------
cudaError_t launch_neumann_compat(int nx, int ny, int nz, const double* rhs, Faces f, const double* dx,
                                  const double* dy, const double* dz, int uniform, double area_uniform,
                                  SolveScalars* S, const RedBuf& rb, cudaStream_t st);
typedef double (*ReadRes)(SolveScalars*, cudaStream_t, int);
int neumann_uniform_iterate(int nx, int ny, int nz, double* phi, const double* rhs, Faces f, double dx, double dy,
                            double dz, double tol, int max_it, int ci, double* a, double* b, SolveScalars* S,
                            const RedBuf& rb, cudaStream_t st, ReadRes read_res, int* iterations,
                            double* final_residual);
int neumann_nonuniform_iterate(int nx, int ny, int nz, double* phi, const double* rhs, Faces f, const Axes& ax,
                               double tol, int max_it, int ci, double* b, double* coef, SolveScalars* S,
                               const RedBuf& rb, cudaStream_t st, ReadRes read_res, int* iterations,
                               double* final_residual);
cudaError_t launch_terms_uniform(int nx, int ny, int nz, const double* phi, const Flow& fl, const int32_t* fluid,
                                 double dx, double dy, double dz, const TermsOut& o, SolveScalars* S,
                                 const RedBuf& rb, cudaStream_t st);
cudaError_t launch_terms_nonuniform(int nx, int ny, int nz, const double* phi, const Flow& fl, const int32_t* fluid,
                                    const Axes& ax, const Faces& f, const double bounds[6], const TermsOut& o,
                                    SolveScalars* S, const RedBuf& rb, cudaStream_t st);

// ---- 2-D force partition (fpm_partition2d.cu) ------------------------------
struct Part2D {
  const double *phi, *u, *v, *xf, *yf, *ring;
  const uint8_t* solid;
  double g0, g1, k1, k2, k3, k4, k5, k6, dt, nu;
  int nx, ny, slip;
};
cudaError_t launch_partition_2d(const Part2D& p, double* nxf, double* nyf, double* gpx, double* gpy,
                                double* vif_density, double* omega, SolveScalars* S, const RedBuf& rb,
                                cudaStream_t st);

// Allocation-free max-norm operator residual (fpm_noalloc.cu); returns a
// status code and fills *msg on failure.
int operator_residual_noalloc(const double* phi, const double* src, const double* diag, const Axes& ax, int nx, int ny,
                              int nz, double* value, cudaStream_t st, std::string* msg);

// Host-side count of kernel launches made by this library (fpm_capi.cu).
void note_launch();

// ---- aggregation multigrid preconditioner (fpm_mg.cu) ---------------------
// Every right-hand side has its own vectors on every level; the kernels of a
// V-cycle cover all of them in one launch (blockIdx.z = chunk + chunks x rhs).
struct MgLevel {
  int nx, ny, nz;
  int zc;                      // planes per thread in the one-thread-per-cell kernels: nz / zc
  long long off, sy, sz;       // cell (i, j, k) (0-based) at off + i + sy j + sz k
  long long alloc;             // elements per array
  float *te, *tn, *tt, *dinv;  // face transmissibilities, inverse diagonal (level 0: omega x inverse diagonal)
  float *x[kMaxRhs], *b[kMaxRhs], *t[kMaxRhs];  // per right-hand side (levels >= 1): solution, right-hand side,
                                                // scratch
  __host__ __device__ long long n() const { return (long long)nx * ny * nz; }
};
constexpr int kMgMaxLevels = 16;
// Tensor maps of the level-0 TMA passes: the level-0 vectors z, p and r and
// the level-1 solution x1 of each right-hand side, level 0's omega D^-1 and
// the open-face bits.
struct MgMaps {
  CUtensorMap z[kMaxRhs], p[kMaxRhs], r[kMaxRhs], x1[kMaxRhs], q[kMaxRhs], p2[kMaxRhs], r2[kMaxRhs], dinv, fb;
};
struct MgHierarchy {
  int nlev, nrhs;
  int kc0;            // planes per CTA of the level-0 TMA passes (even: whole aggregates)
  long long pxb;      // row pitch of the open-face bits (bytes, a multiple of 16)
  MgMaps maps;
  MgLevel lv[kMgMaxLevels];
  MixedGrid g0;       // level 0 uses the FP32 layout of the mixed solver (float4 groups, zero halo)
  // level 0 operator for the float4 kernels: open-face bits per cell (1 east,
  // 2 north, 4 top; the MixedGrid layout with row pitch pxb) and 1-D FP32 axis
  // factors; T_east = dy dz / (xc_{i+1} - xc_i) etc. are rebuilt from them in
  // registers
  uint8_t* fb0;
  float *aex, *dxr;   // row layout (index 3 + i, i 1-based), zero outside
  float *dy, *ayn;    // index j - 1
  float *dz, *azt;    // index k - 1
  // one weighted-Jacobi sweep before and one after each coarse correction
  int gamma;          // cycles on the next coarser problem for the levels l < gamma_depth (1: V-cycle)
  int gamma_depth;
  int coarse_sweeps;  // Jacobi sweeps on the coarsest level (one block per right-hand side)
  float omega;        // Jacobi weight
  float cscale;       // coarse-correction scale (1 = plain Galerkin correction)
};
struct MgVecs {  // level-0 PCG vectors per right-hand side
  float *r[kMaxRhs], *z[kMaxRhs], *p[kMaxRhs], *q[kMaxRhs], *e[kMaxRhs];
  // second r and p buffers of the multigrid PCG: the passes that update r and
  // p read one buffer (with halos) and write the other, alternating with the
  // parity of the inner iteration count
  float *r2[kMaxRhs], *p2[kMaxRhs];
};
struct MgScalars {  // one per right-hand side
  double rz, rz0, pq, alpha, beta, tol2;
  int active, pad0, iters, pad;
};
// Per-right-hand-side grid reductions: partials holds kMaxRhs x (level-0
// blocks per right-hand side) doubles, tickets kMaxRhs counters (zero between
// launches).
struct MgRed {
  double* partials;
  unsigned int* tickets;
  int* err;  // set when a bounded TMA wait gave up
};
long long mg_red_partials(const MgHierarchy& H);
// CTAs of one z-chunk of the level-0 TMA passes (all right-hand sides).
long long mg_tma_ctas_per_chunk(const MixedGrid& G, int nrhs);
// Tensor maps of the level-0 passes (after the level-0 vectors exist).
cudaError_t mg_encode(MgHierarchy& H, const MgVecs& v);
// A launch covers the right-hand sides whose bit is set in mask and whose
// MgScalars::active is set.
cudaError_t mg_setup(MgHierarchy& H, const Dims& d, const int32_t* solid, const Axes& ax, cudaStream_t st);
cudaError_t mg_pcg_start(const MgHierarchy& H, const DPtr4& rv, const double* scale, unsigned mask, MgVecs& v,
                         MgScalars* S, const MgRed& rb, cudaStream_t st);
cudaError_t mg_pcg_iteration(const MgHierarchy& H, MgVecs& v, MgScalars* S, const MgRed& rb, cudaStream_t st);
cudaError_t mg_pcg_apply(const MgHierarchy& H, const Dims& d, const MgVecs& v, const MgScalars* S,
                         const double* scale, unsigned mask, const DPtr4& phi, cudaStream_t st);

// 3-D tensor map with box (b0, b1, 1), no swizzle, zero out-of-bounds fill
// (fpm_jacobi_tma.cu).
bool tma_encode_3d(CUtensorMap* map, CUtensorMapDataType type, void* base, uint64_t d0, uint64_t d1, uint64_t d2,
                   uint64_t stride1_bytes, uint64_t stride2_bytes, uint32_t b0, uint32_t b1);
// Tensor map of `rank` dimensions (dims[0] contiguous; strides[r - 1] is the
// byte stride of dimension r), the given box, no swizzle, zero out-of-bounds
// fill (fpm_jacobi_tma.cu).
bool tma_encode(CUtensorMap* map, CUtensorMapDataType type, int rank, void* base, const uint64_t* dims,
                const uint64_t* strides, const uint32_t* box);

// ---- learned initial guess (fpm_learned.cu, fpm_net.cu) -------------------
cudaError_t launch_learn_inputs(const Dims& d, const double* src, const double* diag, const Axes& ax, uint8_t* fluid,
                                float* mx, float* my, float* mz, float* b, double* bmax, const RedBuf& rb,
                                cudaStream_t st);
cudaError_t launch_learn_apply(const Dims& d, const float* y, const double* src, const double* diag, const Coefs& c,
                               const Axes& ax, double* phi, double* dots, const RedBuf& rb, cudaStream_t st);
cudaError_t launch_energy(const Dims& d, const double* phi, const double* src, const double* diag, const Coefs& c,
                          const Axes& ax, double* out2, const RedBuf& rb, cudaStream_t st);
// Learned flexible CG: work arrays of the preconditioner (compact cell order).
struct FcgWork {
  uint8_t* fluid;            // network inputs prepared once per solve
  float *mx, *my, *mz;
  float *b, *y;              // network input channel (r / max |r|) and output
  double* ay;                // A y_f
  double* sc;                // [0] max |r|, [2..3] (y.r, y.Ay), [4..5] (z.r, z.r_prev)
};
cudaError_t launch_fcg_precond(const Dims& d, void* net, const double* r, const double* rprev, const double* diag,
                               const double* rdiag, const Coefs& c, const Axes& ax, const FcgWork& w, double* z,
                               const RedBuf& rb, cudaStream_t st, std::string* err, int* status);
cudaError_t launch_fcg_direction(const Dims& d, const double* z, double* p, double beta, cudaStream_t st);
cudaError_t launch_fcg_update(const Dims& d, double* phi, const double* p, const double* q, double* r, double* rprev,
                              const SolveScalars* S, cudaStream_t st);
cudaError_t launch_pcg_spmv(const Dims& d, const double* p, double* q, const double* diag, const Coefs& c,
                            const Axes& ax, SolveScalars* S, const RedBuf& rb, cudaStream_t st);
namespace net {
// Network forward pass into out (FP32, one value per cell); returns an FPM_*
// status and fills *err on failure.
int forward_into(void* net, int nx, int ny, int nz, const uint8_t* fluid, const float* mx, const float* my,
                 const float* mz, const float* rhs, float* out, cudaStream_t st, std::string* err);
}  // namespace net

// ---- 3-D four-term partition (fpm_partition3d.cu) --------------------------
struct Part3D {
  const double *phi, *u, *v, *w, *xf, *yf, *zf, *kin, *shell;
  const uint8_t* solid;
  double g[3], dt, nu;
  int nx, ny, nz, slip;
};
cudaError_t launch_partition_3d(const Part3D& p, double* scratch, double* vif, double* omega, SolveScalars* S,
                                const RedBuf& rb, cudaStream_t st);

// ---- error reporting (fpm_capi.cu) ----------------------------------------
void set_error(const std::string& msg);

}  // namespace fpm
