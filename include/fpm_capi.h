/*
 * fpm_capi.h -- C ABI of the GB300 FlowFPM++ hot path (libfpm_gb300.so).
 *
 * Each entry point replaces one procedure of the reference's Fortran API and
 * keeps its argument meaning, order and array layout, so that a Fortran
 * ISO_C_BINDING interface (or ctypes, or any C caller) can pass its arrays
 * through unchanged.  The reference procedure each one replaces is cited as
 * path:line in the reference repository.
 *
 * Conventions
 *  - Arrays are Fortran column-major (x fastest) with the reference's bounds:
 *      padded 3-D  (0:nx+1, 0:ny+1, 1:nz)   phi, solid of the stair-step API
 *      interior    (1:nx, 1:ny, 1:nz)        rhs and all flow / output fields
 *      faces       xlo,xhi(ny,nz) ylo,yhi(nx,nz) zlo,zhi(nx,ny)
 *      axes        xc(0:nx+1) yc(0:ny+1) zc(nz) dx(nx) dy(ny) dz(nz)
 *    solid is int32 (1 solid, 0 fluid).
 *  - One GPU, one rank: every side of the grid is a physical boundary (the
 *    reference's west..north == MPI_PROC_NULL).  Domain decomposition is not
 *    supported; a Fortran shim rejects a communicator with more than one rank.
 *  - Plain entry points take HOST pointers, copy to the GPU, run, copy back
 *    and return when the results are on the host.  Entry points ending in
 *    _dev take DEVICE pointers (cudaMalloc'd) and a cudaStream_t passed as
 *    void* (NULL = default stream); they return after the stream has drained,
 *    with scalar results on the host.
 *  - Every entry point returns FPM_OK (0) or a status code below; the
 *    message is available from fpm_last_error() on the calling thread.  The
 *    reference stops the program (error stop) in the same situations.
 *    Non-convergence is not an error: check the returned residual/sweeps.
 *  - There is no CPU fallback: without a usable GPU every entry point returns
 *    FPM_E_CUDA or FPM_E_NO_DEVICE.
 */
#ifndef FPM_CAPI_H
#define FPM_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define FPM_OK 0
#define FPM_E_METHOD 1        /* 'stair-step method must be pcg or jacobi'                 (fpm_stairstep_mpi_3d.f90:127) */
#define FPM_E_SIZE 2          /* 'stair-step solve needs nz>=2 and nonempty ranks'         (fpm_stairstep_mpi_3d.f90:130),
                                 'nonuniform 3-D FPM kernel requires at least two cells'   (fpm_terms_3d.f90:54) */
#define FPM_E_ISOLATED 3      /* 'stair-step fluid cell has no fluid neighbour'            (fpm_stairstep_mpi_3d.f90:151) */
#define FPM_E_NO_OUTER_FACE 4 /* 'stair-step compatibility needs at least one fluid outer face' (fpm_stairstep_mpi_3d.f90:56) */
#define FPM_E_ARG 5           /* null pointer or invalid argument */
#define FPM_E_CUDA 6          /* CUDA runtime error (message has the CUDA error string) */
#define FPM_E_NO_DEVICE 7     /* no CUDA device visible */
#define FPM_E_LIMIT 8         /* a size exceeds a documented limit */
#define FPM_E_TIMEOUT 9       /* a bounded device-side wait gave up (no GPU hang: the kernel returned) */

/* ---- solver methods (the reference's method='pcg' | 'jacobi') ---------- */
#define FPM_METHOD_PCG 0        /* diagonal PCG, FP64 throughout (reference 'pcg') */
#define FPM_METHOD_JACOBI 1     /* weighted Jacobi 0.2/0.8, FP64, bit-identical per sweep to a serial
                                   -ffp-contract=off evaluation (reference 'jacobi') */
#define FPM_METHOD_JACOBI_DF 2  /* weighted Jacobi in double-float (f32 pair, 48-bit significand)
                                   arithmetic with FP64 residual checks: same iteration, HBM-bound on GB300 */
#define FPM_METHOD_PCG_MIXED 3  /* FP64 iterative refinement (true residual, max-norm test, phi update in FP64)
                                   around FP32 diagonal PCG; max_sweeps caps the FP32 iterations */
#define FPM_METHOD_PCG_MG 4     /* the refinement of FPM_METHOD_PCG_MIXED around FP32 PCG preconditioned by an
                                   aggregation multigrid V-cycle (no reference counterpart) */
#define FPM_METHOD_FCG_LEARNED 5 /* FP64 flexible CG with the learned network as preconditioner (one diagonal
                                    step on what the network leaves); FP64 PCG finishes if it stalls.  Only
                                    through fpm_solve_stairstep_learned_dev (it needs the network) */
#define FPM_METHOD_JACOBI_FMA 6 /* weighted Jacobi 0.2/0.8 in FP64 storage and arithmetic with fused multiply-adds
                                   (the reference's summation order, one rounding per multiply-add); differs
                                   from FPM_METHOD_JACOBI in the last bits, twice as fast on GB300's FP64 pipe */
#define FPM_METHOD_JACOBI_TF 7  /* weighted Jacobi 0.2/0.8 with FP64 storage and triple-float arithmetic on the
                                   FP32 pipe: inputs split exactly into three FP32 limbs, products and sums
                                   error-free down to about 2^-60 relative, each result rounded to FP64 */

/* ---- diagnostics -------------------------------------------------------- */
const char* fpm_last_error(void);
/* Library version as 10000*major + 100*minor + patch. */
int fpm_version(void);
/* CUDA-event timing of the hot loops on the stream they run on (off by
 * default).  fpm_timing_read resolves the recorded events and returns, for
 * kernel `which` (FPM_TIMER_*), the number of launches and their total
 * device time; reset != 0 clears that counter afterwards. */
#define FPM_TIMER_JACOBI_DF 0   /* double-float Jacobi sweep (TMA-streamed) */
#define FPM_TIMER_JACOBI_F64 1  /* FP64 Jacobi sweep (FPM_METHOD_JACOBI or FPM_METHOD_JACOBI_FMA) */
#define FPM_TIMER_PCG_ITER 2    /* one FP64 PCG iteration (three kernels) */
#define FPM_TIMER_PCG_MIXED_ITER 3 /* one FP32 inner PCG iteration over all right-hand sides */
#define FPM_TIMER_FRAMES_ITER 4 /* one batched FP32 PCG iteration over every frame of a 2-D batch */
#define FPM_TIMER_JACOBI_TF 5    /* Jacobi sweep with FP64 storage and triple-float arithmetic (TMA-streamed) */
#define FPM_TIMER_COUNT 6
int fpm_timing_enable(int on);
/* Number of kernels this library has launched in this process. */
long long fpm_kernel_launches(void);
int fpm_timing_read(int which, long long* launches, double* total_ms, int reset);
/* Tile shape (x, y) and planes per CTA the double-float Jacobi autotuner chose
 * for an nx*ny*nz grid (after a double-float run at that size). */
int fpm_jacobi_df_config(int nx, int ny, int nz, int* tile_x, int* tile_y, int* kchunk);
/* Measures the device's FP64 fused multiply-add rate (instructions per
 * second, best of two timed launches of independent FMA chains): the peak of
 * the FP64-pipe roofline that FP64 kernels are reported against.  No
 * reference counterpart (a measurement utility). */
int fpm_measure_fp64_rate(double* instr_per_s, void* stream);
/* Pinned (page-locked) host memory for fast transfers; NULL on failure. */
void* fpm_host_alloc(size_t bytes);
void fpm_host_free(void* p);

/* ---- fpm_stairstep_mpi_3d ----------------------------------------------
 * exchange_solid_halo_3d (src/fpm_stairstep_mpi_3d.f90:25-36): zeroes the
 * physical-boundary halo of solid (padded, host array). */
int fpm_exchange_solid_halo_3d(int32_t* solid, int nx, int ny, int nz);

/* enforce_stairstep_compatibility_3d (src/fpm_stairstep_mpi_3d.f90:41-92):
 * shifts the six outer-face arrays in place by one uniform correction so the
 * outer plus body flux balances the fluid source. */
int fpm_enforce_stairstep_compatibility_3d(const double* rhs, const int32_t* solid, const double* body_grad,
                                           double* xlo, double* xhi, double* ylo, double* yhi, double* zlo,
                                           double* zhi, const double* dx, const double* dy, const double* dz, int nx,
                                           int ny, int nz, double* correction, double* imbalance);
int fpm_enforce_stairstep_compatibility_3d_dev(const double* rhs, const int32_t* solid, const double* body_grad,
                                               double* xlo, double* xhi, double* ylo, double* yhi, double* zlo,
                                               double* zhi, const double* dx, const double* dy, const double* dz,
                                               int nx, int ny, int nz, double* correction, double* imbalance,
                                               void* stream);

/* solve_stairstep_poisson_3d (src/fpm_stairstep_mpi_3d.f90:106-330): solves
 * the stair-step pure-Neumann problem on fluid cells (phi in: initial guess,
 * out: solution with the fluid-volume mean removed).  tolerance < 0 runs
 * exactly max_sweeps iterations.  body_grad has 3 entries (host memory in
 * both forms).  method: FPM_METHOD_*. */
int fpm_solve_stairstep_poisson_3d(double* phi, const double* rhs, const int32_t* solid, const double* body_grad,
                                   const double* xlo, const double* xhi, const double* ylo, const double* yhi,
                                   const double* zlo, const double* zhi, const double* xc, const double* yc,
                                   const double* zc, const double* dx, const double* dy, const double* dz, int nx,
                                   int ny, int nz, double tolerance, int max_sweeps, int check_interval, int method,
                                   int* sweeps, double* residual);
int fpm_solve_stairstep_poisson_3d_dev(double* phi, const double* rhs, const int32_t* solid, const double* body_grad,
                                       const double* xlo, const double* xhi, const double* ylo, const double* yhi,
                                       const double* zlo, const double* zhi, const double* xc, const double* yc,
                                       const double* zc, const double* dx, const double* dy, const double* dz, int nx,
                                       int ny, int nz, double tolerance, int max_sweeps, int check_interval,
                                       int method, int* sweeps, double* residual, void* stream);

/* Several right-hand sides (1..4; e.g. the phi_x, phi_y, phi_z influence
 * fields) on one grid: solve_stairstep_poisson_3d for each, in one call.
 * phi[m], rhs[m] are device pointers; faces[6*m + f] the six face arrays of
 * right-hand side m (xlo, xhi, ylo, yhi, zlo, zhi); body_grads[3*m + q] is host
 * memory; solid and the axes are shared.  FPM_METHOD_PCG_MIXED iterates all
 * right-hand sides together (shared operator reads); the FP64 methods solve
 * them one after the other.  sweeps[m], residual[m] per right-hand side. */
int fpm_solve_stairstep_multi_dev(int nrhs, double* const* phi, const double* const* rhs, const int32_t* solid,
                                  const double* body_grads, const double* const* faces, const double* xc,
                                  const double* yc, const double* zc, const double* dx, const double* dy,
                                  const double* dz, int nx, int ny, int nz, double tolerance, int max_sweeps,
                                  int check_interval, int method, int* sweeps, double* residual, void* stream);

/* stairstep_residual_3d (src/fpm_stairstep_mpi_3d.f90:403-419): independent
 * max-norm residual of L(phi)-f from face gradients. */
int fpm_stairstep_residual_3d(const double* phi, const double* rhs, const int32_t* solid, const double* body_grad,
                              const double* xlo, const double* xhi, const double* ylo, const double* yhi,
                              const double* zlo, const double* zhi, const double* xc, const double* yc,
                              const double* zc, const double* dx, const double* dy, const double* dz, int nx, int ny,
                              int nz, double* value);

/* compute_stairstep_fpm_terms_3d (src/fpm_stairstep_mpi_3d.f90:426-469):
 * gradients, vortex = -(omega x u).grad(phi), advection = -a.grad(phi) and
 * their integrals over fluid cells with centres strictly inside bounds(6). */
int fpm_compute_stairstep_fpm_terms_3d(const double* phi, const double* u, const double* v, const double* w,
                                       const double* ox, const double* oy, const double* oz, const double* ax,
                                       const double* ay, const double* az, const int32_t* solid,
                                       const double* body_grad, const double* xc, const double* yc, const double* zc,
                                       const double* dx, const double* dy, const double* dz, const double* xlo,
                                       const double* xhi, const double* ylo, const double* yhi, const double* zlo,
                                       const double* zhi, const double* bounds, double* gx, double* gy, double* gz,
                                       double* vortex, double* advection, double* totals, int nx, int ny, int nz);
int fpm_compute_stairstep_fpm_terms_3d_dev(const double* phi, const double* u, const double* v, const double* w,
                                           const double* ox, const double* oy, const double* oz, const double* ax,
                                           const double* ay, const double* az, const int32_t* solid,
                                           const double* body_grad, const double* xc, const double* yc,
                                           const double* zc, const double* dx, const double* dy, const double* dz,
                                           const double* xlo, const double* xhi, const double* ylo,
                                           const double* yhi, const double* zlo, const double* zhi,
                                           const double* bounds, double* gx, double* gy, double* gz, double* vortex,
                                           double* advection, double* totals, int nx, int ny, int nz, void* stream);
/* compute_stairstep_fpm_terms_3d (src/fpm_stairstep_mpi_3d.f90:426-497) for
 * npot (1..4) potentials of one grid and flow in one pass, device arrays:
 * the nine flow fields and solid are read once for all potentials.
 * phi[m] (padded), body_grad[3m..3m+2] (host), faces[6m..6m+5] = xlo, xhi,
 * ylo, yhi, zlo, zhi of potential m; outs[5m..5m+4] = gx, gy, gz, vortex,
 * advection; totals[2m], totals[2m+1] (host) = its two integrals.  The
 * per-cell arithmetic is double-float (48-bit significand; densities within
 * about 1e-14 relative of the FP64 evaluation), not bit-identical to the
 * single-potential call. */
int fpm_compute_stairstep_fpm_terms_3d_multi_dev(int npot, const double* const* phi, const double* u,
                                                 const double* v, const double* w, const double* ox,
                                                 const double* oy, const double* oz, const double* ax,
                                                 const double* ay, const double* az, const int32_t* solid,
                                                 const double* body_grad, const double* xc, const double* yc,
                                                 const double* zc, const double* dx, const double* dy,
                                                 const double* dz, const double* const* faces, const double* bounds,
                                                 double* const* outs, double* totals, int nx, int ny, int nz,
                                                 void* stream);


/* ---- fpm_laplace_3d (no body; src/fpm_laplace_3d.f90) -------------------
 * enforce_neumann_compatibility_3d (:9-53): uniform spacing dx, dy, dz. */
int fpm_enforce_neumann_compatibility_3d(const double* rhs, double* xlo, double* xhi, double* ylo, double* yhi,
                                         double* zlo, double* zhi, int nx, int ny, int nz, double dx, double dy,
                                         double dz, double* correction, double* imbalance);
/* solve_neumann_poisson_3d (:55-107): undamped Jacobi with clamped neighbours,
 * mean removal and ghost fill; phi is (0:nx+1, 0:ny+1, 0:nz+1). */
int fpm_solve_neumann_poisson_3d(double* phi, const double* rhs, const double* xlo, const double* xhi,
                                 const double* ylo, const double* yhi, const double* zlo, const double* zhi, int nx,
                                 int ny, int nz, double dx, double dy, double dz, double tolerance, int max_iterations,
                                 int check_interval, int* iterations, double* final_residual);
/* enforce_neumann_compatibility_nonuniform_3d (:150-217). */
int fpm_enforce_neumann_compatibility_nonuniform_3d(const double* rhs, double* xlo, double* xhi, double* ylo,
                                                    double* yhi, double* zlo, double* zhi, const double* dx,
                                                    const double* dy, const double* dz, int nx, int ny, int nz,
                                                    double* correction, double* imbalance);
/* solve_neumann_poisson_nonuniform_3d (:219-293): weighted 0.2/0.8 Jacobi,
 * volume-weighted gauge; phi is (nx, ny, nz), xc(nx), yc(ny), zc(nz). */
int fpm_solve_neumann_poisson_nonuniform_3d(double* phi, const double* rhs, const double* xlo, const double* xhi,
                                            const double* ylo, const double* yhi, const double* zlo,
                                            const double* zhi, const double* xc, const double* yc, const double* zc,
                                            const double* dx, const double* dy, const double* dz, int nx, int ny,
                                            int nz, double tolerance, int max_iterations, int check_interval,
                                            int* iterations, double* final_residual);

/* ---- fpm_terms_3d (no body; src/fpm_terms_3d.f90) -----------------------
 * compute_fpm_terms_uniform_3d (:8-37): central differences on phi
 * (0:nx+1, 0:ny+1, 0:nz+1); fluid is int32 (nx,ny,nz), 1 fluid / 0 masked. */
int fpm_compute_fpm_terms_uniform_3d(const double* phi, const double* u, const double* v, const double* w,
                                     const double* ox, const double* oy, const double* oz, const double* ax,
                                     const double* ay, const double* az, const int32_t* fluid, double* gx, double* gy,
                                     double* gz, double* vortex, double* advection, double* totals, int nx, int ny,
                                     int nz, double dx, double dy, double dz);
/* compute_fpm_terms_nonuniform_3d (:39-88): face-gradient averages with the
 * outer-face data, integrals over cells strictly inside bounds(6);
 * phi (nx,ny,nz), xc(nx), yc(ny), zc(nz).  Needs >= 2 cells per direction. */
int fpm_compute_fpm_terms_nonuniform_3d(const double* phi, const double* u, const double* v, const double* w,
                                        const double* ox, const double* oy, const double* oz, const double* ax,
                                        const double* ay, const double* az, const int32_t* fluid, const double* xc,
                                        const double* yc, const double* zc, const double* dx, const double* dy,
                                        const double* dz, const double* xlo, const double* xhi, const double* ylo,
                                        const double* yhi, const double* zlo, const double* zhi,
                                        const double* bounds, double* gx, double* gy, double* gz, double* vortex,
                                        double* advection, double* totals, int nx, int ny, int nz);

/* ---- fpm_partition_2d (src/fpm_partition_2d.f90:35-154) -----------------
 * fpm_partition_terms_2d: terms[4] = [F_KINE, F_VIF, F_VIS, F_BOUND],
 * vif_density and omega (nx,ny).  phi, u, v (nx,ny); g[2]; solid (nx,ny)
 * uint8, nonzero = solid (the reference's logical); xf(0:nx), yf(0:ny);
 * kin[6]; ring(2nx+2ny, 2, 2); slip_body 0/1. */
int fpm_partition_terms_2d(const double* phi, const double* g, const double* u, const double* v,
                           const uint8_t* solid, const double* xf, const double* yf, const double* kin,
                           const double* ring, double dt, double nu, int nx, int ny, double* terms,
                           double* vif_density, double* omega, int slip_body);

/* ---- 3-D four-term partition ---------------------------------------------
 * The divergence-form force partition of fpm_partition_terms_2d
 * (src/fpm_partition_2d.f90:35-154) on the six faces of every cell of a 3-D
 * stair-step grid (the reference provides it in 2-D only).  phi, u, v, w and
 * solid (uint8, nonzero = solid) are (nx,ny,nz); xf(0:nx), yf(0:ny), zf(0:nz)
 * cell faces; g[3] the body face gradient of phi; kin[12] = rigid body motion
 * about the origin: velocity V(3), angular velocity W(3), acceleration A(3),
 * angular acceleration Al(3) (U_B = V + W x r, a_B = A + Al x r + W x (W x r));
 * shell (L,3,2), L = 2 ny nz + 2 nx nz + 2 nx ny: the velocity of the outer
 * cells (west face (j,k), east, south (i,k), north, bottom (i,j), top) at
 * t - dt and t + dt for Du/Dt on the outer boundary, or NULL for zero.
 * Outputs terms[4] = [F_KINE, F_VIF, F_VIS, F_BOUND], vif_density (nx,ny,nz)
 * and, unless NULL, omega (nx,ny,nz,3). */
int fpm_partition_terms_3d(const double* phi, const double* g, const double* u, const double* v, const double* w,
                           const uint8_t* solid, const double* xf, const double* yf, const double* zf,
                           const double* kin, const double* shell, double dt, double nu, int nx, int ny, int nz,
                           double* terms, double* vif_density, double* omega, int slip_body);

/* ---- batched 2-D frames (examples/flapping_foil_fpm.f90:61-81 per frame) ---
 * For each of nframes independent 2-D frames (cells nx[f] x ny[f], faces
 * xf[f](0:nx), yf[f](0:ny), velocity u[f], v[f] (nx,ny), solid[f] (nx,ny)
 * uint8, ring[f](2nx+2ny,2,2), kin[6f..6f+5], dt[f]): the influence
 * potentials phi_x and phi_y as the reference's foil example computes them
 * (nz = 2, dz = 0.5, zero outer data, compatibility, solve to `tolerance`),
 * then fpm_partition_terms_2d (src/fpm_partition_2d.f90:35-154) for each.
 * All frames are solved together (mixed-precision PCG, FP64 refinement and
 * max-norm test per frame and direction).  Outputs, host memory:
 * terms[8f + 4r + t] (r = 0 x, 1 y; t = KINE, VIF, VIS, BOUND), sweeps[2f + r]
 * (FP32 iterations), residual[2f + r] (final max-norm), and, when phi_out and
 * phi_out[f] are non-NULL, layer 1 of phi_x then phi_y as 2 x (nx,ny). */
int fpm_partition_frames_2d(int nframes, const int* nx, const int* ny, const double* const* xf,
                            const double* const* yf, const double* const* u, const double* const* v,
                            const uint8_t* const* solid, const double* const* ring, const double* kin,
                            const double* dt, double nu, double tolerance, int max_sweeps, int check_interval,
                            double* terms, int* sweeps, double* residual, double* const* phi_out);

/* ---- operator-level entry points (device arrays) ------------------------
 * The private building blocks of solve_stairstep_poisson_3d, exposed so a
 * caller can keep the operator resident and drive sweeps itself.
 * build_operator (src/fpm_stairstep_mpi_3d.f90:336-379): src, diag, rdiag
 * (interior arrays); rdiag = 1/(V diag) if for_pcg else 0.8/diag; *isolated
 * receives the number of fluid cells without a fluid neighbour. */
int fpm_stairstep_build_operator_dev(const double* rhs, const int32_t* solid, const double* body_grad,
                                     const double* xlo, const double* xhi, const double* ylo, const double* yhi,
                                     const double* zlo, const double* zhi, const double* xc, const double* yc,
                                     const double* zc, const double* dx, const double* dy, const double* dz, int nx,
                                     int ny, int nz, int for_pcg, double* src, double* diag, double* rdiag,
                                     int* isolated, void* stream);
/* jacobi_sweep (src/fpm_stairstep_mpi_3d.f90:384-399), nsweeps times,
 * alternating a -> b -> a ...  (padded arrays with zero physical halo and
 * zero solid cells, as after the solver's init loop).  The latest iterate is
 * in a when nsweeps is even, else in b.  method FPM_METHOD_JACOBI (FP64,
 * bit-identical per sweep), FPM_METHOD_JACOBI_FMA (FP64 with fused
 * multiply-adds), FPM_METHOD_JACOBI_TF (FP64 storage, triple-float
 * arithmetic) or FPM_METHOD_JACOBI_DF (double-float arithmetic; for the last
 * two, a and b are copied into and out of the kernel's layout once per call). */
int fpm_stairstep_jacobi_sweeps_dev(double* a, double* b, const double* src, const double* rdiag, const double* xc,
                                    const double* yc, const double* zc, const double* dx, const double* dy,
                                    const double* dz, int nx, int ny, int nz, int nsweeps, int method, void* stream);
/* operator_residual (src/fpm_stairstep_mpi_3d.f90:514-530): max over diag>0
 * of |src + sum(c_nb phi_nb) - diag phi|. */
int fpm_stairstep_operator_residual_dev(const double* phi, const double* src, const double* diag, const double* xc,
                                        const double* yc, const double* zc, const double* dx, const double* dy,
                                        const double* dz, int nx, int ny, int nz, double* value, void* stream);

/* Allocation-free form of fpm_stairstep_operator_residual_dev.  No counterpart
 * in the reference: it exists for callers that cannot allocate GPU memory
 * while they run (a fixed memory pool, an allocator policy that forbids
 * cudaMalloc, or a hard cap on the process's GPU footprint).  It calls no
 * cudaMalloc, cudaFree or allocating library routine: its scratch is a fixed
 * file-scope device array (about 200 KB, held on every GPU that loads the
 * library until the process exits).  Limit: nx + ny + nz <= 12288, else
 * FPM_E_LIMIT.  The first call on a device looks the array's address up
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls share the array, so calls whose GPU
 * work overlaps (different streams or host threads) race: serialise them.
 * Same arguments and result as fpm_stairstep_operator_residual_dev; like it,
 * the call copies the result to *value and waits for the stream before it
 * returns. */
int fpm_stairstep_operator_residual_noalloc_dev(const double* phi, const double* src, const double* diag,
                                                const double* xc, const double* yc, const double* zc,
                                                const double* dx, const double* dy, const double* dz, int nx, int ny,
                                                int nz, double* value, void* stream);

/* ---- learned initial guess (no counterpart in the reference) ---------------
 * A small 3-D convolutional encoder-decoder (4 levels, 16-64 channels, 3x3x3
 * convolutions, BF16 tensor-core kernels with FP32 accumulation, FP32 master
 * weights and Adam) that maps the fluid mask, the cell-size metrics and the
 * right-hand side to an initial guess for the stair-step solve.  Grids must
 * have nx, ny, nz multiples of 8.  All arrays of the _dev functions are
 * device pointers in the solver's compact cell order (x fastest); stream is
 * a cudaStream_t (NULL = legacy default stream).
 *
 * Parameters are exchanged as one flat FP32 array: for each of the 8 layers,
 * its weights [27][cout][cin] (tap t = (dk+1)*9 + (dj+1)*3 + (di+1)) and then
 * its biases [cout]. */
int fpm_net_create(unsigned long long seed, void** net);
int fpm_net_destroy(void* net);
long long fpm_net_param_count(void* net);
int fpm_net_get_params(void* net, float* host, long long n);
int fpm_net_set_params(void* net, const float* host, long long n);
/* Gradients of the last fpm_net_backward_dev / fpm_net_train_step_dev. */
int fpm_net_get_grads(void* net, float* host, long long n);
/* Network inputs of a stair-step problem from its operator (src, diag of
 * fpm_stairstep_build_operator_dev with for_pcg = 1): fluid = diag > 0,
 * mx = w_min / dx (w_min = smallest cell width), my, mz likewise, and
 * b = V src / max |V src| on fluid cells (0 elsewhere). */
int fpm_net_prepare_inputs_dev(const double* src, const double* diag, const double* dx, const double* dy,
                               const double* dz, int nx, int ny, int nz, uint8_t* fluid, float* mx, float* my,
                               float* mz, float* b, void* stream);
/* out (FP32, nx*ny*nz) = network output for the inputs. */
int fpm_net_forward_dev(void* net, int nx, int ny, int nz, const uint8_t* fluid, const float* mx, const float* my,
                        const float* mz, const float* rhs, float* out, void* stream);
/* Forward, loss (1 - cos^2 of the angle between output and target over fluid
 * cells, both with their fluid mean removed) and parameter gradients; no
 * update. */
int fpm_net_backward_dev(void* net, int nx, int ny, int nz, const uint8_t* fluid, const float* mx, const float* my,
                         const float* mz, const float* rhs, const float* target, double* loss, void* stream);
/* fpm_net_backward_dev followed by one Adam step (beta 0.9 / 0.999). */
int fpm_net_train_step_dev(void* net, int nx, int ny, int nz, const uint8_t* fluid, const float* mx,
                           const float* my, const float* mz, const float* rhs, const float* target, float lr,
                           double* loss, void* stream);
/* fpm_solve_stairstep_multi_dev with the network's initial guess: for each
 * right-hand side, phi0 = gamma * net(...) (gamma from the A-norm projection)
 * replaces the caller's phi unless it is not closer to the solution in the
 * energy norm ||phi - phi*||_A (the norm CG minimises, compared through
 * phi.A phi / 2 - phi.b), in which case the caller's phi is kept and
 * fallbacks[m] = 1 (fallbacks may be NULL).  Any method; nx, ny, nz
 * multiples of 8. */
int fpm_solve_stairstep_learned_dev(void* net, int nrhs, double* const* phi, const double* const* rhs,
                                    const int32_t* solid, const double* body_grads, const double* const* faces,
                                    const double* xc, const double* yc, const double* zc, const double* dx,
                                    const double* dy, const double* dz, int nx, int ny, int nz, double tolerance,
                                    int max_sweeps, int check_interval, int method, int* sweeps, double* residual,
                                    int* fallbacks, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FPM_CAPI_H */
