/*
 * fpm_oracle.c -- CPU restatement of FlowFPM++'s hot path, used ONLY as the
 * parity oracle and as the timed CPU baseline (test infrastructure: nothing
 * in the product library links or calls this file).
 *
 * Each function follows the reference Fortran routine named in its comment,
 * loop for loop: same index bounds and clamps, same expression evaluation
 * order (Fortran evaluates left to right; parentheses are written out here),
 * and the serial CPU reduction order (k outer, j, i inner).  Compiled with
 * -ffp-contract=off so no multiply-add is fused, which makes the fixed-work
 * Jacobi sweep bit-for-bit reproducible against any other correctly rounded
 * implementation of the same expression.
 *
 * Parity pins: tests/test_oracle_pins.py checks this restatement against every
 * known answer the reference's own tests and README hold for this path
 * (exact phi = g.x on the 24x20x10 four-body grid with its iteration counts,
 * the manufactured uniform and non-uniform Neumann solutions, the 2-D
 * rotation / uniform-flow / accelerating-cylinder partition cases, the sphere
 * dipole convergence table with its printed RMS, far-field and C_m digits,
 * and the flapping-foil frame terms).
 *
 * Layout (Fortran column-major, x fastest):
 *   padded 3-D  (0:nx+1, 0:ny+1, 1:nz)    phi, next, solid      PH(i,j,k)
 *   interior    (1:nx, 1:ny, 1:nz)         rhs, src, diag, ...   IN(i,j,k)
 *   faces       xlo/xhi(ny,nz) ylo/yhi(nx,nz) zlo/zhi(nx,ny)
 *   axes        xc(0:nx+1) yc(0:ny+1) zc(1:nz) dx(1:nx) dy(1:ny) dz(1:nz)
 * One rank: every side is a physical boundary (MPI_PROC_NULL neighbours), so
 * halo exchanges are no-ops and every MPI_Allreduce is the identity.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PH(i, j, k) ((size_t)(i) + (size_t)(nx + 2) * ((size_t)(j) + (size_t)(ny + 2) * (size_t)((k) - 1)))
#define IN(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1)))
#define XF(j, k) ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1))
#define YF(i, k) ((size_t)((i) - 1) + (size_t)nx * (size_t)((k) - 1))
#define ZF(i, j) ((size_t)((i) - 1) + (size_t)nx * (size_t)((j) - 1))
#define DX(i) dx[(i) - 1]
#define DY(j) dy[(j) - 1]
#define DZ(k) dz[(k) - 1]
#define ZC(k) zc[(k) - 1]

enum { ORC_OK = 0, ORC_E_METHOD = 1, ORC_E_SIZE = 2, ORC_E_ISOLATED = 3, ORC_E_NO_OUTER = 4, ORC_E_ALLOC = 5 };

static int g_threads = 1;
/* Number of OpenMP threads for the loops that are order-independent (the
 * Jacobi sweep, copies, max-norm residuals) and, when > 1, for the sum
 * reductions too (then sums are no longer in serial order). */
void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int orc_get_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* src/fpm_stairstep_mpi_3d.f90:25-36 exchange_solid_halo_3d (one rank):
 * zero the physical-boundary halo of the solid flag. */
void orc_exchange_solid_halo_3d(int32_t *solid, int nx, int ny, int nz) {
    for (int k = 1; k <= nz; k++)
        for (int j = 0; j <= ny + 1; j++) {
            solid[PH(0, j, k)] = 0;
            solid[PH(nx + 1, j, k)] = 0;
        }
    for (int k = 1; k <= nz; k++)
        for (int i = 0; i <= nx + 1; i++) {
            solid[PH(i, 0, k)] = 0;
            solid[PH(i, ny + 1, k)] = 0;
        }
}

/* total_flux, contained in enforce_stairstep_compatibility_3d
 * (src/fpm_stairstep_mpi_3d.f90:69-91). */
static void stairstep_total_flux(const int32_t *solid, const double *bg, const double *xlo, const double *xhi,
                                 const double *ylo, const double *yhi, const double *zlo, const double *zhi,
                                 const double *dx, const double *dy, const double *dz, int nx, int ny, int nz,
                                 double *flux_out, double *area_out) {
    double flux = 0, area = 0, a;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                if (solid[PH(i, j, k)] != 0) continue;
                a = DY(j) * DZ(k);
                if (i == 1) { flux = flux - xlo[XF(j, k)] * a; area = area + a; }
                else if (solid[PH(i - 1, j, k)] != 0) { flux = flux - bg[0] * a; }
                if (i == nx) { flux = flux + xhi[XF(j, k)] * a; area = area + a; }
                else if (solid[PH(i + 1, j, k)] != 0) { flux = flux + bg[0] * a; }
                a = DX(i) * DZ(k);
                if (j == 1) { flux = flux - ylo[YF(i, k)] * a; area = area + a; }
                else if (solid[PH(i, j - 1, k)] != 0) { flux = flux - bg[1] * a; }
                if (j == ny) { flux = flux + yhi[YF(i, k)] * a; area = area + a; }
                else if (solid[PH(i, j + 1, k)] != 0) { flux = flux + bg[1] * a; }
                a = DX(i) * DY(j);
                if (k == 1) { flux = flux - zlo[ZF(i, j)] * a; area = area + a; }
                else if (solid[PH(i, j, k - 1)] != 0) { flux = flux - bg[2] * a; }
                if (k == nz) { flux = flux + zhi[ZF(i, j)] * a; area = area + a; }
                else if (solid[PH(i, j, k + 1)] != 0) { flux = flux + bg[2] * a; }
            }
    *flux_out = flux;
    *area_out = area;
}

/* src/fpm_stairstep_mpi_3d.f90:41-92 enforce_stairstep_compatibility_3d. */
int orc_enforce_stairstep_compatibility_3d(const double *rhs, const int32_t *solid, const double *bg, double *xlo,
                                           double *xhi, double *ylo, double *yhi, double *zlo, double *zhi,
                                           const double *dx, const double *dy, const double *dz, int nx, int ny,
                                           int nz, double *correction, double *imbalance) {
    double source = 0, flux, area, c;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++)
                if (solid[PH(i, j, k)] == 0) source = source + rhs[IN(i, j, k)] * DX(i) * DY(j) * DZ(k);
    stairstep_total_flux(solid, bg, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz, nx, ny, nz, &flux, &area);
    if (area <= 0) return ORC_E_NO_OUTER;
    c = -(flux - source) / area;
    for (size_t m = 0; m < (size_t)ny * nz; m++) { xlo[m] = xlo[m] - c; xhi[m] = xhi[m] + c; }
    for (size_t m = 0; m < (size_t)nx * nz; m++) { ylo[m] = ylo[m] - c; yhi[m] = yhi[m] + c; }
    for (size_t m = 0; m < (size_t)nx * ny; m++) { zlo[m] = zlo[m] - c; zhi[m] = zhi[m] + c; }
    stairstep_total_flux(solid, bg, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz, nx, ny, nz, &flux, &area);
    *correction = c;
    *imbalance = flux - source;
    return ORC_OK;
}

/* src/fpm_stairstep_mpi_3d.f90:499-510 axis_coefficients (both sides physical). */
static void axis_coefficients(const double *center, const double *width, int n, double *cl, double *cu) {
    for (int m = 1; m <= n; m++) {
        cl[m - 1] = 1 / (width[m - 1] * (center[m] - center[m - 1]));
        cu[m - 1] = 1 / (width[m - 1] * (center[m + 1] - center[m]));
    }
    cl[0] = 0;
    cu[n - 1] = 0;
}

/* z coefficients, src/fpm_stairstep_mpi_3d.f90:138-142. */
static void z_coefficients(const double *zc, const double *dz, int nz, double *cb, double *ct) {
    for (int k = 1; k <= nz; k++) {
        cb[k - 1] = 0;
        ct[k - 1] = 0;
        if (k > 1) cb[k - 1] = 1 / (DZ(k) * (ZC(k) - ZC(k - 1)));
        if (k < nz) ct[k - 1] = 1 / (DZ(k) * (ZC(k + 1) - ZC(k)));
    }
}

/* Exported for the kernel-level parity tests: the six 1-D coefficient arrays
 * (cw, ce | cs, cn | cb, ct) the stair-step operator is built from. */
void orc_stairstep_coefficients(const double *xc, const double *yc, const double *zc, const double *dx,
                                const double *dy, const double *dz, int nx, int ny, int nz, double *cw, double *ce,
                                double *cs, double *cn, double *cb, double *ct) {
    axis_coefficients(xc, dx, nx, cw, ce);
    axis_coefficients(yc, dy, ny, cs, cn);
    z_coefficients(zc, dz, nz, cb, ct);
}

/* src/fpm_stairstep_mpi_3d.f90:336-379 build_operator (one rank). */
int orc_build_operator(const double *rhs, const int32_t *solid, const double *bg, const double *xlo,
                       const double *xhi, const double *ylo, const double *yhi, const double *zlo,
                       const double *zhi, const double *cw, const double *ce, const double *cs, const double *cn,
                       const double *cb, const double *ct, const double *dx, const double *dy, const double *dz,
                       int nx, int ny, int nz, int for_pcg, double *src, double *diag, double *rdiag) {
    int isolated = 0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double s = 0, d = 0;
                if (solid[PH(i, j, k)] == 0) {
                    s = -rhs[IN(i, j, k)];
                    if (i == 1) s = s - xlo[XF(j, k)] / DX(i);
                    else if (solid[PH(i - 1, j, k)] != 0) s = s - bg[0] / DX(i);
                    else d = d + cw[i - 1];
                    if (i == nx) s = s + xhi[XF(j, k)] / DX(i);
                    else if (solid[PH(i + 1, j, k)] != 0) s = s + bg[0] / DX(i);
                    else d = d + ce[i - 1];
                    if (j == 1) s = s - ylo[YF(i, k)] / DY(j);
                    else if (solid[PH(i, j - 1, k)] != 0) s = s - bg[1] / DY(j);
                    else d = d + cs[j - 1];
                    if (j == ny) s = s + yhi[YF(i, k)] / DY(j);
                    else if (solid[PH(i, j + 1, k)] != 0) s = s + bg[1] / DY(j);
                    else d = d + cn[j - 1];
                    if (k == 1) s = s - zlo[ZF(i, j)] / DZ(k);
                    else if (solid[PH(i, j, k - 1)] != 0) s = s - bg[2] / DZ(k);
                    else d = d + cb[k - 1];
                    if (k == nz) s = s + zhi[ZF(i, j)] / DZ(k);
                    else if (solid[PH(i, j, k + 1)] != 0) s = s + bg[2] / DZ(k);
                    else d = d + ct[k - 1];
                    if (d <= 0) isolated++;
                }
                size_t c = IN(i, j, k);
                src[c] = s;
                diag[c] = d;
                if (d <= 0) rdiag[c] = 0;
                else if (for_pcg) rdiag[c] = 1 / (DX(i) * DY(j) * DZ(k) * d);
                else rdiag[c] = 0.8 / d;
            }
    return isolated;
}

/* src/fpm_stairstep_mpi_3d.f90:384-399 jacobi_sweep: a -> b over the interior. */
void orc_jacobi_sweep(const double *a, double *b, const double *src, const double *rdiag, const double *cw,
                      const double *ce, const double *cs, const double *cn, const double *cb, const double *ct,
                      int nx, int ny, int nz) {
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
    for (int k = 1; k <= nz; k++) {
        int kb = k - 1 < 1 ? 1 : k - 1, kt = k + 1 > nz ? nz : k + 1;
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                size_t c = IN(i, j, k);
                double s = src[c] + cw[i - 1] * a[PH(i - 1, j, k)];
                s = s + ce[i - 1] * a[PH(i + 1, j, k)];
                s = s + cs[j - 1] * a[PH(i, j - 1, k)];
                s = s + cn[j - 1] * a[PH(i, j + 1, k)];
                s = s + cb[k - 1] * a[PH(i, j, kb)];
                s = s + ct[k - 1] * a[PH(i, j, kt)];
                b[PH(i, j, k)] = 0.2 * a[PH(i, j, k)] + rdiag[c] * s;
            }
    }
}

/* src/fpm_stairstep_mpi_3d.f90:514-530 operator_residual: max over diag>0 of
 * |src + sum(c_nb phi_nb) - diag phi|.  (A NaN never exceeds the running max,
 * matching the reference's remark that max() may drop it.) */
double orc_operator_residual(const double *phi, const double *src, const double *diag, const double *cw,
                             const double *ce, const double *cs, const double *cn, const double *cb,
                             const double *ct, int nx, int ny, int nz) {
    double value = 0;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1) reduction(max : value)
    for (int k = 1; k <= nz; k++) {
        int kb = k - 1 < 1 ? 1 : k - 1, kt = k + 1 > nz ? nz : k + 1;
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                size_t c = IN(i, j, k);
                if (diag[c] > 0) {
                    double t = src[c] + cw[i - 1] * phi[PH(i - 1, j, k)];
                    t = t + ce[i - 1] * phi[PH(i + 1, j, k)];
                    t = t + cs[j - 1] * phi[PH(i, j - 1, k)];
                    t = t + cn[j - 1] * phi[PH(i, j + 1, k)];
                    t = t + cb[k - 1] * phi[PH(i, j, kb)];
                    t = t + ct[k - 1] * phi[PH(i, j, kt)];
                    t = t - diag[c] * phi[PH(i, j, k)];
                    t = fabs(t);
                    if (t > value) value = t;
                }
            }
    }
    return value;
}

typedef struct {
    int nx, ny, nz, check_interval, max_sweeps;
    double tolerance;
    double *phi, *next, *src, *diag, *rdiag, *r, *q;
    const double *cw, *ce, *cs, *cn, *cb, *ct, *dx, *dy, *dz;
    int sweeps;
    double residual;
} solve_state;

/* jacobi_iterate, src/fpm_stairstep_mpi_3d.f90:200-225. */
static void jacobi_iterate(solve_state *S) {
    int nx = S->nx, ny = S->ny, nz = S->nz;
    while (S->sweeps < S->max_sweeps && S->residual > S->tolerance) {
        int ci = S->check_interval < 1 ? 1 : S->check_interval;
        int nsteps = ci < S->max_sweeps - S->sweeps ? ci : S->max_sweeps - S->sweeps;
        for (int step = 1; step <= nsteps; step++) {
            if (step % 2 == 1)
                orc_jacobi_sweep(S->phi, S->next, S->src, S->rdiag, S->cw, S->ce, S->cs, S->cn, S->cb, S->ct, nx,
                                 ny, nz);
            else
                orc_jacobi_sweep(S->next, S->phi, S->src, S->rdiag, S->cw, S->ce, S->cs, S->cn, S->cb, S->ct, nx,
                                 ny, nz);
            S->sweeps++;
        }
        if (nsteps % 2 == 1) {
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
            for (int k = 1; k <= nz; k++)
                for (int j = 1; j <= ny; j++)
                    for (int i = 1; i <= nx; i++) S->phi[PH(i, j, k)] = S->next[PH(i, j, k)];
        }
        S->residual = orc_operator_residual(S->phi, S->src, S->diag, S->cw, S->ce, S->cs, S->cn, S->cb, S->ct, nx,
                                            ny, nz);
    }
}

/* true_residual, src/fpm_stairstep_mpi_3d.f90:297-329. */
static void true_residual(solve_state *S, int reset, double *rz_out, double *res_out) {
    int nx = S->nx, ny = S->ny, nz = S->nz;
    const double *phi = S->phi, *src = S->src, *diag = S->diag, *rdiag = S->rdiag;
    const double *cw = S->cw, *ce = S->ce, *cs = S->cs, *cn = S->cn, *cb = S->cb, *ct = S->ct;
    const double *dx = S->dx, *dy = S->dy, *dz = S->dz;
    double *r = S->r, *next = S->next;
    *res_out = orc_operator_residual(phi, src, diag, cw, ce, cs, cn, cb, ct, nx, ny, nz);
    double red1 = 0, red2 = 0;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1) reduction(+ : red1, red2)
    for (int k = 1; k <= nz; k++) {
        int kb = k - 1 < 1 ? 1 : k - 1, kt = k + 1 > nz ? nz : k + 1;
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                size_t c = IN(i, j, k);
                r[c] = 0;
                if (diag[c] > 0) {
                    double vol = DX(i) * DY(j) * DZ(k);
                    double t = src[c] + cw[i - 1] * phi[PH(i - 1, j, k)];
                    t = t + ce[i - 1] * phi[PH(i + 1, j, k)];
                    t = t + cs[j - 1] * phi[PH(i, j - 1, k)];
                    t = t + cn[j - 1] * phi[PH(i, j + 1, k)];
                    t = t + cb[k - 1] * phi[PH(i, j, kb)];
                    t = t + ct[k - 1] * phi[PH(i, j, kt)];
                    t = t - diag[c] * phi[PH(i, j, k)];
                    r[c] = vol * t;
                    red1 = red1 + r[c];
                    red2 = red2 + 1;
                }
            }
    }
    double shift = red1 / red2, rz = 0;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1) reduction(+ : rz)
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                size_t c = IN(i, j, k);
                if (diag[c] > 0) r[c] = r[c] - shift;
                if (reset) next[PH(i, j, k)] = rdiag[c] * r[c];
                rz = rz + rdiag[c] * r[c] * r[c];
            }
    *rz_out = rz;
}

/* pcg_iterate, src/fpm_stairstep_mpi_3d.f90:235-293. */
static void pcg_iterate(solve_state *S) {
    int nx = S->nx, ny = S->ny, nz = S->nz;
    double *phi = S->phi, *next = S->next, *r = S->r, *q = S->q;
    const double *diag = S->diag, *rdiag = S->rdiag;
    const double *cw = S->cw, *ce = S->ce, *cs = S->cs, *cn = S->cn, *cb = S->cb, *ct = S->ct;
    const double *dx = S->dx, *dy = S->dy, *dz = S->dz;
    double rz, rz_new, pq, alpha, beta, res, best;
    int it, restarts, stalled;
    true_residual(S, 1, &rz, &res);
    it = 0;
    restarts = 0;
    stalled = 0;
    best = res;
    while (S->sweeps < S->max_sweeps && res > S->tolerance) {
        pq = 0;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1) reduction(+ : pq)
        for (int k = 1; k <= nz; k++) {
            int kb = k - 1 < 1 ? 1 : k - 1, kt = k + 1 > nz ? nz : k + 1;
            for (int j = 1; j <= ny; j++)
                for (int i = 1; i <= nx; i++) {
                    size_t c = IN(i, j, k);
                    double vol = DX(i) * DY(j) * DZ(k);
                    double t = diag[c] * next[PH(i, j, k)] - cw[i - 1] * next[PH(i - 1, j, k)];
                    t = t - ce[i - 1] * next[PH(i + 1, j, k)];
                    t = t - cs[j - 1] * next[PH(i, j - 1, k)];
                    t = t - cn[j - 1] * next[PH(i, j + 1, k)];
                    t = t - cb[k - 1] * next[PH(i, j, kb)];
                    t = t - ct[k - 1] * next[PH(i, j, kt)];
                    q[c] = diag[c] > 0 ? vol * t : 0.0;
                    pq = pq + next[PH(i, j, k)] * q[c];
                }
        }
        if (!(pq > 0) || !(rz > 0)) {
            restarts++;
            if (restarts > 1) break;
            true_residual(S, 1, &rz, &res);
            continue;
        }
        restarts = 0;
        alpha = rz / pq;
        rz_new = 0;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1) reduction(+ : rz_new)
        for (int k = 1; k <= nz; k++)
            for (int j = 1; j <= ny; j++)
                for (int i = 1; i <= nx; i++) {
                    size_t c = IN(i, j, k), p = PH(i, j, k);
                    phi[p] = phi[p] + alpha * next[p];
                    r[c] = r[c] - alpha * q[c];
                    rz_new = rz_new + rdiag[c] * r[c] * r[c];
                }
        if (!(rz_new >= 0)) break;
        beta = rz_new / rz;
        rz = rz_new;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
        for (int k = 1; k <= nz; k++)
            for (int j = 1; j <= ny; j++)
                for (int i = 1; i <= nx; i++) {
                    size_t c = IN(i, j, k), p = PH(i, j, k);
                    next[p] = rdiag[c] * r[c] + beta * next[p];
                }
        S->sweeps++;
        it++;
        int ci = S->check_interval < 1 ? 1 : S->check_interval;
        if (it % ci == 0 || S->sweeps == S->max_sweeps) {
            true_residual(S, 0, &rz, &res);
            if (res < 0.99 * best) { best = res; stalled = 0; }
            else stalled++;
            if (stalled >= 50 || !(res == res)) break;
        }
    }
    S->residual = res;
}

/* src/fpm_stairstep_mpi_3d.f90:106-330 solve_stairstep_poisson_3d (one rank).
 * method: 0 = 'pcg', 1 = 'jacobi'.  Returns 0, or an error code mirroring the
 * reference's error stops (bad method, nz<2/empty, isolated fluid cell). */
int orc_solve_stairstep_poisson_3d(double *phi, const double *rhs, const int32_t *solid, const double *bg,
                                   const double *xlo, const double *xhi, const double *ylo, const double *yhi,
                                   const double *zlo, const double *zhi, const double *xc, const double *yc,
                                   const double *zc, const double *dx, const double *dy, const double *dz, int nx,
                                   int ny, int nz, double tolerance, int max_sweeps, int check_interval, int method,
                                   int *sweeps, double *residual) {
    if (method != 0 && method != 1) return ORC_E_METHOD;
    if (nx < 1 || ny < 1 || nz < 2) return ORC_E_SIZE;
    int use_pcg = method == 0;
    size_t nh = (size_t)(nx + 2) * (ny + 2) * nz, ni = (size_t)nx * ny * nz;
    solve_state S;
    memset(&S, 0, sizeof(S));
    S.nx = nx; S.ny = ny; S.nz = nz;
    S.check_interval = check_interval; S.max_sweeps = max_sweeps; S.tolerance = tolerance;
    S.phi = phi;
    S.next = (double *)malloc(nh * sizeof(double));
    S.src = (double *)malloc(ni * sizeof(double));
    S.diag = (double *)malloc(ni * sizeof(double));
    S.rdiag = (double *)malloc(ni * sizeof(double));
    S.r = use_pcg ? (double *)malloc(ni * sizeof(double)) : NULL;
    S.q = use_pcg ? (double *)malloc(ni * sizeof(double)) : NULL;
    double *coef = (double *)malloc((size_t)(2 * nx + 2 * ny + 2 * nz) * sizeof(double));
    if (!S.next || !S.src || !S.diag || !S.rdiag || !coef || (use_pcg && (!S.r || !S.q))) {
        free(S.next); free(S.src); free(S.diag); free(S.rdiag); free(S.r); free(S.q); free(coef);
        return ORC_E_ALLOC;
    }
    double *cw = coef, *ce = cw + nx, *cs = ce + nx, *cn = cs + ny, *cb = cn + ny, *ct = cb + nz;
    axis_coefficients(xc, dx, nx, cw, ce);
    axis_coefficients(yc, dy, ny, cs, cn);
    z_coefficients(zc, dz, nz, cb, ct);
    S.cw = cw; S.ce = ce; S.cs = cs; S.cn = cn; S.cb = cb; S.ct = ct;
    S.dx = dx; S.dy = dy; S.dz = dz;
    S.sweeps = 0;
    S.residual = HUGE_VAL;
    int err = ORC_OK;
    int isolated = orc_build_operator(rhs, solid, bg, xlo, xhi, ylo, yhi, zlo, zhi, cw, ce, cs, cn, cb, ct, dx, dy,
                                      dz, nx, ny, nz, use_pcg, S.src, S.diag, S.rdiag);
    if (isolated > 0) { err = ORC_E_ISOLATED; goto done; }
    /* init loop, :154-160 */
    for (int k = 1; k <= nz; k++)
        for (int j = 0; j <= ny + 1; j++)
            for (int i = 0; i <= nx + 1; i++) {
                size_t p = PH(i, j, k);
                if (solid[p] != 0 || i == 0 || i == nx + 1 || j == 0 || j == ny + 1) phi[p] = 0;
                S.next[p] = phi[p];
            }
    if (use_pcg) pcg_iterate(&S);
    else jacobi_iterate(&S);
    /* gauge, :170-187 */
    {
        double l1 = 0, l2 = 0;
        for (int k = 1; k <= nz; k++)
            for (int j = 1; j <= ny; j++)
                for (int i = 1; i <= nx; i++)
                    if (solid[PH(i, j, k)] == 0) {
                        l1 = l1 + phi[PH(i, j, k)] * DX(i) * DY(j) * DZ(k);
                        l2 = l2 + DX(i) * DY(j) * DZ(k);
                    }
        double mean_value = l1 / l2;
        for (int k = 1; k <= nz; k++)
            for (int j = 1; j <= ny; j++)
                for (int i = 1; i <= nx; i++)
                    if (solid[PH(i, j, k)] == 0) phi[PH(i, j, k)] = phi[PH(i, j, k)] - mean_value;
        S.residual = orc_operator_residual(phi, S.src, S.diag, cw, ce, cs, cn, cb, ct, nx, ny, nz);
    }
done:
    *sweeps = S.sweeps;
    *residual = S.residual;
    free(S.next); free(S.src); free(S.diag); free(S.rdiag); free(S.r); free(S.q); free(coef);
    return err;
}

/* face_gradients, src/fpm_stairstep_mpi_3d.f90:472-497 (one rank). */
static void face_gradients(const double *phi, const int32_t *solid, const double *bg, const double *xlo,
                           const double *xhi, const double *ylo, const double *yhi, const double *zlo,
                           const double *zhi, const double *xc, const double *yc, const double *zc, int nx, int ny,
                           int nz, int i, int j, int k, double *g) {
    if (i == 1) g[0] = xlo[XF(j, k)];
    else if (solid[PH(i - 1, j, k)] != 0) g[0] = bg[0];
    else g[0] = (phi[PH(i, j, k)] - phi[PH(i - 1, j, k)]) / (xc[i] - xc[i - 1]);
    if (i == nx) g[1] = xhi[XF(j, k)];
    else if (solid[PH(i + 1, j, k)] != 0) g[1] = bg[0];
    else g[1] = (phi[PH(i + 1, j, k)] - phi[PH(i, j, k)]) / (xc[i + 1] - xc[i]);
    if (j == 1) g[2] = ylo[YF(i, k)];
    else if (solid[PH(i, j - 1, k)] != 0) g[2] = bg[1];
    else g[2] = (phi[PH(i, j, k)] - phi[PH(i, j - 1, k)]) / (yc[j] - yc[j - 1]);
    if (j == ny) g[3] = yhi[YF(i, k)];
    else if (solid[PH(i, j + 1, k)] != 0) g[3] = bg[1];
    else g[3] = (phi[PH(i, j + 1, k)] - phi[PH(i, j, k)]) / (yc[j + 1] - yc[j]);
    if (k == 1) g[4] = zlo[ZF(i, j)];
    else if (solid[PH(i, j, k - 1)] != 0) g[4] = bg[2];
    else g[4] = (phi[PH(i, j, k)] - phi[PH(i, j, k - 1)]) / (ZC(k) - ZC(k - 1));
    if (k == nz) g[5] = zhi[ZF(i, j)];
    else if (solid[PH(i, j, k + 1)] != 0) g[5] = bg[2];
    else g[5] = (phi[PH(i, j, k + 1)] - phi[PH(i, j, k)]) / (ZC(k + 1) - ZC(k));
}

/* src/fpm_stairstep_mpi_3d.f90:403-419 stairstep_residual_3d. */
double orc_stairstep_residual_3d(const double *phi, const double *rhs, const int32_t *solid, const double *bg,
                                 const double *xlo, const double *xhi, const double *ylo, const double *yhi,
                                 const double *zlo, const double *zhi, const double *xc, const double *yc,
                                 const double *zc, const double *dx, const double *dy, const double *dz, int nx,
                                 int ny, int nz) {
    double local = 0, g[6];
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                if (solid[PH(i, j, k)] != 0) continue;
                face_gradients(phi, solid, bg, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, nx, ny, nz, i, j, k, g);
                double t = (g[1] - g[0]) / DX(i) + (g[3] - g[2]) / DY(j) + (g[5] - g[4]) / DZ(k) - rhs[IN(i, j, k)];
                t = fabs(t);
                if (t > local) local = t;
            }
    return local;
}

/* src/fpm_stairstep_mpi_3d.f90:426-469 compute_stairstep_fpm_terms_3d. */
void orc_compute_stairstep_fpm_terms_3d(const double *phi, const double *u, const double *v, const double *w,
                                        const double *ox, const double *oy, const double *oz, const double *ax,
                                        const double *ay, const double *az, const int32_t *solid, const double *bg,
                                        const double *xc, const double *yc, const double *zc, const double *dx,
                                        const double *dy, const double *dz, const double *xlo, const double *xhi,
                                        const double *ylo, const double *yhi, const double *zlo, const double *zhi,
                                        const double *bounds, double *gx, double *gy, double *gz, double *vortex,
                                        double *advection, double *totals, int nx, int ny, int nz) {
    double vt = 0, at = 0, g[6];
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                size_t c = IN(i, j, k);
                face_gradients(phi, solid, bg, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, nx, ny, nz, i, j, k, g);
                double mask = solid[PH(i, j, k)] == 0 ? 1.0 : 0.0;
                gx[c] = mask * 0.5 * (g[0] + g[1]);
                gy[c] = mask * 0.5 * (g[2] + g[3]);
                gz[c] = mask * 0.5 * (g[4] + g[5]);
                double cx = w[c] * oy[c] - v[c] * oz[c];
                double cy = u[c] * oz[c] - w[c] * ox[c];
                double cz = v[c] * ox[c] - u[c] * oy[c];
                vortex[c] = -(cx * gx[c] + cy * gy[c] + cz * gz[c]);
                advection[c] = -(ax[c] * gx[c] + ay[c] * gy[c] + az[c] * gz[c]);
                int inside = xc[i] > bounds[0] && xc[i] < bounds[1] && yc[j] > bounds[2] && yc[j] < bounds[3] &&
                             ZC(k) > bounds[4] && ZC(k) < bounds[5];
                double volume = inside ? DX(i) * DY(j) * DZ(k) : 0.0;
                vt = vt + volume * vortex[c];
                at = at + volume * advection[c];
            }
    totals[0] = vt;
    totals[1] = at;
}

/* ---------------- fpm_laplace_3d (no body) ---------------- */
#define P3(i, j, k) ((size_t)(i) + (size_t)(nx + 2) * ((size_t)(j) + (size_t)(ny + 2) * (size_t)(k)))

/* src/fpm_laplace_3d.f90:9-53 enforce_neumann_compatibility_3d. */
void orc_enforce_neumann_compatibility_3d(const double *rhs, double *xlo, double *xhi, double *ylo, double *yhi,
                                          double *zlo, double *zhi, int nx, int ny, int nz, double dx, double dy,
                                          double dz, double *correction, double *imbalance) {
    double source = 0, flux = 0, area, c;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) source = source + rhs[IN(i, j, k)] * dx * dy * dz;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) flux = flux + (-xlo[XF(j, k)] + xhi[XF(j, k)]) * dy * dz;
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) flux = flux + (-ylo[YF(i, k)] + yhi[YF(i, k)]) * dx * dz;
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) flux = flux + (-zlo[ZF(i, j)] + zhi[ZF(i, j)]) * dx * dy;
    area = 2.0 * ((double)(ny * nz) * dy * dz + (double)(nx * nz) * dx * dz + (double)(nx * ny) * dx * dy);
    c = -(flux - source) / area;
    for (size_t m = 0; m < (size_t)ny * nz; m++) { xlo[m] = xlo[m] - c; xhi[m] = xhi[m] + c; }
    for (size_t m = 0; m < (size_t)nx * nz; m++) { ylo[m] = ylo[m] - c; yhi[m] = yhi[m] + c; }
    for (size_t m = 0; m < (size_t)nx * ny; m++) { zlo[m] = zlo[m] - c; zhi[m] = zhi[m] + c; }
    flux = 0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) flux = flux + (-xlo[XF(j, k)] + xhi[XF(j, k)]) * dy * dz;
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) flux = flux + (-ylo[YF(i, k)] + yhi[YF(i, k)]) * dx * dz;
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) flux = flux + (-zlo[ZF(i, j)] + zhi[ZF(i, j)]) * dx * dy;
    *correction = c;
    *imbalance = flux - source;
}

/* src/fpm_laplace_3d.f90:109-132 residual_norm. */
double orc_residual_norm_uniform(const double *phi, const double *rhs, const double *xlo, const double *xhi,
                                 const double *ylo, const double *yhi, const double *zlo, const double *zhi, int nx,
                                 int ny, int nz, double dx, double dy, double dz) {
    double value = 0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double p = phi[P3(i, j, k)];
                double xm = phi[P3(i - 1 < 1 ? 1 : i - 1, j, k)], xp = phi[P3(i + 1 > nx ? nx : i + 1, j, k)];
                double ym = phi[P3(i, j - 1 < 1 ? 1 : j - 1, k)], yp = phi[P3(i, j + 1 > ny ? ny : j + 1, k)];
                double zm = phi[P3(i, j, k - 1 < 1 ? 1 : k - 1)], zp = phi[P3(i, j, k + 1 > nz ? nz : k + 1)];
                if (i == 1) xm = p - xlo[XF(j, k)] * dx;
                if (i == nx) xp = p + xhi[XF(j, k)] * dx;
                if (j == 1) ym = p - ylo[YF(i, k)] * dy;
                if (j == ny) yp = p + yhi[YF(i, k)] * dy;
                if (k == 1) zm = p - zlo[ZF(i, j)] * dz;
                if (k == nz) zp = p + zhi[ZF(i, j)] * dz;
                double res = (xm - 2.0 * p + xp) / (dx * dx) + (ym - 2.0 * p + yp) / (dy * dy) +
                             (zm - 2.0 * p + zp) / (dz * dz) - rhs[IN(i, j, k)];
                res = fabs(res);
                if (res > value) value = res;
            }
    return value;
}

/* src/fpm_laplace_3d.f90:55-107 solve_neumann_poisson_3d: undamped Jacobi with
 * clamped neighbours and copy-back, unweighted mean gauge, ghost fill.
 * phi is (0:nx+1, 0:ny+1, 0:nz+1). */
void orc_solve_neumann_poisson_3d(double *phi, const double *rhs, const double *xlo, const double *xhi,
                                  const double *ylo, const double *yhi, const double *zlo, const double *zhi, int nx,
                                  int ny, int nz, double dx, double dy, double dz, double tolerance,
                                  int max_iterations, int check_interval, int *iterations, double *final_residual) {
    size_t ni = (size_t)nx * ny * nz;
    double *next = (double *)calloc(ni, sizeof(double));
    double idx2 = 1.0 / (dx * dx), idy2 = 1.0 / (dy * dy), idz2 = 1.0 / (dz * dz);
    double invdiag = 1.0 / (2.0 * (idx2 + idy2 + idz2));
    int it = 0;
    double fr = HUGE_VAL;
    while (it < max_iterations && fr > tolerance) {
        int ci = check_interval < 1 ? 1 : check_interval;
        int nsteps = ci < max_iterations - it ? ci : max_iterations - it;
        for (int step = 1; step <= nsteps; step++) {
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
            for (int k = 1; k <= nz; k++)
                for (int j = 1; j <= ny; j++)
                    for (int i = 1; i <= nx; i++) {
                        double p = phi[P3(i, j, k)];
                        double xm = phi[P3(i - 1 < 1 ? 1 : i - 1, j, k)], xp = phi[P3(i + 1 > nx ? nx : i + 1, j, k)];
                        double ym = phi[P3(i, j - 1 < 1 ? 1 : j - 1, k)], yp = phi[P3(i, j + 1 > ny ? ny : j + 1, k)];
                        double zm = phi[P3(i, j, k - 1 < 1 ? 1 : k - 1)], zp = phi[P3(i, j, k + 1 > nz ? nz : k + 1)];
                        if (i == 1) xm = p - xlo[XF(j, k)] * dx;
                        if (i == nx) xp = p + xhi[XF(j, k)] * dx;
                        if (j == 1) ym = p - ylo[YF(i, k)] * dy;
                        if (j == ny) yp = p + yhi[YF(i, k)] * dy;
                        if (k == 1) zm = p - zlo[ZF(i, j)] * dz;
                        if (k == nz) zp = p + zhi[ZF(i, j)] * dz;
                        next[IN(i, j, k)] =
                            ((xm + xp) * idx2 + (ym + yp) * idy2 + (zm + zp) * idz2 - rhs[IN(i, j, k)]) * invdiag;
                    }
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
            for (int k = 1; k <= nz; k++)
                for (int j = 1; j <= ny; j++)
                    for (int i = 1; i <= nx; i++) phi[P3(i, j, k)] = next[IN(i, j, k)];
            it++;
        }
        fr = orc_residual_norm_uniform(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, nx, ny, nz, dx, dy, dz);
    }
    double mean_value = 0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) mean_value = mean_value + phi[P3(i, j, k)];
    mean_value = mean_value / (double)(nx * ny * nz);
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) phi[P3(i, j, k)] = phi[P3(i, j, k)] - mean_value;
    /* set_ghosts, :134-148 */
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) {
            phi[P3(0, j, k)] = phi[P3(1, j, k)] - xlo[XF(j, k)] * dx;
            phi[P3(nx + 1, j, k)] = phi[P3(nx, j, k)] + xhi[XF(j, k)] * dx;
        }
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) {
            phi[P3(i, 0, k)] = phi[P3(i, 1, k)] - ylo[YF(i, k)] * dy;
            phi[P3(i, ny + 1, k)] = phi[P3(i, ny, k)] + yhi[YF(i, k)] * dy;
        }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            phi[P3(i, j, 0)] = phi[P3(i, j, 1)] - zlo[ZF(i, j)] * dz;
            phi[P3(i, j, nz + 1)] = phi[P3(i, j, nz)] + zhi[ZF(i, j)] * dz;
        }
    fr = orc_residual_norm_uniform(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, nx, ny, nz, dx, dy, dz);
    *iterations = it;
    *final_residual = fr;
    free(next);
}

/* src/fpm_laplace_3d.f90:150-217 enforce_neumann_compatibility_nonuniform_3d. */
void orc_enforce_neumann_compatibility_nonuniform_3d(const double *rhs, double *xlo, double *xhi, double *ylo,
                                                     double *yhi, double *zlo, double *zhi, const double *dx,
                                                     const double *dy, const double *dz, int nx, int ny, int nz,
                                                     double *correction, double *imbalance) {
    double source = 0, flux = 0, area = 0, c;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) source = source + rhs[IN(i, j, k)] * DX(i) * DY(j) * DZ(k);
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) {
            flux = flux + (-xlo[XF(j, k)] + xhi[XF(j, k)]) * DY(j) * DZ(k);
            area = area + 2.0 * DY(j) * DZ(k);
        }
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) {
            flux = flux + (-ylo[YF(i, k)] + yhi[YF(i, k)]) * DX(i) * DZ(k);
            area = area + 2.0 * DX(i) * DZ(k);
        }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            flux = flux + (-zlo[ZF(i, j)] + zhi[ZF(i, j)]) * DX(i) * DY(j);
            area = area + 2.0 * DX(i) * DY(j);
        }
    c = -(flux - source) / area;
    for (size_t m = 0; m < (size_t)ny * nz; m++) { xlo[m] = xlo[m] - c; xhi[m] = xhi[m] + c; }
    for (size_t m = 0; m < (size_t)nx * nz; m++) { ylo[m] = ylo[m] - c; yhi[m] = yhi[m] + c; }
    for (size_t m = 0; m < (size_t)nx * ny; m++) { zlo[m] = zlo[m] - c; zhi[m] = zhi[m] + c; }
    flux = 0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) flux = flux + (-xlo[XF(j, k)] + xhi[XF(j, k)]) * DY(j) * DZ(k);
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) flux = flux + (-ylo[YF(i, k)] + yhi[YF(i, k)]) * DX(i) * DZ(k);
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) flux = flux + (-zlo[ZF(i, j)] + zhi[ZF(i, j)]) * DX(i) * DY(j);
    *correction = c;
    *imbalance = flux - source;
}

#define Q3(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1)))

/* src/fpm_laplace_3d.f90:295-315 residual_nonuniform.  phi is (nx,ny,nz) and
 * xc(nx), yc(ny), zc(nz) carry no halo here. */
double orc_residual_nonuniform(const double *phi, const double *rhs, const double *xlo, const double *xhi,
                               const double *ylo, const double *yhi, const double *zlo, const double *zhi,
                               const double *xc, const double *yc, const double *zc, const double *dx,
                               const double *dy, const double *dz, int nx, int ny, int nz) {
    double value = 0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double gw, ge, gs, gn, gb, gt;
                double p = phi[Q3(i, j, k)];
                if (i == 1) gw = xlo[XF(j, k)]; else gw = (p - phi[Q3(i - 1, j, k)]) / (xc[i - 1] - xc[i - 2]);
                if (i == nx) ge = xhi[XF(j, k)]; else ge = (phi[Q3(i + 1, j, k)] - p) / (xc[i] - xc[i - 1]);
                if (j == 1) gs = ylo[YF(i, k)]; else gs = (p - phi[Q3(i, j - 1, k)]) / (yc[j - 1] - yc[j - 2]);
                if (j == ny) gn = yhi[YF(i, k)]; else gn = (phi[Q3(i, j + 1, k)] - p) / (yc[j] - yc[j - 1]);
                if (k == 1) gb = zlo[ZF(i, j)]; else gb = (p - phi[Q3(i, j, k - 1)]) / (zc[k - 1] - zc[k - 2]);
                if (k == nz) gt = zhi[ZF(i, j)]; else gt = (phi[Q3(i, j, k + 1)] - p) / (zc[k] - zc[k - 1]);
                double res = (ge - gw) / dx[i - 1] + (gn - gs) / dy[j - 1] + (gt - gb) / dz[k - 1] - rhs[IN(i, j, k)];
                res = fabs(res);
                if (res > value) value = res;
            }
    return value;
}

/* src/fpm_laplace_3d.f90:219-293 solve_neumann_poisson_nonuniform_3d: weighted
 * 0.2/0.8 Jacobi with boundary branches, copy-back, volume-weighted gauge. */
void orc_solve_neumann_poisson_nonuniform_3d(double *phi, const double *rhs, const double *xlo, const double *xhi,
                                             const double *ylo, const double *yhi, const double *zlo,
                                             const double *zhi, const double *xc, const double *yc,
                                             const double *zc, const double *dx, const double *dy, const double *dz,
                                             int nx, int ny, int nz, double tolerance, int max_iterations,
                                             int check_interval, int *iterations, double *final_residual) {
    size_t ni = (size_t)nx * ny * nz;
    double *next = (double *)calloc(ni, sizeof(double));
    int it = 0;
    double fr = HUGE_VAL;
    while (it < max_iterations && fr > tolerance) {
        int ci = check_interval < 1 ? 1 : check_interval;
        int nsteps = ci < max_iterations - it ? ci : max_iterations - it;
        for (int step = 1; step <= nsteps; step++) {
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
            for (int k = 1; k <= nz; k++)
                for (int j = 1; j <= ny; j++)
                    for (int i = 1; i <= nx; i++) {
                        double aw = 0, ae = 0, as = 0, an = 0, ab = 0, at = 0, diag, numer;
                        if (i > 1) aw = 1.0 / (dx[i - 1] * (xc[i - 1] - xc[i - 2]));
                        if (i < nx) ae = 1.0 / (dx[i - 1] * (xc[i] - xc[i - 1]));
                        if (j > 1) as = 1.0 / (dy[j - 1] * (yc[j - 1] - yc[j - 2]));
                        if (j < ny) an = 1.0 / (dy[j - 1] * (yc[j] - yc[j - 1]));
                        if (k > 1) ab = 1.0 / (dz[k - 1] * (zc[k - 1] - zc[k - 2]));
                        if (k < nz) at = 1.0 / (dz[k - 1] * (zc[k] - zc[k - 1]));
                        diag = aw + ae + as + an + ab + at;
                        numer = -rhs[IN(i, j, k)];
                        if (i > 1) numer = numer + aw * phi[Q3(i - 1, j, k)];
                        if (i < nx) numer = numer + ae * phi[Q3(i + 1, j, k)];
                        if (j > 1) numer = numer + as * phi[Q3(i, j - 1, k)];
                        if (j < ny) numer = numer + an * phi[Q3(i, j + 1, k)];
                        if (k > 1) numer = numer + ab * phi[Q3(i, j, k - 1)];
                        if (k < nz) numer = numer + at * phi[Q3(i, j, k + 1)];
                        if (i == 1) numer = numer - xlo[XF(j, k)] / dx[i - 1];
                        if (i == nx) numer = numer + xhi[XF(j, k)] / dx[i - 1];
                        if (j == 1) numer = numer - ylo[YF(i, k)] / dy[j - 1];
                        if (j == ny) numer = numer + yhi[YF(i, k)] / dy[j - 1];
                        if (k == 1) numer = numer - zlo[ZF(i, j)] / dz[k - 1];
                        if (k == nz) numer = numer + zhi[ZF(i, j)] / dz[k - 1];
                        next[Q3(i, j, k)] = 0.2 * phi[Q3(i, j, k)] + 0.8 * numer / diag;
                    }
            memcpy(phi, next, ni * sizeof(double));
            it++;
        }
        fr = orc_residual_nonuniform(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, nx, ny, nz);
    }
    double ws = 0, vs = 0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                ws = ws + phi[Q3(i, j, k)] * dx[i - 1] * dy[j - 1] * dz[k - 1];
                vs = vs + dx[i - 1] * dy[j - 1] * dz[k - 1];
            }
    double mean_value = ws / vs;
    for (size_t m = 0; m < ni; m++) phi[m] = phi[m] - mean_value;
    fr = orc_residual_nonuniform(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, nx, ny, nz);
    *iterations = it;
    *final_residual = fr;
    free(next);
}

/* ---------------- fpm_terms_3d (no body) ---------------- */

/* src/fpm_terms_3d.f90:8-37 compute_fpm_terms_uniform_3d; phi (0:nx+1,0:ny+1,0:nz+1). */
void orc_compute_fpm_terms_uniform_3d(const double *phi, const double *u, const double *v, const double *w,
                                      const double *ox, const double *oy, const double *oz, const double *ax,
                                      const double *ay, const double *az, const int32_t *fluid, double *gx,
                                      double *gy, double *gz, double *vortex, double *advection, double *totals,
                                      int nx, int ny, int nz, double dx, double dy, double dz) {
    double vt = 0, at = 0, volume = dx * dy * dz;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                size_t c = IN(i, j, k);
                gx[c] = (phi[P3(i + 1, j, k)] - phi[P3(i - 1, j, k)]) / (2.0 * dx);
                gy[c] = (phi[P3(i, j + 1, k)] - phi[P3(i, j - 1, k)]) / (2.0 * dy);
                gz[c] = (phi[P3(i, j, k + 1)] - phi[P3(i, j, k - 1)]) / (2.0 * dz);
                double cx = w[c] * oy[c] - v[c] * oz[c];
                double cy = u[c] * oz[c] - w[c] * ox[c];
                double cz = v[c] * ox[c] - u[c] * oy[c];
                double mask = (double)fluid[c];
                vortex[c] = -(mask * (cx * gx[c] + cy * gy[c] + cz * gz[c]));
                advection[c] = -(mask * (ax[c] * gx[c] + ay[c] * gy[c] + az[c] * gz[c]));
                vt = vt + volume * vortex[c];
                at = at + volume * advection[c];
            }
    totals[0] = vt;
    totals[1] = at;
}

/* src/fpm_terms_3d.f90:39-88 compute_fpm_terms_nonuniform_3d; phi (nx,ny,nz).
 * Returns ORC_E_SIZE for fewer than two cells per direction. */
int orc_compute_fpm_terms_nonuniform_3d(const double *phi, const double *u, const double *v, const double *w,
                                        const double *ox, const double *oy, const double *oz, const double *ax,
                                        const double *ay, const double *az, const int32_t *fluid, const double *xc,
                                        const double *yc, const double *zc, const double *dx, const double *dy,
                                        const double *dz, const double *xlo, const double *xhi, const double *ylo,
                                        const double *yhi, const double *zlo, const double *zhi,
                                        const double *bounds, double *gx, double *gy, double *gz, double *vortex,
                                        double *advection, double *totals, int nx, int ny, int nz) {
    if (nx < 2 || ny < 2 || nz < 2) return ORC_E_SIZE;
    double vt = 0, at = 0;
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                size_t c = IN(i, j, k);
                double p = phi[c], we, ea, so, no, bo, to;
                if (i == 1) we = xlo[XF(j, k)]; else we = (p - phi[Q3(i - 1, j, k)]) / (xc[i - 1] - xc[i - 2]);
                if (i == nx) ea = xhi[XF(j, k)]; else ea = (phi[Q3(i + 1, j, k)] - p) / (xc[i] - xc[i - 1]);
                if (j == 1) so = ylo[YF(i, k)]; else so = (p - phi[Q3(i, j - 1, k)]) / (yc[j - 1] - yc[j - 2]);
                if (j == ny) no = yhi[YF(i, k)]; else no = (phi[Q3(i, j + 1, k)] - p) / (yc[j] - yc[j - 1]);
                if (k == 1) bo = zlo[ZF(i, j)]; else bo = (p - phi[Q3(i, j, k - 1)]) / (zc[k - 1] - zc[k - 2]);
                if (k == nz) to = zhi[ZF(i, j)]; else to = (phi[Q3(i, j, k + 1)] - p) / (zc[k] - zc[k - 1]);
                gx[c] = 0.5 * (we + ea);
                gy[c] = 0.5 * (so + no);
                gz[c] = 0.5 * (bo + to);
                double cx = w[c] * oy[c] - v[c] * oz[c];
                double cy = u[c] * oz[c] - w[c] * ox[c];
                double cz = v[c] * ox[c] - u[c] * oy[c];
                double mask = (double)fluid[c];
                vortex[c] = -(mask * (cx * gx[c] + cy * gy[c] + cz * gz[c]));
                advection[c] = -(mask * (ax[c] * gx[c] + ay[c] * gy[c] + az[c] * gz[c]));
                double inside = (xc[i - 1] > bounds[0] && xc[i - 1] < bounds[1] && yc[j - 1] > bounds[2] &&
                                 yc[j - 1] < bounds[3] && zc[k - 1] > bounds[4] && zc[k - 1] < bounds[5])
                                    ? 1.0
                                    : 0.0;
                double volume = inside * dx[i - 1] * dy[j - 1] * dz[k - 1];
                vt = vt + volume * vortex[c];
                at = at + volume * advection[c];
            }
    totals[0] = vt;
    totals[1] = at;
    return ORC_OK;
}

/* ---------------- fpm_partition_2d ---------------- */

/* src/fpm_partition_2d.f90:35-154 fpm_partition_terms_2d (one rank, host).
 * phi, u, v, solid (uint8 0/1) are (nx,ny); xf(0:nx), yf(0:ny); kin(6);
 * ring(2nx+2ny, 2, 2); terms(4) = [KINE, VIF, VIS, BOUND]. */
int orc_fpm_partition_terms_2d(const double *phi, const double *g, const double *u, const double *v,
                               const uint8_t *solid, const double *xf, const double *yf, const double *kin,
                               const double *ring, double dt, double nu, int nx, int ny, double *terms,
                               double *vif_density, double *omega, int slip) {
#define C2(i, j) ((size_t)((i) - 1) + (size_t)nx * (size_t)((j) - 1))
#define RING(m, c, t) ring[(size_t)((m) - 1) + (size_t)L * ((size_t)((c) - 1) + 2 * (size_t)((t) - 1))]
    size_t n2 = (size_t)nx * ny, L = 2 * (size_t)nx + 2 * (size_t)ny;
    double *xc = (double *)malloc(nx * sizeof(double)), *yc = (double *)malloc(ny * sizeof(double));
    double *dx = (double *)malloc(nx * sizeof(double)), *dy = (double *)malloc(ny * sizeof(double));
    double *nxf = (double *)calloc(n2, sizeof(double)), *nyf = (double *)calloc(n2, sizeof(double));
    double *gpx = (double *)calloc(n2, sizeof(double)), *gpy = (double *)calloc(n2, sizeof(double));
    if (!xc || !yc || !dx || !dy || !nxf || !nyf || !gpx || !gpy) {
        free(xc); free(yc); free(dx); free(dy); free(nxf); free(nyf); free(gpx); free(gpy);
        return ORC_E_ALLOC;
    }
    for (int i = 1; i <= nx; i++) { dx[i - 1] = xf[i] - xf[i - 1]; xc[i - 1] = 0.5 * (xf[i - 1] + xf[i]); }
    for (int j = 1; j <= ny; j++) { dy[j - 1] = yf[j] - yf[j - 1]; yc[j - 1] = 0.5 * (yf[j - 1] + yf[j]); }
    terms[0] = terms[1] = terms[2] = terms[3] = 0;
    for (size_t m = 0; m < n2; m++) { vif_density[m] = 0; omega[m] = 0; }
    const double k1 = kin[0], k2 = kin[1], k3 = kin[2], k4 = kin[3], k5 = kin[4], k6 = kin[5];
    /* Pass 1 */
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            if (solid[C2(i, j)]) continue;
            double fu[4], fv[4], fp[4];
            for (int f = 1; f <= 4; f++) {
                int ii = i, jj = j, axis;
                double sgn, hw, len, d, fx, fy;
                if (f == 1) { ii = i + 1; axis = 1; sgn = 1; }
                else if (f == 2) { ii = i - 1; axis = 1; sgn = -1; }
                else if (f == 3) { jj = j + 1; axis = 2; sgn = 1; }
                else { jj = j - 1; axis = 2; sgn = -1; }
                if (axis == 1) {
                    hw = 0.5 * dx[i - 1]; len = dy[j - 1]; fx = xc[i - 1] + sgn * hw; fy = yc[j - 1];
                    d = hw; if (ii >= 1 && ii <= nx) d = fabs(xc[ii - 1] - xc[i - 1]);
                } else {
                    hw = 0.5 * dy[j - 1]; len = dx[i - 1]; fx = xc[i - 1]; fy = yc[j - 1] + sgn * hw;
                    d = hw; if (jj >= 1 && jj <= ny) d = fabs(yc[jj - 1] - yc[j - 1]);
                }
                (void)len;
                if (ii < 1 || ii > nx || jj < 1 || jj > ny) {
                    fu[f - 1] = u[C2(i, j)]; fv[f - 1] = v[C2(i, j)]; fp[f - 1] = 0;
                } else if (solid[C2(ii, jj)]) {
                    if (slip) { fu[f - 1] = u[C2(i, j)]; fv[f - 1] = v[C2(i, j)]; }
                    else { fu[f - 1] = k1 - k3 * fy; fv[f - 1] = k2 + k3 * fx; }
                    fp[f - 1] = g[axis - 1];
                } else {
                    fu[f - 1] = u[C2(i, j)] + (u[C2(ii, jj)] - u[C2(i, j)]) * hw / d;
                    fv[f - 1] = v[C2(i, j)] + (v[C2(ii, jj)] - v[C2(i, j)]) * hw / d;
                    fp[f - 1] = sgn * (phi[C2(ii, jj)] - phi[C2(i, j)]) / d;
                }
            }
            size_t c = C2(i, j);
            nxf[c] = u[c] * (fu[0] - fu[1]) / dx[i - 1] + v[c] * (fu[2] - fu[3]) / dy[j - 1];
            nyf[c] = u[c] * (fv[0] - fv[1]) / dx[i - 1] + v[c] * (fv[2] - fv[3]) / dy[j - 1];
            omega[c] = (fv[0] - fv[1]) / dx[i - 1] - (fu[2] - fu[3]) / dy[j - 1];
            gpx[c] = 0.5 * (fp[0] + fp[1]);
            gpy[c] = 0.5 * (fp[2] + fp[3]);
        }
    /* Pass 2 */
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            if (solid[C2(i, j)]) continue;
            size_t c = C2(i, j);
            double div = 0, lapu = 0, lapv = 0;
            for (int f = 1; f <= 4; f++) {
                int ii = i, jj = j, axis;
                double sgn, hw, len, d, fx, fy;
                if (f == 1) { ii = i + 1; axis = 1; sgn = 1; }
                else if (f == 2) { ii = i - 1; axis = 1; sgn = -1; }
                else if (f == 3) { jj = j + 1; axis = 2; sgn = 1; }
                else { jj = j - 1; axis = 2; sgn = -1; }
                if (axis == 1) {
                    hw = 0.5 * dx[i - 1]; len = dy[j - 1]; fx = xc[i - 1] + sgn * hw; fy = yc[j - 1];
                    d = hw; if (ii >= 1 && ii <= nx) d = fabs(xc[ii - 1] - xc[i - 1]);
                } else {
                    hw = 0.5 * dy[j - 1]; len = dx[i - 1]; fx = xc[i - 1]; fy = yc[j - 1] + sgn * hw;
                    d = hw; if (jj >= 1 && jj <= ny) d = fabs(yc[jj - 1] - yc[j - 1]);
                }
                if (ii < 1 || ii > nx || jj < 1 || jj > ny) {
                    double nn = axis == 1 ? nxf[c] : nyf[c];
                    div = div + sgn * nn * len;
                    int m;
                    if (f == 2) m = j;
                    else if (f == 1) m = ny + j;
                    else if (f == 4) m = 2 * ny + i;
                    else m = 2 * ny + nx + i;
                    double dudt = (RING(m, 1, 2) - RING(m, 1, 1)) / (2 * dt);
                    double dvdt = (RING(m, 2, 2) - RING(m, 2, 1)) / (2 * dt);
                    terms[3] = terms[3] - sgn * (axis == 1 ? dudt + nxf[c] : dvdt + nyf[c]) * phi[c] * len;
                } else if (solid[C2(ii, jj)]) {
                    double ubx = k1 - k3 * fy, uby = k2 + k3 * fx;
                    double bax = k4 - k6 * fy - k3 * k3 * fx, bay = k5 + k6 * fx - k3 * k3 * fy;
                    double phif = phi[c] + sgn * hw * g[axis - 1];
                    terms[0] = terms[0] - sgn * (axis == 1 ? bax : bay) * phif * len;
                    if (slip) {
                        div = div + sgn * (axis == 1 ? nxf[c] : nyf[c]) * len;
                    } else {
                        div = div + sgn * (axis == 1 ? -(k3 * uby) : k3 * ubx) * len;
                        lapu = lapu + (ubx - u[c]) / hw * len;
                        lapv = lapv + (uby - v[c]) / hw * len;
                    }
                } else {
                    size_t c2 = C2(ii, jj);
                    double val = axis == 1 ? nxf[c] + (nxf[c2] - nxf[c]) * hw / d : nyf[c] + (nyf[c2] - nyf[c]) * hw / d;
                    div = div + sgn * val * len;
                    lapu = lapu + (u[c2] - u[c]) / d * len;
                    lapv = lapv + (v[c2] - v[c]) / d * len;
                }
            }
            vif_density[c] = phi[c] * div / (dx[i - 1] * dy[j - 1]);
            terms[1] = terms[1] + phi[c] * div;
            terms[2] = terms[2] + nu * (lapu * gpx[c] + lapv * gpy[c]);
        }
    free(xc); free(yc); free(dx); free(dy); free(nxf); free(nyf); free(gpx); free(gpy);
    return ORC_OK;
#undef C2
#undef RING
}

/* ---------------- test-grid helpers (tests/fpm_test_grid.f90) ---------------- */

/* tests/fpm_test_grid.f90:11-27 stretched_axis: face(0:n), center(n), width(n). */
void orc_stretched_axis(int n, double lo, double hi, double amplitude, double *face, double *center, double *width) {
    double *weight = (double *)malloc((size_t)n * sizeof(double));
    double pi = acos(-1.0), sum = 0;
    for (int m = 1; m <= n; m++) weight[m - 1] = 1 + amplitude * sin(2 * pi * (m - 0.5) / n);
    for (int m = 1; m <= n; m++) sum = sum + weight[m - 1];
    face[0] = lo;
    for (int m = 1; m <= n; m++) {
        width[m - 1] = (hi - lo) * weight[m - 1] / sum;
        face[m] = face[m - 1] + width[m - 1];
        center[m - 1] = 0.5 * (face[m - 1] + face[m]);
    }
    face[n] = hi;
    free(weight);
}

/* tests/fpm_test_grid.f90:31-43 local_axis: centres (0:n+1) with mirrored halo
 * centres, widths (n), for global cells offset+1..offset+n. */
void orc_local_axis(int gn, const double *gcenter, const double *gwidth, int offset, int n, double *center,
                    double *width) {
    for (int m = 0; m <= n + 1; m++) {
        int g = offset + m;
        if (g < 1) center[m] = gcenter[0] - gwidth[0];
        else if (g > gn) center[m] = gcenter[gn - 1] + gwidth[gn - 1];
        else center[m] = gcenter[g - 1];
    }
    for (int m = 1; m <= n; m++) width[m - 1] = gwidth[offset + m - 1];
}

/* ---------------- 3-D four-term partition ----------------
 * The 3-D counterpart of fpm_partition_terms_2d (src/fpm_partition_2d.f90:35-154),
 * which the reference provides in 2-D only: the same face-flux discretisation
 * on the six faces of every fluid cell.  Rigid body motion about the origin:
 * U_B = V + W x r, a_B = A + Al x r + W x (W x r), (U_B.grad)U_B = W x U_B,
 * kin = [V(3), W(3), A(3), Al(3)].  Outer faces: the cell's own u and
 * (u.grad)u, zero viscous flux, Du/Dt from shell(t+dt) - shell(t-dt) over 2 dt
 * plus (u.grad)u.  shell(L,3,2), L = 2 ny nz + 2 nx nz + 2 nx ny, lists the
 * outer cells of the west face (j,k), east, south (i,k), north, bottom (i,j),
 * top; NULL means Du/Dt = 0 there.  Faces f = 1..6: east, west, north, south,
 * top, bottom (outward sign +, -, +, -, +, -).  terms = [KINE, VIF, VIS, BOUND]. */
int orc_fpm_partition_terms_3d(const double *phi, const double *g, const double *u, const double *v,
                               const double *w, const uint8_t *solid, const double *xf, const double *yf,
                               const double *zf, const double *kin, const double *shell, double dt, double nu,
                               int nx, int ny, int nz, double *terms, double *vif_density, double *omega, int slip) {
#define C3(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1)))
    size_t n3 = (size_t)nx * ny * nz;
    size_t L = 2 * (size_t)ny * nz + 2 * (size_t)nx * nz + 2 * (size_t)nx * ny;
    double *N[3], *gp[3];
    for (int a = 0; a < 3; a++) {
        N[a] = (double *)calloc(n3, sizeof(double));
        gp[a] = (double *)calloc(n3, sizeof(double));
        if (!N[a] || !gp[a]) return ORC_E_ALLOC;
    }
    const double *vel[3] = {u, v, w};
    terms[0] = terms[1] = terms[2] = terms[3] = 0;
    for (size_t m = 0; m < n3; m++) {
        vif_density[m] = 0;
        if (omega) omega[m] = omega[n3 + m] = omega[2 * n3 + m] = 0;
    }
    const double V0 = kin[0], V1 = kin[1], V2 = kin[2], W0 = kin[3], W1 = kin[4], W2 = kin[5];
    const double A0 = kin[6], A1 = kin[7], A2 = kin[8], B0 = kin[9], B1 = kin[10], B2 = kin[11];
    for (int pass = 1; pass <= 2; pass++)
        for (int k = 1; k <= nz; k++)
            for (int j = 1; j <= ny; j++)
                for (int i = 1; i <= nx; i++) {
                    size_t c = C3(i, j, k);
                    if (solid[c]) continue;
                    double dxi = xf[i] - xf[i - 1], dyj = yf[j] - yf[j - 1], dzk = zf[k] - zf[k - 1];
                    double xc = 0.5 * (xf[i - 1] + xf[i]), yc = 0.5 * (yf[j - 1] + yf[j]), zc = 0.5 * (zf[k - 1] + zf[k]);
                    double fvel[3][6], fp[6], div = 0, lap[3] = {0, 0, 0};
                    for (int f = 1; f <= 6; f++) {
                        int ii = i, jj = j, kk = k, axis;
                        double sgn = (f % 2 == 1) ? 1.0 : -1.0, hw, area, d, fx = xc, fy = yc, fz = zc;
                        if (f <= 2) {
                            axis = 0; ii = i + (int)sgn; hw = 0.5 * dxi; area = dyj * dzk; fx = xc + sgn * hw; d = hw;
                            if (ii >= 1 && ii <= nx) d = fabs(0.5 * (xf[ii - 1] + xf[ii]) - xc);
                        } else if (f <= 4) {
                            axis = 1; jj = j + (int)sgn; hw = 0.5 * dyj; area = dxi * dzk; fy = yc + sgn * hw; d = hw;
                            if (jj >= 1 && jj <= ny) d = fabs(0.5 * (yf[jj - 1] + yf[jj]) - yc);
                        } else {
                            axis = 2; kk = k + (int)sgn; hw = 0.5 * dzk; area = dxi * dyj; fz = zc + sgn * hw; d = hw;
                            if (kk >= 1 && kk <= nz) d = fabs(0.5 * (zf[kk - 1] + zf[kk]) - zc);
                        }
                        int outer = ii < 1 || ii > nx || jj < 1 || jj > ny || kk < 1 || kk > nz;
                        size_t c2 = outer ? c : C3(ii, jj, kk);
                        /* rigid body velocity and acceleration at the face centre */
                        double ub[3] = {V0 + (W1 * fz - W2 * fy), V1 + (W2 * fx - W0 * fz), V2 + (W0 * fy - W1 * fx)};
                        if (pass == 1) {
                            if (outer) {
                                for (int a = 0; a < 3; a++) fvel[a][f - 1] = vel[a][c];
                                fp[f - 1] = 0;
                            } else if (solid[c2]) {
                                for (int a = 0; a < 3; a++) fvel[a][f - 1] = slip ? vel[a][c] : ub[a];
                                fp[f - 1] = g[axis];
                            } else {
                                for (int a = 0; a < 3; a++) fvel[a][f - 1] = vel[a][c] + (vel[a][c2] - vel[a][c]) * hw / d;
                                fp[f - 1] = sgn * (phi[c2] - phi[c]) / d;
                            }
                        } else {
                            if (outer) {
                                div = div + sgn * N[axis][c] * area;
                                double dudt = 0;
                                if (shell) {
                                    size_t m;
                                    if (f == 2) m = (size_t)(j - 1) + (size_t)ny * (k - 1);
                                    else if (f == 1) m = (size_t)ny * nz + (size_t)(j - 1) + (size_t)ny * (k - 1);
                                    else if (f == 4) m = 2 * (size_t)ny * nz + (size_t)(i - 1) + (size_t)nx * (k - 1);
                                    else if (f == 3) m = 2 * (size_t)ny * nz + (size_t)nx * nz + (size_t)(i - 1) + (size_t)nx * (k - 1);
                                    else if (f == 6) m = 2 * (size_t)ny * nz + 2 * (size_t)nx * nz + (size_t)(i - 1) + (size_t)nx * (j - 1);
                                    else m = 2 * (size_t)ny * nz + 2 * (size_t)nx * nz + (size_t)nx * ny + (size_t)(i - 1) + (size_t)nx * (j - 1);
                                    dudt = (shell[m + L * ((size_t)axis + 3)] - shell[m + L * (size_t)axis]) / (2 * dt);
                                }
                                terms[3] = terms[3] - sgn * (dudt + N[axis][c]) * phi[c] * area;
                            } else if (solid[c2]) {
                                double rx = fx, ry = fy, rz = fz;
                                double wr[3] = {W1 * rz - W2 * ry, W2 * rx - W0 * rz, W0 * ry - W1 * rx};
                                double ab[3] = {A0 + (B1 * rz - B2 * ry) + (W1 * wr[2] - W2 * wr[1]),
                                                A1 + (B2 * rx - B0 * rz) + (W2 * wr[0] - W0 * wr[2]),
                                                A2 + (B0 * ry - B1 * rx) + (W0 * wr[1] - W1 * wr[0])};
                                double phif = phi[c] + sgn * hw * g[axis];
                                terms[0] = terms[0] - sgn * ab[axis] * phif * area;
                                if (slip) {
                                    div = div + sgn * N[axis][c] * area;
                                } else {
                                    double cb[3] = {W1 * ub[2] - W2 * ub[1], W2 * ub[0] - W0 * ub[2], W0 * ub[1] - W1 * ub[0]};
                                    div = div + sgn * cb[axis] * area;
                                    for (int a = 0; a < 3; a++) lap[a] = lap[a] + (ub[a] - vel[a][c]) / hw * area;
                                }
                            } else {
                                div = div + sgn * (N[axis][c] + (N[axis][c2] - N[axis][c]) * hw / d) * area;
                                for (int a = 0; a < 3; a++) lap[a] = lap[a] + (vel[a][c2] - vel[a][c]) / d * area;
                            }
                        }
                    }
                    if (pass == 1) {
                        for (int a = 0; a < 3; a++)
                            N[a][c] = u[c] * (fvel[a][0] - fvel[a][1]) / dxi + v[c] * (fvel[a][2] - fvel[a][3]) / dyj +
                                      w[c] * (fvel[a][4] - fvel[a][5]) / dzk;
                        if (omega) {
                            omega[c] = (fvel[2][2] - fvel[2][3]) / dyj - (fvel[1][4] - fvel[1][5]) / dzk;
                            omega[n3 + c] = (fvel[0][4] - fvel[0][5]) / dzk - (fvel[2][0] - fvel[2][1]) / dxi;
                            omega[2 * n3 + c] = (fvel[1][0] - fvel[1][1]) / dxi - (fvel[0][2] - fvel[0][3]) / dyj;
                        }
                        gp[0][c] = 0.5 * (fp[0] + fp[1]);
                        gp[1][c] = 0.5 * (fp[2] + fp[3]);
                        gp[2][c] = 0.5 * (fp[4] + fp[5]);
                    } else {
                        vif_density[c] = phi[c] * div / (dxi * dyj * dzk);
                        terms[1] = terms[1] + phi[c] * div;
                        terms[2] = terms[2] + nu * (lap[0] * gp[0][c] + lap[1] * gp[1][c] + lap[2] * gp[2][c]);
                    }
                }
    for (int a = 0; a < 3; a++) { free(N[a]); free(gp[a]); }
    return ORC_OK;
#undef C3
}
