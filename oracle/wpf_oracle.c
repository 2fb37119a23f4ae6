/*
 * wpf_oracle.c -- CPU oracle for the wPFAW3D time step (TEST INFRASTRUCTURE).
 *
 * A plain-C restatement of the reference routines, one function per
 * reference subroutine, each citing the wPFAW3D.f90 lines it follows.  It is
 * the parity checker for the CUDA path and the timed CPU baseline; the
 * product library never links it.  Compiled with -ffp-contract=off so every
 * floating-point operation rounds as written (the order of operations follows
 * the Fortran expressions left to right).
 *
 * Parity unpinned against the reference binary (it cannot be built here);
 * pinned by analytic cases and by a scipy.sparse direct solve of the matrix
 * orc_assemble() produces (the assembly of wPFAW3D.f90:629-936).
 */
#include "wpf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_version(void) { return 3; }

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---- indexing --------------------------------------------------------- */
#define PX(p) ((long)(p)->nx + 2)
#define PY(p) ((long)(p)->ny + 2)
#define IDX(p, i, j, k) ((long)(i) + PX(p) * ((long)(j) + PY(p) * (long)(k)))
static long gsize(const orc_params* p) { return PX(p) * PY(p) * ((long)p->nz + 2); }

/* ---- wells (wPFAW3D.f90:451-483) -------------------------------------- */
void orc_build_lw(orc_state* s) {
    const orc_params* p = &s->p;
    long G = gsize(p);
    for (long n = 0; n < G; ++n) s->lw[n] = 0;
    for (int iw = 0; iw < s->nwell; ++iw) {          /* :453-461 (later wells win) */
        int ix = s->well[iw].ix, iy = s->well[iw].iy, iz = s->well[iw].iz;
        if (0 <= ix && ix <= p->nx + 1 && 0 <= iy && iy <= p->ny + 1 && 0 <= iz && iz <= p->nz + 1)
            s->lw[IDX(p, ix, iy, iz)] = iw + 1;
    }
}

/* Field initialisation of loadConfig, wPFAW3D.f90:464-471. */
void orc_init_fields(orc_state* s, double init_permeab, double init_phase, double init_concent,
                     double pini) {
    long G = gsize(&s->p);
    for (long n = 0; n < G; ++n) {
        s->permeab_rock[n] = init_permeab;
        s->pressure[n] = pini;
        s->phase[n] = init_phase;
        s->concent[n] = init_concent;
        s->dphasedt[n] = 0.0;
        s->dconcentdt[n] = 0.0;
        for (int m = 0; m < 4; ++m) s->permeab[4 * n + m] = 0.0;
        for (int m = 0; m < 3; ++m) s->velocity[3 * n + m] = 0.0;
    }
}

/* Fixed phase / concentration at interior well cells, wPFAW3D.f90:474-483. */
void orc_apply_well_values(orc_state* s) {
    const orc_params* p = &s->p;
    for (int iw = 0; iw < s->nwell; ++iw) {
        int ix = s->well[iw].ix, iy = s->well[iw].iy, iz = s->well[iw].iz;
        if (1 <= ix && ix <= p->nx && 1 <= iy && iy <= p->ny && 1 <= iz && iz <= p->nz) {
            s->phase[IDX(p, ix, iy, iz)] = s->well[iw].phase;
            s->concent[IDX(p, ix, iy, iz)] = s->well[iw].concent;
        }
    }
}

/* ---- updateHalo, wPFAW3D.f90:1645-1657 (single domain: all edges global) */
void orc_update_halo(const orc_params* p, double* f) {
    int nx = p->nx, ny = p->ny, nz = p->nz;
    for (int k = 0; k <= nz + 1; ++k)                 /* :1651-1652 x planes */
        for (int j = 0; j <= ny + 1; ++j) {
            f[IDX(p, 0, j, k)] = f[IDX(p, 1, j, k)];
            f[IDX(p, nx + 1, j, k)] = f[IDX(p, nx, j, k)];
        }
    for (int k = 0; k <= nz + 1; ++k)                 /* :1653-1654 y planes */
        for (int i = 0; i <= nx + 1; ++i) {
            f[IDX(p, i, 0, k)] = f[IDX(p, i, 1, k)];
            f[IDX(p, i, ny + 1, k)] = f[IDX(p, i, ny, k)];
        }
    for (int j = 0; j <= ny + 1; ++j)                 /* :1655-1656 z planes */
        for (int i = 0; i <= nx + 1; ++i) {
            f[IDX(p, i, j, 0)] = f[IDX(p, i, j, 1)];
            f[IDX(p, i, j, nz + 1)] = f[IDX(p, i, j, nz)];
        }
}

/* ---- calcPermeability, wPFAW3D.f90:561-599 ----------------------------- */
static double harmonic_mean(double a, double b) { return 2.0 / (1.0 / a + 1.0 / b); } /* :593-598 */

void orc_calc_permeability(orc_state* s) {
    const orc_params* p = &s->p;
    int nx = p->nx, ny = p->ny, nz = p->nz;
    double* K = s->permeab;
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= nz + 1; ++k)                 /* :567-574 */
        for (int j = 0; j <= ny + 1; ++j)
            for (int i = 0; i <= nx + 1; ++i) {
                long n = IDX(p, i, j, k);
                double f = 0.5 * (1.0 + s->phase[n]);
                K[4 * n] = p->permeab_hole * f + s->permeab_rock[n] * (1.0 - f);
            }
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= nz; ++k)                     /* :577-585 */
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                long n = IDX(p, i, j, k);
                K[4 * n + 1] = harmonic_mean(K[4 * n], K[4 * IDX(p, i + 1, j, k)]);
                K[4 * n + 2] = harmonic_mean(K[4 * n], K[4 * IDX(p, i, j + 1, k)]);
                K[4 * n + 3] = harmonic_mean(K[4 * n], K[4 * IDX(p, i, j, k + 1)]);
            }
}

/* ---- solvePressure helpers, wPFAW3D.f90:1099-1159 ---------------------- */
static int onBoundary(const orc_state* s, long n) {  /* :1099-1110 */
    int iw = s->lw[n];
    return iw > 0 ? (s->well[iw - 1].pressure != 0.0) : 0;
}
static int onInlet(const orc_state* s, long n) {     /* :1133-1144 */
    int iw = s->lw[n];
    return iw > 0 ? (s->well[iw - 1].injection != 0.0) : 0;
}
static double valuePressure(const orc_state* s, long n) { return s->well[s->lw[n] - 1].pressure; }
static double valueInjection(const orc_state* s, long n) { return s->well[s->lw[n] - 1].injection; }

/* Global serial index index3D_g - 1 (single domain), wPFAW3D.f90:1086-1091. */
static long gidx(const orc_params* p, int i, int j, int k) {
    return (long)(i - 1) + (long)(j - 1) * p->nx + (long)(k - 1) * (long)p->nx * p->ny;
}

/*
 * Assemble the reference system exactly as wPFAW3D.f90:629-936 does: entries
 * in the same order (z-, y-, x-, diag, x+, y+, z+ per row), the Dirichlet rows
 * as identity rows, and the symmetric elimination of Dirichlet neighbours
 * into b.  irn/jcn are 0-based global indices.  Pass irn == NULL to count.
 * Returns nnz.
 */
long orc_assemble(const orc_state* s, int32_t* irn, int32_t* jcn, double* val, double* b) {
    const orc_params* p = &s->p;
    int nx = p->nx, ny = p->ny, nz = p->nz;
    const double* K = s->permeab;
    double mu = p->viscosity, dx = p->dx;
    long nnz = 0;
#define PUT(r, c, v)                                          \
    do {                                                      \
        if (irn) { irn[nnz] = (int32_t)(r); jcn[nnz] = (int32_t)(c); val[nnz] = (v); } \
        ++nnz;                                                \
    } while (0)
    for (int iz = 1; iz <= nz; ++iz)
        for (int iy = 1; iy <= ny; ++iy)
            for (int ix = 1; ix <= nx; ++ix) {
                long n = IDX(p, ix, iy, iz);
                long row = gidx(p, ix, iy, iz);
                /* right-hand side, :803-825 */
                double bb;
                if (onBoundary(s, n)) bb = valuePressure(s, n);
                else if (onInlet(s, n)) bb = -valueInjection(s, n) * (dx * dx / (dx * dx * dx));
                else bb = 0.0;
                if (onBoundary(s, n)) {                                  /* :837-840 */
                    PUT(row, row, 1.0);
                } else {                                                  /* :841-931 */
                    double txp = ix < nx ? K[4 * n + 1] / mu : 0.0;
                    double txm = ix > 1 ? K[4 * IDX(p, ix - 1, iy, iz) + 1] / mu : 0.0;
                    double typ = iy < ny ? K[4 * n + 2] / mu : 0.0;
                    double tym = iy > 1 ? K[4 * IDX(p, ix, iy - 1, iz) + 2] / mu : 0.0;
                    double tzp = iz < nz ? K[4 * n + 3] / mu : 0.0;
                    double tzm = iz > 1 ? K[4 * IDX(p, ix, iy, iz - 1) + 3] / mu : 0.0;
                    double tc = -(txp + txm + typ + tym + tzp + tzm);
                    if (iz - 1 >= 1) {
                        long m = IDX(p, ix, iy, iz - 1);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * tzm;
                        else PUT(row, gidx(p, ix, iy, iz - 1), tzm);
                    }
                    if (iy - 1 >= 1) {
                        long m = IDX(p, ix, iy - 1, iz);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * tym;
                        else PUT(row, gidx(p, ix, iy - 1, iz), tym);
                    }
                    if (ix - 1 >= 1) {
                        long m = IDX(p, ix - 1, iy, iz);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * txm;
                        else PUT(row, gidx(p, ix - 1, iy, iz), txm);
                    }
                    PUT(row, row, tc);
                    if (ix + 1 <= nx) {
                        long m = IDX(p, ix + 1, iy, iz);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * txp;
                        else PUT(row, gidx(p, ix + 1, iy, iz), txp);
                    }
                    if (iy + 1 <= ny) {
                        long m = IDX(p, ix, iy + 1, iz);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * typ;
                        else PUT(row, gidx(p, ix, iy + 1, iz), typ);
                    }
                    if (iz + 1 <= nz) {
                        long m = IDX(p, ix, iy, iz + 1);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * tzp;
                        else PUT(row, gidx(p, ix, iy, iz + 1), tzp);
                    }
                }
                if (b) b[row] = bb;
            }
#undef PUT
    return nnz;
}

/*
 * Matrix-free form of the assembled system: 7 coefficient arrays over the N
 * global rows (cB=z-, cS=y-, cW=x-, cC=diag, cE=x+, cN=y+, cT=z+), built by
 * the same rules as orc_assemble.  Row products sum in the CSR column order.
 */
typedef struct {
    long N;
    int nx, ny, nz;
    double *cB, *cS, *cW, *cC, *cE, *cN, *cT, *b;
    unsigned char* dir;     /* 1 on Dirichlet rows */
} sysmat;

static void sys_build(const orc_state* s, sysmat* A) {
    const orc_params* p = &s->p;
    int nx = p->nx, ny = p->ny, nz = p->nz;
    long N = (long)nx * ny * nz;
    A->N = N; A->nx = nx; A->ny = ny; A->nz = nz;
    double** arrs[8] = {&A->cB, &A->cS, &A->cW, &A->cC, &A->cE, &A->cN, &A->cT, &A->b};
    for (int a = 0; a < 8; ++a) *arrs[a] = (double*)calloc((size_t)N, sizeof(double));
    A->dir = (unsigned char*)calloc((size_t)N, 1);
    const double* K = s->permeab;
    double mu = p->viscosity, dx = p->dx;
#pragma omp parallel for schedule(static)
    for (int iz = 1; iz <= nz; ++iz)
        for (int iy = 1; iy <= ny; ++iy)
            for (int ix = 1; ix <= nx; ++ix) {
                long n = IDX(p, ix, iy, iz);
                long row = gidx(p, ix, iy, iz);
                double bb;
                if (onBoundary(s, n)) bb = valuePressure(s, n);
                else if (onInlet(s, n)) bb = -valueInjection(s, n) * (dx * dx / (dx * dx * dx));
                else bb = 0.0;
                if (onBoundary(s, n)) {
                    A->cC[row] = 1.0;
                    A->dir[row] = 1;
                } else {
                    double txp = ix < nx ? K[4 * n + 1] / mu : 0.0;
                    double txm = ix > 1 ? K[4 * IDX(p, ix - 1, iy, iz) + 1] / mu : 0.0;
                    double typ = iy < ny ? K[4 * n + 2] / mu : 0.0;
                    double tym = iy > 1 ? K[4 * IDX(p, ix, iy - 1, iz) + 2] / mu : 0.0;
                    double tzp = iz < nz ? K[4 * n + 3] / mu : 0.0;
                    double tzm = iz > 1 ? K[4 * IDX(p, ix, iy, iz - 1) + 3] / mu : 0.0;
                    A->cC[row] = -(txp + txm + typ + tym + tzp + tzm);
                    if (iz > 1) { long m = IDX(p, ix, iy, iz - 1);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * tzm; else A->cB[row] = tzm; }
                    if (iy > 1) { long m = IDX(p, ix, iy - 1, iz);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * tym; else A->cS[row] = tym; }
                    if (ix > 1) { long m = IDX(p, ix - 1, iy, iz);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * txm; else A->cW[row] = txm; }
                    if (ix < nx) { long m = IDX(p, ix + 1, iy, iz);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * txp; else A->cE[row] = txp; }
                    if (iy < ny) { long m = IDX(p, ix, iy + 1, iz);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * typ; else A->cN[row] = typ; }
                    if (iz < nz) { long m = IDX(p, ix, iy, iz + 1);
                        if (onBoundary(s, m)) bb = bb - valuePressure(s, m) * tzp; else A->cT[row] = tzp; }
                }
                A->b[row] = bb;
            }
}

static void sys_free(sysmat* A) {
    free(A->cB); free(A->cS); free(A->cW); free(A->cC); free(A->cE); free(A->cN); free(A->cT);
    free(A->b); free(A->dir);
}

/* y = A x (MatMult, row sums in column order). */
static void sys_mult(const sysmat* A, const double* x, double* y) {
    long sx = 1, sy = A->nx, sz = (long)A->nx * A->ny, N = A->N;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < N; ++r) {
        double sum = 0.0;
        if (A->cB[r] != 0.0) sum += A->cB[r] * x[r - sz];
        if (A->cS[r] != 0.0) sum += A->cS[r] * x[r - sy];
        if (A->cW[r] != 0.0) sum += A->cW[r] * x[r - sx];
        sum += A->cC[r] * x[r];
        if (A->cE[r] != 0.0) sum += A->cE[r] * x[r + sx];
        if (A->cN[r] != 0.0) sum += A->cN[r] * x[r + sy];
        if (A->cT[r] != 0.0) sum += A->cT[r] * x[r + sz];
        y[r] = sum;
    }
}

/* Off-diagonal row sum Σ_{j≠r} a_rj x_j restricted to columns in [lo,hi);
 * columns outside take their value from xg (the ghost snapshot). */
static inline double offsum(const sysmat* A, long r, const double* x, const double* xg, long lo,
                            long hi) {
    long sy = A->nx, sz = (long)A->nx * A->ny;
    double sum = 0.0;
#define T(c, off) if (A->c[r] != 0.0) { long q = r + (off); sum += A->c[r] * ((q >= lo && q < hi) ? x[q] : xg[q]); }
    T(cB, -sz) T(cS, -sy) T(cW, -1) T(cE, 1) T(cN, sy) T(cT, sz)
#undef T
    return sum;
}

/*
 * PCSOR with its=10, lits=1, omega=1.7, default SOR_LOCAL_SYMMETRIC_SWEEP,
 * zero initial guess (wPFAW3D.f90:994-996): z = B r.  "Local" means each of
 * the nblocks contiguous row blocks (the row-block distribution of PETSc with
 * nblocks MPI ranks) sweeps with its own rows; couplings to other blocks use
 * the values from the previous outer iteration (block Jacobi between ranks).
 */
static void pc_sor(const sysmat* A, const double* r, double* z, double* zg, int nblocks) {
    const double omega = 1.7;
    const int its = 10;
    long N = A->N;
    if (nblocks < 1) nblocks = 1;
    for (long q = 0; q < N; ++q) z[q] = 0.0;
    for (int it = 0; it < its; ++it) {
        memcpy(zg, z, (size_t)N * sizeof(double));
#pragma omp parallel for schedule(static, 1)
        for (int blk = 0; blk < nblocks; ++blk) {
            long lo = N * blk / nblocks, hi = N * (blk + 1) / nblocks;
            for (long q = lo; q < hi; ++q) {          /* forward sweep */
                double d = A->cC[q];
                z[q] = (1.0 - omega) * z[q] + omega * (r[q] - offsum(A, q, z, zg, lo, hi)) / d;
            }
            for (long q = hi - 1; q >= lo; --q) {     /* backward sweep */
                double d = A->cC[q];
                z[q] = (1.0 - omega) * z[q] + omega * (r[q] - offsum(A, q, z, zg, lo, hi)) / d;
            }
        }
    }
}

static double dot(const double* a, const double* b, long N) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long q = 0; q < N; ++q) s += a[q] * b[q];
    return s;
}

/*
 * KSPBCGS with left preconditioning (PETSc's BiCGStab recurrence), initial
 * guess nonzero, convergence ||B r_k|| <= rtol*||B b|| (KSPConvergedDefault
 * with a user-provided initial guess), maxit iterations.
 */
static int solve_bcgs(const sysmat* A, double* x, double rtol, int maxit, int nblocks,
                      orc_solve_info* info) {
    long N = A->N;
    double *r = malloc(N * sizeof(double)), *rp = malloc(N * sizeof(double)),
           *pv = calloc(N, sizeof(double)), *v = calloc(N, sizeof(double)),
           *sv = malloc(N * sizeof(double)), *t = malloc(N * sizeof(double)),
           *w = malloc(N * sizeof(double)), *zg = malloc(N * sizeof(double));
    /* ||B b|| */
    pc_sor(A, A->b, w, zg, nblocks);
    double bnorm = sqrt(dot(w, w, N));
    double ttol = rtol * bnorm;
    if (ttol < 1e-50) ttol = 1e-50;
    /* r = B (b - A x) */
    sys_mult(A, x, t);
    for (long q = 0; q < N; ++q) t[q] = A->b[q] - t[q];
    pc_sor(A, t, r, zg, nblocks);
    memcpy(rp, r, N * sizeof(double));
    double dp = sqrt(dot(r, r, N));
    double rhoold = 1.0, alpha = 1.0, omegaold = 1.0;
    int it = 0, conv = dp <= ttol;
    while (!conv && it < maxit) {
        double rho = dot(r, rp, N);
        if (rho == 0.0) break;
        double beta = (rho / rhoold) * (alpha / omegaold);
#pragma omp parallel for schedule(static)
        for (long q = 0; q < N; ++q) pv[q] = r[q] + beta * (pv[q] - omegaold * v[q]);
        sys_mult(A, pv, w);
        pc_sor(A, w, v, zg, nblocks);
        double d1 = dot(v, rp, N);
        if (d1 == 0.0) break;
        alpha = rho / d1;
#pragma omp parallel for schedule(static)
        for (long q = 0; q < N; ++q) sv[q] = r[q] - alpha * v[q];
        sys_mult(A, sv, w);
        pc_sor(A, w, t, zg, nblocks);
        double d1b = dot(sv, t, N), d2 = dot(t, t, N);
        if (d2 == 0.0) {
            for (long q = 0; q < N; ++q) x[q] += alpha * pv[q];
            ++it;
            dp = sqrt(dot(sv, sv, N));
            conv = 1;
            break;
        }
        double omega = d1b / d2;
#pragma omp parallel for schedule(static)
        for (long q = 0; q < N; ++q) {
            x[q] = x[q] + alpha * pv[q] + omega * sv[q];
            r[q] = sv[q] - omega * t[q];
        }
        dp = sqrt(dot(r, r, N));
        rhoold = rho;
        omegaold = omega;
        ++it;
        conv = dp <= ttol;
        if (!(dp == dp) || isinf(dp)) break;
    }
    info->iterations = it;
    info->converged = conv;
    info->rnorm = dp;
    info->bnorm = bnorm;
    free(r); free(rp); free(pv); free(v); free(sv); free(t); free(w); free(zg);
    return conv ? 0 : 1;
}

/*
 * Jacobi-preconditioned CG on the SPD free-row system (-A restricted to the
 * non-Dirichlet rows; Dirichlet rows are the identity and stay at b), run to
 * ||b - A x|| <= rtol*||b|| in the true residual.  Used for parity runs.
 */
static int solve_cg(const sysmat* A, double* x, double rtol, int maxit, orc_solve_info* info) {
    long N = A->N;
    double *r = malloc(N * sizeof(double)), *z = malloc(N * sizeof(double)),
           *pv = malloc(N * sizeof(double)), *q = malloc(N * sizeof(double));
    double bnorm = sqrt(dot(A->b, A->b, N));
    for (long n = 0; n < N; ++n) if (A->dir[n]) x[n] = A->b[n];
    double tol = rtol * bnorm;
    int it = 0, conv = 0;
    double rnorm = 0.0;
    for (int restart = 0; restart < 50 && !conv; ++restart) {
        /* true residual of the negated system: r = -(b - A x) on free rows */
        sys_mult(A, x, q);
#pragma omp parallel for schedule(static)
        for (long n = 0; n < N; ++n) r[n] = A->dir[n] ? 0.0 : -(A->b[n] - q[n]);
        rnorm = sqrt(dot(r, r, N));
        if (rnorm <= tol) { conv = 1; break; }
        if (!(rnorm == rnorm) || isinf(rnorm)) break;   /* non-finite: give up */
        if (it >= maxit) break;
#pragma omp parallel for schedule(static)
        for (long n = 0; n < N; ++n) z[n] = A->dir[n] ? 0.0 : r[n] / (-A->cC[n]);
        memcpy(pv, z, N * sizeof(double));
        double rz = dot(r, z, N);
        int inner = 0;
        while (it < maxit && inner < 2000) {
            sys_mult(A, pv, q);     /* (-A) p on free rows */
#pragma omp parallel for schedule(static)
            for (long n = 0; n < N; ++n) q[n] = A->dir[n] ? 0.0 : -q[n];
            double pq = dot(pv, q, N);
            if (pq == 0.0) break;
            double al = rz / pq;
#pragma omp parallel for schedule(static)
            for (long n = 0; n < N; ++n) {
                x[n] += al * pv[n];   /* x solves (-A) x = -b, i.e. A x = b */
                r[n] -= al * q[n];
            }
            ++it; ++inner;
            double rr = sqrt(dot(r, r, N));
            if (rr <= 0.5 * tol || !(rr == rr) || isinf(rr)) break;
#pragma omp parallel for schedule(static)
            for (long n = 0; n < N; ++n) z[n] = A->dir[n] ? 0.0 : r[n] / (-A->cC[n]);
            double rz2 = dot(r, z, N);
            double be = rz2 / rz;
            rz = rz2;
#pragma omp parallel for schedule(static)
            for (long n = 0; n < N; ++n) pv[n] = z[n] + be * pv[n];
        }
    }
    info->iterations = it;
    info->converged = conv;
    info->rnorm = rnorm;
    info->bnorm = bnorm;
    free(r); free(z); free(pv); free(q);
    return conv ? 0 : 1;
}

/*
 * Multigrid-preconditioned CG on the same SPD free-row system as solve_cg,
 * stopped by the same test on the true residual ||b - A x|| <= rtol*||b||.
 * Only the speed differs: at 128^3 Jacobi-PCG needs ~1300 iterations per
 * solve, this ~15.  The converged pressure is a property of the assembled
 * system (sys_build, wPFAW3D.f90:629-936), not of the solver.
 *
 * Preconditioner: one W-cycle over a hierarchy of 2x2x2 box aggregates
 * (piecewise-constant interpolation P, coarse operator the Galerkin product
 * P^T M P), symmetric red-black Gauss-Seidel (nu sweeps red->black before,
 * black->red after), zero start on every level, exact solve on the final
 * single cell; the whole cycle is a symmetric positive definite operator, as
 * CG requires.  Cells with a zero diagonal (Dirichlet rows and aggregates of
 * them) are inert.  The matrix is stored as a diagonal d > 0 and the six
 * neighbour couplings c >= 0 (M x = d x - sum c x_nb).
 */
typedef struct {
    int nx, ny, nz;
    long N;
    double *d, *ce, *cn, *ct;   /* couplings toward x+, y+, z+ (the x- coupling of cell q
                                  is ce[q - 1], and so on: M is symmetric) */
    double *x, *r, *t;
} mg_level;

#define MG_MAX_LEVELS 24
#define MG_SERIAL_CELLS 32768   /* smaller levels run on one thread (fork/join costs more) */

static double mg_row(const mg_level* L, long q, int i, int j, int k, const double* x) {
    long sy = L->nx, sz = (long)L->nx * L->ny;
    double s = 0.0;
    if (i > 0) s += L->ce[q - 1] * x[q - 1];
    if (i < L->nx - 1) s += L->ce[q] * x[q + 1];
    if (j > 0) s += L->cn[q - sy] * x[q - sy];
    if (j < L->ny - 1) s += L->cn[q] * x[q + sy];
    if (k > 0) s += L->ct[q - sz] * x[q - sz];
    if (k < L->nz - 1) s += L->ct[q] * x[q + sz];
    return s;
}

/* One colour of a Gauss-Seidel sweep: x = (r + sum c x_nb) / d on the cells
 * with (i + j + k) % 2 == colour. */
static void mg_colour(mg_level* L, int colour) {
#pragma omp parallel for schedule(static) if (L->N > MG_SERIAL_CELLS)
    for (int k = 0; k < L->nz; ++k)
        for (int j = 0; j < L->ny; ++j)
            for (int i = (j + k + colour) & 1; i < L->nx; i += 2) {
                long q = i + (long)L->nx * (j + (long)L->ny * k);
                if (L->d[q] > 0.0) L->x[q] = (L->r[q] + mg_row(L, q, i, j, k, L->x)) / L->d[q];
            }
}

/* t = r - M x */
static void mg_resid(mg_level* L) {
#pragma omp parallel for schedule(static) if (L->N > MG_SERIAL_CELLS)
    for (int k = 0; k < L->nz; ++k)
        for (int j = 0; j < L->ny; ++j)
            for (int i = 0; i < L->nx; ++i) {
                long q = i + (long)L->nx * (j + (long)L->ny * k);
                L->t[q] = L->d[q] > 0.0 ? L->r[q] - (L->d[q] * L->x[q] - mg_row(L, q, i, j, k, L->x))
                                        : 0.0;
            }
}

static long mg_parent(const mg_level* F, const mg_level* Cl, long q) {
    long i = q % F->nx, j = (q / F->nx) % F->ny, k = q / ((long)F->nx * F->ny);
    return (i >> 1) + (long)Cl->nx * ((j >> 1) + (long)Cl->ny * (k >> 1));
}

static void mg_alloc(mg_level* L, int nx, int ny, int nz) {
    L->nx = nx; L->ny = ny; L->nz = nz;
    L->N = (long)nx * ny * nz;
    double** a[7] = {&L->d, &L->ce, &L->cn, &L->ct, &L->x, &L->r, &L->t};
    for (int m = 0; m < 7; ++m) *a[m] = (double*)calloc((size_t)L->N, sizeof(double));
}

static void mg_free(mg_level* L) {
    free(L->d); free(L->ce); free(L->cn); free(L->ct);
    free(L->x); free(L->r); free(L->t);
}

/* Galerkin coarse operator of 2x2x2 aggregation: the diagonal of aggregate I
 * is sum_{i,j in I} M_ij, its coupling toward the next aggregate along an
 * axis is the sum of the fine couplings across the shared face.  Gathered
 * per coarse cell (the fine cells of one aggregate are its children). */
static void mg_coarsen(const mg_level* F, mg_level* Cl) {
    mg_alloc(Cl, (F->nx + 1) / 2, (F->ny + 1) / 2, (F->nz + 1) / 2);
#pragma omp parallel for schedule(static) if (F->N > MG_SERIAL_CELLS)
    for (int K = 0; K < Cl->nz; ++K)
        for (int J = 0; J < Cl->ny; ++J)
            for (int I = 0; I < Cl->nx; ++I) {
                long P = I + (long)Cl->nx * (J + (long)Cl->ny * K);
                double d = 0.0, ce = 0.0, cn = 0.0, ct = 0.0;
                for (int k = 2 * K; k < 2 * K + 2 && k < F->nz; ++k)
                    for (int j = 2 * J; j < 2 * J + 2 && j < F->ny; ++j)
                        for (int i = 2 * I; i < 2 * I + 2 && i < F->nx; ++i) {
                            long q = i + (long)F->nx * (j + (long)F->ny * k);
                            if (!(F->d[q] > 0.0)) continue;
                            d += F->d[q];
                            /* a face inside the aggregate counts twice against the
                               diagonal (once from each side); a face toward a dead
                               neighbour carries no coupling (c = 0) */
                            if (i + 1 < F->nx) {
                                if (i == 2 * I + 1) ce += F->ce[q]; else d -= 2.0 * F->ce[q];
                            }
                            if (j + 1 < F->ny) {
                                if (j == 2 * J + 1) cn += F->cn[q]; else d -= 2.0 * F->cn[q];
                            }
                            if (k + 1 < F->nz) {
                                if (k == 2 * K + 1) ct += F->ct[q]; else d -= 2.0 * F->ct[q];
                            }
                        }
                Cl->d[P] = d > 1e-300 ? d : 0.0;
                Cl->ce[P] = I < Cl->nx - 1 ? ce : 0.0;
                Cl->cn[P] = J < Cl->ny - 1 ? cn : 0.0;
                Cl->ct[P] = K < Cl->nz - 1 ? ct : 0.0;
            }
}

/* Cl->r = P^T t (sum of the live children's residuals). */
static void mg_restrict(const mg_level* F, mg_level* Cl) {
#pragma omp parallel for schedule(static) if (F->N > MG_SERIAL_CELLS)
    for (int K = 0; K < Cl->nz; ++K)
        for (int J = 0; J < Cl->ny; ++J)
            for (int I = 0; I < Cl->nx; ++I) {
                double s = 0.0;
                for (int k = 2 * K; k < 2 * K + 2 && k < F->nz; ++k)
                    for (int j = 2 * J; j < 2 * J + 2 && j < F->ny; ++j)
                        for (int i = 2 * I; i < 2 * I + 2 && i < F->nx; ++i) {
                            long q = i + (long)F->nx * (j + (long)F->ny * k);
                            if (F->d[q] > 0.0) s += F->t[q];
                        }
                Cl->r[I + (long)Cl->nx * (J + (long)Cl->ny * K)] = s;
            }
}

/* One W-cycle for M_l x = r_l from the current x of level l: the coarse
 * problem is visited twice (its second visit continues from the first). */
static void mg_cycle(mg_level* lv, int nlev, int l, int nu) {
    mg_level* L = &lv[l];
    if (l == nlev - 1) {                      /* the single-cell level: exact */
        for (int s = 0; s < 2; ++s) { mg_colour(L, 0); mg_colour(L, 1); mg_colour(L, 1); mg_colour(L, 0); }
        return;
    }
    mg_level* Cl = &lv[l + 1];
    for (int s = 0; s < nu; ++s) { mg_colour(L, 0); mg_colour(L, 1); }
    mg_resid(L);
    mg_restrict(L, Cl);
    memset(Cl->x, 0, (size_t)Cl->N * sizeof(double));
    mg_cycle(lv, nlev, l + 1, nu);
    if (l + 1 < nlev - 1) mg_cycle(lv, nlev, l + 1, nu);
#pragma omp parallel for schedule(static) if (L->N > MG_SERIAL_CELLS)
    for (long q = 0; q < L->N; ++q) if (L->d[q] > 0.0) L->x[q] += Cl->x[mg_parent(L, Cl, q)];
    for (int s = 0; s < nu; ++s) { mg_colour(L, 1); mg_colour(L, 0); }
}

static int solve_mgcg(const sysmat* A, double* x, double rtol, int maxit, orc_solve_info* info) {
    long N = A->N;
    mg_level lv[MG_MAX_LEVELS];
    int nlev = 1;
    mg_alloc(&lv[0], A->nx, A->ny, A->nz);
    for (long q = 0; q < N; ++q) {
        if (A->dir[q]) continue;
        lv[0].d[q] = -A->cC[q];
        lv[0].ce[q] = A->cE[q]; lv[0].cn[q] = A->cN[q]; lv[0].ct[q] = A->cT[q];
    }
    while (nlev < MG_MAX_LEVELS && lv[nlev - 1].N > 1) {
        mg_coarsen(&lv[nlev - 1], &lv[nlev]);
        ++nlev;
    }
    double *r = malloc(N * sizeof(double)), *pv = malloc(N * sizeof(double)),
           *q = malloc(N * sizeof(double));
    double* z = lv[0].x;
    double bnorm = sqrt(dot(A->b, A->b, N));
    for (long n = 0; n < N; ++n) if (A->dir[n]) x[n] = A->b[n];
    double tol = rtol * bnorm;
    int it = 0, conv = 0;
    double rnorm = 0.0;
    for (int restart = 0; restart < 50 && !conv; ++restart) {
        sys_mult(A, x, q);
#pragma omp parallel for schedule(static)
        for (long n = 0; n < N; ++n) r[n] = A->dir[n] ? 0.0 : (A->b[n] - q[n]);
        rnorm = sqrt(dot(r, r, N));
        if (rnorm <= tol) { conv = 1; break; }
        if (!(rnorm == rnorm) || isinf(rnorm)) break;
        if (it >= maxit) break;
        /* M = -A on free rows: x solves M x = -b, whose residual is -r_A. */
        for (long n = 0; n < N; ++n) r[n] = -r[n];
        memcpy(lv[0].r, r, N * sizeof(double));
        memset(z, 0, N * sizeof(double));
        mg_cycle(lv, nlev, 0, 1);
        memcpy(pv, z, N * sizeof(double));
        double rz = dot(r, z, N);
        int inner = 0;
        while (it < maxit && inner < 200) {
            sys_mult(A, pv, q);
#pragma omp parallel for schedule(static)
            for (long n = 0; n < N; ++n) q[n] = A->dir[n] ? 0.0 : -q[n];
            double pq = dot(pv, q, N);
            if (pq == 0.0) break;
            double al = rz / pq;
#pragma omp parallel for schedule(static)
            for (long n = 0; n < N; ++n) {
                x[n] += al * pv[n];
                r[n] -= al * q[n];
            }
            ++it; ++inner;
            double rr = sqrt(dot(r, r, N));
            if (rr <= 0.5 * tol || !(rr == rr) || isinf(rr)) break;
            memcpy(lv[0].r, r, N * sizeof(double));
            memset(z, 0, N * sizeof(double));
            mg_cycle(lv, nlev, 0, 1);
            double rz2 = dot(r, z, N);
            double be = rz2 / rz;
            rz = rz2;
#pragma omp parallel for schedule(static)
            for (long n = 0; n < N; ++n) pv[n] = z[n] + be * pv[n];
        }
    }
    info->iterations = it;
    info->converged = conv;
    info->rnorm = rnorm;
    info->bnorm = bnorm;
    free(r); free(pv); free(q);
    for (int l = 0; l < nlev; ++l) mg_free(&lv[l]);
    return conv ? 0 : 1;
}

/*
 * solvePressure, wPFAW3D.f90:603-1160: build the system (:629-936), solve it
 * warm-started from the current pressure (:977-986), copy the result into
 * the interior (:1048) and refresh the halo (:1050).
 */
int orc_solve_pressure(orc_state* s, int mode, double rtol, int maxit, int nblocks,
                       orc_solve_info* info) {
    const orc_params* p = &s->p;
    int nx = p->nx, ny = p->ny, nz = p->nz;
    sysmat A;
    sys_build(s, &A);
    long N = A.N;
    double* x = malloc(N * sizeof(double));
    for (int iz = 1; iz <= nz; ++iz)
        for (int iy = 1; iy <= ny; ++iy)
            for (int ix = 1; ix <= nx; ++ix) x[gidx(p, ix, iy, iz)] = s->pressure[IDX(p, ix, iy, iz)];
    orc_solve_info tmp;
    if (!info) info = &tmp;
    memset(info, 0, sizeof(*info));
    int rc = mode == ORC_SOLVE_BCGS_SOR ? solve_bcgs(&A, x, rtol, maxit, nblocks, info)
             : mode == ORC_SOLVE_MGCG   ? solve_mgcg(&A, x, rtol, maxit, info)
                                        : solve_cg(&A, x, rtol, maxit, info);
    /* true relative residual of the returned iterate */
    double* y = malloc(N * sizeof(double));
    sys_mult(&A, x, y);
    for (long n = 0; n < N; ++n) y[n] = A.b[n] - y[n];
    double bn = sqrt(dot(A.b, A.b, N));
    info->true_relres = bn > 0 ? sqrt(dot(y, y, N)) / bn : 0.0;
    for (int iz = 1; iz <= nz; ++iz)
        for (int iy = 1; iy <= ny; ++iy)
            for (int ix = 1; ix <= nx; ++ix) s->pressure[IDX(p, ix, iy, iz)] = x[gidx(p, ix, iy, iz)];
    orc_update_halo(p, s->pressure);
    free(x); free(y);
    sys_free(&A);
    return rc;
}

/* ---- calcVelocity, wPFAW3D.f90:1164-1193 ------------------------------- */
void orc_calc_velocity(orc_state* s) {
    const orc_params* p = &s->p;
    int nx = p->nx, ny = p->ny, nz = p->nz;
    const double* P = s->pressure;
    const double* K = s->permeab;
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                long n = IDX(p, i, j, k);
                double g1 = (P[IDX(p, i + 1, j, k)] - P[n]) / p->dx;   /* :1189 */
                double g2 = (P[IDX(p, i, j + 1, k)] - P[n]) / p->dx;   /* :1190 */
                double g3 = (P[IDX(p, i, j, k + 1)] - P[n]) / p->dx;   /* :1191 */
                s->velocity[3 * n + 0] = -(K[4 * n + 1] / p->viscosity * g1);  /* :1173 */
                s->velocity[3 * n + 1] = -(K[4 * n + 2] / p->viscosity * g2);
                s->velocity[3 * n + 2] = -(K[4 * n + 3] / p->viscosity * g3);
            }
}

/* ---- calcPhaseDeriv, wPFAW3D.f90:1197-1440 ----------------------------- */
double orc_calc_phase_deriv(orc_state* s, long* overshoot) {
    const orc_params* p = &s->p;
    int nx = p->nx, ny = p->ny, nz = p->nz;
    const double* ph = s->phase;
    const double* V = s->velocity;
    const double dx = p->dx;
    const double phi_0 = 0.0, theta0 = 0.0;             /* :1219-1220 */
    const double w0 = 2.0 * dx;                          /* :1221 */
    const double maxdphi = 2.0 / (2.0 * dx);             /* :1225 */
    double taumin = 1.0e6;                               /* :1223 */
    long nover = 0;
#define PH(a, b, c) ph[IDX(p, (a), (b), (c))]
#pragma omp parallel for schedule(static) reduction(min : taumin) reduction(+ : nover)
    for (int iz = 1; iz <= nz; ++iz)
        for (int iy = 1; iy <= ny; ++iy)
            for (int ix = 1; ix <= nx; ++ix) {
                long n = IDX(p, ix, iy, iz);
                /* grad_phase, :1468-1475 */
                double gpf1 = (PH(ix + 1, iy, iz) - PH(ix - 1, iy, iz)) / (2.0 * dx);
                double gpf2 = (PH(ix, iy + 1, iz) - PH(ix, iy - 1, iz)) / (2.0 * dx);
                double gpf3 = (PH(ix, iy, iz + 1) - PH(ix, iy, iz - 1)) / (2.0 * dx);
                double dpf = sqrt(gpf1 * gpf1 + gpf2 * gpf2 + gpf3 * gpf3);   /* :1232 */
                double vs, vt;
                if (dpf > 1.0e-6) {                                            /* :1234-1244 */
                    double n1 = gpf1 / dpf, n2 = gpf2 / dpf, n3 = gpf3 / dpf;
                    double vx = 0.5 * (V[3 * n + 0] + V[3 * IDX(p, ix - 1, iy, iz) + 0]);
                    double vy = 0.5 * (V[3 * n + 1] + V[3 * IDX(p, ix, iy - 1, iz) + 1]);
                    double vz = 0.5 * (V[3 * n + 2] + V[3 * IDX(p, ix, iy, iz - 1) + 2]);
                    vs = vx * n1 + vy * n2 + vz * n3;
                    vt = 0.0;
                } else {
                    vs = 0.0;
                    vt = 0.0;
                }
                double kxx;
                if (vs >= 0.0) kxx = p->diffusion;                              /* :1246-1252 */
                else kxx = p->diffusion + fabs(s->concent[n]) * p->epsilon *
                                             (p->ral * (vs * vs) + p->rat * (vt * vt)) /
                                             sqrt(vs * vs + vt * vt);
                double tau = 5.0 / 3.0 * p->alpha * p->lambda * (p->epsilon * p->epsilon) / kxx; /* :1254 */
                if (tau < taumin) taumin = tau;                                 /* :1255 */
                if (s->lw[n] > 0) { s->dphasedt[n] = 0.0; continue; }           /* :1257-1261 */

                double phix = gpf1, phiy = gpf2, phiz = gpf3;                   /* :1264-1266 */
                double c0 = PH(ix, iy, iz);
                double phixx = (PH(ix + 1, iy, iz) - 2.0 * c0 + PH(ix - 1, iy, iz)) / (dx * dx);
                double phiyy = (PH(ix, iy + 1, iz) - 2.0 * c0 + PH(ix, iy - 1, iz)) / (dx * dx);
                double phizz = (PH(ix, iy, iz + 1) - 2.0 * c0 + PH(ix, iy, iz - 1)) / (dx * dx);
                double phixy = (PH(ix + 1, iy + 1, iz) - PH(ix + 1, iy - 1, iz) - PH(ix - 1, iy + 1, iz) +
                                PH(ix - 1, iy - 1, iz)) / (4.0 * (dx * dx));
                double phiyz = (PH(ix, iy + 1, iz + 1) - PH(ix, iy - 1, iz + 1) - PH(ix, iy + 1, iz - 1) +
                                PH(ix, iy - 1, iz - 1)) / (4.0 * (dx * dx));
                double phizx = (PH(ix + 1, iy, iz + 1) - PH(ix - 1, iy, iz + 1) - PH(ix + 1, iy, iz - 1) +
                                PH(ix - 1, iy, iz - 1)) / (4.0 * (dx * dx));
                if (phix == 0 && phiy == 0 && phiz == 0 && phixx == 0 && phiyy == 0 && phizz == 0 &&
                    phixy == 0 && phiyz == 0 && phizx == 0) {                   /* :1283-1286 */
                    s->dphasedt[n] = 0;
                    continue;
                }
                double theta = atan(phiy / (phix + 1.0e-20));                   /* :1289 */
                double phi_ = acos(phiz / (dpf + 1.0e-20));                     /* :1290 */
                double dtheta = theta - theta0, dphi_ = phi_ - phi_0;
                double eps = p->epsilon;                                        /* :1298 */
                double c = cos(dtheta), sn = sin(dtheta);
                double c2 = c * c, s2 = sn * sn, c4 = c2 * c2, s4 = s2 * s2;
                double c4phi = cos(4.0 * dphi_), s4phi = sin(4.0 * dphi_);
                double w = w0 * (1.0 + eps * (7.0 * c4 - 6.0 * c2 + s4 * c4phi));               /* :1309 */
                double dwdtheta = w0 * (4.0 * eps * sn * c * (-7.0 * c2 + 3.0 + s2 * c4phi));     /* :1312 */
                double ddwdtheta = w0 * (4.0 * eps * (cos(2.0 * dtheta) * (-7.0 * c2 + 3.0 + s2 * c4phi) +
                                                      2.0 * s2 * c2 * (7.0 + c4phi)));            /* :1316 */
                double dwdphi_ = w0 * (-4.0 * eps * s4 * s4phi);                                   /* :1320 */
                double ddwdphi_ = w0 * (-16.0 * eps * s4 * c4phi);                                 /* :1323 */
                double ddwdthetadphi_ = w0 * (-16.0 * eps * (s2 * sn) * c * s4phi);                 /* :1326 */

                double dthetadx = 0.0, dthetady = 0.0, dthetadz = 0.0;          /* :1330-1337 */
                if (phix > maxdphi || phiy > maxdphi) {
                    dthetadx = (phixy * phix - phiy * phixx) / (phix * phix + phiy * phiy + 1.0e-20);
                    dthetady = (phiyy * phix - phiy * phixy) / (phix * phix + phiy * phiy + 1.0e-20);
                    dthetadz = (phiyz * phix - phiy * phizx) / (phix * phix + phiy * phiy + 1.0e-20);
                }
                double dphi_dx = 0, dphi_dy = 0, dphi_dz = 0;                  /* :1339-1351 */
                if (phix > maxdphi || phiy > maxdphi || phiz > maxdphi) {
                    double den = (phix * phix + phiy * phiy + phiz * phiz) * sqrt(phix * phix + phiy * phiy) + 1.0e-20;
                    dphi_dx = (phiz * (phix * phixx + phiy * phixy) - (phix * phix + phiy * phiy) * phizx) / den;
                    dphi_dy = (phiz * (phix * phixy + phiy * phiyy) - (phix * phix + phiy * phiy) * phiyz) / den;
                    dphi_dz = (phiz * (phix * phizx + phiy * phiyz) - (phix * phix + phiy * phiy) * phizz) / den;
                }
                double dthetaddpdx = 0.0, dthetaddpdy = 0.0;                    /* :1353-1359 */
                if (phix > maxdphi || phiy > maxdphi) {
                    dthetaddpdx = -phiy * (phix * phix + phiy * phiy + phiz * phiz) / ((phix * phix + phiy * phiy) + 1.0e-20);
                    dthetaddpdy = phix * (phix * phix + phiy * phiy + phiz * phiz) / ((phix * phix + phiy * phiy) + 1.0e-20);
                }
                double dthetaddpdz = 0.0;
                double rxy = sqrt(phix * phix + phiy * phiy);                   /* :1363-1365 */
                double dphi_ddpdx = phix * phiz / (rxy * dpf + 1.0e-20);
                double dphi_ddpdy = phiy * phiz / (rxy * dpf + 1.0e-20);
                double dphi_ddpdz = -rxy / (dpf + 1.0e-20);

                double dwdx = dwdtheta * dthetadx + dwdphi_ * dphi_dx;          /* :1367-1377 */
                double dwdy = dwdtheta * dthetady + dwdphi_ * dphi_dy;
                double dwdz = dwdtheta * dthetadz + dwdphi_ * dphi_dz;
                double ddwdthetax = ddwdtheta * dthetadx + ddwdthetadphi_ * dphi_dx;
                double ddwdthetay = ddwdtheta * dthetady + ddwdthetadphi_ * dphi_dy;
                double ddwdthetaz = ddwdtheta * dthetadz + ddwdthetadphi_ * dphi_dz;
                double ddwdphi_x = ddwdphi_ * dphi_dx + ddwdthetadphi_ * dthetadx;
                double ddwdphi_y = ddwdphi_ * dphi_dy + ddwdthetadphi_ * dthetady;
                double ddwdphi_z = ddwdphi_ * dphi_dz + ddwdthetadphi_ * dthetadz;

                double f1 = (1.0 - c0 * c0) * (c0 - p->lambda * s->concent[n]);              /* :1381 */
                double f2 = 2.0 * w * (dwdx * phix + dwdy * phiy + dwdz * phiz);              /* :1386 */
                double lap = (PH(ix + 1, iy, iz) + PH(ix - 1, iy, iz) + PH(ix, iy + 1, iz) + PH(ix, iy - 1, iz) +
                              PH(ix, iy, iz + 1) + PH(ix, iy, iz - 1) - 6 * c0) / (dx * dx);  /* :1451-1460 */
                double f3 = (w * w) * lap;                                                    /* :1390 */
                double d2 = dpf * dpf;
                double f4 = dwdx * (dwdtheta * dthetaddpdx * d2 + dwdphi_ * dphi_ddpdx * d2) +
                            w * (ddwdthetax * dthetaddpdx * d2 + ddwdphi_x * dphi_ddpdx * d2);   /* :1395 */
                double f5 = dwdy * (dwdtheta * dthetaddpdy * d2 + dwdphi_ * dphi_ddpdy * d2) +
                            w * (ddwdthetay * dthetaddpdy * d2 + ddwdphi_y * dphi_ddpdy * d2);   /* :1401 */
                double f6 = dwdz * (dwdtheta * dthetaddpdz * d2 + dwdphi_ * dphi_ddpdz * d2) +
                            w * (ddwdthetaz * dthetaddpdz * d2 + ddwdphi_z * dphi_ddpdz * d2);   /* :1407 */
                double f7 = 0;                                                                /* :1412 */
                s->dphasedt[n] = (f1 + f2 + f3 + f4 + f5 + f6 + f7) / tau;                   /* :1414 */
                if (c0 > 1 || c0 < -1) ++nover;                                               /* :1425-1427 */
            }
#undef PH
    if (overshoot) *overshoot = nover;
    return taumin;   /* single domain: the MPI MIN of :1440 is the identity */
}

/* ---- calcConcentDeriv, wPFAW3D.f90:1554-1624 --------------------------- */
void orc_calc_concent_deriv(orc_state* s) {
    const orc_params* p = &s->p;
    int nx = p->nx, ny = p->ny, nz = p->nz;
    const double* C = s->concent;
    const double* V = s->velocity;
    const double dx = p->dx;
#define CC(a, b, c) C[IDX(p, (a), (b), (c))]
#define VV(m, a, b, c) V[3 * IDX(p, (a), (b), (c)) + (m)]
#pragma omp parallel for schedule(static)
    for (int iz = 1; iz <= nz; ++iz)
        for (int iy = 1; iy <= ny; ++iy)
            for (int ix = 1; ix <= nx; ++ix) {
                long n = IDX(p, ix, iy, iz);
                if (s->lw[n] > 0) { s->dconcentdt[n] = 0.0; continue; }        /* :1562-1566 */
                double c0 = CC(ix, iy, iz);
                double lap = (CC(ix + 1, iy, iz) + CC(ix - 1, iy, iz) + CC(ix, iy + 1, iz) + CC(ix, iy - 1, iz) +
                              CC(ix, iy, iz + 1) + CC(ix, iy, iz - 1) - 6 * c0) / (dx * dx);   /* :1614-1623 */
                /* div_flow, :1586-1606 */
                double uxp = VV(0, ix, iy, iz), uxm = VV(0, ix - 1, iy, iz);
                double uyp = VV(1, ix, iy, iz), uym = VV(1, ix, iy - 1, iz);
                double uzp = VV(2, ix, iy, iz), uzm = VV(2, ix, iy, iz - 1);
                double fxp = uxp * (uxp > 0.0 ? c0 : CC(ix + 1, iy, iz));
                double fxm = uxm * (uxm > 0.0 ? CC(ix - 1, iy, iz) : c0);
                double fyp = uyp * (uyp > 0.0 ? c0 : CC(ix, iy + 1, iz));
                double fym = uym * (uym > 0.0 ? CC(ix, iy - 1, iz) : c0);
                double fzp = uzp * (uzp > 0.0 ? c0 : CC(ix, iy, iz + 1));
                double fzm = uzm * (uzm > 0.0 ? CC(ix, iy, iz - 1) : c0);
                double div = (fxp - fxm) / dx + (fyp - fym) / dx + (fzp - fzm) / dx;
                double c1 = p->diffusion * lap;                                  /* :1568-1573 */
                double c2 = p->alpha * s->dphasedt[n];
                double c3 = 0.0;
                double c7 = -div;
                s->dconcentdt[n] = c1 + c2 + c3 + c7;
            }
#undef CC
#undef VV
}

/* ---- evolvePhase / evolveConcent, wPFAW3D.f90:1628-1640 ---------------- */
void orc_evolve_phase(orc_state* s, double dtime) {
    long G = gsize(&s->p);
    for (long n = 0; n < G; ++n) s->phase[n] = s->phase[n] + s->dphasedt[n] * dtime;
    orc_update_halo(&s->p, s->phase);
}
void orc_evolve_concent(orc_state* s, double dtime) {
    long G = gsize(&s->p);
    for (long n = 0; n < G; ++n) s->concent[n] = s->concent[n] + s->dconcentdt[n] * dtime;
    orc_update_halo(&s->p, s->concent);
}

/* ---- time-step law, wPFAW3D.f90:2227-2230 ------------------------------ */
double orc_next_dtime(const orc_params* p, double tfac, int itime, double dtime, double taumin) {
    if (itime >= 3) {
        double e2 = p->epsilon * p->epsilon;
        double a = e2 / p->diffusion;
        return tfac * 0.5 * (p->dx * p->dx) / e2 * (a < taumin ? a : taumin);
    }
    return dtime;
}

/* ---- showProgress reductions, wPFAW3D.f90:1695, 1756-1801 -------------- */
void orc_diagnostics(const orc_state* s, orc_diag* d) {
    const orc_params* p = &s->p;
    int nx = p->nx, ny = p->ny, nz = p->nz;
    double dx = p->dx, sum_m = 0.0, sum_p = 0.0, r2whmax = 0.0;
    double xref = dx * (p->ix_ref - 1) + 0.5 * dx;
    double yref = dx * (p->iy_ref - 1) + 0.5 * dx;
    double zref = dx * (p->iz_ref - 1) + 0.5 * dx;
    for (int iz = 1; iz <= nz; ++iz)
        for (int iy = 1; iy <= ny; ++iy)
            for (int ix = 1; ix <= nx; ++ix) {
                double f = s->phase[IDX(p, ix, iy, iz)];
                sum_m += 1.0 - f;
                sum_p += 1.0 + f;
                if (f > 0.0) {
                    double x = dx * (ix - 1) + 0.5 * dx, y = dx * (iy - 1) + 0.5 * dx,
                           z = dx * (iz - 1) + 0.5 * dx;
                    double r2 = (x - xref) * (x - xref) + (y - yref) * (y - yref) + (z - zref) * (z - zref);
                    if (r2 > r2whmax) r2whmax = r2;
                }
            }
    d->pv = dx * dx * dx * p->porosity * 0.5 * sum_m;
    d->vcal = dx * dx * dx * (1.0 - p->porosity) * 0.5 * sum_p;
    d->rwhmax = sqrt(r2whmax);
    long G = gsize(p);
    double pmax = s->phase[0], pmin = s->phase[0], cmax = s->concent[0], cmin = s->concent[0];
    for (long n = 0; n < G; ++n) {
        if (s->phase[n] > pmax) pmax = s->phase[n];
        if (s->phase[n] < pmin) pmin = s->phase[n];
        if (s->concent[n] > cmax) cmax = s->concent[n];
        if (s->concent[n] < cmin) cmin = s->concent[n];
    }
    d->phase_max = pmax; d->phase_min = pmin; d->concent_max = cmax; d->concent_min = cmin;
}

/* getPressure, wPFAW3D.f90:2151-2166 (single domain). */
double orc_get_pressure(const orc_state* s, int ix, int iy, int iz) {
    const orc_params* p = &s->p;
    if (1 <= ix && ix <= p->nx && 1 <= iy && iy <= p->ny && 1 <= iz && iz <= p->nz)
        return s->pressure[IDX(p, ix, iy, iz)];
    return 0.0;
}
