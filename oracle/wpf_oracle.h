/*
 * wpf_oracle.h -- CPU oracle for the wPFAW3D time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * Fortran routines (wPFAW3D.f90) used as the parity checker for the CUDA
 * path and as the timed CPU baseline.  Only tests/, __graft_entry__.smoke()
 * and bench.py (cpu_baseline / --impl reference) may load it.  The product
 * library never links or calls it.
 *
 * Parity status: the reference cannot be built or run in this environment
 * (Fortran + Intel MPI + PETSc 3.22, none present), and it ships no golden
 * vectors, so the oracle is "parity unpinned" against the reference binary.
 * It is pinned instead by analytic known-answer cases and by an independent
 * scipy.sparse direct solve of the matrix assembled exactly as
 * wPFAW3D.f90:629-936 assembles it (tests/test_oracle_*.py).
 *
 * Array convention (identical to the reference arrays): every field carries a
 * one-cell halo and is stored Fortran order, x fastest,
 *     idx(i,j,k) = i + (nx+2)*(j + (ny+2)*k),   i in 0..nx+1 (etc.)
 * permeab is (0:3, G) with the component fastest (permeab[4*idx+m]) and
 * velocity is (1:3, G) (velocity[3*idx+m-1]), as in wPFAW3D.f90:97-99.
 */
#ifndef WPF_ORACLE_H
#define WPF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    int32_t nx, ny, nz;      /* interior cells (single domain: local == global) */
    int32_t ix_ref, iy_ref, iz_ref;
    double dx;               /* grid spacing = dxw * epsilon                  */
    double epsilon;          /* interface width w (also anisotropy strength)  */
    double lambda;           /* phase / concentration coupling                */
    double porosity;
    double viscosity;
    double diffusion;
    double ral, rat;         /* dispersivities                                */
    double permeab_hole;     /* kwh                                           */
    double alpha;            /* 0.5/b/kc, derived                             */
} orc_params;

typedef struct orc_well {
    int32_t ix, iy, iz;      /* global 1-based cell index                     */
    int32_t pad;
    double pressure;         /* fixed pressure (Dirichlet iff != 0)           */
    double injection;        /* injection rate (inlet iff != 0)               */
    double phase, concent;   /* fixed phase-field / concentration             */
} orc_well;

typedef struct orc_state {
    orc_params p;
    int32_t nwell;
    int32_t pad;
    const orc_well* well;    /* well[0..nwell-1] (Fortran well(1..nwell))     */
    int32_t* lw;             /* G: 1-based well index or 0                   */
    double* permeab_rock;    /* G                                             */
    double* permeab;         /* 4*G                                           */
    double* pressure;        /* G                                             */
    double* velocity;        /* 3*G                                           */
    double* phase;           /* G                                             */
    double* concent;         /* G                                             */
    double* dphasedt;        /* G                                             */
    double* dconcentdt;      /* G                                             */
} orc_state;

/* Solver modes of orc_solve_pressure. */
#define ORC_SOLVE_BCGS_SOR 0   /* mirror of KSPBCGS + PCSOR(10,1,1.7), wPFAW3D.f90:988-1004 */
#define ORC_SOLVE_CG       1   /* Jacobi-PCG on the SPD free-cell system, tight true residual */
#define ORC_SOLVE_MGCG     2   /* the same system and stopping test, multigrid-preconditioned CG */

typedef struct orc_solve_info {
    int32_t iterations;
    int32_t converged;       /* 1 if the tolerance was met                    */
    double rnorm;            /* final residual norm used by the test          */
    double bnorm;            /* reference norm (||B b|| or ||b||)             */
    double true_relres;      /* ||b - A x|| / ||b|| of the returned iterate  */
} orc_solve_info;

typedef struct orc_diag {
    double pv;               /* pore volume, wPFAW3D.f90:1695                 */
    double vcal;             /* dissolved volume, :1776                       */
    double rwhmax;           /* max wormhole radius, :1756-1775               */
    double phase_max, phase_min, concent_max, concent_min;   /* :1798-1801    */
} orc_diag;

int    orc_version(void);
void   orc_set_threads(int n);
void   orc_build_lw(orc_state* s);
void   orc_init_fields(orc_state* s, double init_permeab, double init_phase,
                       double init_concent, double pini);
void   orc_apply_well_values(orc_state* s);
void   orc_update_halo(const orc_params* p, double* f);
void   orc_calc_permeability(orc_state* s);
long   orc_assemble(const orc_state* s, int32_t* irn, int32_t* jcn, double* val, double* b);
int    orc_solve_pressure(orc_state* s, int mode, double rtol, int maxit, int nblocks,
                          orc_solve_info* info);
void   orc_calc_velocity(orc_state* s);
double orc_calc_phase_deriv(orc_state* s, long* overshoot);
void   orc_calc_concent_deriv(orc_state* s);
void   orc_evolve_phase(orc_state* s, double dtime);
void   orc_evolve_concent(orc_state* s, double dtime);
double orc_next_dtime(const orc_params* p, double tfac, int itime, double dtime, double taumin);
void   orc_diagnostics(const orc_state* s, orc_diag* d);
double orc_get_pressure(const orc_state* s, int ix, int iy, int iz);

#ifdef __cplusplus
}
#endif
#endif
