/*
 * wpf.h -- C ABI of the GB300-native wPFAW3D time step (libwpf_gb300.so).
 *
 * The reference (hfuki/mizuho_edit, wPFAW3D.f90) runs its time step as
 * argument-less module subroutines over module-global Fortran arrays
 * (wPFAW3D.f90:95-103, called from program main at :2249-2280).  This header
 * is the drop-in boundary for that path: the host keeps the driver (config,
 * time loop, output) and the device owns every field between wpf_upload()
 * and wpf_download().  One entry point exists per reference routine, plus a
 * fused wpf_step() that performs the whole loop body with fused kernels.
 *
 * Conventions
 *   - Every function returns an int status, WPF_OK (0) on success.
 *   - Host arrays are borrowed for the duration of a call only.
 *   - Field arrays use the reference layout exactly: one-cell halo, Fortran
 *     order (x fastest), G = (nx+2)*(ny+2)*(nz+2) float64 values, so
 *     element (i,j,k) with 0 <= i <= nx+1 ... is at i + (nx+2)*(j + (ny+2)*k).
 *     permeab is (0:3, G) with the component fastest, velocity is (1:3, G).
 *   - One handle per host thread; all device work of a handle is ordered on
 *     the handle's CUDA stream, and calls return after that work finishes.
 *   - There is no CPU fallback: without a usable CUDA device wpf_create()
 *     fails with WPF_ERR_CUDA.
 */
#ifndef WPF_H
#define WPF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define WPF_OK                 0
#define WPF_ERR_ARG            1   /* invalid argument or state                    */
#define WPF_ERR_CUDA           2   /* CUDA runtime error / no device               */
#define WPF_ERR_NOT_CONVERGED  3   /* solve hit maxit; the best iterate is kept     */
#define WPF_ERR_NONFINITE      4   /* NaN/Inf in a residual or a reduction         */
#define WPF_ERR_TIMEOUT        5   /* a bounded device wait expired                */
#define WPF_ERR_NOMEM          6   /* device allocation failed                     */
#define WPF_ERR_SINGULAR       7   /* no Dirichlet cell: the Darcy system is singular */
#define WPF_ERR_TOO_LARGE      8   /* grid beyond the fixed scratch of wpf_reduce_noalloc */

/* ---- solver modes ------------------------------------------------------ */
#define WPF_SOLVER_FP64   0   /* plain FP64 MG-PCG (the drop-in form)                     */
#define WPF_SOLVER_MIXED  1   /* FP32 MG-PCG inside FP64 iterative refinement             */

typedef struct wpf_handle wpf_handle;

/* Scalars of Param_type that the step uses (wPFAW3D.f90:27-76). */
typedef struct wpf_params {
    int32_t nx, ny, nz;        /* interior grid (single domain)                       */
    int32_t ix_ref, iy_ref, iz_ref;  /* reference cell of showProgress / getPressure  */
    double dx;                 /* dxw * epsilon                                        */
    double epsilon;            /* interface width w (also the anisotropy strength)     */
    double lambda;             /* phase-concentration coupling                         */
    double porosity;
    double viscosity;
    double diffusion;          /* D                                                    */
    double ral, rat;           /* dispersivities                                       */
    double permeab_hole;       /* kwh                                                  */
    double alpha;              /* 0.5 / b / kc                                         */
    double tfac;               /* time-step factor of the dt law                       */
} wpf_params;

/* Well_type (wPFAW3D.f90:82-90): ix/iy/iz are global 1-based indices. */
typedef struct wpf_well {
    int32_t ix, iy, iz, pad;
    double pressure;           /* Dirichlet iff != 0 (wPFAW3D.f90:1106)                */
    double injection;          /* inlet iff != 0 (wPFAW3D.f90:1140)                    */
    double phase, concent;     /* fixed values (applied by the host at load time)      */
} wpf_well;

/* Darcy solver options. */
typedef struct wpf_solver_opts {
    int32_t mode;              /* WPF_SOLVER_FP64 or WPF_SOLVER_MIXED                   */
    int32_t max_outer;         /* FP64 refinement passes (default 20)                  */
    int32_t max_inner;         /* PCG iterations per pass (default 500)                */
    int32_t smooth_sweeps;     /* red-black Gauss-Seidel sweeps per V-cycle side (2)   */
    double rtol;               /* ||b - A p|| <= rtol * ||b|| (true FP64 residual)      */
    double inner_rtol;         /* inner PCG reduction per pass in MIXED mode (1e-4)    */
    int64_t sweep_min_cells;   /* levels with at least this many cells use the pipelined
                                  one-pass sweep kernel (0 = default 2^23)              */
    int32_t w_from_level;      /* levels >= this (and below the pipelined ones) recurse
                                  twice: a W-cycle (0 = default 2; large = V-cycle)     */
    int32_t flags;             /* WPF_SOLVER_NO_GRAPHS: launch each preconditioner
                                  cycle kernel by kernel instead of replaying it as a
                                  captured CUDA graph (same arithmetic)                 */
    int32_t sweep_zchunk;      /* z planes per block of the pipelined sweep (0: the
                                  chunk that fills whole waves of resident blocks)      */
    int32_t row_blocks_per_sm; /* grid of the row-patch kernels (4 x 2 rows of x per
                                  block, grid-stride) in blocks per SM (0: 8)           */
} wpf_solver_opts;

#define WPF_SOLVER_NO_GRAPHS 1
/* WPF_SOLVER_EXTRAPOLATE: start each solve from p + e, e extrapolated in time
 * from the pressure increments of the last two solves (quadratic in t with the
 * step sizes wpf_step knows; equal steps assumed by wpf_solve_pressure), and
 * fall back to the previous pressure (the reference's x0, wPFAW3D.f90:980)
 * whenever p + e has the larger FP64 residual.  The solve still ends at the
 * same rtol on the true FP64 residual, so only the iteration count changes.
 * The increment history survives wpf_upload and is cleared by wpf_set_wells
 * and wpf_set_solver.  No counterpart in the reference.                    */
#define WPF_SOLVER_EXTRAPOLATE 2
/* WPF_SOLVER_NO_TMA: stage the finest-level sweep with per-thread cp.async
 * copies instead of bulk-tensor (TMA) copies (same arithmetic, same results). */
#define WPF_SOLVER_NO_TMA 4
/* WPF_SOLVER_STEP_GRAPH: run wpf_step (from itime >= 3, once the extrapolated
 * start holds two increments when WPF_SOLVER_EXTRAPOLATE is set) as one CUDA
 * graph launch: the dt law, calcPermeability, the whole solve with its
 * convergence tests on the device (conditional graph nodes: a WHILE node over
 * the refinement passes holding a WHILE node over the PCG iterations) and the
 * fused update, with one read-back per step.  The kernels, their order and so
 * the results are those of the host-driven step.  With a warm-start net
 * attached (wpf_net.h) its features, forward pass and prolongation are part
 * of the graph and the step taken along its correction is decided on the
 * device.  wpf_ensemble_run then advances all such members in one launch of
 * one graph.  Ignored while kernel timing is on.                           */
#define WPF_SOLVER_STEP_GRAPH 8
/* WPF_SOLVER_NET_ALWAYS: with a warm-start net attached (wpf_net.h), evaluate
 * its correction at every solve with two increments held, not only when the
 * extrapolated start misses rtol by at most 1.02x (the default gate, where the
 * correction can save a refinement pass).  For measuring the net and for
 * tests; the solves end at the same rtol either way.                       */
#define WPF_SOLVER_NET_ALWAYS 16
/* WPF_SOLVER_FP64_UPDATE: in the FP32-refined form (WPF_SOLVER_MIXED), keep
 * the fused update's rates in FP64.  By default that form takes the rates of
 * its concentration-only cells and of its interface cells on the guard-free
 * phase path in FP32 from FP64 differences of the state (the rate added to
 * the FP64 field as x + dt * rate), which removes most of the update's FP64
 * work; the plain FP64 form and the per-routine entry points are always
 * FP64.                                                                    */
#define WPF_SOLVER_FP64_UPDATE 32
/* WPF_SOLVER_NET_COARSE: in a solve whose learned correction was evaluated,
 * also use the net's output w (computed on the half-resolution grid and
 * prolongated) as a one-vector coarse space of the PCG: deflated PCG, whose
 * start takes the coarse-grid correction w (w.r)/(w.A w) and whose search
 * directions are kept A-orthogonal to w.  The solve ends at the same rtol;
 * the error after k iterations is never above that of PCG without w.      */
#define WPF_SOLVER_NET_COARSE 64
/* WPF_SOLVER_FIXED_START: with WPF_SOLVER_EXTRAPOLATE, start from the
 * quadratic-in-time extrapolation e = a d1 + b d2 of the last two increments
 * with a, b fixed by the step sizes.  By default the FP32-refined form, when
 * it holds the FP64 residual of the previous pressure under the new
 * transmissibilities (its kept residual) and the last step's was below 100
 * rtol, takes the a, b that minimise the residual ||r(p) - A (a d1 + b d2)||
 * instead (never larger than the fixed choice's, which lies in the same
 * span).                                                                   */
#define WPF_SOLVER_FIXED_START 128

/* Per-step / per-solve statistics. */
typedef struct wpf_step_stats {
    int32_t outer_iterations;  /* FP64 residual evaluations after the first            */
    int32_t inner_iterations;  /* total PCG iterations                                 */
    int32_t converged;         /* 1 if rtol was met                                    */
    int32_t overshoot_cells;   /* cells with |phase| > 1 seen by calcPhaseDeriv (:1425) */
    double relres;             /* final ||b - A p|| / ||b||                             */
    double taumin;             /* min relaxation time of this step (:1255)              */
    double dtime;              /* dt used by this step                                  */
    double max_courant;        /* max |u| * dt / dx over faces (advection CFL)          */
    double solve_ms;           /* device time of the Darcy solve                       */
    double update_ms;          /* device time of the fused update kernel               */
    int32_t kernel_launches;   /* kernels this call launched                           */
    int32_t warm_start;        /* 1: the solve started from the extrapolated p + e;
                                  -1: it was tried and rejected; 0: not tried         */
    double relres0;            /* relative residual of the warm start                  */
    int32_t active_cells;      /* cells the fused update evaluated in FP64 (interface and
                                  concentration work lists; the rest were copies)       */
    int32_t device_resident;   /* 1: the step ran as one graph launch (STEP_GRAPH)      */
    int32_t interface_cells;   /* of active_cells, those on the interface list (the
                                  phase-field path; the rest are concentration-only)    */
} wpf_step_stats;

/* showProgress reductions (wPFAW3D.f90:1695, 1756-1810) + inlet flux. */
typedef struct wpf_diag {
    double pv;                 /* dx^3 * poro * 0.5 * sum(1 - phase), interior          */
    double vcal;               /* dx^3 * (1-poro) * 0.5 * sum(1 + phase), interior      */
    double rwhmax;             /* max distance of a phase > 0 cell from the ref cell    */
    double phase_max, phase_min, concent_max, concent_min;   /* over G incl. halo      */
    double pressure_ref;       /* getPressure(ix_ref, iy_ref, iz_ref) (:2151-2166)      */
    double inlet_flux;         /* sum of u_x across the faces ix = 1 | 2, times dx^2    */
    double phase_max_outlet;   /* max phase over the plane ix = nx - ceil(2 w / dx), the
                                  closest the dissolved region gets to outlet wells that
                                  pin phase = -1 on ix = nx: breakthrough when > 0 (no
                                  counterpart in the reference, whose showProgress cannot
                                  report it under Dirichlet BCs); NaN from
                                  wpf_reduce_noalloc                                    */
} wpf_diag;

/* ---- lifetime ------------------------------------------------------------
 * wpf_create replaces allocate(...) of loadConfig (wPFAW3D.f90:441-449) with
 * device allocations; wpf_destroy replaces freeField (:2145-2149).           */
int wpf_create(const wpf_params* p, wpf_handle** out);
int wpf_destroy(wpf_handle* h);
const char* wpf_strerror(int status);
int wpf_device_bytes(const wpf_handle* h, int64_t* bytes);

/* Well table: builds lw (later wells win, wPFAW3D.f90:451-461) and the
 * Dirichlet / inlet masks used by solvePressure (:1099-1159).               */
int wpf_set_wells(wpf_handle* h, const wpf_well* wells, int32_t nwell);

/* Upload / download G-sized halo arrays (any pointer may be NULL to skip).
 * Upload replaces the module arrays permeab_rock, phase, concent, pressure
 * (loadConfig :464-496 / loadField :547-554); the halos are refreshed on the
 * device (updateHalo, :1645-1657) and Dirichlet cells get their well pressure.
 * Download copies them back (permeab is 4*G, velocity 3*G, as the reference). */
int wpf_upload(wpf_handle* h, const double* permeab_rock, const double* phase,
               const double* concent, const double* pressure);
int wpf_download(wpf_handle* h, double* phase, double* concent, double* pressure,
                 double* permeab, double* velocity, double* dphasedt, double* dconcentdt);

int wpf_set_solver(wpf_handle* h, const wpf_solver_opts* o);
int wpf_get_solver(const wpf_handle* h, wpf_solver_opts* o);

/* ---- the reference routines, one entry point each ------------------------ */
int wpf_calc_permeability(wpf_handle* h);                          /* :561-599   */
int wpf_solve_pressure(wpf_handle* h, wpf_step_stats* st);         /* :603-1160  */
int wpf_calc_velocity(wpf_handle* h);                              /* :1164-1193 */
int wpf_calc_phase_deriv(wpf_handle* h, double* taumin,
                         int32_t* overshoot_cells);                /* :1197-1440 */
int wpf_calc_concent_deriv(wpf_handle* h);                         /* :1554-1624 */
int wpf_evolve_phase(wpf_handle* h, double dtime);                 /* :1628-1632 */
int wpf_evolve_concent(wpf_handle* h, double dtime);               /* :1636-1640 */

/* One pass of the main-loop body (wPFAW3D.f90:2226-2280) with fused kernels:
 * dt law (:2227-2230; *dtime_inout is the previous dt on entry, this step's on
 * return), calcPermeability, solvePressure, then one fused kernel for
 * calcVelocity + calcPhaseDeriv + calcConcentDeriv + evolve + updateHalo.
 * itime is the 1-based step number.  st may be NULL.                        */
int wpf_step(wpf_handle* h, int32_t itime, double* dtime_inout, wpf_step_stats* st);

/* nsteps consecutive steps starting at itime0 (no host sync between steps
 * unless the solver needs one); *dtime_inout as in wpf_step.               */
int wpf_run(wpf_handle* h, int32_t itime0, int32_t nsteps, double* dtime_inout,
            wpf_step_stats* last);

/* Diagnostics of showProgress / getPressure on the device.                  */
int wpf_reduce(wpf_handle* h, wpf_diag* d);

/* Allocation-free diagnostics.  No counterpart in the reference: an addition
 * for callers that cannot call cudaMalloc -- code whose device memory belongs
 * to another runtime's pool allocator (which must account for every byte the
 * process takes), and latency-critical code that cannot afford cudaMalloc's
 * implicit device synchronisation.  It computes pv, vcal, rwhmax and the
 * phase / concentration max and min of wpf_diag (pressure_ref and inlet_flux
 * are returned as 0, phase_max_outlet as NaN) from device arrays the caller
 * already holds: d_phase and d_concent are G-sized float64 arrays in the
 * reference layout (Fortran order with the one-cell halo).  Its scratch is one
 * fixed file-scope device array of WPF_NOALLOC_MAX_PLANES records (about
 * 360 KB), reserved on every GPU that loads the library until the process
 * exits; grids with nz + 2 > WPF_NOALLOC_MAX_PLANES are rejected with
 * WPF_ERR_TOO_LARGE.  The first call on a device (and the first after a
 * device reset) looks up the scratch's device address.  Work is ordered on
 * `stream` (a cudaStream_t; NULL = the default stream) and the call returns
 * after it finishes.  Every call shares the one scratch array, so calls that
 * overlap on the GPU race.                                                  */
#define WPF_NOALLOC_MAX_PLANES 4096
int wpf_reduce_noalloc(const wpf_params* p, const double* d_phase, const double* d_concent,
                       wpf_diag* out, void* stream);

/* Last taumin on the device (the lagged input of the dt law).               */
int wpf_get_taumin(const wpf_handle* h, double* taumin);
/* Set that lagged taumin, for a run that resumes at itime >= 3 from a saved
 * state: the first resumed wpf_step then takes the step size the continuous
 * run would have taken (wPFAW3D.f90:2227-2230).  The reference restarts from
 * loadField (:509-557) at itime 0 and takes the configured dt for two steps;
 * this is an addition.  taumin must be positive and finite.               */
int wpf_set_taumin(wpf_handle* h, double taumin);

/* The handle's CUDA stream (cudaStream_t), for callers that order their own
 * work or timing events with the library's; and the number of kernels the
 * handle has launched so far.                                                */
int wpf_get_stream(const wpf_handle* h, void** stream);
int wpf_launch_count(const wpf_handle* h, int64_t* n);

/* Per-kernel-class device timers (CUDA events around each launch of the
 * classes in `mask`; bit c = class c): 0 permeability, 1 FP64 residual,
 * 2 solver coefficients, 3 finest-level smoother, 4 other multigrid kernels,
 * 5 PCG operator apply, 6 PCG vector kernels, 7 fused update, 8 other,
 * 9 single-block bottom cycle of the multigrid hierarchy.
 * Setting the mask resets the totals; wpf_kernel_times returns the summed
 * milliseconds and launch counts of the first n classes.                  */
int wpf_set_kernel_timing(wpf_handle* h, uint32_t mask);
int wpf_kernel_times(wpf_handle* h, double* ms, int64_t* counts, int32_t n);

/* Page-locked host buffers for callers that stream fields every step (the
 * copies in wpf_upload / wpf_download then run at full link bandwidth).     */
int wpf_host_alloc(int64_t bytes, void** ptr);
int wpf_host_free(void* ptr);

/* Asynchronous single-precision snapshot of the four fields saveResult writes
 * (wPFAW3D.f90:1934-2037: pressure, phase, concentration and the cell
 * permeability permeab(0) of the phase the last step started from), for a
 * GiD result writer.  `out` (page-locked, 4 * nx*ny*nz floats) receives them
 * one after the other, interior cells in Fortran order, converted like the
 * reference's real(x, kind=4).  The call packs the fields on the device and
 * queues the copy on a side stream, then returns: the simulation can go on
 * stepping while the copy runs.  wpf_snapshot_wait blocks until the last
 * snapshot has landed in `out`.                                            */
int wpf_snapshot(wpf_handle* h, float* out);
int wpf_snapshot_wait(wpf_handle* h);

/* Ensemble of independent domains (no counterpart in the reference, which
 * runs one domain): nsteps wpf_step calls on each of the n members (steps
 * itime0 .. itime0+nsteps-1), dtime[m] in/out per member as for wpf_step,
 * stats[m] (may be NULL) the last step's.  A pool of nthreads host threads
 * owns the members round-robin; each member runs on its own stream, so the
 * kernels of some members fill the GPU while others wait on a read-back.
 * status[m] (may be NULL) gets each member's status; a member that failed
 * stops.  Returns WPF_OK, or the first failure other than
 * WPF_ERR_NOT_CONVERGED, else that.  A step in which every member can take
 * the device-resident step (WPF_SOLVER_STEP_GRAPH) is instead one launch of
 * one graph holding all members' steps as independent branches, followed by
 * one synchronisation; the graphs are cached per buffer assignment.        */
int wpf_ensemble_run(wpf_handle** members, int32_t n, int32_t itime0, int32_t nsteps, int32_t nthreads,
                     double* dtime, wpf_step_stats* stats, int32_t* status);

/* Self-check of the FP64 <-> FP32 conversions the kernels perform on the
 * integer pipe (GB300 issues the hardware conversions on its narrow FP64
 * pipe): converts each of the n host values both ways on the current device
 * and counts, in *mismatches, the results that differ from the hardware
 * conversions (arguments below 2^-126 in magnitude flush to zero by design). */
int wpf_check_conversions(const double* host_values, int64_t n, int64_t* mismatches);

/* Self-check of the reciprocal the harmonic means of calcPermeability use (a
 * Newton-Raphson refinement of the hardware's approximate FP64 reciprocal,
 * the IEEE division outside [2^-1000, 2^1000]): for each of the n host values
 * compares it with the IEEE 1/x on the current device; *max_ulp is the largest
 * distance in units in the last place, *mismatches the results that differ in
 * class (finite / infinite / NaN) or sign. */
int wpf_check_reciprocal(const double* host_values, int64_t n, int64_t* max_ulp, int64_t* mismatches);

/* FP64 fused multiply-add throughput of the current device, in TFLOP/s
 * (2 per FMA) in *tflops: eight independent FMA chains per thread, 2048
 * threads on every SM, timed with CUDA events after one untimed run.  The
 * ceiling of the kernels bound by the FP64 pipe (the outer FP64 residual,
 * calcPermeability's harmonic means, the FP64 form's update).              */
int wpf_measure_fp64_rate(double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* WPF_H */
