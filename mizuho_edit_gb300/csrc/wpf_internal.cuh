// wpf_internal.cuh -- device layout, handle and shared helpers of libwpf_gb300.
//
// Device layout ("pitched halo grid").  Every cell field, FP64 state and FP32
// solver vectors alike, keeps the reference's one-cell halo (cells 0..n+1 per
// axis) but with the x rows padded to a pitch P that is a multiple of 16
// elements and shifted by XOFF = 15, so the first interior cell of every row
// (i = 1) starts on a 128-byte boundary for FP64 (64-byte for FP32):
//     at(i,j,k) = XOFF + k*S + j*P + i,   S = P*(ny+2)
// A warp of 32 threads over i = 1..32 then touches exactly two 128-byte lines
// of an FP64 field.  The padding columns are allocated but never read.
#pragma once

#include <cuda.h>   // CUtensorMap
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "../../include/wpf.h"

namespace wpf {

constexpr int XOFF = 15;

struct Grid {
    int nx, ny, nz;
    long long P, S, total;   // pitch (elements), plane stride, allocation (elements)
    __host__ __device__ __forceinline__ long long at(int i, int j, int k) const {
        return XOFF + (long long)k * S + (long long)j * P + i;
    }
};

inline Grid make_grid(int nx, int ny, int nz) {
    Grid g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.P = ((long long)nx + 2 + XOFF + 15) / 16 * 16;
    g.S = g.P * (ny + 2);
    g.total = g.S * (nz + 2) + 32;
    return g;
}

// Cell flags (one byte per cell).
enum : uint8_t {
    F_WELL = 1,    // lw > 0: phase / concentration fixed (wPFAW3D.f90:1257, 1562)
    F_DIR = 2,     // Dirichlet pressure (well%pressure /= 0, :1106)
    F_INLET = 4,   // injection (well%injection /= 0, :1140)
};

// Device scalar slots (doubles) used by reductions and the solver.
enum Slot {
    S_TAUMIN_KEY = 0,   // ordered-bits key of the running min of tau (uint64 in a double slot)
    S_OVERSHOOT,        // overshoot count (uint64)
    S_UMAX_BITS,        // max |u| (bits of a non-negative double)
    S_RR64,             // ||r||^2 of the FP64 residual
    S_BB64,             // ||b||^2 of the reference right-hand side
    S_RR0WS,            // ||r(p)||^2 when the solve tries an extrapolated start
    S_RW, S_WW,         // r_ext . A'e_net and ||A'e_net||^2 (step length of the learned start)
    S_PQ,               // PCG p.q
    S_RR,               // PCG r.r
    S_RZ0, S_RZ1,       // PCG r.z (double buffered)
    S_SUM0, S_SUM1, S_SUM2, S_SUM3,   // diagnostics
    S_MAX0, S_MAX1, S_MAX2, S_MAX3, S_MAX4,
    S_NWORK,            // work-list counts of the fused update: interface cells and
                        // concentration-only cells (two ints in a double slot)
    S_WSS2,             // sum of the squared last increment (input scale of the learned start)
    S_WSD2,             // sum of the squared change of the increment (its output scale)
    S_DPH2,             // sum of the squared phase change of the last step (its scale)
    S_KLOG0, S_KLOG1,   // sum of log K_rock and of its square (input normalisation)
    S_KERR,             // set (int) by a kernel whose bounded wait ran out
    S_UPL0, S_UPL1,     // wpf_upload: one int per field whose values changed (4 ints)
    S_WAW,              // e_net . A'e_net (the learned coarse space's 1x1 operator)
    S_WR, S_WQ,         // e_net . r and e_net . q of the PCG with the learned coarse space
    S_GAM,              // its coefficient e_net . r / e_net . A'e_net in this iteration
    S_LS0,              // the least-squares start: r.A'd1, r.A'd2, |A'd1|^2, A'd1.A'd2, |A'd2|^2,
    S_LS5 = S_LS0 + 5,  // |r|^2 (r = r(p), scaled)
    S_LSSCALE,          // the power of two its dots scale r and A'd by
    S_COUNT = 48
};

// Physics parameters in the form the kernels use.
struct Phys {
    double dx, inv_dx, inv_2dx, inv_dx2, inv_4dx2;
    double epsilon, lambda, alpha, diffusion, ral, rat, kwh, viscosity;
    double tau_num;        // 5/3*alpha*lambda*eps^2 (numerator of tau, :1254)
    double tau0;           // tau at kxx = D
    double inv_tau_num, inv_tau0;
    double w0, maxdphi;
    double qscale;         // dx*dx/dx**3 of the injection term (:817)
};

template <typename R>
struct Level {
    Grid g;
    R *cx, *cy, *cz, *diag, *idiag;   // couplings to +x/+y/+z, diagonal, 1/diagonal (0 if dead)
    R *x, *b;                        // unknown (the V-cycle's output) and right-hand side
    R* xs;                           // second buffer: smoothing sweeps read one, write the other
};

constexpr int MAX_LEVELS = 16;

// Bulk-tensor maps of one level for the TMA-staged sweep kernel: the x input
// and the five operator arrays (cx, cy, cz, 1/diag, b).
struct SweepMaps {
    CUtensorMap x, cx, cy, cz, id, b;
};

// cuTensorMapEncodeTiled, fetched once through the runtime's driver entry
// points (the library links the runtime only); nullptr when unavailable.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);
EncodeTiledFn tensor_map_encoder();

// Control block of the device-resident step (WPF_SOLVER_STEP_GRAPH): the
// decisions the host-driven step takes after each read-back, taken instead by
// one-thread kernels inside the step graph.  Copied back once per step.
struct StepCtl {
    double dt;               // this step's dt (the dt law on the device)
    double h1, h2;           // step sizes of the last two increments
    float wa, wb;            // extrapolation coefficients e = wa d1 + wb d2
    float alpha;             // step of the learned correction (0: none taken)
    float alpha_pad;
    double bnorm, relres, relres0;
    double r0, tol;          // PCG: ||r_0|| and the relative tolerance of this pass
    int pass;                // refinement pass whose residual was taken last
    int outer, inner;        // refinement passes with a PCG, PCG iterations in all
    int it;                  // iterations of the current PCG
    int need_pcg;            // this pass runs a PCG (else it adds the accepted start only)
    int accept;              // extrapolated start accepted, not yet added to p
    int used;                // 1 start used, -1 rejected, 0 not tried
    int status;              // WPF_OK / WPF_ERR_NOT_CONVERGED / WPF_ERR_NONFINITE
    int pcgs;                // PCG runs
    int net_runs;            // the learned correction was evaluated this step (0 / 1)
    int ls;                  // the least-squares start is taken this step (0 / 1)
    int ls_skip;             // its predicted residual meets rtol: pass 0's residual kernel is skipped
    double rp_rel;           // ||r(p)|| / ||b|| of the last pass 0 (kept across steps)
    double bnorm_prev;       // ||b|| of the last step (the least-squares dots' scale)
};

// Builds a CUDA graph from stream-captured segments and conditional nodes.
// `graph` is the graph being extended (the top graph or a conditional body),
// `deps` the nodes the next segment depends on.
struct GraphBuilder {
    cudaGraph_t graph = nullptr;
    cudaGraph_t top = nullptr;    // owner of the conditional handles
    cudaStream_t s = nullptr;
    cudaGraphNode_t deps[8];
    int ndeps = 0;
    bool capturing = false;
};
int gb_begin(GraphBuilder& b);   // capture s into graph after deps
int gb_end(GraphBuilder& b);     // end the capture; deps = its leaves
// A conditional handle on the top graph (reset to 0 at each launch); the
// kernels that set it take it as an argument, so it exists before their capture.
int gb_handle(GraphBuilder& b, cudaGraphConditionalHandle* hd);
// Append a conditional node (WHILE or IF) on handle hd after deps; `body` is
// set up to build its body graph.
int gb_cond(GraphBuilder& b, cudaGraphConditionalNodeType type, cudaGraphConditionalHandle hd,
            GraphBuilder* body);

constexpr int STEP_KEY = 10;  // buffer pointers and modes a captured step depends on
constexpr int BRICK_X = 32, BRICK_Y = 4, BRICK_Z = 2;   // fused-update bricks (one RB-thread block)

// Kernels launched per step by a captured device-resident step:
//   fixed + passes * per_pass + iterations * per_iter.
struct StepCounts {
    long long fixed = 0, per_pass = 0, per_iter = 0, per_net = 0;
};

// The learned correction is tried only when the extrapolated start misses the
// tolerance by at most this factor: there a small reduction of the start's
// residual can save a refinement pass; further out the PCG runs anyway.  The
// trained net lowers the start's residual by 0.7 % on unseen seeds (9.14e-8 ->
// 9.07e-8, mean over ten 128^3 steps), so a start more than 2 % above the
// tolerance is out of its reach.
constexpr double NET_WINDOW = 1.02;
__host__ __device__ inline bool net_gate(double rr_ext, double bb, double rtol) {
    const double rel = bb > 0.0 ? sqrt(rr_ext / bb) : sqrt(rr_ext);
    return rel > rtol && rel <= NET_WINDOW * rtol;
}

template <typename R>
struct Hierarchy {
    int nlev = 0;
    Level<R> lv[MAX_LEVELS];
    // per level: maps with the x input in xs ([0]) or in x ([1]); tm_ok when encoded
    SweepMaps tm[MAX_LEVELS][2];
    bool tm_ok[MAX_LEVELS] = {};
    // PCG vectors on the fine grid (level 0 aliases: lv[0].b = r, lv[0].x = z);
    // p is double buffered (p, p2) because the operator kernel forms the new
    // search direction of a cell's neighbours on the fly from z and the old p.
    R *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *p2 = nullptr, *q = nullptr;
    // The preconditioner cycle captured as a CUDA graph, one per r.z slot, with
    // the kernels it holds and the event pairs of the kernel-class timers
    // recorded inside it (captured with timing mask cyc_mask).
    static constexpr int MAX_CYC_TIMERS = 256;
    cudaGraphExec_t cyc[2] = {nullptr, nullptr};
    long long cyc_kernels[2] = {0, 0};
    int cyc_ntimers[2] = {0, 0};
    int cyc_cls[2][MAX_CYC_TIMERS] = {};
    cudaEvent_t cyc_ev[2][2 * MAX_CYC_TIMERS] = {};
    unsigned cyc_mask = 0;
};

}  // namespace wpf

struct wpf_handle {
    wpf_params prm;
    wpf::Phys phys;
    wpf::Grid g;
    int device;
    int nsm;                 // streaming multiprocessors of the device
    cudaStream_t stream;
    cudaEvent_t ev[4];
    // FP64 state (pitched halo grid)
    double *krock, *phase, *concent, *pressure, *phase_n, *concent_n;
    double *T[3];            // K_f / mu at interior faces, 0 on the global boundary faces
    double *Tv[3];           // T / dx: the fused update's face velocity is -(Tv (p_nb - p))
    // materialised only by the per-routine entry points / downloads
    double *K0, *Kf[3], *vel[3], *dphasedt, *dconcentdt;
    uint8_t* flags;
    // wells
    int32_t ndir, ninlet;
    long long* dir_idx;      // Dirichlet cells (pitched index) and their pressure
    double* dir_val;
    double* qterm;           // G-sized injection term (nullptr if no inlet)
    bool have_wells;
    // solver
    wpf_solver_opts opts;
    wpf::Hierarchy<double> h64;
    wpf::Hierarchy<float> h32;
    double* dsum;            // FP64 sum of a live cell's six face T (mixed mode: the
                             // diagonal of the outer residual's diagonal-sum form)
    // FP64 outer residual of the current pressure under the current T (mixed
    // mode with the extrapolated start): written by every plain residual pass,
    // corrected face by face when calcPermeability changes T incrementally,
    // read as r(p) by the next solve's pass 0.  rkeep_ok: it matches p and T.
    double* rkeep;
    bool rkeep_ok;
    // level-0 operator kept up to date cell by cell: calcPermeability's
    // incremental form marks both cells of every face it recomputes
    // (l0mark), and the next level-0 build rebuilds only the marked cells and
    // clears them.  l0_inc_ok: the level-0 arrays of the l0_mode hierarchy
    // match T except at the marked cells.
    uint8_t* l0mark;
    bool l0_inc_ok;
    int l0_mode;
    // extrapolated warm start (WPF_SOLVER_EXTRAPOLATE): the pressure increments
    // of the last two solves (ws[0] newest) and this solve's (ws[2]), FP32
    float* ws[3];
    int ws_hist;             // increments held (0..2)
    int ws_used;             // this solve started from p + e
    double ws_hn, ws_h1, ws_h2;   // step sizes: this step, previous, one before (0 = unknown)
    long long ws_fallbacks;  // solves whose extrapolated start was rejected
    double* staging;         // dense halo-array staging for host copies (lazily allocated)
    bool host_pageable_direct;   // kernels reach pageable host memory in place (host page tables)
    struct wpf_net* ws_net;  // learned warm start (not owned), or null
    const struct wpf_net* ws_net_warm;   // the net whose kernels ran once outside a capture
    float* ws_e[3];          // materialised starts: e_ext = a d1 + b d2, e_net (prolonged net output),
                             // and A'e_net (the deflated PCG's coarse space)
    uint16_t* ws_in;         // net input (bf16, net grid, 16 channels)
    float* ws_out;           // net output channel 0 (net grid)
    float* ws_klog;          // net input channel 0, normalised log K_rock (net grid; K_rock is
                             // fixed between uploads, so it is made once)
    bool ws_klog_ready;      // S_KLOG0/1 hold the statistics of log K_rock
    // asynchronous output snapshots: FP32 device staging, side stream, events
    float* snap;
    cudaStream_t side;
    cudaEvent_t snap_ready, snap_done;
    bool snap_pending;
    double* dsc;             // device scalar slots
    double* hsc;             // pinned host mirror of the scalar slots
    double* partials;        // per-block partial sums of the diagnostics
    int npartials;
    double taumin_last;      // taumin of the last phase-derivative pass
    int64_t bytes;           // device bytes allocated
    bool vel_valid;
    bool kf_valid;           // Kf/K0 hold calcPermeability of the current phase
    bool t_current;          // T was computed from the current phase / permeab_rock
    bool t_from_prev;        // T was computed from the phase now held in phase_n
    int* work;               // active-cell work list of the fused update
    // per brick of the fused update (32 x 4 x 2 cells): any cell in a work
    // list in the last update ([0]) / in this one ([1]); bact_ok: [0] is valid
    // (the fields changed only through fused updates since it was written)
    uint8_t* bact[2];
    bool bact_ok;
    int last_active;         // its length in the last step
    int last_interface;      // of which interface cells
    double ls_rp_rel;        // host-driven solve: ||r(p)|| / ||b|| of the last pass 0
    double ls_bnorm;         // and ||b|| of the last solve (the least-squares start's inputs)
    wpf::Phys* dphys;        // device copy of phys
    long long nlaunch;       // kernels launched on this handle so far
    // per-kernel-class event timers (enabled by wpf_set_kernel_timing)
    unsigned timing_mask;
    int npend;
    int pend_cls[256];
    cudaEvent_t pend_ev[512];
    double kt_ms[16];
    long long kt_count[16];
    // timers while a graph is being captured (event record nodes: cap_ev is
    // non-null only during a capture) and the pairs of launched graphs still
    // to be read
    int* cap_ntimers;
    int* cap_cls;
    cudaEvent_t* cap_ev;
    int cap_max;
    int ngpend;
    int gpend_cls[512];
    cudaEvent_t gpend_a[512], gpend_b[512];
    // device-resident step: control block (device, pinned mirror), pinned
    // copy of the scalar slots, and the instantiated step graphs, one per
    // assignment of the ping-pong buffers (phase, concentration, increments)
    wpf::StepCtl* gctl;
    wpf::StepCtl* gctl_host;
    double* gdsc_host;
    bool gctl_dirty;         // the host-driven path ran since the last graph step
    cudaStream_t cap_side;   // second branch of a captured step
    cudaEvent_t cap_fork, cap_join;
    // the fused update's classification, captured on its own stream into a
    // child graph that runs beside the solve: the nodes it waits for
    // (calcPermeability) until it is added to the step graph
    cudaStream_t cap_split;
    cudaGraph_t split_graph;
    // the extrapolated start's build, captured beside calcPermeability on
    // cap_ws and joined before the pass-0 residual (ws_early: it was)
    cudaStream_t cap_ws;
    cudaEvent_t cap_ws_fork, cap_ws_join;
    bool ws_early;
    cudaGraphNode_t split_deps[8];
    int nsplit_deps;
    static constexpr int MAX_STEP_GRAPHS = 12;
    struct StepGraph {
        const void* key[wpf::STEP_KEY];
        cudaGraphExec_t exec;
        wpf::StepCounts n;
    } sg[MAX_STEP_GRAPHS];
    int nsg;
    unsigned long long uid;  // unique per handle over the process (ensemble graph keys)
    unsigned long long epoch;   // bumped whenever captured graphs become invalid
};

namespace wpf {
// Kernel classes for the event timers (bit i of wpf_set_kernel_timing's mask).
enum KClass {
    KC_PERM = 0,      // calcPermeability face kernel
    KC_RESID64,       // FP64 outer residual
    KC_COEF,          // level-0 coefficients + coarsening
    KC_SMOOTH0,       // red-black Gauss-Seidel on the finest level
    KC_MGREST,        // other multigrid kernels (restrict, prolong, coarse levels)
    KC_APPLY,         // PCG operator apply + dot
    KC_VEC,           // PCG vector updates / dots / correction
    KC_FUSED,         // fused velocity + phase + concentration + Euler + halo
    KC_OTHER,         // halo, Dirichlet, reductions
    KC_BOTTOM,        // single-block bottom cycle of the hierarchy
    KC_COUNT
};
// Record a start event for class c (if timed); returns the slot or -1.
int timer_start(wpf_handle* h, int c);
void timer_stop(wpf_handle* h, int slot);
void timer_flush(wpf_handle* h);   // after a synchronisation: fold finished pairs
}  // namespace wpf

// Launch a kernel on the handle's stream: counts it and, if its class is
// timed, brackets it with a pair of events.
#define WPF_LAUNCH(h, cls, ...)                               \
    do {                                                      \
        const int ts_ = ::wpf::timer_start((h), (cls));       \
        ++(h)->nlaunch;                                       \
        __VA_ARGS__;                                          \
        ::wpf::timer_stop((h), ts_);                          \
    } while (0)

namespace wpf {

// ---- error helpers --------------------------------------------------------
#define WPF_CUDA(call)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return WPF_ERR_CUDA;      \
    } while (0)

// ---- ordered keys for atomic min / max of doubles --------------------------
__device__ __forceinline__ unsigned long long dkey(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double dkey_inv(unsigned long long k) {
    unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    double v;
    memcpy(&v, &b, 8);
    return v;
}
inline unsigned long long dkey_host(double v) {
    unsigned long long b;
    memcpy(&b, &v, 8);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

// ---- FP64 <-> FP32 conversions on the integer pipe ---------------------------
// GB300 issues the hardware FP64<->FP32 conversions on its narrow FP64 pipe, at
// a fraction of even the FP64 FMA rate; the kernels that convert a field per
// cell use these instead, built from the IEEE 754 binary64 / binary32
// layouts.  f64_to_f32: round to nearest, ties to even, for every argument of
// magnitude at least 2^-126 (FP32's normal range); smaller arguments flush to
// zero, overflow gives infinity, NaN stays NaN.  f32_to_f64: exact for normal
// numbers; FP32 subnormals flush to zero.
__device__ __forceinline__ float f64_to_f32(double x) {
    // 32-bit operations on the two halves only (64-bit integer arithmetic
    // can also land on the FP64 pipe)
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned ahi = hi & 0x7fffffffu;
    unsigned f;
    if (ahi >= 0x47f00000u) {                  // |x| >= 2^128, Inf, NaN
        f = (ahi > 0x7ff00000u || (ahi == 0x7ff00000u && lo)) ? 0x7fc00000u : 0x7f800000u;
    } else if (ahi < 0x38100000u) {            // |x| < 2^-126
        f = 0u;
    } else {
        // exponent rebiased (1023 -> 127), the top 23 mantissa bits, and the
        // 29 dropped bits rounded to nearest, ties to even (a carry runs into
        // the exponent, and to Inf past the largest finite value)
        f = ((ahi - 0x38000000u) << 3) | (lo >> 29);
        const unsigned rem = lo & 0x1fffffffu;
        f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
    }
    return __uint_as_float(f | (hi & 0x80000000u));
}
// 1/x (the harmonic means of calcPermeability) by the Newton-Raphson iteration y <- y + y (1 - x y) from the
// hardware's approximate reciprocal (PTX rcp.approx.ftz.f64): two iterations
// square its relative error twice, to within an ulp or two of 1/x (not
// correctly rounded).  Arguments whose exponent is outside [2^-1000, 2^1000]
// (zero, subnormal, huge, Inf, NaN) take the IEEE division.
__device__ __forceinline__ double rcp_nr(double x) {
    const unsigned e = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
    if (e < 23u || e > 2023u) return 1.0 / x;
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double r = fma(-x, y, 1.0);
    y = fma(y, r, y);
    r = fma(-x, y, 1.0);
    return fma(y, r, y);
}
__device__ __forceinline__ double f32_to_f64(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned a = u & 0x7fffffffu;
    unsigned hi, lo;
    if (a >= 0x7f800000u) {                    // Inf, NaN (payload kept)
        hi = 0x7ff00000u | ((a & 0x7fffffu) >> 3);
        lo = a << 29;
    } else if (a < 0x00800000u) {              // zero and FP32 subnormals
        hi = 0u;
        lo = 0u;
    } else {
        hi = (a >> 3) + 0x38000000u;
        lo = a << 29;
    }
    return __hiloint2double((int)(hi | (u & 0x80000000u)), (int)lo);
}
template <typename R>
__device__ __forceinline__ R from_f64(double x);
template <>
__device__ __forceinline__ float from_f64<float>(double x) { return f64_to_f32(x); }
template <>
__device__ __forceinline__ double from_f64<double>(double x) { return x; }
template <typename R>
__device__ __forceinline__ double to_f64(R x);
template <>
__device__ __forceinline__ double to_f64<float>(float x) { return f32_to_f64(x); }
template <>
__device__ __forceinline__ double to_f64<double>(double x) { return x; }
template <typename R>
__device__ __forceinline__ R from_f32(float x);
template <>
__device__ __forceinline__ float from_f32<float>(float x) { return x; }
template <>
__device__ __forceinline__ double from_f32<double>(float x) { return f32_to_f64(x); }
template <typename R>
__device__ __forceinline__ float to_f32(R x);
template <>
__device__ __forceinline__ float to_f32<float>(float x) { return x; }
template <>
__device__ __forceinline__ float to_f32<double>(double x) { return f64_to_f32(x); }

// ---- block reductions -----------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { T w = __shfl_xor_sync(0xffffffffu, v, o); v = w < v ? w : v; }
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { T w = __shfl_xor_sync(0xffffffffu, v, o); v = w > v ? w : v; }
    return v;
}

// Sum over the block; the result is valid in thread 0.  blockDim.x*y*z <= 1024.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* sm /* >= 32 */) {
    int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    int nthr = blockDim.x * blockDim.y * blockDim.z;
    v = warp_sum(v);
    __syncthreads();
    if ((tid & 31) == 0) sm[tid >> 5] = v;
    __syncthreads();
    T s = 0;
    if (tid < 32) {
        s = tid < (nthr + 31) / 32 ? sm[tid] : T(0);
        s = warp_sum(s);
    }
    return s;
}
template <typename T>
__device__ __forceinline__ T block_min(T v, T* sm, T ident) {
    int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    int nthr = blockDim.x * blockDim.y * blockDim.z;
    v = warp_min(v);
    __syncthreads();
    if ((tid & 31) == 0) sm[tid >> 5] = v;
    __syncthreads();
    T s = ident;
    if (tid < 32) {
        s = tid < (nthr + 31) / 32 ? sm[tid] : ident;
        s = warp_min(s);
    }
    return s;
}
template <typename T>
__device__ __forceinline__ T block_max(T v, T* sm, T ident) {
    int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    int nthr = blockDim.x * blockDim.y * blockDim.z;
    v = warp_max(v);
    __syncthreads();
    if ((tid & 31) == 0) sm[tid >> 5] = v;
    __syncthreads();
    T s = ident;
    if (tid < 32) {
        s = tid < (nthr + 31) / 32 ? sm[tid] : ident;
        s = warp_max(s);
    }
    return s;
}

// ---- persistent row loops ----------------------------------------------------
// Reduction and vector kernels run a bounded grid (a few blocks per SM) of
// RB-thread blocks: warps walk the (j,k) rows of the interior, lanes walk x
// (coalesced), and each block issues one atomic per reduced quantity.
constexpr int RB = 256;

// A block's 8 warps take a 4 (y) x 2 (z) patch of rows, so the y and z
// neighbours of a warp's row are mostly rows of the same block (L1 reuse).
#define ROW_LOOP(g)                                                                        \
    const int nby_ = ((g).ny + 3) >> 2, npatch_ = nby_ * (((g).nz + 1) >> 1);             \
    const int lane_ = threadIdx.x & 31, wy_ = (threadIdx.x >> 5) & 3, wz_ = threadIdx.x >> 7; \
    for (int t_ = blockIdx.x; t_ < npatch_; t_ += gridDim.x)                               \
        for (int k = 1 + (t_ / nby_) * 2 + wz_, j = 1 + (t_ % nby_) * 4 + wy_,             \
                 i = (j <= (g).ny && k <= (g).nz) ? 1 + lane_ : (g).nx + 1;                \
             i <= (g).nx; i += 32)

// The same walk with the x loop unrolled 4 times (light streaming kernels:
// more independent loads in flight per warp).
#define ROW_LOOP_U4(g)                                                                     \
    const int nby_ = ((g).ny + 3) >> 2, npatch_ = nby_ * (((g).nz + 1) >> 1);             \
    const int lane_ = threadIdx.x & 31, wy_ = (threadIdx.x >> 5) & 3, wz_ = threadIdx.x >> 7; \
    for (int t_ = blockIdx.x; t_ < npatch_; t_ += gridDim.x)                               \
        _Pragma("unroll 4")                                                                \
        for (int k = 1 + (t_ / nby_) * 2 + wz_, j = 1 + (t_ % nby_) * 4 + wy_,             \
                 i = (j <= (g).ny && k <= (g).nz) ? 1 + lane_ : (g).nx + 1;                \
             i <= (g).nx; i += 32)

inline unsigned row_blocks(const wpf_handle* h, const Grid& g, int per_sm = 0) {
    if (per_sm <= 0) per_sm = h->opts.row_blocks_per_sm > 0 ? h->opts.row_blocks_per_sm : 8;
    const long long patches = (long long)((g.ny + 3) / 4) * ((g.nz + 1) / 2);
    const long long cap = (long long)h->nsm * per_sm;
    return (unsigned)(patches < cap ? patches : cap);
}

// Blocks of `threads` threads (and `smem` dynamic shared bytes) of kernel f
// that one SM holds at once, at most cap (cap when the query fails); cached
// per kernel.  A grid-stride kernel launched with more blocks per SM than fit
// runs the rest as a second, partial wave: with 8 per SM where 5 fit, the
// last 3 start when the first 5 end, and the pass takes two block lifetimes
// instead of 8/5 of one.
int resident_blocks(const void* f, int threads, size_t smem, int cap);

// row_blocks for the row-patch kernel f: as many blocks per SM as stay
// resident (at most 8), unless the caller set row_blocks_per_sm.
template <typename F>
inline unsigned row_blocks_for(const wpf_handle* h, const Grid& g, F f) {
    const int per_sm = h->opts.row_blocks_per_sm > 0 ? h->opts.row_blocks_per_sm
                                                     : resident_blocks((const void*)f, RB, 0, 8);
    return row_blocks(h, g, per_sm);
}

template <typename T>
__device__ __forceinline__ void block_add(T v, double* acc) {
    __shared__ T sm_add[32];
    v = block_sum(v, sm_add);
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) atomicAdd(acc, (double)v);
}

// ---- cross-file entry points (implemented in wpf_physics.cu / wpf_solver.cu)
int phys_permeability(wpf_handle* h, bool materialise);
int breakthrough_plane(const wpf_params& p);   // ix of the breakthrough plane (wpf_diag)
int phys_velocity(wpf_handle* h);
int phys_phase_deriv(wpf_handle* h, double* taumin, int32_t* overshoot);
int phys_concent_deriv(wpf_handle* h);
int phys_evolve(wpf_handle* h, bool phase, double dtime);
int phys_fused_update(wpf_handle* h, double dtime, double* taumin, int32_t* overshoot,
                      double* umax);
int phys_halo(wpf_handle* h, double* f);
int phys_set_dirichlet(wpf_handle* h);
int phys_reduce(wpf_handle* h, wpf_diag* d);
int solver_setup(wpf_handle* h);
int solver_free(wpf_handle* h);
void solver_drop_graphs(wpf_handle* h);   // after an options change
int solve_pressure(wpf_handle* h, wpf_step_stats* st);
// extrapolated / learned start (wpf_solver.cu, wpf_net.cu)
void ws_coeffs(const wpf_handle* h, float* a, float* b);
int ws_build_ext(wpf_handle* h, float a, float b,      // ws_e[0] = a d1 + b d2, S_WSS2 = sum d1^2;
                 float* dnew = nullptr);               // dnew: a copy of it there too
int ws_net_correction(wpf_handle* h);                   // ws_e[1] from the attached net

int ensure_per_routine_arrays(wpf_handle* h);
int dev_alloc(wpf_handle* h, void** p, size_t bytes);
int update_alloc(wpf_handle* h);           // work list + brick activity of the fused update
void update_advance_bricks(wpf_handle* h); // after an update: its activity becomes the last one

// device-resident step (wpf_graph.cu, wpf_solver.cu, wpf_physics.cu)
// capture the solve and the fused update (Dirichlet values .. new phase and
// concentration) into b, in capture on entry and exit
int solve_capture(wpf_handle* h, GraphBuilder& b, StepCounts* n);
// the next level-0 build may rebuild only the cells calcPermeability marked
bool l0_incremental(const wpf_handle* h);
// capture the extrapolated start's build (e = wa d1 + wb d2 with the device
// coefficients) on h->cap_ws, forked from h->stream; false if the solve has
// no extrapolated start
int ws_capture_early(wpf_handle* h, bool* launched);
// capture the classification half of the fused update (step slots reset,
// k_update_split) on stream s (launches only)
int phys_capture_split(wpf_handle* h, cudaStream_t s);
// capture the fused update on stream s with dt read from *dtp (launches
// only); split_done: its classification is already in the graph
int phys_capture_update(wpf_handle* h, const double* dtp, cudaStream_t s, bool split_done);
// add h->split_graph (if any) to b as a child graph node after
// h->split_deps, and make the next segment of b wait for it too
int gb_add_split(wpf_handle* h, GraphBuilder& b, bool* added);
// a second stream joins / leaves the capture running on h->stream
int gb_fork(wpf_handle* h);
int gb_join(wpf_handle* h);
bool step_graph_ready(const wpf_handle* h, int itime);
int step_graph_prepare(wpf_handle* h);           // allocations a capture needs
int step_graph_capture(wpf_handle* h, GraphBuilder& b, StepCounts* n);
int step_graph_finish(wpf_handle* h, const StepCounts& n, wpf_step_stats* st, double* dt_out);
int step_graph_run(wpf_handle* h, wpf_step_stats* st, double* dt_out);
// The learned start inside a captured step: features, forward pass and
// prolongation of the attached net on stream s, with no synchronisation
// (ws_net_prepare, outside any capture, allocates the buffers, takes the
// log-K statistics and runs the net's kernels once); ws_net_check reads the
// net's bounded-wait error flag after the step.
int ws_net_prepare(wpf_handle* h);
int ws_net_capture(wpf_handle* h, cudaStream_t s);
int ws_net_check(wpf_handle* h);
void step_graph_key(const wpf_handle* h, const void** k);   // STEP_KEY buffer pointers
int step_graph_sync_ctl(wpf_handle* h);          // upload host-side history if stale
void step_graphs_drop(wpf_handle* h);
void abandon_capture(cudaStream_t s);
void ensemble_graphs_forget(const wpf_handle* h);   // wpf_ensemble.cu

inline dim3 cell_block() { return dim3(32, 4, 2); }
inline dim3 cell_grid(int nx, int ny, int nz) {
    dim3 b = cell_block();
    return dim3((nx + b.x - 1) / b.x, (ny + b.y - 1) / b.y, (nz + b.z - 1) / b.z);
}

}  // namespace wpf
