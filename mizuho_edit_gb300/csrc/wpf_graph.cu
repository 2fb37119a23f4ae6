// wpf_graph.cu -- the device-resident step (WPF_SOLVER_STEP_GRAPH).
//
// wpf_step's host-driven form (wPFAW3D.f90:2227-2280: dt law,
// calcPermeability, solvePressure, the fused velocity/phase/concentration
// update) reads a scalar back after every residual and every PCG iteration to
// decide what to launch next.  Here the whole step is one CUDA graph: the dt
// law and the solver's decisions run in one-thread control kernels, the two
// solver loops are conditional WHILE nodes whose handles those kernels set,
// and the step ends with two device-to-host copies (the control block and the
// scalar slots) read after the one synchronisation of the step.  The kernels
// are those of the host-driven step, so are the results; only the fused
// update's classification and the extrapolated start's build run on side
// branches (beside the solve and beside calcPermeability).
//
// A graph bakes in the buffers it was captured with; the step's ping-pong
// buffers (phase, concentration and, with the extrapolated start, the three
// increment buffers) cycle with period 6, so a handle keeps instantiated
// graphs keyed by the assignment of those buffers (and by whether the face
// transmissibilities can be updated from the last step's phase, which a
// wpf_upload of the phase rules out: up to 12 graphs).
#include <math.h>
#include <string.h>

#include "wpf_internal.cuh"

namespace wpf {

// ---- graph building ----------------------------------------------------------
int gb_begin(GraphBuilder& b) {
    WPF_CUDA(cudaStreamBeginCaptureToGraph(b.s, b.graph, b.ndeps ? b.deps : nullptr, nullptr, (size_t)b.ndeps,
                                           cudaStreamCaptureModeThreadLocal));
    b.capturing = true;
    return WPF_OK;
}

int gb_end(GraphBuilder& b) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    const cudaError_t e1 = cudaStreamGetCaptureInfo(b.s, &cs, nullptr, nullptr, &deps, nullptr, &nd);
    const bool fits = e1 == cudaSuccess && nd <= 8;
    if (fits) {
        for (size_t q = 0; q < nd; ++q) b.deps[q] = deps[q];
        b.ndeps = (int)nd;
    }
    cudaGraph_t out = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(b.s, &out);
    b.capturing = false;
    if (!fits || e2 != cudaSuccess || cs != cudaStreamCaptureStatusActive) {
        cudaGetLastError();
        return WPF_ERR_CUDA;
    }
    return WPF_OK;
}

int gb_handle(GraphBuilder& b, cudaGraphConditionalHandle* hd) {
    WPF_CUDA(cudaGraphConditionalHandleCreate(hd, b.top, 0, cudaGraphCondAssignDefault));
    return WPF_OK;
}

int gb_cond(GraphBuilder& b, cudaGraphConditionalNodeType type, cudaGraphConditionalHandle hd,
            GraphBuilder* body) {
    // (the parameter union has no default constructor: zeroed raw storage)
    alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)];
    memset(raw, 0, sizeof(raw));
    cudaGraphNodeParams& p = *reinterpret_cast<cudaGraphNodeParams*>(raw);
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = hd;
    p.conditional.type = type;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    WPF_CUDA(cudaGraphAddNode(&node, b.graph, b.ndeps ? b.deps : nullptr, nullptr, (size_t)b.ndeps, &p));
    body->graph = p.conditional.phGraph_out[0];
    body->top = b.top;
    body->s = b.s;
    body->ndeps = 0;
    body->capturing = false;
    b.deps[0] = node;
    b.ndeps = 1;
    return WPF_OK;
}

// A second stream forks from / joins the capture on h->stream (dependency
// edges only: the events are recorded without the external flag).
int gb_fork(wpf_handle* h) {
    WPF_CUDA(cudaEventRecord(h->cap_fork, h->stream));
    WPF_CUDA(cudaStreamWaitEvent(h->cap_side, h->cap_fork, 0));
    return WPF_OK;
}

int gb_join(wpf_handle* h) {
    WPF_CUDA(cudaEventRecord(h->cap_join, h->cap_side));
    WPF_CUDA(cudaStreamWaitEvent(h->stream, h->cap_join, 0));
    return WPF_OK;
}

// The fused update's classification reads the new phase and concentration
// and writes the other ping-pong buffers, the work lists and the quiescent-
// brick flags, none of which the solve touches; it only has to follow
// calcPermeability (which reads the previous phase from those buffers).  A
// fork joined inside the capture would make the solver loops wait for it, so
// it is captured on its own into a child graph, added after the nodes that
// calcPermeability left, and the update's segment waits for it.  At its full
// grid beside the solve: 288.6 -> 295.5 steps/s at 256^3 (2.4 %); with two
// blocks per SM it gained 0.2 %.
static int capture_split_beside(wpf_handle* h) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    WPF_CUDA(cudaStreamGetCaptureInfo(h->stream, &cs, nullptr, nullptr, &deps, nullptr, &nd));
    if (cs != cudaStreamCaptureStatusActive || nd > 8) return WPF_ERR_CUDA;
    for (size_t q = 0; q < nd; ++q) h->split_deps[q] = deps[q];
    h->nsplit_deps = (int)nd;
    WPF_CUDA(cudaStreamBeginCapture(h->cap_split, cudaStreamCaptureModeThreadLocal));
    const int rc = phys_capture_split(h, h->cap_split);
    cudaGraph_t sg = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->cap_split, &sg);
    if (rc || e != cudaSuccess) {
        if (sg) cudaGraphDestroy(sg);
        cudaGetLastError();
        return rc ? rc : WPF_ERR_CUDA;
    }
    h->split_graph = sg;
    return WPF_OK;
}

static void drop_split(wpf_handle* h) {
    if (h->split_graph) cudaGraphDestroy(h->split_graph);
    h->split_graph = nullptr;
}

int gb_add_split(wpf_handle* h, GraphBuilder& b, bool* added) {
    *added = false;
    if (!h->split_graph) return WPF_OK;
    cudaGraphNode_t node = nullptr;
    const cudaError_t e = b.ndeps < 8 ? cudaGraphAddChildGraphNode(&node, b.graph, h->split_deps,
                                                                   (size_t)h->nsplit_deps, h->split_graph)
                                      : cudaErrorInvalidValue;
    drop_split(h);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return WPF_ERR_CUDA;
    }
    b.deps[b.ndeps++] = node;
    *added = true;
    return WPF_OK;
}

// ---- step control kernels ------------------------------------------------------
// The dt law of wPFAW3D.f90:2227-2230, dt = dt_c * min(dt_a, taumin), with
// dt_c = tfac * dx^2 / (2 eps^2) and dt_a = eps^2 / D, taumin from the key the
// previous update left in S_TAUMIN_KEY; the extrapolation coefficients of
// ws_coeffs for two held increments; the solve's control state and slots reset.
__global__ void k_step_begin(StepCtl* c, double* dsc, double dt_c, double dt_a) {
    if (threadIdx.x) return;
    const double tm = dkey_inv(reinterpret_cast<const unsigned long long*>(dsc)[S_TAUMIN_KEY]);
    const double dt = dt_c * (dt_a < tm ? dt_a : tm);
    c->dt = dt;
    const double hn = dt, h1 = c->h1, h2 = c->h2;
    if (!(hn > 0 && h1 > 0 && h2 > 0)) {
        c->wa = 2.f;
        c->wb = -1.f;
    } else {
        const double q = hn * (hn + h1) / (h1 + h2);
        c->wa = (float)(hn / h1 + q / h1);
        c->wb = (float)(-q / h2);
    }
    c->bnorm_prev = c->bnorm;   // the least-squares start's scale (k_ctl_ls_begin)
    c->bnorm = c->relres = c->relres0 = c->r0 = c->tol = 0.0;
    c->pass = c->outer = c->inner = c->it = c->need_pcg = c->accept = c->used = c->pcgs = c->net_runs = 0;
    c->alpha = 0.f;
    c->status = WPF_ERR_NOT_CONVERGED;
    for (int q = 0; q < 5; ++q) dsc[S_RR64 + q] = 0.0;   // RR64 BB64 RR0WS RW WW
    dsc[S_WSS2] = 0.0;
    dsc[S_WSD2] = 0.0;
}

// A converged solve's increment becomes the newest of the history.
__global__ void k_step_end(StepCtl* c) {
    if (threadIdx.x) return;
    if (c->status == WPF_OK) {
        c->h2 = c->h1;
        c->h1 = c->dt;
    }
}

// ---- host side ------------------------------------------------------------------
static bool ws_enabled(const wpf_handle* h) { return (h->opts.flags & WPF_SOLVER_EXTRAPOLATE) != 0; }

bool step_graph_ready(const wpf_handle* h, int itime) {
    const int f = h->opts.flags;
    return (f & WPF_SOLVER_STEP_GRAPH) && !(f & WPF_SOLVER_NO_GRAPHS) && itime >= 3 && h->timing_mask == 0 &&
           h->opts.max_outer >= 1 && h->have_wells && h->ndir > 0 &&
           (!ws_enabled(h) || h->ws_hist == 2);
}

int step_graph_prepare(wpf_handle* h) {
    int rc = solver_setup(h);
    if (rc) return rc;
    const Grid& g = h->g;
    if ((rc = update_alloc(h))) return rc;
    if (ws_enabled(h) && !h->ws_e[0] && (rc = dev_alloc(h, (void**)&h->ws_e[0], sizeof(float) * g.total)))
        return rc;
    if (!h->gctl) {
        if ((rc = dev_alloc(h, (void**)&h->gctl, sizeof(StepCtl)))) return rc;
        WPF_CUDA(cudaMallocHost((void**)&h->gctl_host, sizeof(StepCtl)));
        memset(h->gctl_host, 0, sizeof(StepCtl));
        WPF_CUDA(cudaMallocHost((void**)&h->gdsc_host, S_COUNT * sizeof(double)));
        h->gctl_dirty = true;
    }
    if (h->ws_net && ws_enabled(h) && (rc = ws_net_prepare(h))) return rc;
    if (!h->cap_split) WPF_CUDA(cudaStreamCreateWithFlags(&h->cap_split, cudaStreamNonBlocking));
    if (!h->cap_ws) {
        WPF_CUDA(cudaStreamCreateWithFlags(&h->cap_ws, cudaStreamNonBlocking));
        WPF_CUDA(cudaEventCreateWithFlags(&h->cap_ws_fork, cudaEventDisableTiming));
        WPF_CUDA(cudaEventCreateWithFlags(&h->cap_ws_join, cudaEventDisableTiming));
    }
    if (!h->cap_side) {
        WPF_CUDA(cudaStreamCreateWithFlags(&h->cap_side, cudaStreamNonBlocking));
        WPF_CUDA(cudaEventCreateWithFlags(&h->cap_fork, cudaEventDisableTiming));
        WPF_CUDA(cudaEventCreateWithFlags(&h->cap_join, cudaEventDisableTiming));
    }
    return WPF_OK;
}

// Capture one step of h into b (b not capturing on entry or exit).  The
// capture-time calls are launches only; the host flags phys_permeability
// sets are restored, since the graph runs later.
int step_graph_capture(wpf_handle* h, GraphBuilder& b, StepCounts* n) {
    cudaStream_t s = h->stream;
    const wpf_params& p = h->prm;
    const double e2 = p.epsilon * p.epsilon;
    const double dt_c = p.tfac * 0.5 * (p.dx * p.dx) / e2;
    const double dt_a = e2 / p.diffusion;
    StepCtl* c = h->gctl;
    int rc;
    if ((rc = gb_begin(b))) return rc;
    long long l0 = h->nlaunch;
    WPF_LAUNCH(h, KC_OTHER, k_step_begin<<<1, 32, 0, s>>>(c, h->dsc, dt_c, dt_a));
    // the extrapolated start needs only the dt law's coefficients: it is
    // built beside calcPermeability (HBM-bound beside FP64-bound)
    if ((rc = ws_capture_early(h, &h->ws_early))) return rc;
    const bool tc = h->t_current, tp = h->t_from_prev, kv = h->kf_valid, rko = h->rkeep_ok;
    const bool l0ok = h->l0_inc_ok;
    const int l0m = h->l0_mode;
    rc = phys_permeability(h, false);
    h->t_current = tc;
    h->t_from_prev = tp;
    h->kf_valid = kv;
    if (!rc) rc = capture_split_beside(h);
    if (rc) {
        h->rkeep_ok = rko;
        h->l0_inc_ok = l0ok;
        h->ws_early = false;
        drop_split(h);
        return rc;
    }
    n->fixed += h->nlaunch - l0;
    rc = solve_capture(h, b, n);   // the solve and the fused update (reads rkeep_ok as set above)
    h->rkeep_ok = rko;
    h->l0_inc_ok = l0ok;   // set when the graph has run (step_graph_finish)
    h->l0_mode = l0m;
    h->ws_early = false;
    drop_split(h);
    if (rc) return rc;
    l0 = h->nlaunch;
    WPF_LAUNCH(h, KC_OTHER, k_step_end<<<1, 32, 0, s>>>(c));
    WPF_CUDA(cudaGetLastError());
    WPF_CUDA(cudaMemcpyAsync(h->gctl_host, c, sizeof(StepCtl), cudaMemcpyDeviceToHost, s));
    WPF_CUDA(cudaMemcpyAsync(h->gdsc_host, h->dsc, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
    n->fixed += h->nlaunch - l0;
    return gb_end(b);
}

// End a capture left open by a failure, so that the stream is usable again.
void abandon_capture(cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
        cudaGraph_t t = nullptr;
        cudaStreamEndCapture(s, &t);
    }
    cudaGetLastError();
}

// Host state after a device-resident step, as the host-driven step leaves it.
int step_graph_finish(wpf_handle* h, const StepCounts& n, wpf_step_stats* st, double* dt_out) {
    const StepCtl c = *h->gctl_host;
    const double* d = h->gdsc_host;
    unsigned long long key, ov, um;
    memcpy(&key, d + S_TAUMIN_KEY, 8);
    memcpy(&ov, d + S_OVERSHOOT, 8);
    memcpy(&um, d + S_UMAX_BITS, 8);
    double umax;
    memcpy(&umax, &um, 8);
    int nw[2], kerr = 0;
    memcpy(nw, d + S_NWORK, sizeof(nw));
    memcpy(&kerr, d + S_KERR, sizeof(int));
    const double taumin = dkey_inv(key);
    h->taumin_last = taumin;
    h->ls_rp_rel = c.rp_rel;   // the least-squares start's record, for a host-driven next step
    h->ls_bnorm = c.bnorm;
    h->last_active = nw[0] + nw[1];
    h->last_interface = nw[0];
    h->ws_hn = c.dt;
    h->ws_used = c.used;
    if (c.used < 0) ++h->ws_fallbacks;
    if (ws_enabled(h) && h->ws[0]) {
        if (c.status == WPF_OK) {
            float* t = h->ws[1];
            h->ws[1] = h->ws[0];
            h->ws[0] = h->ws[2];
            h->ws[2] = t;
            h->ws_hist = h->ws_hist < 2 ? h->ws_hist + 1 : 2;
            h->ws_h2 = h->ws_h1;
            h->ws_h1 = c.dt;
        } else {
            h->ws_hist = 0;
        }
    }
    double* t = h->phase; h->phase = h->phase_n; h->phase_n = t;
    t = h->concent; h->concent = h->concent_n; h->concent_n = t;
    update_advance_bricks(h);
    h->vel_valid = false;
    h->kf_valid = false;
    h->t_from_prev = true;   // T came from the phase now in phase_n
    h->t_current = false;
    // every graph step ends on a plain residual pass of the final pressure
    h->rkeep_ok = h->rkeep && h->opts.mode == WPF_SOLVER_MIXED && c.status != WPF_ERR_NONFINITE;
    h->l0_inc_ok = h->l0mark != nullptr;   // the step rebuilt the level-0 operator
    h->l0_mode = h->opts.mode;
    const long long launches = n.fixed + (long long)c.pass * n.per_pass + (long long)c.inner * n.per_iter +
                               (long long)c.net_runs * n.per_net;
    h->nlaunch += launches;
    int rc = c.status;
    if (h->ws_net && ws_enabled(h) && rc != WPF_ERR_CUDA) {   // the net's kernels' bounded waits
        const int nrc = ws_net_check(h);
        if (nrc) rc = nrc;
    }
    if (kerr) {   // a sweep whose bounded staging wait ran out left its flag
        WPF_CUDA(cudaMemsetAsync(h->dsc + S_KERR, 0, sizeof(double), h->stream));
        WPF_CUDA(cudaStreamSynchronize(h->stream));
        rc = WPF_ERR_TIMEOUT;
    }
    if (st) {
        st->outer_iterations = c.outer;
        st->inner_iterations = c.inner;
        st->converged = c.status == WPF_OK;
        st->relres = c.relres;
        st->relres0 = c.relres0;
        st->warm_start = c.used;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
        st->solve_ms = ms;
        ms = 0.f;
        cudaEventElapsedTime(&ms, h->ev[2], h->ev[3]);
        st->update_ms = ms;
        st->taumin = taumin;
        st->overshoot_cells = (int32_t)ov;
        st->dtime = c.dt;
        st->max_courant = umax * c.dt / h->prm.dx;
        st->kernel_launches = (int32_t)launches;
        st->active_cells = (int32_t)h->last_active;
        st->interface_cells = (int32_t)h->last_interface;
        st->device_resident = 1;
    }
    cudaGetLastError();
    if (dt_out) *dt_out = c.dt;
    return rc;
}

void step_graph_key(const wpf_handle* h, const void** k) {
    const bool ws = ws_enabled(h);
    k[0] = h->phase;
    k[1] = h->concent;
    k[2] = ws ? h->ws[0] : nullptr;
    k[3] = ws ? h->ws[1] : nullptr;
    k[4] = ws ? h->ws[2] : nullptr;
    // calcPermeability recomputes only the faces whose cells changed phase when
    // T came from the phase now in phase_n (the last step), else every face
    k[5] = h->t_from_prev ? h->phase_n : nullptr;
    // and then corrects the kept FP64 residual, which pass 0 reads
    k[6] = (h->t_from_prev && h->rkeep && h->rkeep_ok) ? h->rkeep : nullptr;
    // the update skips the bricks that were quiescent in the last update
    k[7] = h->bact_ok ? h->bact[0] : nullptr;
    // the level-0 build rebuilds only the cells of recomputed faces
    k[8] = (h->t_from_prev && l0_incremental(h)) ? h->l0mark : nullptr;
    // the learned correction of the start, when a net is attached
    k[9] = ws ? (const void*)h->ws_net : nullptr;
}

// Upload the increment step sizes when the host-driven path changed them.
int step_graph_sync_ctl(wpf_handle* h) {
    if (!h->gctl_dirty) return WPF_OK;
    h->gctl_host->h1 = h->ws_h1;
    h->gctl_host->h2 = h->ws_h2;
    h->gctl_host->rp_rel = h->ls_rp_rel;   // the host-driven solves' record for the least-squares start
    h->gctl_host->bnorm = h->ls_bnorm;
    WPF_CUDA(cudaMemcpyAsync(h->gctl, h->gctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice, h->stream));
    h->gctl_dirty = false;
    return WPF_OK;
}

int step_graph_run(wpf_handle* h, wpf_step_stats* st, double* dt_out) {
    int rc = step_graph_prepare(h);
    if (rc) return rc;
    const void* key[STEP_KEY];
    step_graph_key(h, key);
    int slot = -1;
    for (int q = 0; q < h->nsg; ++q)
        if (!memcmp(h->sg[q].key, key, sizeof(key))) slot = q;
    if (slot < 0) {
        if (h->nsg == wpf_handle::MAX_STEP_GRAPHS) {   // drop the oldest
            cudaGraphExecDestroy(h->sg[0].exec);
            memmove(&h->sg[0], &h->sg[1], sizeof(h->sg[0]) * (wpf_handle::MAX_STEP_GRAPHS - 1));
            --h->nsg;
        }
        GraphBuilder b;
        WPF_CUDA(cudaGraphCreate(&b.graph, 0));
        b.top = b.graph;
        b.s = h->stream;
        StepCounts n;
        const long long saved = h->nlaunch;
        rc = step_graph_capture(h, b, &n);
        h->nlaunch = saved;
        if (b.capturing || rc) abandon_capture(h->stream);
        cudaGraphExec_t exec = nullptr;
        if (!rc && cudaGraphInstantiate(&exec, b.graph, 0) != cudaSuccess) {
            cudaGetLastError();
            rc = WPF_ERR_CUDA;
        }
        cudaGraphDestroy(b.graph);
        if (rc) return rc;
        slot = h->nsg++;
        memcpy(h->sg[slot].key, key, sizeof(key));
        h->sg[slot].exec = exec;
        h->sg[slot].n = n;
    }
    if ((rc = step_graph_sync_ctl(h))) return rc;
    WPF_CUDA(cudaGraphLaunch(h->sg[slot].exec, h->stream));
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    return step_graph_finish(h, h->sg[slot].n, st, dt_out);
}

void step_graphs_drop(wpf_handle* h) {
    for (int q = 0; q < h->nsg; ++q)
        if (h->sg[q].exec) cudaGraphExecDestroy(h->sg[q].exec);
    h->nsg = 0;
    ++h->epoch;
    h->gctl_dirty = true;
    ensemble_graphs_forget(h);
}

}  // namespace wpf
