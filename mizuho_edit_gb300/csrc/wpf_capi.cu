// wpf_capi.cu -- the extern "C" boundary of libwpf_gb300 (declared in include/wpf.h).
//
// Each entry point stands in for one module procedure of wPFAW3D.f90; the
// handle holds what the reference keeps in module-global arrays
// (wPFAW3D.f90:78-103), resident in device memory.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <utility>
#include <vector>

#include "wpf_internal.cuh"

using namespace wpf;

namespace wpf {

int dev_alloc(wpf_handle* h, void** p, size_t bytes) {
    *p = nullptr;
    if (cudaMalloc(p, bytes) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return WPF_ERR_NOMEM;
    }
    if (cudaMemsetAsync(*p, 0, bytes, h->stream) != cudaSuccess) return WPF_ERR_CUDA;
    h->bytes += (int64_t)bytes;
    return WPF_OK;
}

int timer_start(wpf_handle* h, int c) {
    if (!(h->timing_mask & (1u << c))) return -1;
    if (h->cap_ev) {   // capturing a graph: the pair becomes two event record nodes
        if (*h->cap_ntimers >= h->cap_max) return -1;
        const int slot = (*h->cap_ntimers)++;
        h->cap_cls[slot] = c;
        cudaEventRecordWithFlags(h->cap_ev[2 * slot], h->stream, cudaEventRecordExternal);
        return slot;
    }
    if (h->npend >= 256) timer_flush(h);
    if (h->npend >= 256) return -1;
    const int slot = h->npend++;
    h->pend_cls[slot] = c;
    cudaEventRecord(h->pend_ev[2 * slot], h->stream);
    return slot;
}

void timer_stop(wpf_handle* h, int slot) {
    if (slot < 0) return;
    if (h->cap_ev)
        cudaEventRecordWithFlags(h->cap_ev[2 * slot + 1], h->stream, cudaEventRecordExternal);
    else
        cudaEventRecord(h->pend_ev[2 * slot + 1], h->stream);
}

static void fold(wpf_handle* h, int cls, cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) {
        h->kt_ms[cls] += ms;
        h->kt_count[cls] += 1;
    } else {
        cudaGetLastError();
    }
}

void timer_flush(wpf_handle* h) {
    if (h->npend) {
        cudaEventSynchronize(h->pend_ev[2 * h->npend - 1]);
        for (int s = 0; s < h->npend; ++s)
            fold(h, h->pend_cls[s], h->pend_ev[2 * s], h->pend_ev[2 * s + 1]);
        h->npend = 0;
    }
    if (h->ngpend) {
        cudaEventSynchronize(h->gpend_b[h->ngpend - 1]);
        for (int s = 0; s < h->ngpend; ++s) fold(h, h->gpend_cls[s], h->gpend_a[s], h->gpend_b[s]);
        h->ngpend = 0;
    }
}

int ensure_per_routine_arrays(wpf_handle* h) {
    if (h->K0) return WPF_OK;
    const size_t b = sizeof(double) * h->g.total;
    double** arrs[9] = {&h->K0, &h->Kf[0], &h->Kf[1], &h->Kf[2], &h->vel[0], &h->vel[1], &h->vel[2],
                        &h->dphasedt, &h->dconcentdt};
    for (auto a : arrs) {
        int rc = dev_alloc(h, (void**)a, b);
        if (rc) return rc;
    }
    return WPF_OK;
}

int resident_blocks(const void* f, int threads, size_t smem, int cap) {
    static std::mutex mu;
    static std::vector<std::pair<const void*, int>> seen;   // (kernel, blocks per SM) for RB-thread launches
    const bool cacheable = threads == RB && smem == 0;
    std::lock_guard<std::mutex> lock(mu);
    if (cacheable)
        for (const auto& e : seen)
            if (e.first == f) return e.second < cap ? e.second : cap;
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f, threads, smem) != cudaSuccess || b < 1) {
        cudaGetLastError();
        return cap;
    }
    if (cacheable) seen.emplace_back(f, b);
    return b < cap ? b : cap;
}

}  // namespace wpf

static Phys make_phys(const wpf_params& p) {
    Phys P;
    P.dx = p.dx;
    P.inv_dx = 1.0 / p.dx;
    P.inv_2dx = 1.0 / (2.0 * p.dx);
    P.inv_dx2 = 1.0 / (p.dx * p.dx);
    P.inv_4dx2 = 1.0 / (4.0 * (p.dx * p.dx));
    P.epsilon = p.epsilon;
    P.lambda = p.lambda;
    P.alpha = p.alpha;
    P.diffusion = p.diffusion;
    P.ral = p.ral;
    P.rat = p.rat;
    P.kwh = p.permeab_hole;
    P.viscosity = p.viscosity;
    P.tau_num = 5.0 / 3.0 * p.alpha * p.lambda * (p.epsilon * p.epsilon);   // :1254
    P.tau0 = P.tau_num / p.diffusion;
    P.inv_tau_num = 1.0 / P.tau_num;
    P.inv_tau0 = 1.0 / P.tau0;
    P.w0 = 2.0 * p.dx;                                                      // :1221
    P.maxdphi = 2.0 / (2.0 * p.dx);                                          // :1225
    P.qscale = p.dx * p.dx / (p.dx * p.dx * p.dx);                           // :817
    return P;
}

static void free_all(wpf_handle* h) {
    step_graphs_drop(h);
    if (h->gctl) cudaFree(h->gctl);
    if (h->gctl_host) cudaFreeHost(h->gctl_host);
    if (h->gdsc_host) cudaFreeHost(h->gdsc_host);
    if (h->split_graph) cudaGraphDestroy(h->split_graph);
    if (h->cap_split) cudaStreamDestroy(h->cap_split);
    if (h->cap_ws) cudaStreamDestroy(h->cap_ws);
    if (h->cap_ws_fork) cudaEventDestroy(h->cap_ws_fork);
    if (h->cap_ws_join) cudaEventDestroy(h->cap_ws_join);
    if (h->cap_side) cudaStreamDestroy(h->cap_side);
    if (h->cap_fork) cudaEventDestroy(h->cap_fork);
    if (h->cap_join) cudaEventDestroy(h->cap_join);
    double* d[] = {h->krock, h->phase, h->concent, h->pressure, h->phase_n, h->concent_n,
                   h->T[0], h->T[1], h->T[2], h->Tv[0], h->Tv[1], h->Tv[2], h->K0, h->Kf[0], h->Kf[1], h->Kf[2],
                   h->vel[0], h->vel[1], h->vel[2], h->dphasedt, h->dconcentdt, h->dir_val,
                   h->qterm, h->dsc, h->partials, h->staging};
    for (double* p : d)
        if (p) cudaFree(p);
    if (h->flags) cudaFree(h->flags);
    if (h->work) cudaFree(h->work);
    for (int q = 0; q < 2; ++q)
        if (h->bact[q]) cudaFree(h->bact[q]);
    if (h->snap) cudaFree(h->snap);
    if (h->snap_ready) cudaEventDestroy(h->snap_ready);
    if (h->snap_done) cudaEventDestroy(h->snap_done);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->dphys) cudaFree(h->dphys);
    if (h->dir_idx) cudaFree(h->dir_idx);
    solver_free(h);
    if (h->hsc) cudaFreeHost(h->hsc);
    for (int e = 0; e < 4; ++e)
        if (h->ev[e]) cudaEventDestroy(h->ev[e]);
    for (int e = 0; e < 512; ++e)
        if (h->pend_ev[e]) cudaEventDestroy(h->pend_ev[e]);
    if (h->stream) cudaStreamDestroy(h->stream);
}

extern "C" {

const char* wpf_strerror(int s) {
    switch (s) {
        case WPF_OK: return "ok";
        case WPF_ERR_ARG: return "invalid argument";
        case WPF_ERR_CUDA: return "CUDA error (no usable device or a failed launch)";
        case WPF_ERR_NOT_CONVERGED: return "Darcy solve did not reach the tolerance";
        case WPF_ERR_NONFINITE: return "non-finite value in a residual or reduction";
        case WPF_ERR_TIMEOUT: return "bounded device wait expired";
        case WPF_ERR_NOMEM: return "device allocation failed";
        case WPF_ERR_SINGULAR: return "no Dirichlet cell: the Darcy system is singular";
        case WPF_ERR_TOO_LARGE:
            return "grid exceeds the fixed scratch of wpf_reduce_noalloc (nz + 2 > 4096 planes)";
        default: return "unknown status";
    }
}

int wpf_create(const wpf_params* p, wpf_handle** out) {
    if (!p || !out) return WPF_ERR_ARG;
    *out = nullptr;
    if (p->nx < 1 || p->ny < 1 || p->nz < 1 || !(p->dx > 0) || !(p->viscosity != 0) ||
        !(p->diffusion != 0) || !(p->epsilon != 0))
        return WPF_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return WPF_ERR_CUDA;
    }
    wpf_handle* h = (wpf_handle*)calloc(1, sizeof(wpf_handle));
    if (!h) return WPF_ERR_NOMEM;
    new (&h->h64) Hierarchy<double>();
    new (&h->h32) Hierarchy<float>();
    static std::atomic<unsigned long long> next_uid{1};
    h->uid = next_uid++;
    h->prm = *p;
    h->phys = make_phys(*p);
    h->g = make_grid(p->nx, p->ny, p->nz);
    cudaGetDevice(&h->device);
    h->nsm = 1;
    cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device);
    if (h->nsm < 1) h->nsm = 1;
    int pma = 0, pmh = 0;
    cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, h->device);
    cudaDeviceGetAttribute(&pmh, cudaDevAttrPageableMemoryAccessUsesHostPageTables, h->device);
    h->host_pageable_direct = pma == 1 && pmh == 1;
    cudaGetLastError();
    int rc = WPF_OK;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) rc = WPF_ERR_CUDA;
    for (int e = 0; e < 4 && !rc; ++e)
        if (cudaEventCreate(&h->ev[e]) != cudaSuccess) rc = WPF_ERR_CUDA;
    if (!rc && cudaMallocHost((void**)&h->hsc, S_COUNT * sizeof(double)) != cudaSuccess)
        rc = WPF_ERR_CUDA;
    const size_t fb = sizeof(double) * h->g.total;
    double** arrs[12] = {&h->krock, &h->phase, &h->concent, &h->pressure, &h->phase_n, &h->concent_n,
                         &h->T[0], &h->T[1], &h->T[2], &h->Tv[0], &h->Tv[1], &h->Tv[2]};
    for (int a = 0; a < 12 && !rc; ++a) rc = dev_alloc(h, (void**)arrs[a], fb);
    if (!rc) rc = dev_alloc(h, (void**)&h->flags, h->g.total);
    if (!rc) rc = dev_alloc(h, (void**)&h->dsc, S_COUNT * sizeof(double));
    if (!rc) rc = dev_alloc(h, (void**)&h->dphys, sizeof(Phys));
    if (!rc && cudaMemcpyAsync(h->dphys, &h->phys, sizeof(Phys), cudaMemcpyHostToDevice, h->stream) !=
                   cudaSuccess)
        rc = WPF_ERR_CUDA;
    h->opts.mode = WPF_SOLVER_FP64;
    h->opts.max_outer = 20;
    h->opts.max_inner = 500;
    h->opts.smooth_sweeps = 2;
    h->opts.rtol = 1e-8;
    h->opts.inner_rtol = 1e-4;
    h->taumin_last = 1.0e6;
    if (!rc && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = WPF_ERR_CUDA;
    if (rc) {
        free_all(h);
        free(h);
        return rc;
    }
    *out = h;
    return WPF_OK;
}

int wpf_destroy(wpf_handle* h) {
    if (!h) return WPF_ERR_ARG;
    cudaStreamSynchronize(h->stream);
    free_all(h);
    h->h64.~Hierarchy<double>();
    h->h32.~Hierarchy<float>();
    free(h);
    return WPF_OK;
}

int wpf_device_bytes(const wpf_handle* h, int64_t* bytes) {
    if (!h || !bytes) return WPF_ERR_ARG;
    *bytes = h->bytes;
    return WPF_OK;
}

int wpf_set_solver(wpf_handle* h, const wpf_solver_opts* o) {
    if (!h || !o) return WPF_ERR_ARG;
    if (o->mode != WPF_SOLVER_FP64 && o->mode != WPF_SOLVER_MIXED) return WPF_ERR_ARG;
    if (o->max_outer < 0 || o->max_inner < 1 || !(o->rtol > 0) || o->smooth_sweeps < 0 ||
        o->smooth_sweeps > 16 || o->sweep_zchunk < 0 || o->row_blocks_per_sm < 0 || o->row_blocks_per_sm > 64)
        return WPF_ERR_ARG;
    cudaStreamSynchronize(h->stream);
    solver_drop_graphs(h);   // the captured cycles bake in nu, the sweep and W-cycle levels
    h->opts = *o;
    h->ws_hist = 0;          // a new solver starts a new increment history
    h->ws_h1 = h->ws_h2 = 0.0;
    h->rkeep_ok = false;
    h->l0_inc_ok = false;
    if (!(h->opts.inner_rtol > 0 && h->opts.inner_rtol < 1)) h->opts.inner_rtol = 1e-4;
    if (h->opts.smooth_sweeps == 0) h->opts.smooth_sweeps = 2;
    return WPF_OK;
}

int wpf_get_solver(const wpf_handle* h, wpf_solver_opts* o) {
    if (!h || !o) return WPF_ERR_ARG;
    *o = h->opts;
    return WPF_OK;
}

int wpf_set_wells(wpf_handle* h, const wpf_well* wells, int32_t nwell) {
    if (!h || nwell < 0 || (nwell > 0 && !wells)) return WPF_ERR_ARG;
    const Grid& g = h->g;
    const long long nxh = g.nx + 2, nyh = g.ny + 2, nzh = g.nz + 2;
    std::vector<int32_t> lw((size_t)(nxh * nyh * nzh), 0);
    for (int iw = 0; iw < nwell; ++iw) {   // wPFAW3D.f90:453-461 (later wells win)
        const wpf_well& w = wells[iw];
        if (0 <= w.ix && w.ix <= g.nx + 1 && 0 <= w.iy && w.iy <= g.ny + 1 && 0 <= w.iz &&
            w.iz <= g.nz + 1)
            lw[(size_t)(w.ix + nxh * (w.iy + nyh * w.iz))] = iw + 1;
    }
    std::vector<uint8_t> fl((size_t)g.total, 0);
    std::vector<long long> didx;
    std::vector<double> dval;
    std::vector<std::pair<long long, double>> inl;
    for (int k = 0; k <= g.nz + 1; ++k)
        for (int j = 0; j <= g.ny + 1; ++j)
            for (int i = 0; i <= g.nx + 1; ++i) {
                const int iw = lw[(size_t)(i + nxh * (j + nyh * k))];
                if (iw <= 0) continue;
                const wpf_well& w = wells[iw - 1];
                const long long n = g.at(i, j, k);
                uint8_t f = F_WELL;
                const bool interior = i >= 1 && i <= g.nx && j >= 1 && j <= g.ny && k >= 1 && k <= g.nz;
                if (w.pressure != 0.0) {
                    f |= F_DIR;
                    if (interior) { didx.push_back(n); dval.push_back(w.pressure); }
                } else if (w.injection != 0.0) {
                    f |= F_INLET;
                    if (interior) inl.push_back({n, w.injection});
                }
                fl[(size_t)n] = f;
            }
    if (h->dir_idx) { cudaFree(h->dir_idx); h->dir_idx = nullptr; }
    if (h->dir_val) { cudaFree(h->dir_val); h->dir_val = nullptr; }
    if (h->qterm) { cudaFree(h->qterm); h->qterm = nullptr; }
    h->ndir = (int32_t)didx.size();
    h->ninlet = (int32_t)inl.size();
    int rc;
    if (h->ndir) {
        if ((rc = dev_alloc(h, (void**)&h->dir_idx, sizeof(long long) * h->ndir))) return rc;
        if ((rc = dev_alloc(h, (void**)&h->dir_val, sizeof(double) * h->ndir))) return rc;
        WPF_CUDA(cudaMemcpyAsync(h->dir_idx, didx.data(), sizeof(long long) * h->ndir,
                                 cudaMemcpyHostToDevice, h->stream));
        WPF_CUDA(cudaMemcpyAsync(h->dir_val, dval.data(), sizeof(double) * h->ndir,
                                 cudaMemcpyHostToDevice, h->stream));
    }
    if (h->ninlet) {
        std::vector<double> q((size_t)g.total, 0.0);
        for (auto& e : inl) q[(size_t)e.first] = e.second * h->phys.qscale;   // -b of :817
        if ((rc = dev_alloc(h, (void**)&h->qterm, sizeof(double) * g.total))) return rc;
        WPF_CUDA(cudaMemcpyAsync(h->qterm, q.data(), sizeof(double) * g.total, cudaMemcpyHostToDevice,
                                 h->stream));
    }
    WPF_CUDA(cudaMemcpyAsync(h->flags, fl.data(), g.total, cudaMemcpyHostToDevice, h->stream));
    WPF_CUDA(cudaStreamSynchronize(h->stream));   // host vectors go out of scope
    h->have_wells = true;
    h->ws_hist = 0;   // new boundary conditions: the increment history no longer applies
    h->rkeep_ok = false;
    h->l0_inc_ok = false;   // the well flags enter the level-0 operator
    h->bact_ok = false;   // the well flags enter the update's classification
    step_graphs_drop(h);   // the step graphs bake in the well arrays
    return phys_set_dirichlet(h);
}

// Host fields are dense halo arrays (nx+2)(ny+2)(nz+2) in Fortran order; the
// device rows are pitched.  A field crosses the host link as one contiguous
// copy through a dense staging buffer and is re-pitched on the device (block
// = one row of nx+2 values): row-by-row 2D copies of 2 KB rows run far below
// the link's bandwidth.
// Host layout <-> pitched device field as a flat walk over 16-byte pairs of
// the dense array (one row-major index e -> row e / w, column e % w), each
// thread keeping four pairs in flight: the dense side is the caller's host
// array when the device reaches it in place, where many outstanding requests
// keep the link busy.  Needs a 16-byte aligned dense array.
__device__ __forceinline__ long long pitched_of(const Grid& g, unsigned long long e, unsigned w) {
    const unsigned long long r = e / w;
    return g.at(0, 0, 0) + (long long)r * g.P + (long long)(e - r * w);
}

// in: writes only the values that differ bitwise from the device copy and
// flags *changed if any did
__global__ void __launch_bounds__(256) k_dense_in(Grid g, const double2* __restrict__ src,
                                                  double* __restrict__ dst, long long G, int* changed) {
    const unsigned w = g.nx + 2;
    const long long npair = G >> 1, stride = (long long)gridDim.x * blockDim.x;
    int chg = 0;
    auto put = [&](long long o, double v) {
        if (__double_as_longlong(dst[o]) != __double_as_longlong(v)) {
            dst[o] = v;
            chg = 1;
        }
    };
    for (long long q0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; q0 < npair; q0 += 4 * stride) {
        double2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (q0 + u * stride < npair) v[u] = src[q0 + u * stride];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long q = q0 + u * stride;
            if (q >= npair) break;
            put(pitched_of(g, 2ull * q, w), v[u].x);
            put(pitched_of(g, 2ull * q + 1, w), v[u].y);
        }
    }
    if ((G & 1) && blockIdx.x == 0 && threadIdx.x == 0)
        put(pitched_of(g, G - 1, w), reinterpret_cast<const double*>(src)[G - 1]);
    if (__syncthreads_or(chg) && threadIdx.x == 0) *changed = 1;
}

__global__ void __launch_bounds__(256) k_dense_out(Grid g, const double* __restrict__ src,
                                                   double2* __restrict__ dst, long long G) {
    const unsigned w = g.nx + 2;
    const long long npair = G >> 1, stride = (long long)gridDim.x * blockDim.x;
    for (long long q0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; q0 < npair; q0 += 4 * stride) {
        double2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long q = q0 + u * stride;
            if (q < npair) v[u] = make_double2(src[pitched_of(g, 2ull * q, w)], src[pitched_of(g, 2ull * q + 1, w)]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (q0 + u * stride < npair) dst[q0 + u * stride] = v[u];
    }
    if ((G & 1) && blockIdx.x == 0 && threadIdx.x == 0)
        reinterpret_cast<double*>(dst)[G - 1] = src[pitched_of(g, G - 1, w)];
}

// Host layout -> pitched device field, writing only the values that differ
// bitwise from the device copy and flagging *changed if any did (row per
// block: any alignment).
__global__ void k_repitch_in(Grid g, const double* __restrict__ src, double* __restrict__ dst, int* changed) {
    const int w = g.nx + 2;
    const long long row = blockIdx.x;
    const long long dense = row * w, pitched = g.at(0, 0, 0) + row * g.P;
    int chg = 0;
    for (int i = threadIdx.x; i < w; i += blockDim.x) {
        const double v = src[dense + i];
        if (__double_as_longlong(dst[pitched + i]) != __double_as_longlong(v)) {
            dst[pitched + i] = v;
            chg = 1;
        }
    }
    if (__syncthreads_or(chg) && threadIdx.x == 0) *changed = 1;
}

// Pitched device field -> host layout, row per block (any alignment).
__global__ void k_repitch_out(Grid g, const double* __restrict__ src, double* __restrict__ dst) {
    const int w = g.nx + 2;
    const long long row = blockIdx.x;
    const long long dense = row * w, pitched = g.at(0, 0, 0) + row * g.P;
    for (int i = threadIdx.x; i < w; i += blockDim.x) dst[dense + i] = src[pitched + i];
}

// FP32 dense interior copies of pressure, phase, concentration and the cell
// permeability K0 = kwh f + Krock (1 - f), f = (1 + phase)/2 (:567-574) of kph.
__global__ void __launch_bounds__(RB) k_snapshot(Grid g, Phys P, const double* __restrict__ pr,
                                                 const double* __restrict__ ph,
                                                 const double* __restrict__ cc,
                                                 const double* __restrict__ kph,
                                                 const double* __restrict__ kr, float* __restrict__ out) {
    const long long N = (long long)g.nx * g.ny * g.nz;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        const long long d = (i - 1) + (long long)g.nx * ((j - 1) + (long long)g.ny * (k - 1));
        const double f = 0.5 * (1.0 + kph[n]);
        out[d] = (float)pr[n];
        out[N + d] = (float)ph[n];
        out[2 * N + d] = (float)cc[n];
        out[3 * N + d] = (float)(P.kwh * f + kr[n] * (1.0 - f));
    }
}

static int ensure_staging(wpf_handle* h) {
    if (h->staging) return WPF_OK;
    const Grid& g = h->g;
    return dev_alloc(h, (void**)&h->staging, sizeof(double) * (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2));
}

// The address through which a kernel reads or writes the host array p in
// place, or null when it has to go through a staging copy: page-locked
// memory (its mapped device address) always; ordinary pageable memory when
// the device reaches it through the host's page tables (GB300 with its Grace
// host over the coherent NVLink-C2C), which the handle queried at creation.
static const void* host_direct(const wpf_handle* h, const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
    if (a.type == cudaMemoryTypeUnregistered && h->host_pageable_direct) return p;
    return nullptr;
}

// changed: device int set when any value differs from the device copy
static int copy_field_in(wpf_handle* h, double* dst, const double* src, int* changed) {
    const Grid& g = h->g;
    const double* from = static_cast<const double*>(host_direct(h, src));   // read in place
    if (!from) {
        int rc = ensure_staging(h);
        if (rc) return rc;
        const size_t G = (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
        WPF_CUDA(cudaMemcpyAsync(h->staging, src, G * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        from = h->staging;
    }
    const long long G = (long long)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
    if (((uintptr_t)from & 15u) == 0)
        WPF_LAUNCH(h, KC_OTHER, k_dense_in<<<(unsigned)h->nsm * 8, 256, 0, h->stream>>>(
            g, reinterpret_cast<const double2*>(from), dst, G, changed));
    else
        WPF_LAUNCH(h, KC_OTHER, k_repitch_in<<<(unsigned)((g.ny + 2) * (g.nz + 2)), 128, 0, h->stream>>>(
            g, from, dst, changed));
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

static int copy_field_out(wpf_handle* h, double* dst, const double* src) {
    const Grid& g = h->g;
    if (double* hd = static_cast<double*>(const_cast<void*>(host_direct(h, dst)))) {   // write in place
        const long long G = (long long)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
        if (((uintptr_t)hd & 15u) == 0)
            WPF_LAUNCH(h, KC_OTHER, k_dense_out<<<(unsigned)h->nsm * 8, 256, 0, h->stream>>>(
                g, src, reinterpret_cast<double2*>(hd), G));
        else
            WPF_LAUNCH(h, KC_OTHER, k_repitch_out<<<(unsigned)((g.ny + 2) * (g.nz + 2)), 128, 0, h->stream>>>(
                g, src, hd));
        WPF_CUDA(cudaGetLastError());
        return WPF_OK;
    }
    int rc = ensure_staging(h);
    if (rc) return rc;
    const size_t G = (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
    WPF_LAUNCH(h, KC_OTHER, k_repitch_out<<<(unsigned)((g.ny + 2) * (g.nz + 2)), 128, 0, h->stream>>>(
        g, src, h->staging));
    WPF_CUDA(cudaGetLastError());
    WPF_CUDA(cudaMemcpyAsync(dst, h->staging, G * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    return WPF_OK;
}

int wpf_upload(wpf_handle* h, const double* krock, const double* phase, const double* concent,
               const double* pressure) {
    if (!h) return WPF_ERR_ARG;
    int rc;
    // each field is compared bitwise with the device copy as it is written:
    // only a field that changed invalidates the state derived from it (a
    // host driver that sends back what it downloaded keeps the incremental
    // permeability, the kept residual and the quiescent bricks)
    int* chg = reinterpret_cast<int*>(h->dsc + S_UPL0);   // krock, phase, concent, pressure
    WPF_CUDA(cudaMemsetAsync(chg, 0, 4 * sizeof(int), h->stream));
    if (krock) { if ((rc = copy_field_in(h, h->krock, krock, chg + 0))) return rc; if ((rc = phys_halo(h, h->krock))) return rc; }
    if (phase) { if ((rc = copy_field_in(h, h->phase, phase, chg + 1))) return rc; if ((rc = phys_halo(h, h->phase))) return rc; }
    if (concent) { if ((rc = copy_field_in(h, h->concent, concent, chg + 2))) return rc; if ((rc = phys_halo(h, h->concent))) return rc; }
    if (pressure) {
        if ((rc = copy_field_in(h, h->pressure, pressure, chg + 3))) return rc;
        if ((rc = phys_set_dirichlet(h))) return rc;
    }
    WPF_CUDA(cudaMemcpyAsync(h->hsc + S_UPL0, h->dsc + S_UPL0, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                             h->stream));
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    int c[4];
    memcpy(c, h->hsc + S_UPL0, sizeof(c));
    const bool ck = krock && c[0], cp = phase && c[1], cc = concent && c[2], cpr = pressure && c[3];
    if (ck || cp || cpr) {
        h->vel_valid = false;
        h->rkeep_ok = false;   // the kept residual no longer matches p and T
    }
    if (cp || cc) h->bact_ok = false;   // the update's brick activity no longer holds
    if (ck) h->ws_klog_ready = false;   // the learned start's input statistics change
    if (cp || ck) {
        h->kf_valid = false;
        h->t_current = false;
        h->t_from_prev = false;
    }
    return WPF_OK;
}

int wpf_download(wpf_handle* h, double* phase, double* concent, double* pressure, double* permeab,
                 double* velocity, double* dphasedt, double* dconcentdt) {
    if (!h) return WPF_ERR_ARG;
    int rc;
    if (phase && (rc = copy_field_out(h, phase, h->phase))) return rc;
    if (concent && (rc = copy_field_out(h, concent, h->concent))) return rc;
    if (pressure && (rc = copy_field_out(h, pressure, h->pressure))) return rc;
    if (dphasedt || dconcentdt || permeab || velocity) {
        if ((rc = ensure_per_routine_arrays(h))) return rc;
    }
    if (dphasedt && (rc = copy_field_out(h, dphasedt, h->dphasedt))) return rc;
    if (dconcentdt && (rc = copy_field_out(h, dconcentdt, h->dconcentdt))) return rc;
    const Grid& g = h->g;
    const size_t G = (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
    if (permeab || velocity) {
        std::vector<double> tmp(G);
        if (permeab) {
            double* comp[4] = {h->K0, h->Kf[0], h->Kf[1], h->Kf[2]};
            for (int m = 0; m < 4; ++m) {
                if ((rc = copy_field_out(h, tmp.data(), comp[m]))) return rc;
                WPF_CUDA(cudaStreamSynchronize(h->stream));
                for (size_t n = 0; n < G; ++n) permeab[4 * n + m] = tmp[n];
            }
        }
        if (velocity) {
            for (int m = 0; m < 3; ++m) {
                if ((rc = copy_field_out(h, tmp.data(), h->vel[m]))) return rc;
                WPF_CUDA(cudaStreamSynchronize(h->stream));
                for (size_t n = 0; n < G; ++n) velocity[3 * n + m] = tmp[n];
            }
        }
    }
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    return WPF_OK;
}

int wpf_calc_permeability(wpf_handle* h) {
    if (!h) return WPF_ERR_ARG;
    int rc = phys_permeability(h, true);
    if (rc) return rc;
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    return WPF_OK;
}

int wpf_solve_pressure(wpf_handle* h, wpf_step_stats* st) {
    if (!h || !h->have_wells) return WPF_ERR_ARG;
    wpf_step_stats tmp;
    memset(&tmp, 0, sizeof(tmp));
    h->ws_hn = 0.0;   // step size unknown here: the extrapolation assumes equal steps
    int rc = solve_pressure(h, st ? st : &tmp);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess && !rc) rc = WPF_ERR_CUDA;
    return rc;
}

int wpf_calc_velocity(wpf_handle* h) {
    if (!h) return WPF_ERR_ARG;
    int rc = phys_velocity(h);
    if (rc) return rc;
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    return WPF_OK;
}

int wpf_calc_phase_deriv(wpf_handle* h, double* taumin, int32_t* overshoot) {
    if (!h || !h->have_wells) return WPF_ERR_ARG;
    if (!h->vel_valid) return WPF_ERR_ARG;   // calcVelocity must run first (:2251-2252)
    return phys_phase_deriv(h, taumin, overshoot);
}

int wpf_calc_concent_deriv(wpf_handle* h) {
    if (!h || !h->have_wells || !h->vel_valid) return WPF_ERR_ARG;
    int rc = phys_concent_deriv(h);
    if (rc) return rc;
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    return WPF_OK;
}

int wpf_evolve_phase(wpf_handle* h, double dtime) {
    if (!h) return WPF_ERR_ARG;
    int rc = phys_evolve(h, true, dtime);
    if (rc) return rc;
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    return WPF_OK;
}

int wpf_evolve_concent(wpf_handle* h, double dtime) {
    if (!h) return WPF_ERR_ARG;
    int rc = phys_evolve(h, false, dtime);
    if (rc) return rc;
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    return WPF_OK;
}

int wpf_get_taumin(const wpf_handle* h, double* taumin) {
    if (!h || !taumin) return WPF_ERR_ARG;
    *taumin = h->taumin_last;
    return WPF_OK;
}

int wpf_set_taumin(wpf_handle* h, double taumin) {
    if (!h || !(taumin > 0.0) || !(taumin < INFINITY)) return WPF_ERR_ARG;
    h->taumin_last = taumin;   // the host-driven step's dt law
    // and the key the device-resident step's dt law reads (the last update's min)
    const unsigned long long key = dkey_host(taumin);
    memcpy(&h->hsc[S_TAUMIN_KEY], &key, 8);
    WPF_CUDA(cudaMemcpyAsync(h->dsc + S_TAUMIN_KEY, h->hsc + S_TAUMIN_KEY, sizeof(double),
                             cudaMemcpyHostToDevice, h->stream));
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    return WPF_OK;
}

int wpf_step(wpf_handle* h, int32_t itime, double* dtime_inout, wpf_step_stats* st) {
    if (!h || !dtime_inout || !h->have_wells) return WPF_ERR_ARG;
    double dt = *dtime_inout;
    const wpf_params& p = h->prm;
    if (itime >= 3) {   // wPFAW3D.f90:2227-2230, taumin from the previous step
        const double e2 = p.epsilon * p.epsilon;
        const double a = e2 / p.diffusion;
        dt = p.tfac * 0.5 * (p.dx * p.dx) / e2 * (a < h->taumin_last ? a : h->taumin_last);
    }
    wpf_step_stats tmp;
    memset(&tmp, 0, sizeof(tmp));
    wpf_step_stats* s = st ? st : &tmp;
    if (step_graph_ready(h, itime)) {   // the whole step as one graph launch
        memset(s, 0, sizeof(*s));
        return step_graph_run(h, s, dtime_inout);
    }
    const long long l0 = h->nlaunch;
    int rc = phys_permeability(h, false);
    if (rc) return rc;
    h->ws_hn = dt;   // step size of this step, for the extrapolated start
    const int srs = solve_pressure(h, s);
    if (srs && srs != WPF_ERR_NOT_CONVERGED) return srs;
    double taumin = 0, umax = 0;
    int32_t over = 0;
    rc = phys_fused_update(h, dt, &taumin, &over, &umax);   // records ev[2]/ev[3] around the kernel
    if (rc) return rc;
    WPF_CUDA(cudaEventSynchronize(h->ev[3]));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev[2], h->ev[3]);
    s->update_ms = ms;
    s->taumin = taumin;
    s->overshoot_cells = over;
    s->dtime = dt;
    s->max_courant = umax * dt / p.dx;
    s->kernel_launches = (int32_t)(h->nlaunch - l0);
    s->active_cells = (int32_t)h->last_active;
    s->interface_cells = (int32_t)h->last_interface;
    s->device_resident = 0;
    *dtime_inout = dt;
    return srs;
}

int wpf_run(wpf_handle* h, int32_t itime0, int32_t nsteps, double* dtime_inout,
            wpf_step_stats* last) {
    if (!h || nsteps < 0 || !dtime_inout) return WPF_ERR_ARG;
    int rc = WPF_OK;
    for (int s = 0; s < nsteps; ++s) {
        rc = wpf_step(h, itime0 + s, dtime_inout, last);
        if (rc && rc != WPF_ERR_NOT_CONVERGED) return rc;
    }
    return rc;
}

int wpf_set_kernel_timing(wpf_handle* h, uint32_t mask) {
    if (!h) return WPF_ERR_ARG;
    if (mask && !h->pend_ev[0]) {
        for (int e = 0; e < 512; ++e)
            if (cudaEventCreate(&h->pend_ev[e]) != cudaSuccess) return WPF_ERR_CUDA;
    }
    timer_flush(h);
    h->timing_mask = mask & ((1u << KC_COUNT) - 1);
    for (int c = 0; c < 16; ++c) { h->kt_ms[c] = 0.0; h->kt_count[c] = 0; }
    return WPF_OK;
}

int wpf_kernel_times(wpf_handle* h, double* ms, int64_t* counts, int32_t n) {
    if (!h || n < 0 || (n > 0 && (!ms || !counts))) return WPF_ERR_ARG;
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    timer_flush(h);
    for (int c = 0; c < n && c < 16; ++c) { ms[c] = h->kt_ms[c]; counts[c] = h->kt_count[c]; }
    return WPF_OK;
}

int wpf_get_stream(const wpf_handle* h, void** stream) {
    if (!h || !stream) return WPF_ERR_ARG;
    *stream = (void*)h->stream;
    return WPF_OK;
}

int wpf_launch_count(const wpf_handle* h, int64_t* n) {
    if (!h || !n) return WPF_ERR_ARG;
    *n = h->nlaunch;
    return WPF_OK;
}

int wpf_host_alloc(int64_t bytes, void** ptr) {
    if (!ptr || bytes <= 0) return WPF_ERR_ARG;
    if (cudaMallocHost(ptr, (size_t)bytes) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return WPF_ERR_NOMEM;
    }
    return WPF_OK;
}

int wpf_snapshot(wpf_handle* h, float* out) {
    if (!h || !out) return WPF_ERR_ARG;
    const Grid& g = h->g;
    const long long N = (long long)g.nx * g.ny * g.nz;
    if (!h->snap) {
        int rc = dev_alloc(h, (void**)&h->snap, sizeof(float) * 4 * N);
        if (rc) return rc;
        WPF_CUDA(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
        WPF_CUDA(cudaEventCreateWithFlags(&h->snap_ready, cudaEventDisableTiming));
        WPF_CUDA(cudaEventCreateWithFlags(&h->snap_done, cudaEventDisableTiming));
    }
    // the staging buffer is reused: the previous copy must have left it
    if (h->snap_pending) WPF_CUDA(cudaStreamWaitEvent(h->stream, h->snap_done, 0));
    // K0 of the phase the last fused step started from (phase_n after it)
    const double* kph = h->t_from_prev ? h->phase_n : h->phase;
    WPF_LAUNCH(h, KC_OTHER, k_snapshot<<<row_blocks(h, g), RB, 0, h->stream>>>(
        g, h->phys, h->pressure, h->phase, h->concent, kph, h->krock, h->snap));
    WPF_CUDA(cudaGetLastError());
    WPF_CUDA(cudaEventRecord(h->snap_ready, h->stream));
    WPF_CUDA(cudaStreamWaitEvent(h->side, h->snap_ready, 0));
    WPF_CUDA(cudaMemcpyAsync(out, h->snap, sizeof(float) * 4 * N, cudaMemcpyDeviceToHost, h->side));
    WPF_CUDA(cudaEventRecord(h->snap_done, h->side));
    h->snap_pending = true;
    return WPF_OK;
}

int wpf_snapshot_wait(wpf_handle* h) {
    if (!h) return WPF_ERR_ARG;
    if (h->snap_pending) WPF_CUDA(cudaEventSynchronize(h->snap_done));
    h->snap_pending = false;
    return WPF_OK;
}

int wpf_host_free(void* ptr) {
    if (ptr && cudaFreeHost(ptr) != cudaSuccess) return WPF_ERR_CUDA;
    return WPF_OK;
}

int wpf_reduce(wpf_handle* h, wpf_diag* d) {
    if (!h || !d) return WPF_ERR_ARG;
    return phys_reduce(h, d);
}

}  // extern "C"

namespace wpf {
// The integer-pipe conversions against the hardware ones: x -> FP32 must equal
// __double2float_rn(x) wherever that is a normal number, zero, Inf or NaN (an
// FP32-subnormal result flushes to a zero of the same sign), and FP32 -> FP64
// must be exact for every FP32 value that is not subnormal.
__global__ void k_check_conversions(const double* x, long long n, unsigned long long* bad) {
    unsigned long long nb = 0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const double v = x[q];
        const float ref = __double2float_rn(v);
        const float got = f64_to_f32(v);
        const unsigned ur = __float_as_uint(ref), ug = __float_as_uint(got);
        const unsigned ar = ur & 0x7fffffffu;
        const unsigned vhi = (unsigned)__double2hiint(v) & 0x7fffffffu;
        bool ok;
        if (ar > 0x7f800000u) ok = (ug & 0x7fffffffu) > 0x7f800000u;                 // NaN
        else if (vhi < 0x38100000u) ok = ug == (ur & 0x80000000u);                   // |x| < 2^-126: flushed
        else ok = ug == ur;
        if (!ok) ++nb;
        const float f = ref;
        const unsigned af = __float_as_uint(f) & 0x7fffffffu;
        if (!(af != 0u && af < 0x00800000u) && af <= 0x7f800000u) {
            const double back = f32_to_f64(f);
            if (__double_as_longlong(back) != __double_as_longlong((double)f)) ++nb;
        }
    }
    if (nb) atomicAdd(bad, nb);
}

// rcp_nr(x) against the IEEE 1/x: the largest distance in units in the last
// place over the finite results, and the count of results that differ in
// class (finite / infinite / NaN) or sign.
__global__ void k_check_reciprocal(const double* x, long long n, unsigned long long* worst,
                                   unsigned long long* bad) {
    unsigned long long w = 0, nb = 0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const double v = x[q];
        const double ref = 1.0 / v, got = rcp_nr(v);
        const long long br = __double_as_longlong(ref), bg = __double_as_longlong(got);
        const bool fr = isfinite(ref), fg = isfinite(got);
        if (fr != fg || (!fr && !(isnan(ref) && isnan(got)) && br != bg) || (fr && ((br ^ bg) < 0))) {
            ++nb;
        } else if (fr) {
            const unsigned long long d = br > bg ? (unsigned long long)(br - bg) : (unsigned long long)(bg - br);
            if (d > w) w = d;
        }
    }
    if (nb) atomicAdd(bad, nb);
    if (w) atomicMax(worst, w);
}
}  // namespace wpf

extern "C" int wpf_check_reciprocal(const double* host_values, int64_t n, int64_t* max_ulp,
                                    int64_t* mismatches) {
    using namespace wpf;
    if (!host_values || n < 0 || !max_ulp || !mismatches) return WPF_ERR_ARG;
    *max_ulp = 0;
    *mismatches = 0;
    if (n == 0) return WPF_OK;
    double* d = nullptr;
    unsigned long long* acc = nullptr;
    if (cudaMalloc(&d, sizeof(double) * n) != cudaSuccess || cudaMalloc(&acc, 2 * sizeof(*acc)) != cudaSuccess) {
        cudaGetLastError();
        if (d) cudaFree(d);
        return WPF_ERR_NOMEM;
    }
    unsigned long long h[2] = {0, 0};
    int rc = WPF_OK;
    if (cudaMemcpy(d, host_values, sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(acc, 0, 2 * sizeof(*acc)) != cudaSuccess)
        rc = WPF_ERR_CUDA;
    if (!rc) {
        k_check_reciprocal<<<256, 256>>>(d, n, acc, acc + 1);
        if (cudaMemcpy(h, acc, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) rc = WPF_ERR_CUDA;
    }
    cudaFree(d);
    cudaFree(acc);
    *max_ulp = (int64_t)h[0];
    *mismatches = (int64_t)h[1];
    return rc;
}

// FP64 FMA throughput: eight independent chains per thread (a <- a b + c
// converges to c / (1 - b), so the values stay finite); every thread stores
// its sum so that no chain is dead code.
__global__ void __launch_bounds__(256) k_fp64_rate(double* out, int iters, double b, double c) {
    double a[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] = 1e-3 * threadIdx.x + q;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int q = 0; q < 8; ++q) a[q] = fma(a[q], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += a[q];
    out[(long long)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" int wpf_measure_fp64_rate(double* tflops) {
    using namespace wpf;
    if (!tflops) return WPF_ERR_ARG;
    *tflops = 0.0;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1) {
        cudaGetLastError();
        return WPF_ERR_CUDA;
    }
    const unsigned blocks = (unsigned)nsm * 8u;   // 2048 threads per SM
    const int iters = 4096;
    double* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks * 256) != cudaSuccess) {
        cudaGetLastError();
        return WPF_ERR_NOMEM;
    }
    int rc = WPF_OK;
    float ms = 0.f;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = WPF_ERR_CUDA;
    if (!rc) {
        k_fp64_rate<<<blocks, 256>>>(out, iters, 0.999999, 1e-6);   // untimed
        cudaEventRecord(e0);
        for (int r = 0; r < 3; ++r) k_fp64_rate<<<blocks, 256>>>(out, iters, 0.999999, 1e-6);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess ||
            !(ms > 0.f))
            rc = WPF_ERR_CUDA;
    }
    if (!rc) *tflops = 3.0 * 2.0 * 8.0 * iters * (double)blocks * 256.0 / (ms * 1e-3) / 1e12;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    cudaGetLastError();
    return rc;
}

extern "C" int wpf_check_conversions(const double* host_values, int64_t n, int64_t* mismatches) {
    using namespace wpf;
    if (!host_values || n < 0 || !mismatches) return WPF_ERR_ARG;
    *mismatches = 0;
    if (n == 0) return WPF_OK;
    double* d = nullptr;
    unsigned long long* bad = nullptr;
    if (cudaMalloc(&d, sizeof(double) * n) != cudaSuccess || cudaMalloc(&bad, sizeof(*bad)) != cudaSuccess) {
        cudaGetLastError();
        if (d) cudaFree(d);
        return WPF_ERR_NOMEM;
    }
    unsigned long long nb = 0;
    int rc = WPF_OK;
    if (cudaMemcpy(d, host_values, sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(bad, 0, sizeof(*bad)) != cudaSuccess)
        rc = WPF_ERR_CUDA;
    if (!rc) {
        k_check_conversions<<<256, 256>>>(d, n, bad);
        if (cudaMemcpy(&nb, bad, sizeof(nb), cudaMemcpyDeviceToHost) != cudaSuccess) rc = WPF_ERR_CUDA;
    }
    cudaFree(d);
    cudaFree(bad);
    *mismatches = (int64_t)nb;
    return rc;
}
