// wpf_ensemble.cu -- advance an ensemble of independent domains together.
//
// No counterpart in the reference (one domain per run).  Every member is its
// own handle with its own buffers, so members of different grid sizes share
// the GPU.  Two forms of a step:
//   - every member can take the device-resident step (WPF_SOLVER_STEP_GRAPH):
//     one graph holds all members' step graphs as independent branches (each
//     with its own conditional solver loops), launched once and synchronised
//     once; the graphs are cached per (members, buffer assignment);
//   - otherwise (the first steps, a member that fell back): a pool of host
//     threads owns the members round-robin and runs wpf_step on each, so that
//     while one member's host waits on a read-back the kernels of the others
//     keep the device busy.
// Members never touch each other's memory, so no synchronisation is needed
// between them beyond the step's join.
#include <mutex>
#include <thread>
#include <vector>

#include "wpf_internal.cuh"

namespace wpf {
namespace {

struct EnsGraph {
    std::vector<unsigned long long> uid, epoch;
    std::vector<const void*> keys;   // STEP_KEY entries per member
    std::vector<StepCounts> n;
    cudaGraphExec_t exec = nullptr;
    unsigned long long last_use = 0;
};

std::mutex ens_mu;
std::vector<EnsGraph*> ens_cache;
unsigned long long ens_clock = 0;
constexpr size_t ENS_MAX = 8;

void ens_free(EnsGraph* e) {
    if (e->exec) cudaGraphExecDestroy(e->exec);
    delete e;
}

// One step of every listed member as one graph launch on the first member's stream.
int ensemble_graph_step(const std::vector<wpf_handle*>& mem, const std::vector<int>& idx, double* dtime,
                        wpf_step_stats* stats, std::vector<int>& st) {
    const int n = (int)mem.size();
    for (int m = 0; m < n; ++m) {
        const int rc = step_graph_prepare(mem[m]);
        if (rc) return rc;
    }
    std::vector<unsigned long long> uid(n), epoch(n);
    std::vector<const void*> keys((size_t)STEP_KEY * n);
    for (int m = 0; m < n; ++m) {
        uid[m] = mem[m]->uid;
        epoch[m] = mem[m]->epoch;
        step_graph_key(mem[m], &keys[(size_t)STEP_KEY * m]);
    }
    std::lock_guard<std::mutex> lk(ens_mu);
    EnsGraph* e = nullptr;
    for (EnsGraph* c : ens_cache)
        if (c->uid == uid && c->epoch == epoch && c->keys == keys) e = c;
    if (!e) {
        if (ens_cache.size() >= ENS_MAX) {   // drop the least recently used
            size_t lru = 0;
            for (size_t q = 1; q < ens_cache.size(); ++q)
                if (ens_cache[q]->last_use < ens_cache[lru]->last_use) lru = q;
            ens_free(ens_cache[lru]);
            ens_cache.erase(ens_cache.begin() + (long)lru);
        }
        e = new EnsGraph;
        e->uid = uid;
        e->epoch = epoch;
        e->keys = keys;
        e->n.resize(n);
        GraphBuilder top;
        if (cudaGraphCreate(&top.graph, 0) != cudaSuccess) {
            delete e;
            return WPF_ERR_CUDA;
        }
        int rc = WPF_OK;
        for (int m = 0; m < n && !rc; ++m) {
            GraphBuilder b;
            b.graph = top.graph;
            b.top = top.graph;
            b.s = mem[m]->stream;
            const long long saved = mem[m]->nlaunch;
            rc = step_graph_capture(mem[m], b, &e->n[m]);
            mem[m]->nlaunch = saved;
            if (rc || b.capturing) abandon_capture(mem[m]->stream);
        }
        if (!rc && cudaGraphInstantiate(&e->exec, top.graph, 0) != cudaSuccess) {
            cudaGetLastError();
            e->exec = nullptr;
            rc = WPF_ERR_CUDA;
        }
        cudaGraphDestroy(top.graph);
        if (rc) {
            ens_free(e);
            return rc;
        }
        ens_cache.push_back(e);
    }
    e->last_use = ++ens_clock;
    cudaStream_t ls = mem[0]->stream;
    for (int m = 0; m < n; ++m) {
        if (!mem[m]->gctl_dirty) continue;
        const int rc = step_graph_sync_ctl(mem[m]);   // on the member's stream
        if (rc) return rc;
        WPF_CUDA(cudaStreamSynchronize(mem[m]->stream));
    }
    WPF_CUDA(cudaGraphLaunch(e->exec, ls));
    WPF_CUDA(cudaStreamSynchronize(ls));
    for (int m = 0; m < n; ++m) {
        wpf_step_stats tmp;
        const int q = idx[m];
        const int rc = step_graph_finish(mem[m], e->n[m], stats ? &stats[q] : &tmp, &dtime[q]);
        if (rc) st[q] = rc;
    }
    return WPF_OK;
}

}  // namespace

void ensemble_graphs_forget(const wpf_handle* h) {
    std::lock_guard<std::mutex> lk(ens_mu);
    for (size_t q = 0; q < ens_cache.size();) {
        bool has = false;
        for (unsigned long long u : ens_cache[q]->uid) has = has || u == h->uid;
        if (has) {
            ens_free(ens_cache[q]);
            ens_cache.erase(ens_cache.begin() + (long)q);
        } else {
            ++q;
        }
    }
}

}  // namespace wpf

extern "C" int wpf_ensemble_run(wpf_handle** members, int32_t n, int32_t itime0, int32_t nsteps,
                                int32_t nthreads, double* dtime, wpf_step_stats* stats, int32_t* status) {
    using namespace wpf;
    if (!members || n < 1 || nsteps < 0 || !dtime) return WPF_ERR_ARG;
    for (int m = 0; m < n; ++m)
        if (!members[m]) return WPF_ERR_ARG;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > n) nthreads = n;
    std::vector<int> st(n, WPF_OK);
    int dev = 0;
    cudaGetDevice(&dev);
    for (int m = 0; m < n; ++m)   // a graph launch on one member's stream must not overtake the others
        if (cudaStreamSynchronize(members[m]->stream) != cudaSuccess) return WPF_ERR_CUDA;
    auto alive = [&](int m) { return st[m] == WPF_OK || st[m] == WPF_ERR_NOT_CONVERGED; };
    int hard = WPF_OK;
    for (int s = 0; s < nsteps && !hard; ++s) {
        const int itime = itime0 + s;
        std::vector<wpf_handle*> mem;
        std::vector<int> idx;
        bool all = true;
        for (int m = 0; m < n; ++m) {
            if (!alive(m)) continue;
            mem.push_back(members[m]);
            idx.push_back(m);
            all = all && step_graph_ready(members[m], itime);
        }
        if (mem.empty()) break;
        if (all) {
            hard = ensemble_graph_step(mem, idx, dtime, stats, st);
            continue;
        }
        auto work = [&](int t) {
            cudaSetDevice(dev);   // host threads start on device 0; follow the caller
            for (int m = t; m < n; m += nthreads) {
                if (!alive(m)) continue;
                wpf_step_stats tmp;
                const int rc = wpf_step(members[m], itime, &dtime[m], stats ? &stats[m] : &tmp);
                if (rc) st[m] = rc;
            }
        };
        std::vector<std::thread> pool;
        for (int t = 0; t < nthreads; ++t) pool.emplace_back(work, t);
        for (auto& th : pool) th.join();
    }
    int worst = WPF_OK;
    for (int m = 0; m < n; ++m) {
        if (status) status[m] = st[m];
        if (st[m] != WPF_OK && (worst == WPF_OK || worst == WPF_ERR_NOT_CONVERGED)) worst = st[m];
    }
    return hard ? hard : worst;
}
