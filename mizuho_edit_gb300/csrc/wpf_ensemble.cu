// wpf_ensemble.cu -- advance an ensemble of independent domains together.
//
// No counterpart in the reference (one domain per run).  Every member is its
// own handle with its own stream, so members of different grid sizes share
// the GPU: a pool of host threads owns the members round-robin and steps each
// of its members in turn, so that while one member's host waits on a
// convergence read-back, the kernels of the others keep the device busy.
// Members never touch each other's memory, so no synchronisation is needed
// between threads beyond the final join.
#include <thread>
#include <vector>

#include "wpf_internal.cuh"

extern "C" int wpf_ensemble_run(wpf_handle** members, int32_t n, int32_t itime0, int32_t nsteps,
                                int32_t nthreads, double* dtime, wpf_step_stats* stats, int32_t* status) {
    if (!members || n < 1 || nsteps < 0 || !dtime) return WPF_ERR_ARG;
    for (int m = 0; m < n; ++m)
        if (!members[m]) return WPF_ERR_ARG;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > n) nthreads = n;
    std::vector<int> st(n, WPF_OK);
    int dev = 0;
    cudaGetDevice(&dev);
    auto work = [&](int t) {
        cudaSetDevice(dev);   // host threads start on device 0; follow the caller
        for (int s = 0; s < nsteps; ++s)
            for (int m = t; m < n; m += nthreads) {
                if (st[m] != WPF_OK && st[m] != WPF_ERR_NOT_CONVERGED) continue;
                wpf_step_stats tmp;
                const int rc = wpf_step(members[m], itime0 + s, &dtime[m], stats ? &stats[m] : &tmp);
                if (rc) st[m] = rc;
            }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) pool.emplace_back(work, t);
    for (auto& th : pool) th.join();
    int worst = WPF_OK;
    for (int m = 0; m < n; ++m) {
        if (status) status[m] = st[m];
        if (st[m] != WPF_OK && (worst == WPF_OK || worst == WPF_ERR_NOT_CONVERGED)) worst = st[m];
    }
    return worst;
}
