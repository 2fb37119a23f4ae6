// wpf_noalloc.cu -- showProgress diagnostics for callers that cannot allocate.
//
// wpf_reduce (the handle-based entry point) keeps its per-plane partial sums
// in device memory that wpf_create/wpf_reduce allocate.  Some callers cannot
// call cudaMalloc at all: code whose device memory is owned by another
// runtime's pool allocator (a solver framework or a machine learning
// framework's caching allocator, which must see every byte the process
// takes), and code on latency-critical paths where cudaMalloc's implicit
// device synchronisation is not acceptable.  They already hold the
// phase-field and concentration arrays on the device and only need the
// diagnostics of showProgress (wPFAW3D.f90:1695, 1756-1810) from them.
// wpf_reduce_noalloc serves them: its scratch is the fixed file-scope array
// below, reserved on every GPU that loads the library until the process
// exits, and the call allocates nothing.
#include <mutex>

#include "wpf_internal.cuh"

namespace {

// One partial record per z plane: compensated sums of (1-phase), (1+phase),
// the max r^2 of phase > 0 cells and the max/min of phase and concentration.
constexpr int NA_FIELDS = 9;          // s0, c0, s1, c1, r2max, pmax, pmin, cmax, cmin
constexpr int NA_RESULT = 8;
constexpr int NA_SCRATCH = WPF_NOALLOC_MAX_PLANES * NA_FIELDS + NA_RESULT;

// The scratch of every wpf_reduce_noalloc call on a device (360 KB at the
// 4096-plane limit).  Device code could name it directly; host code must use
// the device address obtained by cudaGetSymbolAddress (the symbol itself is
// only a host-side stand-in).  Calls that overlap on the GPU share it and race.
static __device__ __align__(256) double g_noalloc_scratch[NA_SCRATCH];

__device__ __forceinline__ void na_two_sum(double& s, double& c, double v) {
    const double t = s + v;
    const double bp = t - s;
    c += (s - (t - bp)) + (v - bp);
    s = t;
}

// One block per plane k of the reference layout (Fortran order with halo).
// Every record a call uses is written here before the final kernel reads it,
// so nothing in the scratch needs clearing between calls.
__global__ void k_noalloc_partial(int nx, int ny, int nz, double dx, int ix_ref, int iy_ref,
                                  int iz_ref, const double* __restrict__ ph,
                                  const double* __restrict__ cc, double* __restrict__ parts) {
    __shared__ double sm[32];
    const int k = blockIdx.x;
    const long long px = nx + 2, py = ny + 2;
    double s0 = 0, c0 = 0, s1 = 0, c1 = 0, r2max = 0;
    double pmax = -1.0e308, pmin = 1.0e308, cmax = -1.0e308, cmin = 1.0e308;
    const double xref = dx * (ix_ref - 1) + 0.5 * dx, yref = dx * (iy_ref - 1) + 0.5 * dx,
                 zref = dx * (iz_ref - 1) + 0.5 * dx;
    for (int j = threadIdx.y; j <= ny + 1; j += blockDim.y)
        for (int i = threadIdx.x; i <= nx + 1; i += blockDim.x) {
            const long long n = i + px * (j + py * k);
            const double f = ph[n], c = cc[n];
            pmax = fmax(pmax, f); pmin = fmin(pmin, f);
            cmax = fmax(cmax, c); cmin = fmin(cmin, c);
            if (i >= 1 && i <= nx && j >= 1 && j <= ny && k >= 1 && k <= nz) {
                na_two_sum(s0, c0, 1.0 - f);
                na_two_sum(s1, c1, 1.0 + f);
                if (f > 0.0) {
                    const double x = dx * (i - 1) + 0.5 * dx - xref, y = dx * (j - 1) + 0.5 * dx - yref,
                                 z = dx * (k - 1) + 0.5 * dx - zref;
                    r2max = fmax(r2max, x * x + y * y + z * z);
                }
            }
        }
    const double v[NA_FIELDS] = {wpf::block_sum(s0, sm), wpf::block_sum(c0, sm),
                                 wpf::block_sum(s1, sm), wpf::block_sum(c1, sm),
                                 wpf::block_max(r2max, sm, 0.0), wpf::block_max(pmax, sm, -1.0e308),
                                 wpf::block_min(pmin, sm, 1.0e308), wpf::block_max(cmax, sm, -1.0e308),
                                 wpf::block_min(cmin, sm, 1.0e308)};
    if (threadIdx.x == 0 && threadIdx.y == 0)
        for (int f = 0; f < NA_FIELDS; ++f) parts[(long long)k * NA_FIELDS + f] = v[f];
}

__global__ void k_noalloc_final(const double* __restrict__ parts, int nparts, double* out) {
    if (threadIdx.x != 0) return;
    double s0 = 0, c0 = 0, s1 = 0, c1 = 0, r2 = 0;
    double pmax = -1.0e308, pmin = 1.0e308, cmax = -1.0e308, cmin = 1.0e308;
    for (int q = 0; q < nparts; ++q) {
        const double* p = parts + (long long)q * NA_FIELDS;
        na_two_sum(s0, c0, p[0]); c0 += p[1];
        na_two_sum(s1, c1, p[2]); c1 += p[3];
        r2 = fmax(r2, p[4]);
        pmax = fmax(pmax, p[5]); pmin = fmin(pmin, p[6]);
        cmax = fmax(cmax, p[7]); cmin = fmin(cmin, p[8]);
    }
    out[0] = s0 + c0; out[1] = s1 + c1; out[2] = r2; out[3] = pmax;
    out[4] = pmin; out[5] = cmax; out[6] = cmin; out[7] = 0.0;
}

// Device address of g_noalloc_scratch, looked up on the first call made on a
// device (with that device current) and kept with the identity of the CUDA
// context it was looked up in: a device reset ends that context, the next
// call sees a new one and looks the address up again.
constexpr int NA_MAX_DEVICES = 64;
struct NaAddr {
    unsigned long long ctx_id;
    double* addr;
};
std::mutex g_na_mutex;
NaAddr g_na_addr[NA_MAX_DEVICES] = {};

// The current context's process-unique id (cuCtxGetId) through the runtime's
// driver entry points, so that the library links the runtime only.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);
bool current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_cur = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
        cudaGetLastError();
    });
    void* ctx = nullptr;
    return get_cur && get_id && get_cur(&ctx) == 0 && ctx && get_id(ctx, id) == 0;
}

int scratch_address(double** out) {
    int dev = 0;
    // cudaSetDevice makes the device's primary context current (creating it if
    // a reset ended the last one), so the context id below is the one the
    // kernels will run in
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES ||
        cudaSetDevice(dev) != cudaSuccess) {
        cudaGetLastError();
        return WPF_ERR_CUDA;
    }
    unsigned long long ctx = 0;
    const bool known = current_context_id(&ctx);
    std::lock_guard<std::mutex> lock(g_na_mutex);
    NaAddr& a = g_na_addr[dev];
    if (!known || !a.addr || a.ctx_id != ctx) {   // without a context id: look up every call
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return WPF_ERR_CUDA;
        }
        a.addr = static_cast<double*>(p);
        a.ctx_id = known ? ctx : 0;
    }
    *out = a.addr;
    return WPF_OK;
}

}  // namespace

extern "C" int wpf_reduce_noalloc(const wpf_params* p, const double* d_phase,
                                  const double* d_concent, wpf_diag* out, void* stream) {
    if (!p || !out) return WPF_ERR_ARG;
    if (p->nx < 1 || p->ny < 1 || p->nz < 1) return WPF_ERR_ARG;
    if ((long long)p->nz + 2 > WPF_NOALLOC_MAX_PLANES) return WPF_ERR_TOO_LARGE;
    if (!d_phase || !d_concent) return WPF_ERR_ARG;
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nparts = p->nz + 2;
    double* result = scratch + (long long)WPF_NOALLOC_MAX_PLANES * NA_FIELDS;
    k_noalloc_partial<<<nparts, dim3(32, 8), 0, s>>>(p->nx, p->ny, p->nz, p->dx, p->ix_ref,
                                                      p->iy_ref, p->iz_ref, d_phase, d_concent,
                                                      scratch);
    k_noalloc_final<<<1, 32, 0, s>>>(scratch, nparts, result);
    if (cudaGetLastError() != cudaSuccess) return WPF_ERR_CUDA;
    double r[NA_RESULT];
    if (cudaMemcpyAsync(r, result, sizeof(r), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return WPF_ERR_CUDA;
    }
    const double dx3 = p->dx * p->dx * p->dx;
    out->pv = dx3 * p->porosity * 0.5 * r[0];
    out->vcal = dx3 * (1.0 - p->porosity) * 0.5 * r[1];
    out->rwhmax = sqrt(r[2]);
    out->phase_max = r[3];
    out->phase_min = r[4];
    out->concent_max = r[5];
    out->concent_min = r[6];
    out->pressure_ref = 0.0;
    out->inlet_flux = 0.0;
    out->phase_max_outlet = NAN;   // not reduced here (like the two above)
    return WPF_OK;
}
