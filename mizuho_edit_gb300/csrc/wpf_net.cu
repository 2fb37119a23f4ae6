// wpf_net.cu -- the learned warm start: a small 3-D U-Net on tcgen05 tensor
// cores (sm_103a), trained and run on the GPU by these kernels only.
//
// No counterpart in the reference (wPFAW3D.f90:980 starts every solve from the
// previous pressure).  Layout: activations bf16 NDHWC (channel innermost, then
// x, y, z); weights bf16 [Cout][27][Cin], tap t = (dz+1)*9 + (dy+1)*3 + (dx+1);
// FP32 master weights, gradients and Adam moments.
//
// Convolution = implicit GEMM on tcgen05: one CTA of 128 threads owns 128
// output voxels (M = 128, one TMEM lane each) and all Cout channels (N =
// Cout); the K loop runs over the 27 taps, each tap one stage of K = Cin
// (Cin/16 MMAs of K = 16).  Threads gather the A rows (the Cin channels of the
// shifted voxel: Cin/8 16-byte chunks) and the B rows (weights of the tap)
// into shared memory in the no-swizzle K-major core-matrix layout (8 rows x
// 16 bytes per core matrix; LBO = byte stride between core matrices along K,
// SBO = along M/N), two stages in flight: thread 0 issues the MMAs of a stage
// and commits them to the stage's mbarrier, which the gatherers wait on
// before refilling that buffer.  The FP32 accumulator lives in TMEM and is
// read back with tcgen05.ld for the epilogue (bias, ReLU, bf16 store).
// Weight gradient = the same machinery with M = (tap, Cin) rows, N = Cout and
// K = voxels (split over CTAs, FP32 atomics into the gradient).  Data
// gradient = the forward kernel with the flipped, transposed weights.
#include <cuda_bf16.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <random>
#include <vector>

#include "wpf_internal.cuh"
#include "../../include/wpf_net.h"

namespace wpf {
namespace net {

typedef uint16_t bf16_t;
constexpr int CT = 128;                        // threads per CTA = MMA rows
constexpr long long WAIT_LIMIT = 1LL << 24;    // bounded mbarrier waits

__device__ __forceinline__ float bf2f(bf16_t v) { return __uint_as_float((uint32_t)v << 16); }
__device__ __forceinline__ bf16_t f2bf(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }
__device__ __forceinline__ uint32_t pack2(float a, float b) {
    return (uint32_t)f2bf(a) | ((uint32_t)f2bf(b) << 16);
}

// ---- PTX wrappers -------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// Wait for the completion of the barrier phase with the given parity; false
// when the bounded wait runs out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (long long it = 0; it < WAIT_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// whole warp: allocate ncols TMEM columns, address written to *dst
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// D (tmem) (+)= A (smem desc) * B (smem desc)^T, bf16 inputs, f32 accumulate
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}
// 16 consecutive FP32 columns of the warp's 32 TMEM lanes (one row per thread)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15},"
        " [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
// Shared-memory matrix descriptor, no swizzle (layout type 0), version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: D f32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Shared memory of a conv CTA: two stages of A (128 rows) and B (COUT rows),
// plus 1 KB so that every descriptor-addressed read stays inside the
// allocation.  Sized per shape: the 16-channel layers take 10 KB, so many
// CTAs share an SM and hide each other's gather latency.
constexpr int CONV_SMEM_MAX = 96 * 1024;
template <int CIN, int COUT>
constexpr int conv_smem() { return 2 * (CIN * 256 + COUT * CIN * 2) + 1024; }
constexpr int WG_STAGE_ = 32;
template <int CIN, int COUT>
constexpr int wgrad_smem() { return 2 * (128 * WG_STAGE_ * 2 + COUT * WG_STAGE_ * 2) + 1024; }

struct ConvArgs {
    int nx, ny, nz, nvox;
    const bf16_t* in;
    const bf16_t* w;
    const float* bias;
    bf16_t* out16;
    float* out32;
    int relu;
    int* err;
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(CT) k_conv3d(ConvArgs a) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmem_sh;
    constexpr int AB = CIN * 256;        // 128 rows x CIN bf16
    constexpr int BB = COUT * CIN * 2;   // COUT rows x CIN bf16
    constexpr int SB = AB + BB;
    static_assert(2 * SB + 1024 == conv_smem<CIN, COUT>() && conv_smem<CIN, COUT>() <= CONV_SMEM_MAX,
                  "conv stages exceed the shared allocation");
    constexpr uint32_t NCOL = COUT < 32 ? 32 : COUT;
    constexpr uint32_t IDESC = idesc_bf16(128, COUT);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tmem_alloc(&tmem_sh, NCOL);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = tmem_sh;
    const uint32_t sbase = smem_u32(sm);

    const long long v = (long long)blockIdx.x * CT + tid;   // output voxel of row m = tid
    const bool vok = v < a.nvox;
    int x = 0, y = 0, z = 0;
    if (vok) {
        x = (int)(v % a.nx);
        const long long r = v / a.nx;
        y = (int)(r % a.ny);
        z = (int)(r / a.ny);
    }
    bool ok = true;
    for (int t = 0; t < 27; ++t) {
        const int buf = t & 1;
        if (t >= 2 && !mbar_wait(&bar[buf], ((t - 2) >> 1) & 1)) ok = false;
        unsigned char* A = sm + buf * SB;
        unsigned char* B = A + AB;
        const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
        const int xs = x + dx, ys = y + dy, zs = z + dz;
        const bool inb = vok && xs >= 0 && xs < a.nx && ys >= 0 && ys < a.ny && zs >= 0 && zs < a.nz;
        const uint4* src =
            reinterpret_cast<const uint4*>(a.in + (((long long)zs * a.ny + ys) * a.nx + xs) * CIN);
#pragma unroll
        for (int c = 0; c < CIN / 8; ++c) {
            const uint4 q = inb ? src[c] : make_uint4(0u, 0u, 0u, 0u);
            *reinterpret_cast<uint4*>(A + c * 2048 + (tid >> 3) * 128 + (tid & 7) * 16) = q;
        }
        for (int q = tid; q < COUT * CIN / 8; q += CT) {
            const int co = q / (CIN / 8), c = q - co * (CIN / 8);
            const uint4 val = reinterpret_cast<const uint4*>(a.w + ((long long)co * 27 + t) * CIN)[c];
            *reinterpret_cast<uint4*>(B + c * (COUT * 16) + (co >> 3) * 128 + (co & 7) * 16) = val;
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_after();
#pragma unroll
            for (int kk = 0; kk < CIN / 16; ++kk) {
                const uint64_t ad = sdesc(sbase + buf * SB + 2 * kk * 2048, 2048, 128);
                const uint64_t bd = sdesc(sbase + buf * SB + AB + 2 * kk * (COUT * 16), COUT * 16, 128);
                mma_bf16(tmem, ad, bd, IDESC, (t > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(&bar[buf]);
        }
    }
    // the last commit (tap 26: buffer 0, its 14th phase) covers every MMA
    if (!mbar_wait(&bar[0], 1)) ok = false;
    tc_after();
#pragma unroll
    for (int c0 = 0; c0 < COUT; c0 += 16) {
        float acc[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, acc);
        if (vok && ok) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                float s = acc[i] + (a.bias ? a.bias[c0 + i] : 0.f);
                if (a.relu) s = fmaxf(s, 0.f);
                acc[i] = s;
            }
            if (a.out16) {
                uint4* dst = reinterpret_cast<uint4*>(a.out16 + v * COUT + c0);
                dst[0] = make_uint4(pack2(acc[0], acc[1]), pack2(acc[2], acc[3]), pack2(acc[4], acc[5]),
                                    pack2(acc[6], acc[7]));
                dst[1] = make_uint4(pack2(acc[8], acc[9]), pack2(acc[10], acc[11]), pack2(acc[12], acc[13]),
                                    pack2(acc[14], acc[15]));
            } else {
                float4* dst = reinterpret_cast<float4*>(a.out32 + v * COUT + c0);
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    dst[i] = make_float4(acc[4 * i], acc[4 * i + 1], acc[4 * i + 2], acc[4 * i + 3]);
            }
        }
    }
    if (!ok) {   // a wait ran out: give the MMAs in flight a second bounded wait
        mbar_wait(&bar[0], 1);
        if (tid == 0) atomicExch(a.err, 1);
    }
    tc_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, NCOL);
}

// ---- row-tiled convolution of 16-channel inputs, staged by TMA ----------------
// For a level whose nx is a multiple of TX (128, 64, 32 or 16) and whose ny
// is a multiple of TY = 128 / TX, a CTA owns the TX x TY x 1 brick of output
// voxels (x0.., y0.., z0): M = 128 rows in x-fastest order, N = COUT.  Its
// input halo -- 3 z planes x (TY + 2) rows x the brick's x range, both
// 8-channel halves -- is staged once by bulk-tensor copies that fill zeros
// outside the grid (the convolution's zero padding), each half in its own
// "chunk plane" so that 8 consecutive x voxels form one 128-byte core matrix
// of the no-swizzle K-major layout.  Every tap's A operand is then a window
// of that plane: the descriptor's start moves by (dz, dy) rows and, with TY = 1
// (one 130-voxel row), by dx voxels; with TY > 1 the rows of the window must
// be TX apart, so three copies shifted by dx = -1, 0, 1 are staged instead.
// All 27 taps' weights sit in shared memory as B operands; one thread issues
// the 27 MMAs (K = 16 each) back to back and commits them to an mbarrier.
// No per-tap gather and no per-tap block barrier: the 16-channel layers (the
// finest level of the U-Net) were latency-bound on exactly those.
template <int COUT, int TX>
struct RowTile {
    static constexpr int TY = 128 / TX;
    static constexpr bool SHIFT = TY > 1;
    static constexpr int BOXX = SHIFT ? TX : TX + 2;       // x extent of one staged box
    static constexpr int NSH = SHIFT ? 3 : 1;              // staged dx copies
    static constexpr int ROWS = 3 * (TY + 2);               // (z, y) rows of a box
    static constexpr int CH = ROWS * BOXX * 16;             // bytes of one box (8 channels)
    static constexpr int CHP = (CH + 127) / 128 * 128;      // its slot (128-byte aligned)
    static constexpr int ABYTES = NSH * 2 * CHP;
    static constexpr int BBYTES = 27 * 2 * COUT * 16;
    static constexpr int SMEM = ABYTES + BBYTES + 1024;
    static_assert(TX % 8 == 0 && TX * TY == 128, "a brick is 128 voxels, whole core matrices in x");
    static_assert(SMEM <= 200 * 1024, "row conv stage exceeds the shared allocation");
};

struct RowConvArgs {
    int nx, ny, nz;
    const bf16_t* w;
    const float* bias;
    bf16_t* out16;
    float* out32;
    int relu;
    int* err;
};

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

template <int COUT, int TX>
__global__ void __launch_bounds__(CT) k_conv3d_row(RowConvArgs a, const __grid_constant__ CUtensorMap in_map) {
    using T = RowTile<COUT, TX>;
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t bar[2];   // 0: the input halo landed; 1: the MMAs finished
    __shared__ uint32_t tmem_sh;
    constexpr uint32_t NCOL = 32;
    constexpr uint32_t IDESC = idesc_bf16(128, COUT);
    static_assert(COUT == 16 || COUT == 32, "row conv: N = 16 or 32");
    const int tid = threadIdx.x, warp = tid >> 5;
    const int ntx = a.nx / TX, nty = a.ny / T::TY;
    const int bx = blockIdx.x % ntx, by = (blockIdx.x / ntx) % nty, bz = blockIdx.x / (ntx * nty);
    const int x0 = bx * TX, y0 = by * T::TY, z0 = bz;
    unsigned char* Bs = sm + T::ABYTES;
    if (warp == 0) tmem_alloc(&tmem_sh, NCOL);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (tid == 0) {
        mbar_expect_tx(&bar[0], (uint32_t)(T::NSH * 2 * T::CH));
        for (int sh = 0; sh < T::NSH; ++sh)
            for (int c = 0; c < 2; ++c)
                tma_load_4d(sm + (sh * 2 + c) * T::CHP, &in_map, 8 * c, T::SHIFT ? x0 + sh - 1 : x0 - 1, y0 - 1,
                            z0 - 1, &bar[0]);
    }
    // the 27 taps' weights as B operands: tap t, channel half c, row co
    for (int q = tid; q < 27 * 2 * COUT; q += CT) {
        const int t = q / (2 * COUT), r = q - t * (2 * COUT), c = r / COUT, co = r - c * COUT;
        const uint4 val = reinterpret_cast<const uint4*>(a.w + ((long long)co * 27 + t) * 16)[c];
        *reinterpret_cast<uint4*>(Bs + t * (2 * COUT * 16) + c * (COUT * 16) + (co >> 3) * 128 + (co & 7) * 16) =
            val;
    }
    fence_async_smem();
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = tmem_sh;
    const uint32_t sbase = smem_u32(sm);
    bool ok = true;
    if (tid == 0) {
        if (!mbar_wait(&bar[0], 0)) ok = false;
        tc_after();
        if (ok) {
            for (int t = 0; t < 27; ++t) {
                const int dz = t / 9, dy = (t / 3) % 3, dx = t % 3;   // 0..2 (offset + 1)
                const uint32_t arow = (uint32_t)((dz * (T::TY + 2) + dy) * T::BOXX * 16);
                const uint32_t aoff = T::SHIFT ? (uint32_t)(dx * 2 * T::CHP) + arow : arow + (uint32_t)(dx * 16);
                const uint64_t ad = sdesc(sbase + aoff, T::CHP, 128);
                const uint64_t bd = sdesc(sbase + T::ABYTES + t * (2 * COUT * 16), COUT * 16, 128);
                mma_bf16(tmem, ad, bd, IDESC, t > 0 ? 1u : 0u);
            }
        }
        mma_commit(&bar[1]);   // arrives when every MMA issued above has finished (or at once)
    }
    __syncwarp();
    if (!mbar_wait(&bar[1], 0)) ok = false;
    tc_after();
    const int x = x0 + tid % TX, y = y0 + tid / TX;
    const long long v = ((long long)z0 * a.ny + y) * a.nx + x;
#pragma unroll
    for (int c0 = 0; c0 < COUT; c0 += 16) {
        float acc[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, acc);
        if (ok) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                float s = acc[i] + (a.bias ? a.bias[c0 + i] : 0.f);
                if (a.relu) s = fmaxf(s, 0.f);
                acc[i] = s;
            }
            if (a.out16) {
                uint4* dst = reinterpret_cast<uint4*>(a.out16 + v * COUT + c0);
                dst[0] = make_uint4(pack2(acc[0], acc[1]), pack2(acc[2], acc[3]), pack2(acc[4], acc[5]),
                                    pack2(acc[6], acc[7]));
                dst[1] = make_uint4(pack2(acc[8], acc[9]), pack2(acc[10], acc[11]), pack2(acc[12], acc[13]),
                                    pack2(acc[14], acc[15]));
            } else {
                float4* dst = reinterpret_cast<float4*>(a.out32 + v * COUT + c0);
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    dst[i] = make_float4(acc[4 * i], acc[4 * i + 1], acc[4 * i + 2], acc[4 * i + 3]);
            }
        }
    }
    if (!ok) {   // a wait ran out: the copies and MMAs in flight get a second bounded wait
        mbar_wait(&bar[0], 0);
        mbar_wait(&bar[1], 0);
        atomicExch(a.err, 1);
    }
    tc_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, NCOL);
}

// Weight gradient: D[r][co] = sum_v x[v + d_t][ci] gy[v][co], r = t*CIN + ci.
// CTA (blockIdx.x = 128-row tile of r, blockIdx.y = chunk of WG_VOX voxels);
// stages of 32 voxels (two MMAs of K = 16), FP32 atomics into gw.
constexpr int WG_VOX = 2048;
constexpr int WG_STAGE = WG_STAGE_;

struct WgradArgs {
    int nx, ny, nz, nvox;
    const bf16_t* x;
    const bf16_t* gy;
    float* gw;
    int* err;
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(CT) k_conv3d_wgrad(WgradArgs a) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmem_sh;
    constexpr int AB = 128 * WG_STAGE * 2;    // 128 rows x 32 voxels bf16
    constexpr int BB = COUT * WG_STAGE * 2;
    constexpr int SB = AB + BB;
    static_assert(2 * SB + 1024 == wgrad_smem<CIN, COUT>() && wgrad_smem<CIN, COUT>() <= CONV_SMEM_MAX,
                  "wgrad stages exceed the shared allocation");
    constexpr uint32_t NCOL = COUT < 32 ? 32 : COUT;
    constexpr uint32_t IDESC = idesc_bf16(128, COUT);
    constexpr int R = 27 * CIN;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tmem_alloc(&tmem_sh, NCOL);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = tmem_sh;
    const uint32_t sbase = smem_u32(sm);
    const int r = blockIdx.x * CT + tid;
    const bool rok = r < R;
    const int t = rok ? r / CIN : 0, ci = rok ? r - (r / CIN) * CIN : 0;
    const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
    const long long v_begin = (long long)blockIdx.y * WG_VOX;
    const long long v_end = min((long long)a.nvox, v_begin + WG_VOX);
    const int nstage = (int)((v_end - v_begin + WG_STAGE - 1) / WG_STAGE);
    bool ok = true;
    for (int s = 0; s < nstage; ++s) {
        const int buf = s & 1;
        if (s >= 2 && !mbar_wait(&bar[buf], ((s - 2) >> 1) & 1)) ok = false;
        unsigned char* A = sm + buf * SB;
        unsigned char* B = A + AB;
        const long long v0 = v_begin + (long long)s * WG_STAGE;
        // A row r: x[v + d_t][ci] for the stage's 32 voxels (8 per core-matrix row)
        int vx = (int)(v0 % a.nx);
        long long rr = v0 / a.nx;
        int vy = (int)(rr % a.ny), vz = (int)(rr / a.ny);
#pragma unroll
        for (int c = 0; c < WG_STAGE / 8; ++c) {
            uint32_t w4[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                float pair[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const long long vv = v0 + c * 8 + h * 2 + e;
                    float val = 0.f;
                    const int xs = vx + dx, ys = vy + dy, zs = vz + dz;
                    if (rok && vv < v_end && xs >= 0 && xs < a.nx && ys >= 0 && ys < a.ny && zs >= 0 &&
                        zs < a.nz)
                        val = bf2f(a.x[(((long long)zs * a.ny + ys) * a.nx + xs) * CIN + ci]);
                    pair[e] = val;
                    if (++vx == a.nx) {
                        vx = 0;
                        if (++vy == a.ny) { vy = 0; ++vz; }
                    }
                }
                w4[h] = pack2(pair[0], pair[1]);
            }
            *reinterpret_cast<uint4*>(A + c * 2048 + (tid >> 3) * 128 + (tid & 7) * 16) =
                make_uint4(w4[0], w4[1], w4[2], w4[3]);
        }
        // B row co: gy[v][co] for the same voxels
        for (int q = tid; q < COUT * (WG_STAGE / 8); q += CT) {
            const int co = q % COUT, c = q / COUT;
            uint32_t w4[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const long long va = v0 + c * 8 + h * 2;
                const float g0 = va < v_end ? bf2f(a.gy[va * COUT + co]) : 0.f;
                const float g1 = va + 1 < v_end ? bf2f(a.gy[(va + 1) * COUT + co]) : 0.f;
                w4[h] = pack2(g0, g1);
            }
            *reinterpret_cast<uint4*>(B + c * (COUT * 16) + (co >> 3) * 128 + (co & 7) * 16) =
                make_uint4(w4[0], w4[1], w4[2], w4[3]);
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_after();
#pragma unroll
            for (int kk = 0; kk < WG_STAGE / 16; ++kk) {
                const uint64_t ad = sdesc(sbase + buf * SB + 2 * kk * 2048, 2048, 128);
                const uint64_t bd = sdesc(sbase + buf * SB + AB + 2 * kk * (COUT * 16), COUT * 16, 128);
                mma_bf16(tmem, ad, bd, IDESC, (s > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(&bar[buf]);
        }
    }
    const int last = nstage - 1;
    if (nstage > 0 && !mbar_wait(&bar[last & 1], (last >> 1) & 1)) ok = false;
    tc_after();
    if (nstage > 0) {
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            float acc[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, acc);
            if (rok && ok) {
#pragma unroll
                for (int i = 0; i < 16; ++i) atomicAdd(&a.gw[(long long)(c0 + i) * R + r], acc[i]);
            }
        }
    }
    if (!ok) {
        if (nstage > 0) mbar_wait(&bar[last & 1], (last >> 1) & 1);
        if (tid == 0) atomicExch(a.err, 1);
    }
    tc_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, NCOL);
}

// gb[co] += sum_v gy[v][co]
__global__ void k_bias_grad(const bf16_t* __restrict__ gy, int nvox, int cout, float* gb) {
    __shared__ float s[64];
    if (threadIdx.x < 64) s[threadIdx.x] = 0.f;
    __syncthreads();
    const int co = threadIdx.x % cout;
    const int lanes = blockDim.x / cout;
    float acc = 0.f;
    for (long long v = (long long)blockIdx.x * lanes + threadIdx.x / cout; v < nvox;
         v += (long long)gridDim.x * lanes)
        acc += bf2f(gy[v * cout + co]);
    atomicAdd(&s[co], acc);
    __syncthreads();
    if (threadIdx.x < cout) atomicAdd(&gb[threadIdx.x], s[threadIdx.x]);
}

// ---- elementwise pieces of the U-Net ----------------------------------------------
// out = 2x2x2 mean of in (dims of in: nx, ny, nz, even)
// One thread per (coarse voxel, 8-channel chunk): 16-byte loads and stores.
// Per channel the same sum in the same order as the element-wise form.
__device__ __forceinline__ void unpack8(const uint4 q, float* f) {
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        f[2 * i] = bf2f((bf16_t)(w[i] & 0xFFFFu));
        f[2 * i + 1] = bf2f((bf16_t)(w[i] >> 16));
    }
}

__global__ void k_pool2(const bf16_t* __restrict__ in, bf16_t* __restrict__ out, int nx, int ny, int nz,
                        int C) {
    const int hx = nx / 2, hy = ny / 2, hz = nz / 2, C8 = C / 8;
    const long long n = (long long)hx * hy * hz * C8;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(q % C8);
        long long V = q / C8;
        const int X = (int)(V % hx);
        V /= hx;
        const int Y = (int)(V % hy), Z = (int)(V / hy);
        float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int k = 0; k < 2; ++k)
            for (int j = 0; j < 2; ++j)
                for (int i = 0; i < 2; ++i) {
                    const uint4 v = reinterpret_cast<const uint4*>(
                        in + ((((long long)(2 * Z + k) * ny + 2 * Y + j) * nx) + 2 * X + i) * C)[c8];
                    float f[8];
                    unpack8(v, f);
#pragma unroll
                    for (int e = 0; e < 8; ++e) s[e] += f[e];
                }
        reinterpret_cast<uint4*>(out)[q] =
            make_uint4(pack2(0.125f * s[0], 0.125f * s[1]), pack2(0.125f * s[2], 0.125f * s[3]),
                       pack2(0.125f * s[4], 0.125f * s[5]), pack2(0.125f * s[6], 0.125f * s[7]));
    }
}

// out = up2(low) + skip (dims of out / skip: nx, ny, nz); per (voxel, chunk)
__global__ void k_up2_add(const bf16_t* __restrict__ low, const bf16_t* __restrict__ skip,
                          bf16_t* __restrict__ out, int nx, int ny, int nz, int C) {
    const int C8 = C / 8;
    const long long n = (long long)nx * ny * nz * C8;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(q % C8);
        long long v = q / C8;
        const int x = (int)(v % nx);
        v /= nx;
        const int y = (int)(v % ny), z = (int)(v / ny);
        const long long P = (((long long)(z / 2) * (ny / 2) + y / 2) * (nx / 2) + x / 2) * C8 + c8;
        float a[8], b[8];
        unpack8(reinterpret_cast<const uint4*>(low)[P], a);
        unpack8(reinterpret_cast<const uint4*>(skip)[q], b);
        reinterpret_cast<uint4*>(out)[q] = make_uint4(pack2(a[0] + b[0], a[1] + b[1]), pack2(a[2] + b[2], a[3] + b[3]),
                                                      pack2(a[4] + b[4], a[5] + b[5]), pack2(a[6] + b[6], a[7] + b[7]));
    }
}

// g_low[V][c] = (sum over the 8 children of g[v][c]) * (y_low[V][c] > 0)
// (backward of s = up2(a) + skip, a = relu(.), w.r.t. the pre-activation of a)
__global__ void k_bwd_up_relu(const bf16_t* __restrict__ g, const bf16_t* __restrict__ ylow,
                              bf16_t* __restrict__ out, int nx, int ny, int nz, int C) {
    const int hx = nx / 2, hy = ny / 2, hz = nz / 2;
    const long long n = (long long)hx * hy * hz * C;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(q % C);
        long long V = q / C;
        const int X = (int)(V % hx);
        V /= hx;
        const int Y = (int)(V % hy), Z = (int)(V / hy);
        float s = 0.f;
        for (int k = 0; k < 2; ++k)
            for (int j = 0; j < 2; ++j)
                for (int i = 0; i < 2; ++i)
                    s += bf2f(g[((((long long)(2 * Z + k) * ny + 2 * Y + j) * nx) + 2 * X + i) * C + c]);
        out[q] = bf2f(ylow[q]) > 0.f ? f2bf(s) : (bf16_t)0;
    }
}

// g_pre[v][c] = (g_pool[parent][c] / 8 + g_skip[v][c]) * (y[v][c] > 0)   (dims of y: nx, ny, nz)
__global__ void k_bwd_pool_skip_relu(const bf16_t* __restrict__ gpool, const bf16_t* __restrict__ gskip,
                                     const bf16_t* __restrict__ y, bf16_t* __restrict__ out, int nx,
                                     int ny, int nz, int C) {
    const long long n = (long long)nx * ny * nz * C;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(q % C);
        long long v = q / C;
        const int x = (int)(v % nx);
        v /= nx;
        const int yy = (int)(v % ny), z = (int)(v / ny);
        const long long P = (((long long)(z / 2) * (ny / 2) + yy / 2) * (nx / 2) + x / 2) * C + c;
        const float s = 0.125f * bf2f(gpool[P]) + (gskip ? bf2f(gskip[q]) : 0.f);
        out[q] = bf2f(y[q]) > 0.f ? f2bf(s) : (bf16_t)0;
    }
}

// Masked mean-square loss on channel 0 of the FP32 output: sums
// acc[0] += sum mask (o - t)^2, acc[1] += sum mask (a first pass).
__global__ void k_loss_sums(const float* __restrict__ out, int cstride, const float* __restrict__ tgt,
                            const float* __restrict__ mask, int nvox, double* acc) {
    double s = 0.0, m = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox;
         v += (long long)gridDim.x * blockDim.x) {
        const float w = mask ? mask[v] : 1.f;
        const float d = out[v * cstride] - tgt[v];
        s += (double)w * d * d;
        m += w;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        m += __shfl_down_sync(0xffffffffu, m, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], s);
        atomicAdd(&acc[1], m);
    }
}
// g[v][0] = 2 mask (o - t) / sum(mask), g[v][1..C) = 0   (bf16)
__global__ void k_loss_grad(const float* __restrict__ out, int C, const float* __restrict__ tgt,
                            const float* __restrict__ mask, int nvox, const double* acc,
                            bf16_t* __restrict__ g) {
    const float inv = acc[1] > 0.0 ? (float)(1.0 / acc[1]) : 0.f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox;
         v += (long long)gridDim.x * blockDim.x) {
        const float w = mask ? mask[v] : 1.f;
        const float d = out[v * C] - tgt[v];
        g[v * C] = f2bf(2.f * w * d * inv);
        for (int c = 1; c < C; ++c) g[v * C + c] = 0;
    }
}

// Adam on the FP32 parameters.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, long long n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// bf16 copies of one layer's weights: w16[co][t][ci] and the flipped transpose
// wt16[ci][26 - t][co] (the weights of the data-gradient convolution).
__global__ void k_pack_weights(const float* __restrict__ w, int cin, int cout, bf16_t* __restrict__ w16,
                               bf16_t* __restrict__ wt16) {
    const int n = cout * 27 * cin;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int ci = q % cin, t = (q / cin) % 27, co = q / (27 * cin);
        const bf16_t b = f2bf(w[q]);
        w16[q] = b;
        wt16[((long long)ci * 27 + (26 - t)) * cout + co] = b;
    }
}

// channel 0 of an FP32 [v][C] tensor
__global__ void k_channel0(const float* __restrict__ in, int C, int nvox, float* __restrict__ out) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox;
         v += (long long)gridDim.x * blockDim.x)
        out[v] = in[v * C];
}

// ---- host side ----------------------------------------------------------------
struct Layer {
    int cin, cout, level;
    long long woff, boff;   // offsets in the parameter vector
    bf16_t *w16, *wt16;
};

static const int LAYER_CIN[WPF_NET_LAYERS] = {16, 16, 32, 64, 64, 32, 16};
static const int LAYER_COUT[WPF_NET_LAYERS] = {16, 32, 64, 64, 32, 16, 16};
static const int LAYER_LEVEL[WPF_NET_LAYERS] = {0, 1, 2, 3, 2, 1, 0};

template <int CIN, int COUT>
static int launch_conv_t(const ConvArgs& a, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        WPF_CUDA(cudaFuncSetAttribute(k_conv3d<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      conv_smem<CIN, COUT>()));
        attr = true;
    }
    const unsigned grid = (unsigned)((a.nvox + CT - 1) / CT);
    k_conv3d<CIN, COUT><<<grid, CT, conv_smem<CIN, COUT>(), s>>>(a);
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

// The row-tiled kernel on its brick grid; WPF_ERR_CUDA when the tensor map
// cannot be encoded (the caller then uses the gather kernel).
template <int COUT, int TX>
static int launch_conv_row(const ConvArgs& a, cudaStream_t s) {
    using T = RowTile<COUT, TX>;
    static bool attr = false;
    if (!attr) {
        WPF_CUDA(cudaFuncSetAttribute(k_conv3d_row<COUT, TX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      T::SMEM));
        attr = true;
    }
    const EncodeTiledFn f = tensor_map_encoder();
    if (!f) return WPF_ERR_CUDA;
    CUtensorMap m;
    const cuuint64_t dims[4] = {16, (cuuint64_t)a.nx, (cuuint64_t)a.ny, (cuuint64_t)a.nz};
    const cuuint64_t strides[3] = {32, (cuuint64_t)a.nx * 32, (cuuint64_t)a.nx * a.ny * 32};
    const cuuint32_t box[4] = {8, (cuuint32_t)T::BOXX, (cuuint32_t)(T::TY + 2), 3};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    if (f(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)a.in, dims, strides, box, es,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return WPF_ERR_CUDA;
    RowConvArgs r;
    r.nx = a.nx; r.ny = a.ny; r.nz = a.nz;
    r.w = a.w; r.bias = a.bias; r.out16 = a.out16; r.out32 = a.out32; r.relu = a.relu; r.err = a.err;
    const unsigned grid = (unsigned)((a.nx / TX) * (a.ny / T::TY) * a.nz);
    k_conv3d_row<COUT, TX><<<grid, CT, T::SMEM, s>>>(r, m);
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

template <int COUT>
static int try_conv_row(const ConvArgs& a, cudaStream_t s, bool* done) {
    *done = true;
#define WPF_ROW_CASE(TX) \
    if (a.nx % TX == 0 && a.ny % (128 / TX) == 0) return launch_conv_row<COUT, TX>(a, s);
    WPF_ROW_CASE(128) WPF_ROW_CASE(64) WPF_ROW_CASE(32) WPF_ROW_CASE(16)
#undef WPF_ROW_CASE
    *done = false;
    return WPF_OK;
}

static int launch_conv(int cin, int cout, const ConvArgs& a, cudaStream_t s) {
    if (cin == 16 && (cout == 16 || cout == 32) && (long long)a.nx * a.ny * a.nz == a.nvox) {
        bool done = false;
        const int rc = cout == 16 ? try_conv_row<16>(a, s, &done) : try_conv_row<32>(a, s, &done);
        if (done) return rc;
    }
#define WPF_CONV_CASE(I, O) \
    if (cin == I && cout == O) return launch_conv_t<I, O>(a, s);
    WPF_CONV_CASE(16, 16) WPF_CONV_CASE(16, 32) WPF_CONV_CASE(32, 64) WPF_CONV_CASE(64, 64)
    WPF_CONV_CASE(64, 32) WPF_CONV_CASE(32, 16)
#undef WPF_CONV_CASE
    return WPF_ERR_ARG;
}

template <int CIN, int COUT>
static int launch_wgrad_t(const WgradArgs& a, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        WPF_CUDA(cudaFuncSetAttribute(k_conv3d_wgrad<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      wgrad_smem<CIN, COUT>()));
        attr = true;
    }
    const dim3 grid((27 * CIN + CT - 1) / CT, (unsigned)((a.nvox + WG_VOX - 1) / WG_VOX));
    k_conv3d_wgrad<CIN, COUT><<<grid, CT, wgrad_smem<CIN, COUT>(), s>>>(a);
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

static int launch_wgrad(int cin, int cout, const WgradArgs& a, cudaStream_t s) {
#define WPF_WG_CASE(I, O) \
    if (cin == I && cout == O) return launch_wgrad_t<I, O>(a, s);
    WPF_WG_CASE(16, 16) WPF_WG_CASE(16, 32) WPF_WG_CASE(32, 64) WPF_WG_CASE(64, 64)
    WPF_WG_CASE(64, 32) WPF_WG_CASE(32, 16)
#undef WPF_WG_CASE
    return WPF_ERR_ARG;
}

static unsigned ew_grid(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)(b < 4096 ? (b < 1 ? 1 : b) : 4096);
}

}  // namespace net
}  // namespace wpf

using namespace wpf;
using namespace wpf::net;

struct wpf_net {
    int nx[4], ny[4], nz[4];   // grid of each level
    long long nvox[4];
    Layer L[WPF_NET_LAYERS];
    long long nparam;
    float *p, *g, *m, *v;          // FP32 parameters, gradients, Adam moments
    long long step;
    // activations (bf16) and the FP32 output
    bf16_t *y[WPF_NET_LAYERS - 1], *p0, *p1, *p2, *s2, *s1, *s0;
    float* out32;
    // gradients (bf16)
    bf16_t *gout, *gs0, *gs1, *gs2, *gp0, *gp1, *gp2, *gpre[WPF_NET_LAYERS];
    double* dacc;   // loss sums
    int* derr;
    std::vector<void*> allocs;
};

namespace {

template <typename T>
int net_alloc(wpf_net* n, T** p, size_t count) {
    *p = nullptr;
    if (cudaMalloc((void**)p, count * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return WPF_ERR_NOMEM;
    }
    n->allocs.push_back((void*)*p);
    if (cudaMemset(*p, 0, count * sizeof(T)) != cudaSuccess) return WPF_ERR_CUDA;
    return WPF_OK;
}

int check_err(wpf_net* n, cudaStream_t s) {
    int e = 0;
    WPF_CUDA(cudaMemcpyAsync(&e, n->derr, sizeof(int), cudaMemcpyDeviceToHost, s));
    WPF_CUDA(cudaStreamSynchronize(s));
    return e ? WPF_ERR_TIMEOUT : WPF_OK;
}

int conv(wpf_net* n, int l, const bf16_t* in, const bf16_t* w, int cin, int cout, bool relu, bf16_t* out16,
         float* out32, const float* bias, cudaStream_t s) {
    const int lv = n->L[l].level;
    ConvArgs a;
    a.nx = n->nx[lv]; a.ny = n->ny[lv]; a.nz = n->nz[lv]; a.nvox = (int)n->nvox[lv];
    a.in = in; a.w = w; a.bias = bias; a.out16 = out16; a.out32 = out32; a.relu = relu ? 1 : 0;
    a.err = n->derr;
    return launch_conv(cin, cout, a, s);
}

int pack_all(wpf_net* n, cudaStream_t s) {
    for (int l = 0; l < WPF_NET_LAYERS; ++l) {
        const Layer& L = n->L[l];
        k_pack_weights<<<ew_grid((long long)L.cout * 27 * L.cin), 256, 0, s>>>(n->p + L.woff, L.cin, L.cout,
                                                                            L.w16, L.wt16);
    }
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

int forward(wpf_net* n, const bf16_t* x, cudaStream_t s) {
    int rc;
    auto B = [&](int l) { return n->p + n->L[l].boff; };
    // encoder
    if ((rc = conv(n, 0, x, n->L[0].w16, 16, 16, true, n->y[0], nullptr, B(0), s))) return rc;
    k_pool2<<<ew_grid(n->nvox[1] * 16 / 8), 256, 0, s>>>(n->y[0], n->p0, n->nx[0], n->ny[0], n->nz[0], 16);
    if ((rc = conv(n, 1, n->p0, n->L[1].w16, 16, 32, true, n->y[1], nullptr, B(1), s))) return rc;
    k_pool2<<<ew_grid(n->nvox[2] * 32 / 8), 256, 0, s>>>(n->y[1], n->p1, n->nx[1], n->ny[1], n->nz[1], 32);
    if ((rc = conv(n, 2, n->p1, n->L[2].w16, 32, 64, true, n->y[2], nullptr, B(2), s))) return rc;
    k_pool2<<<ew_grid(n->nvox[3] * 64 / 8), 256, 0, s>>>(n->y[2], n->p2, n->nx[2], n->ny[2], n->nz[2], 64);
    if ((rc = conv(n, 3, n->p2, n->L[3].w16, 64, 64, true, n->y[3], nullptr, B(3), s))) return rc;
    // decoder
    k_up2_add<<<ew_grid(n->nvox[2] * 64 / 8), 256, 0, s>>>(n->y[3], n->y[2], n->s2, n->nx[2], n->ny[2], n->nz[2], 64);
    if ((rc = conv(n, 4, n->s2, n->L[4].w16, 64, 32, true, n->y[4], nullptr, B(4), s))) return rc;
    k_up2_add<<<ew_grid(n->nvox[1] * 32 / 8), 256, 0, s>>>(n->y[4], n->y[1], n->s1, n->nx[1], n->ny[1], n->nz[1], 32);
    if ((rc = conv(n, 5, n->s1, n->L[5].w16, 32, 16, true, n->y[5], nullptr, B(5), s))) return rc;
    k_up2_add<<<ew_grid(n->nvox[0] * 16 / 8), 256, 0, s>>>(n->y[5], n->y[0], n->s0, n->nx[0], n->ny[0], n->nz[0], 16);
    if ((rc = conv(n, 6, n->s0, n->L[6].w16, 16, 16, false, nullptr, n->out32, B(6), s))) return rc;
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

int wgrad(wpf_net* n, int l, const bf16_t* x, const bf16_t* gy, cudaStream_t s) {
    const Layer& L = n->L[l];
    const int lv = L.level;
    WgradArgs a;
    a.nx = n->nx[lv]; a.ny = n->ny[lv]; a.nz = n->nz[lv]; a.nvox = (int)n->nvox[lv];
    a.x = x; a.gy = gy; a.gw = n->g + L.woff; a.err = n->derr;
    int rc = launch_wgrad(L.cin, L.cout, a, s);
    if (rc) return rc;
    k_bias_grad<<<256, 256, 0, s>>>(gy, (int)n->nvox[lv], L.cout, n->g + L.boff);
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

int backward(wpf_net* n, const bf16_t* x, cudaStream_t s) {
    int rc;
    const int* X = n->nx; const int* Y = n->ny; const int* Z = n->nz;
    // layer 6 (no ReLU): gradient gout
    if ((rc = wgrad(n, 6, n->s0, n->gout, s))) return rc;
    if ((rc = conv(n, 6, n->gout, n->L[6].wt16, 16, 16, false, n->gs0, nullptr, nullptr, s))) return rc;
    // layer 5
    k_bwd_up_relu<<<ew_grid(n->nvox[1] * 16), 256, 0, s>>>(n->gs0, n->y[5], n->gpre[5], X[0], Y[0], Z[0], 16);
    if ((rc = wgrad(n, 5, n->s1, n->gpre[5], s))) return rc;
    if ((rc = conv(n, 5, n->gpre[5], n->L[5].wt16, 16, 32, false, n->gs1, nullptr, nullptr, s))) return rc;
    // layer 4
    k_bwd_up_relu<<<ew_grid(n->nvox[2] * 32), 256, 0, s>>>(n->gs1, n->y[4], n->gpre[4], X[1], Y[1], Z[1], 32);
    if ((rc = wgrad(n, 4, n->s2, n->gpre[4], s))) return rc;
    if ((rc = conv(n, 4, n->gpre[4], n->L[4].wt16, 32, 64, false, n->gs2, nullptr, nullptr, s))) return rc;
    // layer 3
    k_bwd_up_relu<<<ew_grid(n->nvox[3] * 64), 256, 0, s>>>(n->gs2, n->y[3], n->gpre[3], X[2], Y[2], Z[2], 64);
    if ((rc = wgrad(n, 3, n->p2, n->gpre[3], s))) return rc;
    if ((rc = conv(n, 3, n->gpre[3], n->L[3].wt16, 64, 64, false, n->gp2, nullptr, nullptr, s))) return rc;
    // layer 2
    k_bwd_pool_skip_relu<<<ew_grid(n->nvox[2] * 64), 256, 0, s>>>(n->gp2, n->gs2, n->y[2], n->gpre[2], X[2], Y[2],
                                                                 Z[2], 64);
    if ((rc = wgrad(n, 2, n->p1, n->gpre[2], s))) return rc;
    if ((rc = conv(n, 2, n->gpre[2], n->L[2].wt16, 64, 32, false, n->gp1, nullptr, nullptr, s))) return rc;
    // layer 1
    k_bwd_pool_skip_relu<<<ew_grid(n->nvox[1] * 32), 256, 0, s>>>(n->gp1, n->gs1, n->y[1], n->gpre[1], X[1], Y[1],
                                                                 Z[1], 32);
    if ((rc = wgrad(n, 1, n->p0, n->gpre[1], s))) return rc;
    if ((rc = conv(n, 1, n->gpre[1], n->L[1].wt16, 32, 16, false, n->gp0, nullptr, nullptr, s))) return rc;
    // layer 0
    k_bwd_pool_skip_relu<<<ew_grid(n->nvox[0] * 16), 256, 0, s>>>(n->gp0, n->gs0, n->y[0], n->gpre[0], X[0], Y[0],
                                                                 Z[0], 16);
    if ((rc = wgrad(n, 0, x, n->gpre[0], s))) return rc;
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

}  // namespace

extern "C" {

int wpf_net_create(int32_t nx, int32_t ny, int32_t nz, wpf_net** out) {
    if (!out || nx < 8 || ny < 8 || nz < 8 || nx % 8 || ny % 8 || nz % 8) return WPF_ERR_ARG;
    *out = nullptr;
    wpf_net* n = new wpf_net();
    for (int l = 0; l < 4; ++l) {
        n->nx[l] = nx >> l; n->ny[l] = ny >> l; n->nz[l] = nz >> l;
        n->nvox[l] = (long long)n->nx[l] * n->ny[l] * n->nz[l];
    }
    long long off = 0;
    for (int l = 0; l < WPF_NET_LAYERS; ++l) {
        Layer& L = n->L[l];
        L.cin = LAYER_CIN[l]; L.cout = LAYER_COUT[l]; L.level = LAYER_LEVEL[l];
        L.woff = off; off += (long long)L.cout * 27 * L.cin;
        L.boff = off; off += L.cout;
    }
    n->nparam = off;
    n->step = 0;
    int rc = WPF_OK;
    auto A16 = [&](bf16_t** p, long long c) { if (!rc) rc = net_alloc(n, p, (size_t)c); };
    auto A32 = [&](float** p, long long c) { if (!rc) rc = net_alloc(n, p, (size_t)c); };
    A32(&n->p, off); A32(&n->g, off); A32(&n->m, off); A32(&n->v, off);
    for (int l = 0; l < WPF_NET_LAYERS; ++l) {
        const long long wn = (long long)n->L[l].cout * 27 * n->L[l].cin;
        A16(&n->L[l].w16, wn); A16(&n->L[l].wt16, wn);
    }
    const long long* V = n->nvox;
    for (int l = 0; l < WPF_NET_LAYERS - 1; ++l) A16(&n->y[l], V[LAYER_LEVEL[l]] * LAYER_COUT[l]);
    A16(&n->p0, V[1] * 16); A16(&n->p1, V[2] * 32); A16(&n->p2, V[3] * 64);
    A16(&n->s2, V[2] * 64); A16(&n->s1, V[1] * 32); A16(&n->s0, V[0] * 16);
    A32(&n->out32, V[0] * 16);
    A16(&n->gout, V[0] * 16); A16(&n->gs0, V[0] * 16); A16(&n->gs1, V[1] * 32); A16(&n->gs2, V[2] * 64);
    A16(&n->gp0, V[1] * 16); A16(&n->gp1, V[2] * 32); A16(&n->gp2, V[3] * 64);
    for (int l = 0; l < WPF_NET_LAYERS; ++l)
        A16(&n->gpre[l], V[LAYER_LEVEL[l]] * LAYER_COUT[l]);
    if (!rc) rc = net_alloc(n, &n->dacc, 2);
    if (!rc) rc = net_alloc(n, &n->derr, 1);
    if (rc) {
        wpf_net_destroy(n);
        return rc;
    }
    *out = n;
    return WPF_OK;
}

int wpf_net_destroy(wpf_net* n) {
    if (!n) return WPF_ERR_ARG;
    cudaDeviceSynchronize();
    for (void* p : n->allocs) cudaFree(p);
    delete n;
    return WPF_OK;
}

int wpf_net_param_count(const wpf_net* n, int64_t* c) {
    if (!n || !c) return WPF_ERR_ARG;
    *c = n->nparam;
    return WPF_OK;
}

int wpf_net_init(wpf_net* n, uint64_t seed) {
    if (!n) return WPF_ERR_ARG;
    std::vector<float> h((size_t)n->nparam, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < WPF_NET_LAYERS; ++l) {
        const Layer& L = n->L[l];
        const double sd = sqrt(2.0 / (27.0 * L.cin)) * (l == WPF_NET_LAYERS - 1 ? 0.1 : 1.0);
        std::normal_distribution<double> nd(0.0, sd);
        for (long long q = 0; q < (long long)L.cout * 27 * L.cin; ++q) h[(size_t)(L.woff + q)] = (float)nd(rng);
    }
    return wpf_net_set_params(n, h.data());
}

int wpf_net_get_params(wpf_net* n, float* host) {
    if (!n || !host) return WPF_ERR_ARG;
    WPF_CUDA(cudaMemcpy(host, n->p, sizeof(float) * n->nparam, cudaMemcpyDeviceToHost));
    return WPF_OK;
}

int wpf_net_get_grads(wpf_net* n, float* host) {
    if (!n || !host) return WPF_ERR_ARG;
    WPF_CUDA(cudaMemcpy(host, n->g, sizeof(float) * n->nparam, cudaMemcpyDeviceToHost));
    return WPF_OK;
}

int wpf_net_set_params(wpf_net* n, const float* host) {
    if (!n || !host) return WPF_ERR_ARG;
    WPF_CUDA(cudaMemcpy(n->p, host, sizeof(float) * n->nparam, cudaMemcpyHostToDevice));
    WPF_CUDA(cudaMemset(n->m, 0, sizeof(float) * n->nparam));
    WPF_CUDA(cudaMemset(n->v, 0, sizeof(float) * n->nparam));
    n->step = 0;
    int rc = pack_all(n, 0);
    if (rc) return rc;
    WPF_CUDA(cudaDeviceSynchronize());
    return WPF_OK;
}

int wpf_net_get_activation(wpf_net* n, int32_t layer, uint16_t* host, int64_t count) {
    if (!n || !host || layer < 0 || layer >= WPF_NET_LAYERS) return WPF_ERR_ARG;
    const long long want = n->nvox[LAYER_LEVEL[layer]] * LAYER_COUT[layer];
    if (count != want) return WPF_ERR_ARG;
    if (layer < WPF_NET_LAYERS - 1) {
        WPF_CUDA(cudaMemcpy(host, n->y[layer], sizeof(bf16_t) * want, cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> t((size_t)want);
        WPF_CUDA(cudaMemcpy(t.data(), n->out32, sizeof(float) * want, cudaMemcpyDeviceToHost));
        for (long long q = 0; q < want; ++q) {   // round to nearest even bf16
            uint32_t b;
            memcpy(&b, &t[(size_t)q], 4);
            b += 0x7FFFu + ((b >> 16) & 1u);
            host[q] = (uint16_t)(b >> 16);
        }
    }
    return WPF_OK;
}

int wpf_net_forward(wpf_net* n, const uint16_t* in, float* out, void* stream) {
    if (!n || !in) return WPF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = forward(n, in, s);
    if (rc) return rc;
    if (out) k_channel0<<<ew_grid(n->nvox[0]), 256, 0, s>>>(n->out32, 16, (int)n->nvox[0], out);
    WPF_CUDA(cudaGetLastError());
    return check_err(n, s);
}

int wpf_net_train_step(wpf_net* n, const uint16_t* in, const float* target, const float* mask, float lr,
                       float* loss, void* stream) {
    if (!n || !in || !target || !(lr >= 0.f)) return WPF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = forward(n, in, s);
    if (rc) return rc;
    WPF_CUDA(cudaMemsetAsync(n->dacc, 0, 2 * sizeof(double), s));
    const int nv = (int)n->nvox[0];
    k_loss_sums<<<ew_grid(nv), 256, 0, s>>>(n->out32, 16, target, mask, nv, n->dacc);
    k_loss_grad<<<ew_grid(nv), 256, 0, s>>>(n->out32, 16, target, mask, nv, n->dacc, n->gout);
    WPF_CUDA(cudaMemsetAsync(n->g, 0, sizeof(float) * n->nparam, s));
    if ((rc = backward(n, in, s))) return rc;
    n->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = (float)(1.0 / (1.0 - pow(b1, (double)n->step)));
    const float c2 = (float)(1.0 / (1.0 - pow(b2, (double)n->step)));
    k_adam<<<ew_grid(n->nparam), 256, 0, s>>>(n->p, n->g, n->m, n->v, n->nparam, lr, b1, b2, 1e-8f, c1, c2);
    if ((rc = pack_all(n, s))) return rc;
    WPF_CUDA(cudaGetLastError());
    if (loss) {
        double h[2];
        WPF_CUDA(cudaMemcpyAsync(h, n->dacc, sizeof(h), cudaMemcpyDeviceToHost, s));
        WPF_CUDA(cudaStreamSynchronize(s));
        *loss = h[1] > 0 ? (float)(h[0] / h[1]) : 0.f;
    }
    return check_err(n, s);
}

int wpf_conv3d(int32_t cin, int32_t cout, int32_t nx, int32_t ny, int32_t nz, const uint16_t* in,
               const uint16_t* w, const float* bias, int32_t relu, uint16_t* out16, float* out32, void* stream) {
    if (!in || !w || (!out16 == !out32) || nx < 1 || ny < 1 || nz < 1) return WPF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    static int* derr = nullptr;
    if (!derr) {
        WPF_CUDA(cudaMalloc((void**)&derr, sizeof(int)));
        WPF_CUDA(cudaMemset(derr, 0, sizeof(int)));
    }
    ConvArgs a;
    a.nx = nx; a.ny = ny; a.nz = nz; a.nvox = nx * ny * nz;
    a.in = in; a.w = w; a.bias = bias; a.out16 = out16; a.out32 = out32; a.relu = relu; a.err = derr;
    int rc = launch_conv(cin, cout, a, s);
    if (rc) return rc;
    int e = 0;
    WPF_CUDA(cudaMemcpyAsync(&e, derr, sizeof(int), cudaMemcpyDeviceToHost, s));
    WPF_CUDA(cudaStreamSynchronize(s));
    return e ? WPF_ERR_TIMEOUT : WPF_OK;
}

int wpf_conv3d_wgrad(int32_t cin, int32_t cout, int32_t nx, int32_t ny, int32_t nz, const uint16_t* x,
                     const uint16_t* gy, float* gw, float* gb, void* stream) {
    if (!x || !gy || !gw || nx < 1 || ny < 1 || nz < 1) return WPF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    static int* derr = nullptr;
    if (!derr) {
        WPF_CUDA(cudaMalloc((void**)&derr, sizeof(int)));
        WPF_CUDA(cudaMemset(derr, 0, sizeof(int)));
    }
    WgradArgs a;
    a.nx = nx; a.ny = ny; a.nz = nz; a.nvox = nx * ny * nz;
    a.x = x; a.gy = gy; a.gw = gw; a.err = derr;
    int rc = launch_wgrad(cin, cout, a, s);
    if (rc) return rc;
    if (gb) k_bias_grad<<<256, 256, 0, s>>>(gy, nx * ny * nz, cout, gb);
    WPF_CUDA(cudaGetLastError());
    int e = 0;
    WPF_CUDA(cudaMemcpyAsync(&e, derr, sizeof(int), cudaMemcpyDeviceToHost, s));
    WPF_CUDA(cudaStreamSynchronize(s));
    return e ? WPF_ERR_TIMEOUT : WPF_OK;
}

}  // extern "C"

// ---- the learned start inside a simulation handle ------------------------------------
// The net works on the simulation grid coarsened 2x2x2 (net voxel (X,Y,Z),
// 0-based, covers the fine cells 2X+1..2X+2 etc., 1-based).
namespace wpf {
namespace net {

// sum log K_rock, sum (log K_rock)^2 over the interior
__global__ void __launch_bounds__(RB) k_klog_stats(Grid g, const double* __restrict__ kr, double* dsc) {
    double s = 0.0, s2 = 0.0;
    ROW_LOOP(g) {
        const double v = log(kr[g.at(i, j, k)]);
        s += v;
        s2 += v * v;
    }
    block_add(s, dsc + S_KLOG0);
    block_add(s2, dsc + S_KLOG1);
}

// sum (phase - phase_prev)^2 over the interior
__global__ void __launch_bounds__(RB) k_dphase_stats(Grid g, const double* __restrict__ ph,
                                                     const double* __restrict__ prev, double* dsc) {
    double s2 = 0.0;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        const double d = ph[n] - prev[n];
        s2 += d * d;
    }
    block_add(s2, dsc + S_DPH2);
}

// Scales: s = rms of the last increment d1, q = rms of its change d1 - d2
// (the extrapolation error scales with the changes of the increment, three
// orders of magnitude below the increment itself, so the network sees and
// predicts in units of q; in units of s its target would sit below bf16
// resolution).
__device__ __forceinline__ double ws_scale_s(const Grid& g, const double* dsc) {
    return sqrt(dsc[S_WSS2] / ((double)g.nx * g.ny * g.nz)) + 1e-30;
}
__device__ __forceinline__ double ws_scale_q(const Grid& g, const double* dsc) {
    return sqrt(dsc[S_WSD2] / ((double)g.nx * g.ny * g.nz)) + 1e-30;
}

// Net input: 2x2x2 means of (log K_rock - mean)/sd, phase, pressure, d1/s,
// (d1 - d2)/q, (phase - phase_prev)/s_phi; channels 6..15 zero.
// Channel 0 of the net input, 2x2x2 means of (log K_rock - mean) / sd: K_rock
// only changes with an upload, so this FP64 log pass runs once, not per solve.
__global__ void k_ws_klog_feature(Grid g, int nxn, int nyn, int nzn, const double* __restrict__ kr,
                                  const double* __restrict__ dsc, float* __restrict__ out) {
    const double N = (double)g.nx * g.ny * g.nz;
    const double km = dsc[S_KLOG0] / N;
    const double ksd = sqrt(fmax(dsc[S_KLOG1] / N - km * km, 1e-12));
    const long long nv = (long long)nxn * nyn * nzn;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
         v += (long long)gridDim.x * blockDim.x) {
        const int X = (int)(v % nxn);
        const long long r = v / nxn;
        const int Y = (int)(r % nyn), Z = (int)(r / nyn);
        double f = 0.0;
        for (int c = 0; c < 8; ++c)
            f += log(kr[g.at(2 * X + 1 + (c & 1), 2 * Y + 1 + ((c >> 1) & 1), 2 * Z + 1 + (c >> 2))]);
        out[v] = (float)((f / 8 - km) / ksd);
    }
}

__global__ void k_ws_features(Grid g, int nxn, int nyn, int nzn, const float* __restrict__ klog,
                              const double* __restrict__ ph, const double* __restrict__ prev,
                              const double* __restrict__ pr, const float* __restrict__ d1,
                              const float* __restrict__ d2, const double* __restrict__ dsc,
                              bf16_t* __restrict__ out) {
    const double N = (double)g.nx * g.ny * g.nz;
    const double s = ws_scale_s(g, dsc), q = ws_scale_q(g, dsc);
    const double sp = sqrt(dsc[S_DPH2] / N) + 1e-30;
    const long long nv = (long long)nxn * nyn * nzn;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
         v += (long long)gridDim.x * blockDim.x) {
        const int X = (int)(v % nxn);
        const long long r = v / nxn;
        const int Y = (int)(r % nyn), Z = (int)(r / nyn);
        double f[6] = {0, 0, 0, 0, 0, 0};
        for (int c = 0; c < 8; ++c) {
            const long long n = g.at(2 * X + 1 + (c & 1), 2 * Y + 1 + ((c >> 1) & 1), 2 * Z + 1 + (c >> 2));
            f[1] += ph[n];
            f[2] += pr[n];
            f[3] += d1[n];
            f[4] += (double)d1[n] - (double)d2[n];
            f[5] += ph[n] - prev[n];
        }
        const float ch[6] = {klog[v], (float)(f[1] / 8), (float)(f[2] / 8),
                             (float)(f[3] / 8 / s),           (float)(f[4] / 8 / q), (float)(f[5] / 8 / sp)};
        uint4* o = reinterpret_cast<uint4*>(out + v * 16);
        o[0] = make_uint4(pack2(ch[0], ch[1]), pack2(ch[2], ch[3]), pack2(ch[4], ch[5]), 0u);
        o[1] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// e_net on the fine interior: q * trilinear interpolation of the net output
// between net-voxel centres (clamped at the edges); zero on Dirichlet cells.
__global__ void __launch_bounds__(RB) k_ws_prolong(Grid g, int nxn, int nyn, int nzn,
                                                   const float* __restrict__ o, const uint8_t* __restrict__ fl,
                                                   const double* __restrict__ dsc, float* __restrict__ e2) {
    const float s = (float)ws_scale_q(g, dsc);
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        if (fl[n] & F_DIR) {
            e2[n] = 0.f;
            continue;
        }
        auto axis = [](int fi, int nn, int& a0, int& a1, float& w) {
            const float u = 0.5f * ((float)fi - 1.5f);
            const float fu = floorf(u);
            w = u - fu;
            a0 = (int)fu;
            a1 = a0 + 1;
            if (a0 < 0) { a0 = 0; w = 0.f; }
            if (a1 > nn - 1) { a1 = nn - 1; }
            if (a0 > nn - 1) { a0 = nn - 1; w = 0.f; }
        };
        int x0, x1, y0, y1, z0, z1;
        float wx, wy, wz;
        axis(i, nxn, x0, x1, wx);
        axis(j, nyn, y0, y1, wy);
        axis(k, nzn, z0, z1, wz);
        auto O = [&](int x, int y, int z) { return o[((long long)z * nyn + y) * nxn + x]; };
        const float c00 = O(x0, y0, z0) + wx * (O(x1, y0, z0) - O(x0, y0, z0));
        const float c10 = O(x0, y1, z0) + wx * (O(x1, y1, z0) - O(x0, y1, z0));
        const float c01 = O(x0, y0, z1) + wx * (O(x1, y0, z1) - O(x0, y0, z1));
        const float c11 = O(x0, y1, z1) + wx * (O(x1, y1, z1) - O(x0, y1, z1));
        const float c0 = c00 + wy * (c10 - c00), c1 = c01 + wy * (c11 - c01);
        e2[n] = s * (c0 + wz * (c1 - c0));
    }
}

// Training target: 2x2x2 means of (d_new - e_ext) / q.
__global__ void k_ws_target(Grid g, int nxn, int nyn, int nzn, const float* __restrict__ dnew,
                            const float* __restrict__ e1, const double* __restrict__ dsc,
                            float* __restrict__ out) {
    const double s = ws_scale_q(g, dsc);
    const long long nv = (long long)nxn * nyn * nzn;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
         v += (long long)gridDim.x * blockDim.x) {
        const int X = (int)(v % nxn);
        const long long r = v / nxn;
        const int Y = (int)(r % nyn), Z = (int)(r / nyn);
        double acc = 0.0;
        for (int c = 0; c < 8; ++c) {
            const long long n = g.at(2 * X + 1 + (c & 1), 2 * Y + 1 + ((c >> 1) & 1), 2 * Z + 1 + (c >> 2));
            acc += (double)dnew[n] - (double)e1[n];
        }
        out[v] = (float)(acc / 8.0 / s);
    }
}

}  // namespace net

// The log K_rock channel of the net input (statistics, then the net-grid
// means), made when K_rock changed since the last one.
static int ws_klog_prepare(wpf_handle* h) {
    const Grid& g = h->g;
    cudaStream_t s = h->stream;
    const int nxn = g.nx / 2, nyn = g.ny / 2, nzn = g.nz / 2;
    const long long nv = (long long)nxn * nyn * nzn;
    int rc;
    if (!h->ws_klog && (rc = dev_alloc(h, (void**)&h->ws_klog, sizeof(float) * nv))) return rc;
    if (!h->ws_klog_ready) {
        WPF_CUDA(cudaMemsetAsync(h->dsc + S_KLOG0, 0, 2 * sizeof(double), s));
        WPF_LAUNCH(h, KC_OTHER, net::k_klog_stats<<<row_blocks(h, g), RB, 0, s>>>(g, h->krock, h->dsc));
        WPF_LAUNCH(h, KC_OTHER, net::k_ws_klog_feature<<<net::ew_grid(nv), 256, 0, s>>>(
            g, nxn, nyn, nzn, h->krock, h->dsc, h->ws_klog));
        WPF_CUDA(cudaGetLastError());
        h->ws_klog_ready = true;
    }
    return WPF_OK;
}

// Net input of the coming solve: e_ext (and its scale) for step size hn,
// then the features.
static int ws_prepare_features(wpf_handle* h, double hn, uint16_t* in) {
    const Grid& g = h->g;
    cudaStream_t s = h->stream;
    int rc0 = ws_klog_prepare(h);
    if (rc0) return rc0;
    const double keep = h->ws_hn;
    h->ws_hn = hn;
    float a, b;
    ws_coeffs(h, &a, &b);
    h->ws_hn = keep;
    int rc = ws_build_ext(h, a, b);
    if (rc) return rc;
    WPF_CUDA(cudaMemsetAsync(h->dsc + S_DPH2, 0, sizeof(double), s));
    WPF_LAUNCH(h, KC_OTHER, net::k_dphase_stats<<<row_blocks(h, g), RB, 0, s>>>(g, h->phase, h->phase_n, h->dsc));
    const int nxn = g.nx / 2, nyn = g.ny / 2, nzn = g.nz / 2;
    const long long nv = (long long)nxn * nyn * nzn;
    WPF_LAUNCH(h, KC_OTHER, net::k_ws_features<<<net::ew_grid(nv), 256, 0, s>>>(
        g, nxn, nyn, nzn, h->ws_klog, h->phase, h->phase_n, h->pressure, h->ws[0], h->ws[1], h->dsc, in));
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

// e_net for the solve that is starting: features (e_ext already built by
// the solve), forward pass, prolongation.
int ws_net_correction(wpf_handle* h) {
    const Grid& g = h->g;
    cudaStream_t s = h->stream;
    const int nxn = g.nx / 2, nyn = g.ny / 2, nzn = g.nz / 2;
    const long long nv = (long long)nxn * nyn * nzn;
    int rc;
    if (!h->ws_in && (rc = dev_alloc(h, (void**)&h->ws_in, sizeof(uint16_t) * nv * 16))) return rc;
    if (!h->ws_out && (rc = dev_alloc(h, (void**)&h->ws_out, sizeof(float) * nv))) return rc;
    if (!h->ws_e[1] && (rc = dev_alloc(h, (void**)&h->ws_e[1], sizeof(float) * g.total))) return rc;
    if ((h->opts.flags & WPF_SOLVER_NET_COARSE) && !h->ws_e[2] &&
        (rc = dev_alloc(h, (void**)&h->ws_e[2], sizeof(float) * g.total)))
        return rc;
    if ((rc = ws_klog_prepare(h))) return rc;
    WPF_CUDA(cudaMemsetAsync(h->dsc + S_DPH2, 0, sizeof(double), s));
    WPF_LAUNCH(h, KC_OTHER, net::k_dphase_stats<<<row_blocks(h, g), RB, 0, s>>>(g, h->phase, h->phase_n, h->dsc));
    WPF_LAUNCH(h, KC_OTHER, net::k_ws_features<<<net::ew_grid(nv), 256, 0, s>>>(
        g, nxn, nyn, nzn, h->ws_klog, h->phase, h->phase_n, h->pressure, h->ws[0], h->ws[1], h->dsc,
        h->ws_in));
    rc = wpf_net_forward(h->ws_net, h->ws_in, h->ws_out, (void*)s);
    if (rc) return rc;
    h->nlaunch += 2 * WPF_NET_LAYERS + 1;   // the net's kernels (convolutions, pooling, copies)
    WPF_LAUNCH(h, KC_OTHER, net::k_ws_prolong<<<row_blocks(h, g), RB, 0, s>>>(
        g, nxn, nyn, nzn, h->ws_out, h->flags, h->dsc, h->ws_e[1]));
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

// The device-resident step's learned start.  Buffers, the log-K statistics
// and one run of the net's kernels (their function attributes are set on the
// first launch) happen here, outside any stream capture.
int ws_net_prepare(wpf_handle* h) {
    const Grid& g = h->g;
    cudaStream_t s = h->stream;
    const long long nv = (long long)(g.nx / 2) * (g.ny / 2) * (g.nz / 2);
    int rc;
    if (!h->ws_in && (rc = dev_alloc(h, (void**)&h->ws_in, sizeof(uint16_t) * nv * 16))) return rc;
    if (!h->ws_out && (rc = dev_alloc(h, (void**)&h->ws_out, sizeof(float) * nv))) return rc;
    if (!h->ws_e[1] && (rc = dev_alloc(h, (void**)&h->ws_e[1], sizeof(float) * g.total))) return rc;
    if ((h->opts.flags & WPF_SOLVER_NET_COARSE) && !h->ws_e[2] &&
        (rc = dev_alloc(h, (void**)&h->ws_e[2], sizeof(float) * g.total)))
        return rc;
    if ((rc = ws_klog_prepare(h))) return rc;
    if (h->ws_net_warm != h->ws_net) {
        if ((rc = wpf_net_forward(h->ws_net, h->ws_in, h->ws_out, (void*)s))) return rc;
        h->ws_net_warm = h->ws_net;
    }
    return WPF_OK;
}

// e_net for a captured step: the kernels of ws_net_correction on stream s,
// with no read-back (the net's error flag is read after the step).
int ws_net_capture(wpf_handle* h, cudaStream_t s) {
    const Grid& g = h->g;
    const int nxn = g.nx / 2, nyn = g.ny / 2, nzn = g.nz / 2;
    const long long nv = (long long)nxn * nyn * nzn;
    if (!h->ws_in || !h->ws_out || !h->ws_e[1] || !h->ws_klog || !h->ws_klog_ready) return WPF_ERR_ARG;
    WPF_CUDA(cudaMemsetAsync(h->dsc + S_DPH2, 0, sizeof(double), s));
    WPF_LAUNCH(h, KC_OTHER, net::k_dphase_stats<<<row_blocks(h, g), RB, 0, s>>>(g, h->phase, h->phase_n, h->dsc));
    WPF_LAUNCH(h, KC_OTHER, net::k_ws_features<<<net::ew_grid(nv), 256, 0, s>>>(
        g, nxn, nyn, nzn, h->ws_klog, h->phase, h->phase_n, h->pressure, h->ws[0], h->ws[1], h->dsc,
        h->ws_in));
    wpf_net* n = h->ws_net;
    int rc = forward(n, h->ws_in, s);
    if (rc) return rc;
    k_channel0<<<ew_grid(n->nvox[0]), 256, 0, s>>>(n->out32, 16, (int)n->nvox[0], h->ws_out);
    h->nlaunch += 2 * WPF_NET_LAYERS + 1;   // the net's kernels (convolutions, pooling, copies)
    WPF_LAUNCH(h, KC_OTHER, net::k_ws_prolong<<<row_blocks(h, g), RB, 0, s>>>(
        g, nxn, nyn, nzn, h->ws_out, h->flags, h->dsc, h->ws_e[1]));
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

int ws_net_check(wpf_handle* h) { return h->ws_net ? check_err(h->ws_net, h->stream) : WPF_OK; }

}  // namespace wpf

extern "C" {

int wpf_set_warm_start_net(wpf_handle* h, wpf_net* n) {
    if (!h) return WPF_ERR_ARG;
    if (n && (n->nx[0] * 2 != h->g.nx || n->ny[0] * 2 != h->g.ny || n->nz[0] * 2 != h->g.nz))
        return WPF_ERR_ARG;
    h->ws_net = n;
    return WPF_OK;
}

int wpf_ws_features(wpf_handle* h, double dt_next, uint16_t* in) {
    if (!h || !in || !(h->opts.flags & WPF_SOLVER_EXTRAPOLATE) || h->ws_hist < 2 || !h->ws[0] ||
        h->g.nx % 16 || h->g.ny % 16 || h->g.nz % 16)
        return WPF_ERR_ARG;
    int rc = wpf::ws_prepare_features(h, dt_next, in);
    if (rc) return rc;
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    return WPF_OK;
}

int wpf_ws_target(wpf_handle* h, float* target) {
    if (!h || !target || !h->ws[0] || !h->ws_e[0] || h->ws_hist < 1) return WPF_ERR_ARG;
    const Grid& g = h->g;
    const int nxn = g.nx / 2, nyn = g.ny / 2, nzn = g.nz / 2;
    WPF_LAUNCH(h, KC_OTHER, wpf::net::k_ws_target<<<wpf::net::ew_grid((long long)nxn * nyn * nzn), 256, 0,
                                                    h->stream>>>(g, nxn, nyn, nzn, h->ws[0], h->ws_e[0],
                                                                 h->dsc, target));
    WPF_CUDA(cudaGetLastError());
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    return WPF_OK;
}

}  // extern "C"
