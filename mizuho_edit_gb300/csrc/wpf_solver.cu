// wpf_solver.cu -- matrix-free Darcy solve on sm_103a (replaces solvePressure's
// PETSc assembly + KSPBCGS/PCSOR, wPFAW3D.f90:603-1160).
//
// The system is the reference's: for a free (non-Dirichlet) cell
//     sum_f T_f (p_nb - p_c) = b_c,  T_f = K_f/mu on interior faces,
// Dirichlet cells fixed at their well pressure (identity rows, :840) and
// eliminated symmetrically from their neighbours' rows (:852-931).  On the
// device it is solved in the SPD form A' = -A on the free cells, matrix-free
// from the face array T, never assembled.
//
// Method: FP64 outer residual r = f - A'p (true residual, 7-point, from T and
// the pressure field in which Dirichlet cells hold their well value), then a
// preconditioned CG on A' e = r in precision R (double for the plain form,
// float for the mixed form), p += e, repeated until
//     ||r|| <= rtol * ||b||,   b = the reference right-hand side incl. the
// Dirichlet rows (so the relative residual is the one PETSc's default test
// would see for the unpreconditioned norm).
//
// Preconditioner: one V-cycle of an aggregation multigrid: 2x2x2 aggregates,
// coarse couplings = 0.5 x (sum of the fine couplings across the aggregate
// face) and coarse diagonal = 0.5 x (Galerkin diagonal), i.e. the Galerkin
// operator of piecewise-constant interpolation scaled by 1/2 (a coarse
// correction over-relaxed by 2, which makes piecewise-constant interpolation
// effective); red-black Gauss-Seidel smoothing (symmetric: red-black before,
// black-red after) so the V-cycle is a symmetric preconditioner; coarsening
// down to <= 2 cells per axis, solved by Gauss-Seidel sweeps in one block.
// Dead cells (Dirichlet, or aggregates of only Dirichlet cells) carry a zero
// diagonal and zero couplings and never change.
//
// On the large levels one red-black sweep is one kernel (k_sweep_async): each
// block owns a 32x8 column of cells and a 32-plane chunk of z and marches up
// in z, updating the first colour of plane k+1 and then the second colour of
// plane k, with the planes' x, couplings, 1/diag and b staged in shared memory
// by cp.async two planes ahead.  The first colour is recomputed on a one-cell
// ring around the tile from the old values (it depends on old values only),
// so every block produces exactly the two-kernel red-black result; the sweep
// reads x from one buffer and writes the other, so no block can see another
// block's new values.  Mid-size levels use in-place two-kernel half-sweeps and
// the levels of at most 4096 cells run their whole sub-cycle in one block.
#include <cuda.h>   // CUtensorMap (the encoder is fetched at run time)
#include <math.h>

#include <mutex>
#include <stddef.h>
#include <stdio.h>

#include "wpf_internal.cuh"

namespace wpf {

constexpr double COARSE_SCALE = 0.5;
constexpr int SX = 32, SY = 8;   // sweep tile (x, y); the z chunk is chosen per level (sweep_chunk)
constexpr int FX = SX + 4, FY = SY + 4;    // shared footprint: tile + 2-cell ring

// ---------------------------------------------------------------------------
// FP64 outer residual.  r = qterm + sum_f T_f (p_nb - p_c) on free cells, 0 on
// Dirichlet cells; accumulates ||r||^2 and, when want_b, ||b_ref||^2 with
// b_ref the reference right-hand side (:803-825, :852-931).
//
// With D (the FP64 sum of the six face transmissibilities of each live cell)
// the residual is formed as r = q + sum_f T_f p_nb - D p_c: seven FP64 FMAs
// instead of six subtractions and six multiply-adds (the FP64 pipe bounds
// these kernels on GB300).  The terms T p cancel where the differences T dp
// did not, which raises the rounding floor of ||r||/||b|| by about the ratio
// |p| / |dp| between neighbours (a few hundred on these grids): ~1e-14, far
// below the 1e-8 of the mixed form, which alone uses it.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double resid_cell(double q, double p0, double pxp, double pxm, double pyp,
                                             double pym, double pzp, double pzm, double txp, double txm,
                                             double typ, double tym, double tzp, double tzm,
                                             const double* __restrict__ D, long long n) {
    if (D) {
        double acc = fma(tzm, pzm, q);
        acc = fma(tym, pym, acc);
        acc = fma(txm, pxm, acc);
        acc = fma(txp, pxp, acc);
        acc = fma(typ, pyp, acc);
        acc = fma(tzp, pzp, acc);
        return fma(-D[n], p0, acc);
    }
    return q + (tzm * (pzm - p0) + tym * (pym - p0) + txm * (pxm - p0) + txp * (pxp - p0) +
                typ * (pyp - p0) + tzp * (pzp - p0));
}

template <typename R>
__global__ void __launch_bounds__(RB) k_resid64(Grid g, const double* __restrict__ pr,
                                                const double* __restrict__ Tx,
                                                const double* __restrict__ Ty,
                                                const double* __restrict__ Tz,
                                                const uint8_t* __restrict__ fl,
                                                const double* __restrict__ qterm,
                                                const double* __restrict__ D,
                                                R* __restrict__ rout, double* dsc, int want_b,
                                                const int* skip = nullptr,
                                                float* __restrict__ zero_out = nullptr,
                                                double* __restrict__ rk_out = nullptr,
                                                const int* want_b_dev = nullptr) {
    // skip: a device flag that, when set, makes the launch a no-op (the
    // device-resident step launches this pass unconditionally); zero_out: a
    // field whose interior is cleared on the way; rk_out: the residual kept
    // in FP64 for the next solve's pass 0; want_b_dev: a device flag that
    // also asks for ||b|| (set when pass 0's residual was a prediction)
    if (skip && *skip) return;
    if (want_b_dev && *want_b_dev) want_b = 1;
    double rr = 0.0, bb = 0.0;
    R rrr = 0;
    const long long sy = g.P, sz = g.S;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        const uint8_t f = fl[n];
        if (zero_out) zero_out[n] = 0.f;
        double r = 0.0;
        const double p0 = pr[n];
        if (f & F_DIR) {
            bb += p0 * p0;
        } else {
            const double q = qterm ? qterm[n] : 0.0;
            const double txp = Tx[n], txm = Tx[n - 1], typ = Ty[n], tym = Ty[n - sy];
            const double tzp = Tz[n], tzm = Tz[n - sz];
            const double pxp = pr[n + 1], pxm = pr[n - 1], pyp = pr[n + sy], pym = pr[n - sy];
            const double pzp = pr[n + sz], pzm = pr[n - sz];
            r = resid_cell(q, p0, pxp, pxm, pyp, pym, pzp, pzm, txp, txm, typ, tym, tzp, tzm, D, n);
            if (want_b && (q != 0.0 || ((fl[n - sz] | fl[n - sy] | fl[n - 1] | fl[n + 1] |
                                         fl[n + sy] | fl[n + sz]) & F_DIR))) {
                double bref = -q;
                if (fl[n - sz] & F_DIR) bref -= pzm * tzm;
                if (fl[n - sy] & F_DIR) bref -= pym * tym;
                if (fl[n - 1] & F_DIR) bref -= pxm * txm;
                if (fl[n + 1] & F_DIR) bref -= pxp * txp;
                if (fl[n + sy] & F_DIR) bref -= pyp * typ;
                if (fl[n + sz] & F_DIR) bref -= pzp * tzp;
                bb += bref * bref;
            }
        }
        const R rr_ = from_f64<R>(r);
        rout[n] = rr_;
        if (rk_out) rk_out[n] = r;
        // the FP32 form squares the rounded residual in FP32 (FP64 across
        // threads: ~1e-6 relative in the norm, none of the FP64 pipe)
        if (sizeof(R) == 4) rrr += rr_ * rr_;
        else rr += r * r;
    }
    rr += (double)rrr;
    block_add(rr, dsc + S_RR64);
    if (want_b) block_add(bb, dsc + S_BB64);
}

// p += e on the interior (e is zero on dead cells).
template <typename R>
__global__ void __launch_bounds__(RB) k_add_correction(Grid g, double* __restrict__ pr,
                                                       const R* __restrict__ e) {
    ROW_LOOP_U4(g) {
        const long long n = g.at(i, j, k);
        pr[n] += to_f64<R>(e[n]);
    }
}

// ---- extrapolated / learned warm start ------------------------------------------
// e_ext = a d1 + b d2 from the last two increments (zero on Dirichlet cells,
// where every increment is zero); accumulates sum d1^2 and sum (d1 - d2)^2
// (the scales the learned start works in) into S_WSS2 and S_WSD2.  With ab
// non-null the coefficients are read from the device (ab[0], ab[1]).
// dnew non-null: also e there (the increment record of an accepted start,
// which pass 0's residual kernel writes when it runs)
__global__ void __launch_bounds__(RB) k_ws_build_ext(Grid g, const float* __restrict__ d1,
                                                     const float* __restrict__ d2, float a, float b,
                                                     float* __restrict__ e, double* dsc,
                                                     const float* ab = nullptr, float* __restrict__ dnew = nullptr) {
    if (ab) {
        a = ab[0];
        b = ab[1];
    }
    // the two scales are sums of squares of FP32 data: FP32 per thread (a few
    // hundred terms), FP64 across threads, no FP64 work per cell
    float s2 = 0.f, q2 = 0.f;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        const float v1 = d1[n], v2 = d2[n];
        const float ev = __fmaf_rn(a, v1, __fmul_rn(b, v2));
        e[n] = ev;
        if (dnew) dnew[n] = ev;
        s2 = __fmaf_rn(v1, v1, s2);
        const float dd = v1 - v2;
        q2 = __fmaf_rn(dd, dd, q2);
    }
    block_add((double)s2, dsc + S_WSS2);
    block_add((double)q2, dsc + S_WSD2);
}

template <typename R>
__device__ __forceinline__ R apply_l0(const R* __restrict__ cx, const R* __restrict__ cy,
                                      const R* __restrict__ cz, const R* __restrict__ diag,
                                      const float* __restrict__ e, long long n, long long sy, long long sz) {
    return diag[n] * from_f32<R>(e[n]) -
           (cx[n] * from_f32<R>(e[n + 1]) + cx[n - 1] * from_f32<R>(e[n - 1]) + cy[n] * from_f32<R>(e[n + sy]) +
            cy[n - sy] * from_f32<R>(e[n - sy]) + cz[n] * from_f32<R>(e[n + sz]) +
            cz[n - sz] * from_f32<R>(e[n - sz]));
}

// The least-squares start (the default; WPF_SOLVER_FIXED_START keeps the
// fixed coefficients): the five dots of min_{a,b} ||r - A'(a d1 + b d2)||, r
// the kept FP64 residual of p under this step's transmissibilities, A' the
// level-0 operator; A'd1 and A'd2 formed on the fly, one pass.  r and A'd are
// scaled by a power of two s (from the last step's ||b||, so that they are
// O(1) at the tolerance's scale) and the dots accumulated in FP32 per thread,
// FP64 across threads; the solution does not depend on s.  Dirichlet cells
// carry no residual.  c non-null (the step graph): a no-op unless c->ls.
template <typename R>
__global__ void __launch_bounds__(RB) k_ws_ls_dots(Grid g, const R* __restrict__ cx, const R* __restrict__ cy,
                                                   const R* __restrict__ cz, const R* __restrict__ diag,
                                                   const uint8_t* __restrict__ fl, const float* __restrict__ d1,
                                                   const float* __restrict__ d2, const double* __restrict__ rk,
                                                   const StepCtl* c, double scale, double* dsc) {
    if (c && !c->ls) return;
    const double s = c ? dsc[S_LSSCALE] : scale;
    const float sf = (float)s;
    const long long sy = g.P, sz = g.S;
    float ra = 0.f, rb = 0.f, aa = 0.f, ab = 0.f, bb = 0.f, rr = 0.f;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        if (fl[n] & F_DIR) continue;
        const float u = to_f32<R>(apply_l0(cx, cy, cz, diag, d1, n, sy, sz)) * sf;
        const float v = to_f32<R>(apply_l0(cx, cy, cz, diag, d2, n, sy, sz)) * sf;
        const float r = f64_to_f32(rk[n] * s);
        ra = fmaf(r, u, ra);
        rb = fmaf(r, v, rb);
        aa = fmaf(u, u, aa);
        ab = fmaf(u, v, ab);
        bb = fmaf(v, v, bb);
        rr = fmaf(r, r, rr);
    }
    block_add((double)ra, dsc + S_LS0);
    block_add((double)rb, dsc + S_LS0 + 1);
    block_add((double)aa, dsc + S_LS0 + 2);
    block_add((double)ab, dsc + S_LS0 + 3);
    block_add((double)bb, dsc + S_LS0 + 4);
    block_add((double)rr, dsc + S_LS0 + 5);
}

// The 2x2 normal equations of the least-squares start; a one-direction fit
// when d2 adds nothing to d1, and the given (a, b) kept when neither fits.
__host__ __device__ inline void ws_ls_solve(const double* m, float* a, float* b) {
    const double ra = m[0], rb = m[1], aa = m[2], ab = m[3], bb = m[4];
    const double det = aa * bb - ab * ab;
    if (aa > 0.0 && bb > 0.0 && det > 1e-6 * aa * bb && det == det && ra == ra && rb == rb) {
        *a = (float)((ra * bb - rb * ab) / det);
        *b = (float)((aa * rb - ab * ra) / det);
    } else if (aa > 0.0 && ra == ra) {
        *a = (float)(ra / aa);
        *b = 0.f;
    }
}
// ||r(p) - A'(a d1 + b d2)||^2 from the dots (scaled like them)
__host__ __device__ inline double ws_ls_predict(const double* m, double a, double b) {
    return m[5] - 2.0 * (a * m[0] + b * m[1]) + a * a * m[2] + 2.0 * a * b * m[3] + b * b * m[4];
}
// The predicted start residual at or below LS_SKIP rtol ||b|| (with the last
// step's ||b||) skips pass 0's residual kernel: the start is accepted on the
// prediction and the plain FP64 verification pass decides as always.
constexpr double LS_SKIP = 0.8;

// Whether the least-squares start is taken this step: when the previous
// pressure's residual under the new T (the last pass 0's record) is below
// LS_WINDOW rtol.  Measured at 256^3 (time-steps/s, least-squares start
// always / below 100 rtol / below 10 rtol): kwh 10^3 early in the run, p at
// ~46 rtol, 329.5 / 329.4 / 292.1; late, p at ~1.7 rtol, 363.5 / 362.9 /
// 355.2; kwh 20 early, p at ~390 rtol, 314.7 / 339.8 / 339.5 (the fit
// costs its pass and saves no iteration there); kwh 20 late, p at ~30 rtol,
// 336.6 / 336.6 / 264.4.  And the power of two that brings values of the
// size rtol ||b|| / sqrt(cells) to ~1.
constexpr double LS_WINDOW = 100.0;
__host__ __device__ inline bool ws_ls_wanted(double rp_rel, double bnorm_prev, double rtol) {
    return rp_rel > 0.0 && rp_rel < LS_WINDOW * rtol && bnorm_prev > 0.0;
}
__host__ __device__ inline double ws_ls_scale(double bnorm_prev, double rtol, long long cells) {
    const double v = bnorm_prev * rtol / sqrt((double)(cells > 0 ? cells : 1));
    int e = (v > 0.0 && v == v) ? ilogb(v) : 0;
    e = e < -100 ? -100 : (e > 100 ? 100 : e);
    return ldexp(1.0, -e);
}
__global__ void k_ctl_ls_begin(StepCtl* c, double* dsc, double rtol, long long cells) {
    if (threadIdx.x) return;
    c->ls = ws_ls_wanted(c->rp_rel, c->bnorm_prev, rtol) ? 1 : 0;
    c->ls_skip = 0;
    dsc[S_LSSCALE] = ws_ls_scale(c->bnorm_prev, rtol, cells);
}
// (rtol < 0: never skip)
__global__ void k_ctl_ws_ls(StepCtl* c, double* dsc, double rtol) {
    if (threadIdx.x || !c->ls) return;
    ws_ls_solve(dsc + S_LS0, &c->wa, &c->wb);
    const double s = dsc[S_LSSCALE], bn = c->bnorm_prev;
    const double pred = fmax(ws_ls_predict(dsc + S_LS0, c->wa, c->wb), 0.0) / (s * s);
    if (sqrt(pred) <= LS_SKIP * rtol * bn) {   // the norms pass 0 would have given
        c->ls_skip = 1;
        dsc[S_RR64] = pred;
        dsc[S_RR0WS] = dsc[S_LS5] / (s * s);
        dsc[S_BB64] = bn * bn;
    }
}

// Pass-0 residual of the start p + e_ext: r0 = r(p) in FP64 exactly as
// k_resid64 (||r0||^2 into S_RR0WS, ||b_ref||^2 into S_BB64), then
// r_ext = r0 - A'e_ext with A'e from the level-0 coefficients in precision R
// (e is a small increment, so its rounding stays orders of magnitude below the
// outer tolerance); writes rout = r_ext, dnew = e_ext, ||r_ext||^2 into S_RR64.
// With D (the mixed form) r_ext is formed in R from r0 rounded to R: its
// relative error, ~1e-7 |r0| / |r_ext|, only perturbs the right-hand side of
// the first correction, and the pass that accepts the solve always takes a
// plain FP64 residual.  With rk_in, r0 is read from the kept FP64 residual
// (the last pass's, corrected for this step's change of T by calcPermeability)
// instead of being recomputed.
template <typename R, bool KEPT>
__global__ void __launch_bounds__(RB) k_resid64_ws(Grid g, const double* __restrict__ pr,
                                                   const double* __restrict__ Tx,
                                                   const double* __restrict__ Ty,
                                                   const double* __restrict__ Tz,
                                                   const uint8_t* __restrict__ fl,
                                                   const double* __restrict__ qterm,
                                                   const double* __restrict__ D,
                                                   const R* __restrict__ cx, const R* __restrict__ cy,
                                                   const R* __restrict__ cz,
                                                   const R* __restrict__ diag,
                                                   const float* __restrict__ e1,
                                                   R* __restrict__ rout, float* __restrict__ dnew,
                                                   double* dsc, const double* __restrict__ rk_in = nullptr,
                                                   const int* skip = nullptr) {
    if (skip && *skip) return;   // the least-squares start's prediction stands in (k_ctl_ws_ls)
    double rr1 = 0.0, rr0 = 0.0, bb = 0.0;
    R rr1r = 0;   // the same sum in R (with D)
    float rr0f = 0.f;               // ||r(p)||^2 in FP32 on the kept path (only the fallback test reads it)
    const long long sy = g.P, sz = g.S;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        const uint8_t f = fl[n];
        double r0 = 0.0, r1 = 0.0;
        float e = 0.f;
        if (f & F_DIR) {
            const double p0 = pr[n];
            bb += p0 * p0;
        } else {
            const double q = qterm ? qterm[n] : 0.0;
            // b_ref differs from -q only next to a Dirichlet cell: branch on
            // the neighbour flags so that interior cells issue no FP64 there
            const uint8_t dm = (fl[n - sz] | fl[n - sy] | fl[n - 1] | fl[n + 1] | fl[n + sy] |
                                fl[n + sz]) & F_DIR;
            auto bref_add = [&](double pxp, double pxm, double pyp, double pym, double pzp, double pzm,
                                double txp, double txm, double typ, double tym, double tzp, double tzm) {
                double bref = -q;
                if (fl[n - sz] & F_DIR) bref -= pzm * tzm;
                if (fl[n - sy] & F_DIR) bref -= pym * tym;
                if (fl[n - 1] & F_DIR) bref -= pxm * txm;
                if (fl[n + 1] & F_DIR) bref -= pxp * txp;
                if (fl[n + sy] & F_DIR) bref -= pyp * typ;
                if (fl[n + sz] & F_DIR) bref -= pzp * tzp;
                bb += bref * bref;
            };
            if (KEPT) {
                // r(p) kept from the last residual pass, corrected face by
                // face for the new T: FP64 work only next to a Dirichlet cell
                r0 = rk_in[n];
                if (dm || (qterm && q != 0.0))
                    bref_add(pr[n + 1], pr[n - 1], pr[n + sy], pr[n - sy], pr[n + sz], pr[n - sz], Tx[n],
                             Tx[n - 1], Ty[n], Ty[n - sy], Tz[n], Tz[n - sz]);
            } else {
                const double p0 = pr[n];
                const double txp = Tx[n], txm = Tx[n - 1], typ = Ty[n], tym = Ty[n - sy];
                const double tzp = Tz[n], tzm = Tz[n - sz];
                const double pxp = pr[n + 1], pxm = pr[n - 1], pyp = pr[n + sy], pym = pr[n - sy];
                const double pzp = pr[n + sz], pzm = pr[n - sz];
                r0 = resid_cell(q, p0, pxp, pxm, pyp, pym, pzp, pzm, txp, txm, typ, tym, tzp, tzm, D, n);
                if (dm || q != 0.0) bref_add(pxp, pxm, pyp, pym, pzp, pzm, txp, txm, typ, tym, tzp, tzm);
            }
            e = e1[n];
            if (D) {
                const R r1r = from_f64<R>(r0) - apply_l0(cx, cy, cz, diag, e1, n, sy, sz);
                rout[n] = r1r;
                rr1r += r1r * r1r;
            } else {
                r1 = r0 - to_f64<R>(apply_l0(cx, cy, cz, diag, e1, n, sy, sz));
            }
        }
        if (!D || (f & F_DIR)) {
            rout[n] = from_f64<R>(r1);
            rr1 += r1 * r1;
        }
        dnew[n] = e;
        if (KEPT) {
            const float f0 = f64_to_f32(r0);
            rr0f = fmaf(f0, f0, rr0f);
        } else {
            rr0 += r0 * r0;
        }
    }
    rr1 += (double)rr1r;
    rr0 += (double)rr0f;
    block_add(rr1, dsc + S_RR64);
    block_add(rr0, dsc + S_RR0WS);
    block_add(bb, dsc + S_BB64);
}

// Accept the learned correction with step alpha: r -= alpha A'e_net,
// dnew += alpha e_net.
template <typename R>
__global__ void __launch_bounds__(RB) k_ws_take_net(Grid g, const R* __restrict__ cx, const R* __restrict__ cy,
                                                    const R* __restrict__ cz, const R* __restrict__ diag,
                                                    const uint8_t* __restrict__ fl, float alpha,
                                                    const float* __restrict__ e2, R* __restrict__ r,
                                                    float* __restrict__ dnew) {
    const long long sy = g.P, sz = g.S;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        dnew[n] += alpha * e2[n];
        if (!(fl[n] & F_DIR)) r[n] -= (R)alpha * apply_l0(cx, cy, cz, diag, e2, n, sy, sz);
    }
}

// The learned correction against the extrapolated start's residual: with
// w = A'e_net, r_ext.w into S_RW and w.w into S_WW (per thread in precision
// R, across threads in FP64), from which alpha = r.w / w.w, the step that
// minimises ||r_ext - alpha w||.
template <typename R>
__global__ void __launch_bounds__(RB) k_net_dots(Grid g, const R* __restrict__ cx, const R* __restrict__ cy,
                                                 const R* __restrict__ cz, const R* __restrict__ diag,
                                                 const uint8_t* __restrict__ fl, const float* __restrict__ e2,
                                                 const R* __restrict__ r, double* dsc,
                                                 float* __restrict__ aw = nullptr) {
    const long long sy = g.P, sz = g.S;
    R rw = 0, ww = 0, waw = 0;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        if (fl[n] & F_DIR) {
            if (aw) aw[n] = 0.f;
            continue;
        }
        const R w = apply_l0(cx, cy, cz, diag, e2, n, sy, sz);
        if (aw) aw[n] = to_f32<R>(w);   // A'e_net for the deflated PCG
        rw += r[n] * w;
        ww += w * w;
        waw += (R)e2[n] * w;
    }
    block_add((double)rw, dsc + S_RW);
    block_add((double)ww, dsc + S_WW);
    block_add((double)waw, dsc + S_WAW);   // the learned coarse space's operator
}

// p += e (e1 [+ alpha e2]: the accepted start, added once, when e1 != null)
// + x (the pass's correction, when x != null); dnew accumulates x, so that
// after the last pass it holds this solve's whole increment.
template <typename R>
__global__ void __launch_bounds__(RB) k_add_correction_ws(Grid g, double* __restrict__ pr,
                                                          const R* __restrict__ x,
                                                          const float* __restrict__ e1,
                                                          const float* __restrict__ e2, float alpha,
                                                          float* __restrict__ dnew) {
    ROW_LOOP_U4(g) {
        const long long n = g.at(i, j, k);
        double inc = x ? to_f64<R>(x[n]) : 0.0;
        if (e1) inc += f32_to_f64(e2 ? e1[n] + alpha * e2[n] : e1[n]);
        pr[n] += inc;
        if (x) dnew[n] += to_f32<R>(x[n]);
    }
}

// Level-0 coefficients of A' from T and the Dirichlet flags.
template <typename R>
__global__ void __launch_bounds__(RB) k_l0_coeffs(Grid g, const double* __restrict__ Tx,
                                                  const double* __restrict__ Ty,
                                                  const double* __restrict__ Tz,
                                                  const uint8_t* __restrict__ fl,
                                                  R* __restrict__ cx, R* __restrict__ cy,
                                                  R* __restrict__ cz, R* __restrict__ diag,
                                                  R* __restrict__ idiag, double* __restrict__ dsum,
                                                  uint8_t* __restrict__ mark) {
    const long long sy = g.P, sz = g.S;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        if (mark) {   // incremental: only the cells with a recomputed face
            if (!mark[n]) continue;
            mark[n] = 0;
        }
        const bool live = !(fl[n] & F_DIR);
        const R tx = from_f64<R>(Tx[n]), ty = from_f64<R>(Ty[n]), tz = from_f64<R>(Tz[n]);
        cx[n] = (live && !(fl[n + 1] & F_DIR)) ? tx : (R)0;
        cy[n] = (live && !(fl[n + sy] & F_DIR)) ? ty : (R)0;
        cz[n] = (live && !(fl[n + sz] & F_DIR)) ? tz : (R)0;
        R d;
        if (dsum) {
            // the FP64 diagonal of the outer residual's operator (its
            // diagonal-sum form), from which the R diagonal is rounded
            const double D = live ? Tx[n] + Tx[n - 1] + Ty[n] + Ty[n - sy] + Tz[n] + Tz[n - sz] : 0.0;
            dsum[n] = D;
            d = from_f64<R>(D);
        } else {
            // each face converted once, the six summed in R: the R operator only
            // needs R accuracy (the outer residual is FP64)
            d = tx + from_f64<R>(Tx[n - 1]) + ty + from_f64<R>(Ty[n - sy]) + tz + from_f64<R>(Tz[n - sz]);
        }
        const R dr = live ? d : (R)0;
        diag[n] = dr;
        idiag[n] = (live && dr > (R)0) ? (R)1 / dr : (R)0;
    }
}

// Coarse operator of level l+1 from level l (see the file header).
template <typename R>
__global__ void k_coarsen(Grid f, Grid c, const R* __restrict__ fcx, const R* __restrict__ fcy,
                          const R* __restrict__ fcz, const R* __restrict__ fdiag, R* __restrict__ ccx,
                          R* __restrict__ ccy, R* __restrict__ ccz, R* __restrict__ cdiag,
                          R* __restrict__ cidiag, R scale) {
    const int I = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int J = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int K = 1 + blockIdx.z * blockDim.z + threadIdx.z;
    if (I > c.nx || J > c.ny || K > c.nz) return;
    R D = 0, Cx = 0, Cy = 0, Cz = 0;
    for (int dk = 0; dk < 2; ++dk) {
        const int k = 2 * K - 1 + dk;
        if (k > f.nz) break;
        for (int dj = 0; dj < 2; ++dj) {
            const int j = 2 * J - 1 + dj;
            if (j > f.ny) break;
            for (int di = 0; di < 2; ++di) {
                const int i = 2 * I - 1 + di;
                if (i > f.nx) break;
                const long long n = f.at(i, j, k);
                D += fdiag[n];
                // couplings leaving the aggregate on the + side; internal ones cancel
                if (di == 1) Cx += fcx[n]; else if (i + 1 <= f.nx) D -= 2 * fcx[n];
                if (dj == 1) Cy += fcy[n]; else if (j + 1 <= f.ny) D -= 2 * fcy[n];
                if (dk == 1) Cz += fcz[n]; else if (k + 1 <= f.nz) D -= 2 * fcz[n];
            }
        }
    }
    const long long m = c.at(I, J, K);
    // the + face of the last (single-child) aggregate in a direction is a boundary face
    ccx[m] = (2 * I <= f.nx) ? scale * Cx : (R)0;
    ccy[m] = (2 * J <= f.ny) ? scale * Cy : (R)0;
    ccz[m] = (2 * K <= f.nz) ? scale * Cz : (R)0;
    const R d = scale * D;
    cdiag[m] = d;
    cidiag[m] = d > (R)0 ? (R)1 / d : (R)0;
}

template <typename R>
__device__ __forceinline__ R offsum(const R* __restrict__ cx, const R* __restrict__ cy,
                                    const R* __restrict__ cz, const R* __restrict__ x, long long n,
                                    long long sy, long long sz) {
    return cx[n] * x[n + 1] + cx[n - 1] * x[n - 1] + cy[n] * x[n + sy] + cy[n - sy] * x[n - sy] +
           cz[n] * x[n + sz] + cz[n - sz] * x[n - sz];
}

// ---------------------------------------------------------------------------
// Pipelined red-black sweep for the large levels.  Block = 32x8 threads, tile
// = 32x8 cells of a plane, z chunk of szc planes.  Shared memory holds NSLOT
// plane slots; each slot carries x on the tile + 2-cell ring and the
// couplings / 1/diag / b on the tile + 1-cell ring, filled by cp.async
// (4- or 8-byte async copies, zero-filled outside the halo box) two planes
// ahead of use, so the compute phases read only shared memory.
// ---------------------------------------------------------------------------
constexpr int NSLOT = 7;
constexpr int R1X = SX + 2, R1Y = SY + 2;   // first-colour region: tile + 1-cell ring
constexpr int WX = SX + 8;                  // staged row: i in [i0-4, i0+SX+3], 16-byte aligned

// Each array starts on a 128-byte boundary: the bulk-tensor copies write
// whole boxes there.
template <typename R>
struct alignas(128) SweepSlot {
    alignas(128) R x[FY][WX];         // rows j in [j0-2, j0+SY+1]
    alignas(128) R cx[R1Y][WX];       // rows j in [j0-1, j0+SY]
    alignas(128) R cy[R1Y + 1][WX];   // rows j in [j0-2, j0+SY]
    alignas(128) R cz[R1Y][WX];
    alignas(128) R id[R1Y][WX];
    alignas(128) R b[R1Y][WX];
};
constexpr int SLOT_ROWS = FY + R1Y + (R1Y + 1) + 3 * R1Y;   // 63 staged rows per plane

// element offset in a slot of staged row `row` (rows numbered x, cx, cy, cz, id, b)
template <typename R>
__device__ __forceinline__ int slot_row_offset(int row) {
    typedef SweepSlot<R> S;
    if (row < FY) return (int)(offsetof(S, x) / sizeof(R)) + row * WX;
    row -= FY;
    if (row < R1Y) return (int)(offsetof(S, cx) / sizeof(R)) + row * WX;
    row -= R1Y;
    if (row < R1Y + 1) return (int)(offsetof(S, cy) / sizeof(R)) + row * WX;
    row -= R1Y + 1;
    if (row < R1Y) return (int)(offsetof(S, cz) / sizeof(R)) + row * WX;
    row -= R1Y;
    if (row < R1Y) return (int)(offsetof(S, id) / sizeof(R)) + row * WX;
    return (int)(offsetof(S, b) / sizeof(R)) + (row - R1Y) * WX;
}

// SweepMaps (wpf_internal.cuh): the x input (12-row boxes), cx / cz / 1/diag /
// b (10-row boxes) and cy (11-row boxes), each box WX elements wide; 3-D
// tensors (P, ny+2, nz+2) over the pitched arrays.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(map), "r"(x), "r"(y), "r"(z),
        "r"((unsigned)__cvta_generic_to_shared(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                     (unsigned)__cvta_generic_to_shared(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    for (int it = 0; it < (1 << 20); ++it) {
        unsigned done;
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

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool ok) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem),
                 "r"(ok ? 16 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// ZERO: xin is zero (first pre-smoothing sweep).  dot != null: accumulate
// b.xout.  (The coarse correction before the first post-sweep is a separate
// k_prolong4 pass on the input buffer: added here, per thread on its staged x
// chunks with scattered reads of the coarse level, it made that sweep 45 %
// slower than the others for less than half that as a separate pass.)
// Every staged row is a 16-byte aligned window of WX elements starting at
// i = i0 - 4 (XOFF and the pitches make at(i0-4, j, k) a multiple of 4
// elements).  TMA: one thread stages a plane with five or six bulk-tensor
// copies that complete on the slot's mbarrier (zero fill outside the halo
// box); otherwise each thread owns fixed 16-byte chunks of the slot and
// copies them with cp.async, its addresses precomputed once and advanced by
// one plane stride per plane.
template <typename R, bool ZERO, bool TMA>
__global__ void __launch_bounds__(SX * SY) k_sweep_async(Grid g, const R* __restrict__ cx,
                                                         const R* __restrict__ cy,
                                                         const R* __restrict__ cz,
                                                         const R* __restrict__ idiag,
                                                         const R* __restrict__ b,
                                                         const R* __restrict__ xin,
                                                         R* __restrict__ xout, int c0,
                                                         double* dot,
                                                         const __grid_constant__ SweepMaps maps,
                                                         int* err, int szc) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t mbar[NSLOT];
    // slots on a 128-byte boundary whatever the dynamic window's base (the
    // allocation carries 128 spare bytes)
    const unsigned mis = (unsigned)__cvta_generic_to_shared(smem_raw) & 127u;
    SweepSlot<R>* slots = reinterpret_cast<SweepSlot<R>*>(smem_raw + (mis ? 128u - mis : 0u));
    if (TMA) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            for (int q = 0; q < NSLOT; ++q)
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
                                 (unsigned)__cvta_generic_to_shared(&mbar[q]))
                             : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
    }
    bool wait_ok = true;
    constexpr int NT = SX * SY;
    constexpr int EPC = 16 / sizeof(R);               // elements per 16-byte chunk
    constexpr int CPR = WX / EPC;                     // chunks per staged row
    constexpr int NCH = SLOT_ROWS * CPR;              // chunks per plane
    constexpr int MAXC = (NCH + NT - 1) / NT;         // chunks per thread
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * SX + tx;
    const int i0 = 1 + blockIdx.x * SX, j0 = 1 + blockIdx.y * SY;
    const int k0 = 1 + blockIdx.z * szc;
    const int k1 = min(g.nz, k0 + szc - 1);
    R dacc = 0;

    // this thread's chunks: source array, row offset (plane 0), smem offset, row j
    const R* csrc[MAXC];
    long long coff[MAXC];
    int csm[MAXC];
    bool cx_ok[MAXC], cis_x[MAXC];
#pragma unroll
    for (int s = 0; s < MAXC; ++s) {
        const int q = tid + s * NT;
        csrc[s] = nullptr;
        coff[s] = 0;
        csm[s] = 0;
        cx_ok[s] = false;
        cis_x[s] = false;
        if (q >= NCH) continue;
        const int row = q / CPR, ch = q - row * CPR;
        int j, srow;
        const R* src;
        if (row < FY) { src = xin; j = j0 - 2 + row; srow = row; cis_x[s] = true; }
        else if (row < FY + R1Y) { src = cx; j = j0 - 1 + (row - FY); srow = row; }
        else if (row < FY + 2 * R1Y + 1) { src = cy; j = j0 - 2 + (row - FY - R1Y); srow = row; }
        else {
            const int r3 = row - (FY + 2 * R1Y + 1);
            const int which = r3 / R1Y;
            src = which == 0 ? cz : (which == 1 ? idiag : b);
            j = j0 - 1 + (r3 - which * R1Y);
            srow = row;
        }
        const int e0 = i0 - 4 + ch * EPC;
        csrc[s] = src;
        cx_ok[s] = j >= 0 && j <= g.ny + 1 && e0 <= g.nx + 1;
        coff[s] = XOFF + (long long)j * g.P + e0;
        csm[s] = slot_row_offset<R>(srow) + ch * EPC;
    }
    auto slot_index = [&](int k) { return (k + 2 * NSLOT) % NSLOT; };
    auto slot_base = [&](int k) -> R* { return reinterpret_cast<R*>(&slots[slot_index(k)]); };
    auto slot = [&](int k) -> SweepSlot<R>& { return slots[slot_index(k)]; };
    auto issue = [&](int k) {
        R* base = slot_base(k);
        if (TMA) {
            // the zero-guess sweep stages no x: its rows are zeroed here
            if (ZERO) {
#pragma unroll
                for (int s = 0; s < MAXC; ++s)
                    if (cis_x[s]) {
#pragma unroll
                        for (int e = 0; e < EPC; ++e) base[csm[s] + e] = 0;
                    }
            }
            if (tid == 0) {
                SweepSlot<R>& S = slots[slot_index(k)];
                uint64_t* bar = &mbar[slot_index(k)];
                constexpr unsigned rowb = WX * sizeof(R);
                mbar_expect(bar, rowb * (ZERO ? (SLOT_ROWS - FY) : SLOT_ROWS));
                const int x0 = XOFF + i0 - 4;
                if (!ZERO) tma_load_3d(&S.x[0][0], &maps.x, x0, j0 - 2, k, bar);
                tma_load_3d(&S.cx[0][0], &maps.cx, x0, j0 - 1, k, bar);
                tma_load_3d(&S.cy[0][0], &maps.cy, x0, j0 - 2, k, bar);
                tma_load_3d(&S.cz[0][0], &maps.cz, x0, j0 - 1, k, bar);
                tma_load_3d(&S.id[0][0], &maps.id, x0, j0 - 1, k, bar);
                tma_load_3d(&S.b[0][0], &maps.b, x0, j0 - 1, k, bar);
            }
            return;
        }
        const bool kok = k >= 0 && k <= g.nz + 1;
#pragma unroll
        for (int s = 0; s < MAXC; ++s) {
            if (!csrc[s] && !(ZERO && cis_x[s])) continue;
            if (ZERO && cis_x[s]) {
                R* d = base + csm[s];
#pragma unroll
                for (int e = 0; e < EPC; ++e) d[e] = 0;
                continue;
            }
            const bool ok = kok && cx_ok[s];
            const R* src = ok ? csrc[s] + coff[s] + (long long)k * g.S : csrc[s];
            cp_async16(base + csm[s], src, ok);
        }
        cp_async_commit();
    };
    // plane k staged (TMA: the fill number of its slot gives the phase parity);
    // after one wait has run out the block stops waiting and reports it
    auto landed = [&](int k) {
        if (!wait_ok) return;
        if (!mbar_wait_bounded(&mbar[slot_index(k)], (unsigned)(((k - (k0 - 2)) / NSLOT) & 1))) wait_ok = false;
    };
    // Updated value of the cell at slot column w, slot row c (R1 row) of plane
    // k; neighbours = false when they are all known to be zero (first colour
    // of the zero-guess sweep).
    auto relax = [&](const SweepSlot<R>& S, const SweepSlot<R>& Sm, const SweepSlot<R>& Sp, int c,
                     int w, bool neighbours) -> R {
        R s = S.b[c][w];
        if (neighbours)
            s += S.cx[c][w] * S.x[c + 1][w + 1] + S.cx[c][w - 1] * S.x[c + 1][w - 1] +
                 S.cy[c + 1][w] * S.x[c + 2][w] + S.cy[c][w] * S.x[c][w] +
                 S.cz[c][w] * Sp.x[c + 1][w] + Sm.cz[c][w] * Sm.x[c + 1][w];
        return S.id[c][w] * s;
    };
    // Per-thread constants of the three compute phases (the colour of a cell
    // flips with the plane parity only).
    // First colour of a plane on the tile + ring: thread t < 17*R1Y takes the
    // m-th cell of that colour in R1 row c (every other cell of the row).
    constexpr int PF = R1X / 2;
    const bool f_on = tid < PF * R1Y;
    const int fc = f_on ? tid / PF : 0, fm = tid - fc * PF;
    const int fj = j0 - 1 + fc;
    const int fpar = (c0 - (i0 - 1) - fj) & 1;
    const bool fj_ok = f_on && fj >= 1 && fj <= g.ny;
    // Second colour of a plane on the tile: thread t < 16*SY takes the m-th
    // cell of that colour in tile row r; the values stay in shared memory.
    // (the last PS*SY threads: with the pipelined order of the TMA path the two
    // colours share a phase, and 42 threads then take one cell of each)
    constexpr int PS = SX / 2;
    const int stid = tid - (NT - PS * SY);
    const bool s_on = stid >= 0;
    const int sr = s_on ? stid / PS : 0, sm2 = stid - sr * PS;
    const int sj = j0 + sr;
    const int spar = (c0 + 1 - i0 - sj) & 1;
    const bool sj_ok = s_on && sj <= g.ny;
    // the coalesced store of a finished tile: one cell per thread
    const bool w_on = i0 + tx <= g.nx && j0 + ty <= g.ny;
    R* const wptr = xout + g.at(i0 + tx, j0 + ty, 0);

    auto first_colour = [&](int k, SweepSlot<R>& S, const SweepSlot<R>& Sm, const SweepSlot<R>& Sp) {
        if (!fj_ok || k < 1 || k > g.nz) return;
        const int a = 2 * fm + ((fpar - k) & 1);
        const int i = i0 - 1 + a;
        if (i < 1 || i > g.nx) return;
        S.x[fc + 1][a + 3] = relax(S, Sm, Sp, fc, a + 3, !ZERO);
    };
    auto second_colour = [&](int k, SweepSlot<R>& S, const SweepSlot<R>& Sm, const SweepSlot<R>& Sp) {
        if (!sj_ok) return;
        const int i = i0 + 2 * sm2 + ((spar - k) & 1);
        if (i > g.nx) return;
        const int w = i - i0 + 4;
        S.x[sr + 2][w] = relax(S, Sm, Sp, sr + 1, w, true);
    };
    auto write_out = [&](int k, const SweepSlot<R>& S) {
        if (!w_on) return;
        const R v = S.x[ty + 2][tx + 4];
        wptr[(long long)k * g.S] = v;
        if (dot) dacc += S.b[ty + 1][tx + 4] * v;
    };

    for (int k = k0 - 2; k <= k0 + 3; ++k) issue(k);
    if (TMA) {
        for (int k = k0 - 2; k <= k0 + 1; ++k) landed(k);
    } else {
        cp_async_wait<2>();                   // planes k0-2 .. k0+1 landed
    }
    __syncthreads();
    first_colour(k0 - 1, slot(k0 - 1), slot(k0 - 2), slot(k0));
    __syncthreads();
    first_colour(k0, slot(k0), slot(k0 - 1), slot(k0 + 1));
    int sk = slot_index(k0);                  // slot of plane k, advanced by one per plane
    if (TMA) {
        // One phase and one block barrier per plane: the first colour of plane
        // k+1 and the second colour of plane k-1 share a phase.  The first
        // colour reads only old second-colour values (planes k..k+2), which
        // the second colour of plane k-1 does not write; the second colour of
        // k-1 reads the first colours of planes k-2..k, finished before the
        // last barrier.  Live planes k-2..k+2 plus two in flight fill the
        // seven slots; the copies of plane k+4 go to the slot of plane k-3,
        // whose last readers (second colour of k-2, write-out of k-3) and
        // fenced writers finished before the last barrier.  Every thread
        // waits on the plane's mbarrier itself, which makes the landed copies
        // visible to it.
        for (int k = k0; k <= k1 + 1; ++k) {
            const int skm1 = sk == 0 ? NSLOT - 1 : sk - 1;
            const int skm2 = skm1 == 0 ? NSLOT - 1 : skm1 - 1;
            const int skp1 = sk == NSLOT - 1 ? 0 : sk + 1;
            const int skp2 = skp1 == NSLOT - 1 ? 0 : skp1 + 1;
            fence_proxy_async();              // this thread's generic accesses before the next copies
            if (k <= k1) {
                issue(k + 4);
                landed(k + 2);
            }
            if (k - 2 >= k0) write_out(k - 2, slots[skm2]);
            if (k <= k1) first_colour(k + 1, slots[skp1], slots[sk], slots[skp2]);
            if (k - 1 >= k0) second_colour(k - 1, slots[skm1], slots[skm2], slots[sk]);
            __syncthreads();
            sk = skp1;
        }
    } else {
        for (int k = k0; k <= k1; ++k) {
            const int skm1 = sk == 0 ? NSLOT - 1 : sk - 1;
            const int skp1 = sk == NSLOT - 1 ? 0 : sk + 1;
            const int skp2 = skp1 == NSLOT - 1 ? 0 : skp1 + 1;
            issue(k + 4);                     // the slot of plane k-3, idle since k-2
            cp_async_wait<2>();               // plane k+2 landed
            __syncthreads();
            if (k > k0) write_out(k - 1, slots[skm1]);
            first_colour(k + 1, slots[skp1], slots[sk], slots[skp2]);
            __syncthreads();
            second_colour(k, slots[sk], slots[skm1], slots[skp1]);
            sk = skp1;
        }
        __syncthreads();
    }
    write_out(k1, slot(k1));
    if (TMA) {   // the copies still in flight land before the block exits
        landed(k1 + 3);
        landed(k1 + 4);
        if (!wait_ok && err) atomicExch(err, 1);
    } else {
        cp_async_wait<0>();
    }
    if (dot) block_add(dacc, dot);
}

template <typename R>
constexpr size_t sweep_smem() { return sizeof(SweepSlot<R>) * NSLOT + 128; }

// One colour of red-black Gauss-Seidel in place (mid-size levels).  Thread
// (t,j,k) handles the cell of colour `color` at i = 1 + 2t + ((color+1+j+k) & 1).
template <typename R>
__global__ void k_rbgs(Grid g, const R* __restrict__ cx, const R* __restrict__ cy,
                       const R* __restrict__ cz, const R* __restrict__ idiag, R* __restrict__ x,
                       const R* __restrict__ b, int color) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int k = 1 + blockIdx.z * blockDim.z + threadIdx.z;
    const int i = 1 + 2 * t + ((color + 1 + j + k) & 1);
    if (i > g.nx || j > g.ny || k > g.nz) return;
    const long long n = g.at(i, j, k);
    x[n] = idiag[n] * (b[n] + offsum(cx, cy, cz, x, n, g.P, g.S));
}

// First red sweep from a zero initial guess: red cells get idiag*b, black 0.
template <typename R>
__global__ void k_rbgs_first(Grid g, const R* __restrict__ idiag, R* __restrict__ x,
                             const R* __restrict__ b) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int k = 1 + blockIdx.z * blockDim.z + threadIdx.z;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    const long long n = g.at(i, j, k);
    x[n] = ((i + j + k) & 1) ? (R)0 : idiag[n] * b[n];
}

// x_l += x_{l+1}(parent) on live cells, four cells of a row per thread:
// at(1 + 4q, j, k) is a multiple of 4 elements (XOFF + 1 = 16, pitches
// multiples of 16), so the FP32 form moves 16-byte vectors; the four cells
// take two coarse values.  Rows are walked with the x chunk fastest, so a warp
// streams whole rows.
template <typename R>
__global__ void __launch_bounds__(256) k_prolong4(Grid f, Grid c, const R* __restrict__ idiag,
                                                  R* __restrict__ x, const R* __restrict__ xc) {
    const int nq = (f.nx + 3) >> 2;
    const long long total = (long long)nq * f.ny * f.nz;
    for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < total; t += (long long)gridDim.x * 256) {
        const long long r = t / nq;
        const int q = (int)(t - r * nq);
        const int j = 1 + (int)(r % f.ny), k = 1 + (int)(r / f.ny);
        const int i = 1 + 4 * q;
        const long long n = f.at(i, j, k);
        const R* crow = xc + c.at(0, (j + 1) >> 1, (k + 1) >> 1);
        const R a = crow[1 + 2 * q];
        if constexpr (sizeof(R) == 4) {
            if (i + 3 <= f.nx) {
                const R b = crow[2 + 2 * q];
                const float4 d = *reinterpret_cast<const float4*>(idiag + n);
                float4 v = *reinterpret_cast<float4*>(x + n);
                if (d.x != 0.f) v.x += a;
                if (d.y != 0.f) v.y += a;
                if (d.z != 0.f) v.z += b;
                if (d.w != 0.f) v.w += b;
                *reinterpret_cast<float4*>(x + n) = v;
                continue;
            }
        }
        for (int e = 0; e < 4 && i + e <= f.nx; ++e) {
            const R v = e < 2 ? a : crow[2 + 2 * q];
            if (idiag[n + e] != (R)0) x[n + e] += v;
        }
    }
}

template <typename R>
static void launch_prolong(wpf_handle* h, const Grid& f, const Grid& c, const R* idiag, R* x, const R* xc,
                           cudaStream_t s) {
    const long long total = (long long)((f.nx + 3) >> 2) * f.ny * f.nz;
    const long long cap = (long long)h->nsm * 8;
    const long long blocks = (total + 255) / 256;
    WPF_LAUNCH(h, KC_MGREST, k_prolong4<R><<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(f, c, idiag, x, xc));
}

// Residual of level l restricted (summed over the aggregate) into b of level l+1.
template <typename R>
__global__ void k_resid_restrict(Grid f, Grid c, const R* __restrict__ cx, const R* __restrict__ cy,
                                 const R* __restrict__ cz, const R* __restrict__ diag,
                                 const R* __restrict__ x, const R* __restrict__ b,
                                 R* __restrict__ bc) {
    const int I = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int J = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int K = 1 + blockIdx.z * blockDim.z + threadIdx.z;
    if (I > c.nx || J > c.ny || K > c.nz) return;
    R s = 0;
    for (int dk = 0; dk < 2; ++dk) {
        const int k = 2 * K - 1 + dk;
        if (k > f.nz) break;
        for (int dj = 0; dj < 2; ++dj) {
            const int j = 2 * J - 1 + dj;
            if (j > f.ny) break;
            for (int di = 0; di < 2; ++di) {
                const int i = 2 * I - 1 + di;
                if (i > f.nx) break;
                const long long n = f.at(i, j, k);
                s += b[n] - (diag[n] * x[n] - offsum(cx, cy, cz, x, n, f.P, f.S));
            }
        }
    }
    bc[c.at(I, J, K)] = s;
}

// The coarsest levels (at most bottom_cells<R>() cells on the first of them)
// run their whole sub-cycle in one 1024-thread block, with every array of
// those levels copied into shared memory in a compact halo-free layout
// (neighbours outside the grid read as zero; their couplings are zero).
constexpr int BOTTOM_THREADS = 1024;
constexpr size_t BOTTOM_SMEM_MAX = 200 * 1024;   // bound on the staged bottom levels
template <typename R>
constexpr long long bottom_cells() { return sizeof(R) == 4 ? 4096 : 512; }

template <typename R>
struct BottomArgs {
    int l0, nlev, nu;
    Level<R> lv[MAX_LEVELS];
};

template <typename R>
struct BLevel {
    int nx, ny, nz, n, hx;   // hx = cells of one colour per row, at most
    // q / d = (q * ceil(2^32 / d)) >> 32, exact for q * d < 2^32 (here q, d < 2^13)
    unsigned long long mnx, mny, mhx;
    R *cx, *cy, *cz, *d, *id, *x, *b;
};

__host__ __device__ inline unsigned long long div_magic(unsigned d) {
    return ((1ull << 32) + d - 1) / d;
}
__device__ __forceinline__ int fdiv(int q, unsigned long long m) {
    return (int)(((unsigned long long)(unsigned)q * m) >> 32);
}

template <typename R>
__device__ __forceinline__ R b_offsum(const BLevel<R>& L, int c, int i, int j, int k) {
    const int sy = L.nx, sz = L.nx * L.ny;
    R s = 0;
    if (i + 1 < L.nx) s += L.cx[c] * L.x[c + 1];
    if (i > 0) s += L.cx[c - 1] * L.x[c - 1];
    if (j + 1 < L.ny) s += L.cy[c] * L.x[c + sy];
    if (j > 0) s += L.cy[c - sy] * L.x[c - sy];
    if (k + 1 < L.nz) s += L.cz[c] * L.x[c + sz];
    if (k > 0) s += L.cz[c - sz] * L.x[c - sz];
    return s;
}

// colour of a 0-based cell in the 1-based convention of the other kernels
__device__ __forceinline__ int b_colour(int i, int j, int k) { return (i + j + k + 1) & 1; }

// One colour of Gauss-Seidel on a staged level: thread m takes the m-th cell of
// that colour (row r = (j,k), t-th of the row).  first: the zero-guess first
// sweep, which also zeroes the other colour (x = 0 before it).
template <typename R>
__device__ __forceinline__ void b_sweep(const BLevel<R> L, int color, bool first = false) {
    const int nh = L.hx * L.ny * L.nz;
    for (int m = threadIdx.x; m < nh; m += blockDim.x) {
        const int r = fdiv(m, L.mhx), t = m - r * L.hx, k = fdiv(r, L.mny), j = r - k * L.ny;
        const int par = (color + 1 + j + k) & 1;   // b_colour(i, j, k) == color
        const int i = 2 * t + par;
        const int c = i + L.nx * r;
        if (first) {
            if (i < L.nx) L.x[c] = L.id[c] * L.b[c];
            const int io = 2 * t + (par ^ 1);
            if (io < L.nx) L.x[c - i + io] = 0;
        } else if (i < L.nx) {
            L.x[c] = L.id[c] * (L.b[c] + b_offsum(L, c, i, j, k));
        }
    }
    __syncthreads();
}

// b of level l+1 = residual of level l summed over each aggregate.
template <typename R>
__device__ __forceinline__ void b_restrict(const BLevel<R> L, const BLevel<R> C) {
    for (int q = threadIdx.x; q < C.n; q += blockDim.x) {
        const int rr = fdiv(q, C.mnx), I = q - rr * C.nx, K = fdiv(rr, C.mny), J = rr - K * C.ny;
        R s = 0;
        for (int dk = 0; dk < 2; ++dk) {
            const int k = 2 * K + dk;
            if (k >= L.nz) break;
            for (int dj = 0; dj < 2; ++dj) {
                const int j = 2 * J + dj;
                if (j >= L.ny) break;
                for (int di = 0; di < 2; ++di) {
                    const int i = 2 * I + di;
                    if (i >= L.nx) break;
                    const int c = i + L.nx * (j + L.ny * k);
                    s += L.b[c] - (L.d[c] * L.x[c] - b_offsum(L, c, i, j, k));
                }
            }
        }
        C.b[q] = s;
    }
    __syncthreads();
}

template <typename R>
__device__ __forceinline__ void b_prolong(const BLevel<R> L, const BLevel<R> C) {
    for (int c = threadIdx.x; c < L.n; c += blockDim.x) {
        const int r = fdiv(c, L.mnx), i = c - r * L.nx, k = fdiv(r, L.mny), j = r - k * L.ny;
        if (L.id[c] != (R)0) L.x[c] += C.x[(i >> 1) + C.nx * ((j >> 1) + C.ny * (k >> 1))];
    }
    __syncthreads();
}

// V-cycle over the staged levels l0..last, written as two loops (no device
// recursion, so no call stack): nu symmetric red-black sweeps around each
// coarse correction.  The coarsest level (at most 2 cells per axis) is one
// cell in the usual case, solved exactly; otherwise it gets 4 symmetric
// red-black sweep pairs from zero -- a symmetric operator, like the rest.
template <typename R>
__device__ void b_vcycle(const BLevel<R>* lv, int l0, int last, int nu) {
    for (int l = l0; l < last; ++l) {
        const BLevel<R> L = lv[l];
        b_sweep(L, 0, true);
        b_sweep(L, 1);
        for (int s = 1; s < nu; ++s) { b_sweep(L, 0); b_sweep(L, 1); }
        b_restrict(L, lv[l + 1]);
    }
    {
        const BLevel<R> L = lv[last];
        if (L.n == 1) {
            if (threadIdx.x == 0) L.x[0] = L.id[0] * L.b[0];
            __syncthreads();
        } else {
            b_sweep(L, 0, true);
            b_sweep(L, 1);
            b_sweep(L, 1);
            b_sweep(L, 0);
            for (int s = 1; s < 4; ++s) { b_sweep(L, 0); b_sweep(L, 1); b_sweep(L, 1); b_sweep(L, 0); }
        }
    }
    for (int l = last - 1; l >= l0; --l) {
        const BLevel<R> L = lv[l];
        b_prolong(L, lv[l + 1]);
        for (int s = 0; s < nu; ++s) { b_sweep(L, 1); b_sweep(L, 0); }
    }
}

template <typename R>
__global__ void __launch_bounds__(BOTTOM_THREADS) k_bottom(BottomArgs<R> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* sp = reinterpret_cast<R*>(smem_raw);
    __shared__ BLevel<R> lv[MAX_LEVELS];
    if (threadIdx.x == 0) {
        R* p = sp;
        for (int l = A.l0; l < A.nlev; ++l) {
            const Grid& g = A.lv[l].g;
            BLevel<R>& B = lv[l];
            B.nx = g.nx; B.ny = g.ny; B.nz = g.nz; B.n = g.nx * g.ny * g.nz;
            B.hx = (g.nx + 1) / 2;
            B.mnx = div_magic(g.nx);
            B.mny = div_magic(g.ny);
            B.mhx = div_magic(B.hx);
            R** arrs[7] = {&B.cx, &B.cy, &B.cz, &B.d, &B.id, &B.x, &B.b};
            for (auto a : arrs) { *a = p; p += B.n; }
        }
    }
    __syncthreads();
    for (int l = A.l0; l < A.nlev; ++l) {   // stage the operators and the top right-hand side
        const Level<R>& G = A.lv[l];
        const BLevel<R> B = lv[l];
        for (int c = threadIdx.x; c < B.n; c += blockDim.x) {
            const int r = fdiv(c, B.mnx), i = c - r * B.nx, k = fdiv(r, B.mny), j = r - k * B.ny;
            const long long n = G.g.at(i + 1, j + 1, k + 1);
            const R vx = G.cx[n], vy = G.cy[n], vz = G.cz[n], vd = G.diag[n], vi = G.idiag[n];
            const R vb = l == A.l0 ? G.b[n] : (R)0;
            B.cx[c] = vx; B.cy[c] = vy; B.cz[c] = vz; B.d[c] = vd; B.id[c] = vi;
            if (l == A.l0) B.b[c] = vb;
        }
    }
    __syncthreads();
    b_vcycle(lv, A.l0, A.nlev - 1, A.nu);
    const Level<R>& G = A.lv[A.l0];
    const BLevel<R> B = lv[A.l0];
    for (int c = threadIdx.x; c < B.n; c += blockDim.x) {
        const int r = fdiv(c, B.mnx), i = c - r * B.nx, k = fdiv(r, B.mny), j = r - k * B.ny;
        G.x[G.g.at(i + 1, j + 1, k + 1)] = B.x[c];
    }
}

template <typename R>
static size_t bottom_smem(const Hierarchy<R>& H, int l0) {
    size_t cells = 0;
    for (int l = l0; l < H.nlev; ++l) cells += (size_t)H.lv[l].g.nx * H.lv[l].g.ny * H.lv[l].g.nz;
    return cells * 7 * sizeof(R);
}

// ---- PCG vector kernels (persistent row loops, one atomic per block) -------
// p_new = z + beta p_old (beta = rz_new/rz_old, 0 when first) formed on the
// fly for the cell and its six neighbours; q = A' p_new; accumulates p_new.q.
// With `it` non-null (the device-resident loop) the iteration index comes from
// the device: first = (*it == 0), and on odd iterations pold and pnew swap
// roles, so one captured body serves every iteration.
template <typename R>
__global__ void __launch_bounds__(RB) k_apply_p(Grid g, const R* __restrict__ cx,
                                                const R* __restrict__ cy,
                                                const R* __restrict__ cz,
                                                const R* __restrict__ diag,
                                                const R* __restrict__ z,
                                                R* pold_a, R* pnew_a, R* __restrict__ q,
                                                const double* __restrict__ rz_new,
                                                const double* __restrict__ rz_old, int first_a,
                                                const int* it, double* acc,
                                                const float* __restrict__ w = nullptr,
                                                const double* __restrict__ gam = nullptr,
                                                double* wq = nullptr) {
    __shared__ R sbeta, sgam;
    __shared__ int sfirst, sodd, suse;
    if (threadIdx.x == 0) {
        int f = first_a, odd = 0;
        if (it) {
            const int v = *it;
            f = v == 0;
            odd = v & 1;
        }
        sfirst = f;
        sodd = odd;
        sbeta = f ? (R)0 : (R)(*rz_new / *rz_old);
        const double gv = (w && gam) ? *gam : __longlong_as_double(0x7ff8000000000000LL);
        suse = gv == gv;   // the learned coarse space is on (k_cc_pre)
        sgam = suse ? (R)gv : (R)0;
    }
    __syncthreads();
    const R beta = sbeta;
    const R gm = sgam;
    const bool first = sfirst, usew = suse;
    const R* __restrict__ pold = sodd ? pnew_a : pold_a;
    R* __restrict__ pnew = sodd ? pold_a : pnew_a;
    const long long sy = g.P, sz = g.S;
    R d = 0, dw = 0;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        auto P = [&](long long m) {
            R v = z[m];
            if (usew) v += gm * (R)w[m];
            return first ? v : v + beta * pold[m];
        };
        const R pc = P(n);
        const R v = diag[n] * pc - (cx[n] * P(n + 1) + cx[n - 1] * P(n - 1) + cy[n] * P(n + sy) +
                                    cy[n - sy] * P(n - sy) + cz[n] * P(n + sz) + cz[n - sz] * P(n - sz));
        pnew[n] = pc;
        q[n] = v;
        d += pc * v;
        if (usew) dw += (R)w[n] * v;
    }
    block_add(d, acc);
    if (usew && wq) block_add(dw, wq);
}

// alpha = rz/pq; x += alpha p (x = alpha p when first, unless x_set); r -= alpha q; accumulate r.r
// (it non-null: first and the p buffer from the device iteration index, as k_apply_p)
template <typename R>
__global__ void __launch_bounds__(RB) k_update_xr(Grid g, R* __restrict__ x, R* __restrict__ r,
                                                  const R* p_a, const R* p_odd,
                                                  const R* __restrict__ q,
                                                  const double* __restrict__ rz,
                                                  const double* __restrict__ pq, int first_a,
                                                  const int* it, double* acc, int x_set = 0) {
    __shared__ R salpha;
    __shared__ int sfirst, sodd;
    if (threadIdx.x == 0) {
        salpha = (R)(*rz / *pq);
        sfirst = it ? *it == 0 : first_a;
        sodd = it ? (*it & 1) : 0;
    }
    __syncthreads();
    const R alpha = salpha;
    const bool first = sfirst && !x_set;   // x_set: x holds the deflated start
    const R* __restrict__ p = sodd ? p_odd : p_a;
    R d = 0;
    ROW_LOOP_U4(g) {
        const long long n = g.at(i, j, k);
        x[n] = first ? alpha * p[n] : x[n] + alpha * p[n];
        const R rn = r[n] - alpha * q[n];
        r[n] = rn;
        d += rn * rn;
    }
    block_add(d, acc);
}

template <typename R>
__global__ void __launch_bounds__(RB) k_dot(Grid g, const R* __restrict__ a,
                                            const R* __restrict__ b, double* acc) {
    R d = 0;
    ROW_LOOP_U4(g) {
        const long long n = g.at(i, j, k);
        d += a[n] * b[n];
    }
    block_add(d, acc);
}

// ---- the learned coarse space (WPF_SOLVER_NET_COARSE) ----------------------
// Deflated PCG (Nicolaides' deflation; Saad, Yeung, Erhel and Guyomarc'h's
// deflated CG) with the one-vector coarse space w = e_net, the net's output
// on the half-resolution grid prolongated: the start takes the coarse-grid
// correction, x_0 = g0 w with g0 = w.r / w.A'w and r_0 -= g0 A'w, so that
// w.r_0 = 0, and every search direction is kept A'-orthogonal to w,
// p = z - mu w + beta p with mu = (A'w).z / w.A'w.  The residuals then stay
// orthogonal to w, and the error in the A' norm after k iterations is never
// above that of PCG without w.  (Adding w (w.r)/(w.A'w) to the cycle's
// output instead -- the additive two-level form -- raised the iteration
// count: 38 against 32 over ten 96^3 solves.)  A'w is stored by k_net_dots.
// c non-null (the step graph): active only in a step whose net ran (the IF
// node's condition); the host-driven solve launches these only then.
template <typename R>
__global__ void __launch_bounds__(RB) k_wdot(Grid g, const float* __restrict__ w, const R* __restrict__ r,
                                             const StepCtl* c, double* acc) {
    if (c && !c->net_runs) return;
    R d = 0;
    ROW_LOOP_U4(g) {
        const long long n = g.at(i, j, k);
        d += (R)w[n] * r[n];
    }
    block_add(d, acc);
}
// the deflated start: x = g0 w, r -= g0 A'w (x = 0 when the coarse space is off)
template <typename R>
__global__ void __launch_bounds__(RB) k_defl_start(Grid g, const float* __restrict__ w,
                                                   const float* __restrict__ aw, const StepCtl* c,
                                                   const double* __restrict__ dsc, R* __restrict__ x,
                                                   R* __restrict__ r) {
    __shared__ R sg0;
    if (threadIdx.x == 0) {
        const double waw = dsc[S_WAW], wr = dsc[S_WR];
        const bool on = (!c || c->net_runs) && waw > 0.0 && wr == wr;
        sg0 = on ? (R)(wr / waw) : (R)0;
    }
    __syncthreads();
    const R g0 = sg0;
    ROW_LOOP_U4(g) {
        const long long n = g.at(i, j, k);
        x[n] = g0 * (R)w[n];
        if (g0 != (R)0) r[n] -= g0 * (R)aw[n];
    }
}
// After the cycle that left z and the dot (A'w).z in S_WQ: the coefficient of
// w in p, -mu = -(A'w).z / w.A'w; NaN marks the coarse space off.
__global__ void k_cc_mu(const StepCtl* c, double* dsc) {
    if (threadIdx.x) return;
    const double waw = dsc[S_WAW], awz = dsc[S_WQ];
    const bool on = (!c || c->net_runs) && waw > 0.0 && awz == awz;
    dsc[S_GAM] = on ? -awz / waw : __longlong_as_double(0x7ff8000000000000LL);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <typename R>
static int alloc_hierarchy(wpf_handle* h, Hierarchy<R>& H) {
    if (H.nlev) return WPF_OK;
    Grid g = h->g;
    int nlev = 0;
    while (true) {
        Level<R>& L = H.lv[nlev];
        L = Level<R>();
        L.g = g;
        R** arrs[6] = {&L.cx, &L.cy, &L.cz, &L.diag, &L.idiag, &L.xs};
        for (auto a : arrs) {
            int rc = dev_alloc(h, (void**)a, sizeof(R) * g.total);
            if (rc) return rc;
        }
        if (nlev > 0) {
            int rc = dev_alloc(h, (void**)&L.x, sizeof(R) * g.total);
            if (!rc) rc = dev_alloc(h, (void**)&L.b, sizeof(R) * g.total);
            if (rc) return rc;
        }
        ++nlev;
        if ((g.nx <= 2 && g.ny <= 2 && g.nz <= 2) || nlev == MAX_LEVELS) break;
        g = make_grid((g.nx + 1) / 2, (g.ny + 1) / 2, (g.nz + 1) / 2);
    }
    H.nlev = nlev;
    R** vecs[6] = {&H.x, &H.r, &H.z, &H.p, &H.p2, &H.q};
    for (auto a : vecs) {
        int rc = dev_alloc(h, (void**)a, sizeof(R) * h->g.total);
        if (rc) return rc;
    }
    H.lv[0].b = H.r;
    H.lv[0].x = H.z;
    return WPF_OK;
}

template <typename R>
static void drop_cycles(Hierarchy<R>& H);
template <typename R>
static void free_cycle_events(Hierarchy<R>& H);

template <typename R>
static void free_hierarchy(Hierarchy<R>& H) {
    drop_cycles(H);
    free_cycle_events(H);
    for (int l = 0; l < H.nlev; ++l) {
        Level<R>& L = H.lv[l];
        cudaFree(L.cx); cudaFree(L.cy); cudaFree(L.cz); cudaFree(L.diag); cudaFree(L.idiag);
        cudaFree(L.xs);
        if (l > 0) { cudaFree(L.x); cudaFree(L.b); }
    }
    cudaFree(H.x); cudaFree(H.r); cudaFree(H.z); cudaFree(H.p); cudaFree(H.p2); cudaFree(H.q);
    H = Hierarchy<R>();
}

// The FP64 diagonal sums of the outer residual's diagonal-sum form (mixed form only).
static double* resid_dsum(wpf_handle* h) { return h->opts.mode == WPF_SOLVER_MIXED ? h->dsum : nullptr; }

// Whether the next level-0 build may rebuild only the marked cells.
bool l0_incremental(const wpf_handle* h) {
    return h->l0mark && h->l0_inc_ok && h->l0_mode == h->opts.mode;
}

template <typename R>
static void build_level0(wpf_handle* h, Hierarchy<R>& H, cudaStream_t s) {
    const Grid& g = h->g;
    Level<R>& L0 = H.lv[0];
    const bool inc = l0_incremental(h);
    if (!inc && h->l0mark) cudaMemsetAsync(h->l0mark, 0, (size_t)g.total, s);
    WPF_LAUNCH(h, KC_COEF, k_l0_coeffs<R><<<row_blocks(h, g), RB, 0, s>>>(
        g, h->T[0], h->T[1], h->T[2], h->flags, L0.cx, L0.cy, L0.cz, L0.diag, L0.idiag, resid_dsum(h),
        inc ? h->l0mark : nullptr));
    h->l0_inc_ok = h->l0mark != nullptr;
    h->l0_mode = h->opts.mode;
}

template <typename R>
static void build_coarse(wpf_handle* h, Hierarchy<R>& H, cudaStream_t s) {
    for (int l = 0; l + 1 < H.nlev; ++l) {
        Level<R>& F = H.lv[l];
        Level<R>& C = H.lv[l + 1];
        WPF_LAUNCH(h, KC_COEF, k_coarsen<R><<<cell_grid(C.g.nx, C.g.ny, C.g.nz), cell_block(), 0, s>>>(
            F.g, C.g, F.cx, F.cy, F.cz, F.diag, C.cx, C.cy, C.cz, C.diag, C.idiag, (R)COARSE_SCALE));
    }
}

template <typename R>
static int build_hierarchy(wpf_handle* h, Hierarchy<R>& H) {
    build_level0(h, H, h->stream);
    build_coarse(h, H, h->stream);
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

static dim3 sweep_grid(const Grid& g, int szc) {
    return dim3((g.nx + SX - 1) / SX, (g.ny + SY - 1) / SY, (g.nz + szc - 1) / szc);
}

template <typename R>
static void rbgs_grid(const Grid& g, dim3& gr, dim3& b) {
    b = cell_block();
    const int half = (g.nx + 1) / 2;
    gr = dim3((half + b.x - 1) / b.x, (g.ny + b.y - 1) / b.y, (g.nz + b.z - 1) / b.z);
}

static long long ncells(const Grid& g) { return (long long)g.nx * g.ny * g.nz; }
constexpr long long BIG_CELLS = 1LL << 23;   // default: levels swept by the pipelined kernel

// One preconditioner cycle z = M r (level 0 aliases b = r, x = z); rz != null
// accumulates r.z (in the last level-0 sweep when that level is a big one,
// else by a dot).  Level l recurses gamma(l) times (gamma = 2 from level
// opts.w_from_level on: a W-cycle on the mid levels; 1 above: a V-cycle),
// with symmetric smoothing around each coarse correction, so the cycle stays
// a symmetric preconditioner.  Big levels sweep between their two buffers so
// that the 2*nu sweeps end in the level's output buffer x (the first
// pre-sweep writes xs, the last post-sweep writes x); mid levels sweep x in
// place; the levels from the first one with at most bottom_cells<R>() cells
// run in one k_bottom block.
// ---- bulk-tensor maps of the sweep -------------------------------------------------
EncodeTiledFn tensor_map_encoder() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            cudaGetLastError();
    });
    return fn;
}

// 3-D map (x over the whole pitched row, y = j in 0..ny+1, z = k in 0..nz+1)
// with boxes of WX x rows x 1 elements; outside the tensor the copy fills zeros.
template <typename R>
static bool encode_map(CUtensorMap* m, const R* base, const Grid& g, int rows) {
    const EncodeTiledFn f = tensor_map_encoder();
    if (!f || !base) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.P, (cuuint64_t)(g.ny + 2), (cuuint64_t)(g.nz + 2)};
    const cuuint64_t strides[2] = {(cuuint64_t)g.P * sizeof(R), (cuuint64_t)g.S * sizeof(R)};
    const cuuint32_t box[3] = {(cuuint32_t)WX, (cuuint32_t)rows, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return f(m, sizeof(R) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
             (void*)base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <typename R>
static bool ensure_maps(Hierarchy<R>& H, int l) {
    if (H.tm_ok[l]) return true;
    const Level<R>& L = H.lv[l];
    bool ok = true;
    for (int v = 0; v < 2; ++v) {
        SweepMaps& m = H.tm[l][v];
        ok = ok && encode_map(&m.x, v ? L.x : L.xs, L.g, FY) && encode_map(&m.cx, L.cx, L.g, R1Y) &&
             encode_map(&m.cy, L.cy, L.g, R1Y + 1) && encode_map(&m.cz, L.cz, L.g, R1Y) &&
             encode_map(&m.id, L.idiag, L.g, R1Y) && encode_map(&m.b, L.b, L.g, R1Y);
    }
    H.tm_ok[l] = ok;
    return ok;
}

// One sweep of level l from `in` to `out` (the TMA-staged kernel unless the
// maps are unavailable or the caller asked for the cp.async one).
// z chunk of the pipelined sweep on grid g.  A block marches szc + 5 planes
// (two staged below the chunk, the pipeline's fill and drain above) and the
// blocks run in waves of (resident blocks per SM) x SMs, so the chunk count
// nzc is the one that minimises  waves(tiles * nzc) * (ceil(nz / nzc) + 5):
// at 256^3 seven chunks of 37 planes (1792 blocks, 3.9 waves) rather than
// eight of 32 (2048 blocks, 4.5 waves).
template <typename R>
static int sweep_chunk(const wpf_handle* h, const Grid& g) {
    static int per_sm = 0;   // resident sweep blocks per SM (shared memory bound)
    if (!per_sm) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_sweep_async<R, false, true>, SX * SY,
                                                          sweep_smem<R>()) != cudaSuccess || b < 1) {
            cudaGetLastError();
            b = 1;
        }
        per_sm = b;
    }
    const long long resident = (long long)per_sm * h->nsm;
    const long long tiles = (long long)((g.nx + SX - 1) / SX) * ((g.ny + SY - 1) / SY);
    int best = g.nz, best_nzc = 1;
    long long best_cost = -1;
    for (int nzc = 1; nzc <= g.nz && nzc <= 64; ++nzc) {
        const int szc = (g.nz + nzc - 1) / nzc;
        const int real = (g.nz + szc - 1) / szc;
        const long long waves = (tiles * real + resident - 1) / resident;
        const long long cost = waves * (szc + 5);
        if (best_cost < 0 || cost < best_cost || (cost == best_cost && real < best_nzc)) {
            best_cost = cost;
            best = szc;
            best_nzc = real;
        }
    }
    return best;
}

template <typename R>
static void launch_sweep(wpf_handle* h, Hierarchy<R>& H, int l, int cls, bool zero, const R* in, R* out,
                         int c0, double* dot) {
    Level<R>& L = H.lv[l];
    const Grid& g = L.g;
    cudaStream_t s = h->stream;
    const dim3 sb(SX, SY);
    const bool tma = !(h->opts.flags & WPF_SOLVER_NO_TMA) && ensure_maps(H, l);
    const SweepMaps& m = H.tm[l][in == L.x ? 1 : 0];
    int* err = reinterpret_cast<int*>(h->dsc + S_KERR);
    const size_t sm = sweep_smem<R>();
    const int szc = h->opts.sweep_zchunk > 0 ? (h->opts.sweep_zchunk < g.nz ? h->opts.sweep_zchunk : g.nz)
                                             : sweep_chunk<R>(h, g);
    const dim3 gr = sweep_grid(g, szc);
    if (tma && zero)
        WPF_LAUNCH(h, cls, k_sweep_async<R, true, true><<<gr, sb, sm, s>>>(
            g, L.cx, L.cy, L.cz, L.idiag, L.b, in, out, c0, dot, m, err, szc));
    else if (tma)
        WPF_LAUNCH(h, cls, k_sweep_async<R, false, true><<<gr, sb, sm, s>>>(
            g, L.cx, L.cy, L.cz, L.idiag, L.b, in, out, c0, dot, m, err, szc));
    else if (zero)
        WPF_LAUNCH(h, cls, k_sweep_async<R, true, false><<<gr, sb, sm, s>>>(
            g, L.cx, L.cy, L.cz, L.idiag, L.b, in, out, c0, dot, m, err, szc));
    else
        WPF_LAUNCH(h, cls, k_sweep_async<R, false, false><<<gr, sb, sm, s>>>(
            g, L.cx, L.cy, L.cz, L.idiag, L.b, in, out, c0, dot, m, err, szc));
}

template <typename R>
static void cycle_level(wpf_handle* h, Hierarchy<R>& H, int l, int lb, int nu, long long big,
                        int wfrom, double* rz, bool& need_dot) {
    cudaStream_t s = h->stream;
    const dim3 sb(SX, SY);
    if (l >= lb) {
        BottomArgs<R> A;
        A.l0 = lb;
        A.nlev = H.nlev;
        A.nu = nu;
        for (int q = 0; q < H.nlev; ++q) A.lv[q] = H.lv[q];
        WPF_LAUNCH(h, lb == 0 ? KC_SMOOTH0 : KC_BOTTOM,
                   k_bottom<R><<<1, BOTTOM_THREADS, bottom_smem(H, lb), s>>>(A));
        return;
    }
    Level<R>& L = H.lv[l];
    Level<R>& C = H.lv[l + 1];
    const Grid& g = L.g;
    const int cls = l == 0 ? KC_SMOOTH0 : KC_MGREST;
    const bool is_big = ncells(g) >= big;
    const int gamma = (l >= wfrom && !is_big) ? 2 : 1;
    dim3 hb, hg;
    rbgs_grid<R>(g, hg, hb);
    auto half_pre = [&](bool zero) {
        if (zero)
            WPF_LAUNCH(h, cls, k_rbgs_first<R><<<cell_grid(g.nx, g.ny, g.nz), cell_block(), 0, s>>>(g, L.idiag, L.x, L.b));
        else
            WPF_LAUNCH(h, cls, k_rbgs<R><<<hg, hb, 0, s>>>(g, L.cx, L.cy, L.cz, L.idiag, L.x, L.b, 0));
        WPF_LAUNCH(h, cls, k_rbgs<R><<<hg, hb, 0, s>>>(g, L.cx, L.cy, L.cz, L.idiag, L.x, L.b, 1));
    };
    auto half_post = [&]() {
        WPF_LAUNCH(h, cls, k_rbgs<R><<<hg, hb, 0, s>>>(g, L.cx, L.cy, L.cz, L.idiag, L.x, L.b, 1));
        WPF_LAUNCH(h, cls, k_rbgs<R><<<hg, hb, 0, s>>>(g, L.cx, L.cy, L.cz, L.idiag, L.x, L.b, 0));
    };
    if (is_big) {
        R* buf[2] = {L.xs, L.x};
        for (int it = 0; it < nu; ++it) {
            const R* in = buf[(it + 1) & 1];
            R* out = buf[it & 1];
            launch_sweep(h, H, l, cls, it == 0, in, out, 0, nullptr);
        }
        const R* pre_end = buf[(nu - 1) & 1];
        WPF_LAUNCH(h, KC_MGREST, k_resid_restrict<R><<<cell_grid(C.g.nx, C.g.ny, C.g.nz), cell_block(), 0, s>>>(
            g, C.g, L.cx, L.cy, L.cz, L.diag, pre_end, L.b, C.b));
        cycle_level(h, H, l + 1, lb, nu, big, wfrom, nullptr, need_dot);
        for (int it = 0; it < nu; ++it) {
            const int w = nu + it;   // sweep number in the cycle: writes buf[w & 1]
            R* in = buf[(w + 1) & 1];
            R* out = buf[w & 1];
            const bool last0 = (l == 0 && it == nu - 1 && rz);
            if (last0) need_dot = false;
            if (it == 0)   // the coarse correction, into the first post-sweep's input
                launch_prolong<R>(h, g, C.g, L.idiag, in, C.x, s);
            launch_sweep(h, H, l, cls, false, in, out, 1, last0 ? rz : nullptr);
        }
        return;
    }
    for (int it = 0; it < nu; ++it) half_pre(it == 0);
    for (int rep = 0; rep < gamma; ++rep) {
        WPF_LAUNCH(h, KC_MGREST, k_resid_restrict<R><<<cell_grid(C.g.nx, C.g.ny, C.g.nz), cell_block(), 0, s>>>(
            g, C.g, L.cx, L.cy, L.cz, L.diag, L.x, L.b, C.b));
        cycle_level(h, H, l + 1, lb, nu, big, wfrom, nullptr, need_dot);
        launch_prolong<R>(h, g, C.g, L.idiag, L.x, C.x, s);
        if (rep + 1 < gamma) {
            for (int it = 0; it < nu; ++it) half_post();
            for (int it = 0; it < nu; ++it) half_pre(false);
        }
    }
    for (int it = 0; it < nu; ++it) half_post();
}

template <typename R>
static void vcycle(wpf_handle* h, Hierarchy<R>& H, int nu, double* rz) {
    const long long big = h->opts.sweep_min_cells > 0 ? h->opts.sweep_min_cells : BIG_CELLS;
    const int wfrom = h->opts.w_from_level > 0 ? h->opts.w_from_level : 2;
    int lb = H.nlev - 1;
    while (lb > 0 && ncells(H.lv[lb - 1].g) <= bottom_cells<R>() &&
           bottom_smem(H, lb - 1) <= BOTTOM_SMEM_MAX)
        --lb;
    bool need_dot = rz != nullptr;
    cycle_level(h, H, 0, lb, nu, big, wfrom, rz, need_dot);
    if (need_dot) {
        const Grid& g = H.lv[0].g;
        WPF_LAUNCH(h, KC_VEC, k_dot<R><<<row_blocks(h, g), RB, 0, h->stream>>>(g, H.r, H.z, rz));
    }
}

template <typename R>
static void drop_cycles(Hierarchy<R>& H) {
    for (int c = 0; c < 2; ++c) {
        if (H.cyc[c]) cudaGraphExecDestroy(H.cyc[c]);
        H.cyc[c] = nullptr;
        H.cyc_kernels[c] = 0;
        H.cyc_ntimers[c] = 0;
    }
}

template <typename R>
static void free_cycle_events(Hierarchy<R>& H) {
    for (int c = 0; c < 2; ++c)
        for (int e = 0; e < 2 * Hierarchy<R>::MAX_CYC_TIMERS; ++e)
            if (H.cyc_ev[c][e]) { cudaEventDestroy(H.cyc_ev[c][e]); H.cyc_ev[c][e] = nullptr; }
}

// One preconditioner cycle accumulating r.z into rz slot `slot` (0 or 1).
// The cycle launches tens of small kernels on the coarse levels, so it is
// captured once per slot as a CUDA graph and replayed: the same kernels with
// the same arguments in the same order (the hierarchy's buffers are fixed and
// its coefficients are rebuilt in place every solve).  Kernel-class timers
// become event record nodes of the graph, folded in after each replay.
template <typename R>
static int run_cycle(wpf_handle* h, Hierarchy<R>& H, int nu, int slot) {
    double* rz = h->dsc + S_RZ0 + slot;
    if (h->opts.flags & WPF_SOLVER_NO_GRAPHS) {
        vcycle(h, H, nu, rz);
        WPF_CUDA(cudaGetLastError());
        return WPF_OK;
    }
    if (H.cyc[slot] && H.cyc_mask != h->timing_mask) drop_cycles(H);
    cudaStream_t s = h->stream;
    if (!H.cyc[slot]) {
        if (h->timing_mask && !H.cyc_ev[slot][0])
            for (int e = 0; e < 2 * Hierarchy<R>::MAX_CYC_TIMERS; ++e)
                WPF_CUDA(cudaEventCreate(&H.cyc_ev[slot][e]));
        const long long l0 = h->nlaunch;
        H.cyc_ntimers[slot] = 0;
        WPF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        if (h->timing_mask) {
            h->cap_ntimers = &H.cyc_ntimers[slot];
            h->cap_cls = H.cyc_cls[slot];
            h->cap_max = Hierarchy<R>::MAX_CYC_TIMERS;
            h->cap_ev = H.cyc_ev[slot];
        }
        vcycle(h, H, nu, rz);
        h->cap_ev = nullptr;
        cudaGraph_t graph = nullptr;
        const cudaError_t e1 = cudaStreamEndCapture(s, &graph);
        const long long nk = h->nlaunch - l0;
        h->nlaunch = l0;
        if (e1 != cudaSuccess || !graph) {
            cudaGetLastError();
            return WPF_ERR_CUDA;
        }
        const cudaError_t e2 = cudaGraphInstantiate(&H.cyc[slot], graph, 0);
        cudaGraphDestroy(graph);
        if (e2 != cudaSuccess) {
            H.cyc[slot] = nullptr;
            cudaGetLastError();
            return WPF_ERR_CUDA;
        }
        H.cyc_kernels[slot] = nk;
        H.cyc_mask = h->timing_mask;
    }
    WPF_CUDA(cudaGraphLaunch(H.cyc[slot], s));
    h->nlaunch += H.cyc_kernels[slot];
    for (int t = 0; t < H.cyc_ntimers[slot] && h->ngpend < 512; ++t) {
        h->gpend_cls[h->ngpend] = H.cyc_cls[slot][t];
        h->gpend_a[h->ngpend] = H.cyc_ev[slot][2 * t];
        h->gpend_b[h->ngpend] = H.cyc_ev[slot][2 * t + 1];
        ++h->ngpend;
    }
    return WPF_OK;
}

static int read_slot(wpf_handle* h, int slot, int n = 1) {
    WPF_CUDA(cudaMemcpyAsync(h->hsc + slot, h->dsc + slot, n * sizeof(double), cudaMemcpyDeviceToHost,
                             h->stream));
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    timer_flush(h);
    return WPF_OK;
}

// PCG on A' e = r (H.r holds r on entry); e accumulates in H.x.  Stops when
// ||r_k|| <= tol * ||r_0|| or after maxit iterations.
// wc: the learned coarse space's vector (WPF_SOLVER_NET_COARSE) and awc its
// A'wc, or null: deflated PCG.
template <typename R>
static int pcg(wpf_handle* h, Hierarchy<R>& H, double tol, int maxit, int nu, int* iters,
               double* final_ratio, const float* wc = nullptr, const float* awc = nullptr) {
    const Grid& g = h->g;
    cudaStream_t s = h->stream;
    const unsigned rb = row_blocks(h, g);
    Level<R>& L0 = H.lv[0];
    double* d = h->dsc;
    WPF_CUDA(cudaMemsetAsync(d + S_PQ, 0, 4 * sizeof(double), s));   // PQ, RR, RZ0, RZ1
    WPF_LAUNCH(h, KC_VEC, k_dot<R><<<rb, RB, 0, s>>>(g, H.r, H.r, d + S_RR));
    if (wc) {
        WPF_CUDA(cudaMemsetAsync(d + S_WR, 0, sizeof(double), s));
        WPF_LAUNCH(h, KC_VEC, k_wdot<R><<<rb, RB, 0, s>>>(g, wc, H.r, nullptr, d + S_WR));
        WPF_LAUNCH(h, KC_VEC, k_defl_start<R><<<rb, RB, 0, s>>>(g, wc, awc, nullptr, d, H.x, H.r));
    }
    int rc = read_slot(h, S_RR);
    if (rc) return rc;
    const double r0 = sqrt(h->hsc[S_RR]);
    *iters = 0;
    *final_ratio = 1.0;
    if (!(r0 > 0.0)) return r0 == 0.0 ? WPF_OK : WPF_ERR_NONFINITE;
    rc = run_cycle(h, H, nu, 0);
    if (rc) return rc;
    int cur = 0;          // rz of this iteration in S_RZ0 + cur
    R* pold = H.p2;
    R* pnew = H.p;
    for (int it = 0; it < maxit; ++it) {
        if (wc) {
            WPF_CUDA(cudaMemsetAsync(d + S_WQ, 0, sizeof(double), s));
            WPF_LAUNCH(h, KC_VEC, k_wdot<R><<<rb, RB, 0, s>>>(g, awc, H.z, nullptr, d + S_WQ));
            WPF_LAUNCH(h, KC_OTHER, k_cc_mu<<<1, 32, 0, s>>>(nullptr, d));
        }
        WPF_CUDA(cudaMemsetAsync(d + S_PQ, 0, 2 * sizeof(double), s));   // S_PQ, S_RR
        WPF_LAUNCH(h, KC_APPLY, k_apply_p<R><<<row_blocks_for(h, g, k_apply_p<R>), RB, 0, s>>>(g, L0.cx, L0.cy, L0.cz, L0.diag, H.z, pold, pnew,
                                                 H.q, d + S_RZ0 + cur, d + S_RZ0 + (cur ^ 1),
                                                 it == 0, nullptr, d + S_PQ, wc, d + S_GAM));
        WPF_LAUNCH(h, KC_VEC, k_update_xr<R><<<rb, RB, 0, s>>>(g, H.x, H.r, pnew, pnew, H.q, d + S_RZ0 + cur,
                                                   d + S_PQ, it == 0, nullptr, d + S_RR, wc != nullptr));
        rc = read_slot(h, S_PQ, 2);
        if (rc) return rc;
        *iters = it + 1;
        const double rn = sqrt(h->hsc[S_RR]);
        *final_ratio = rn / r0;
        if (!(rn == rn) || isinf(rn)) return WPF_ERR_NONFINITE;
        if (rn <= tol * r0) return WPF_OK;
        const int nxt = cur ^ 1;
        WPF_CUDA(cudaMemsetAsync(d + S_RZ0 + nxt, 0, sizeof(double), s));
        rc = run_cycle(h, H, nu, nxt);
        if (rc) return rc;
        cur = nxt;
        R* t = pold; pold = pnew; pnew = t;
    }
    return WPF_ERR_NOT_CONVERGED;
}

template <typename R>
static int set_sweep_smem() {
    WPF_CUDA(cudaFuncSetAttribute(k_bottom<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)BOTTOM_SMEM_MAX));
    WPF_CUDA(cudaFuncSetAttribute(k_sweep_async<R, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sweep_smem<R>()));
    WPF_CUDA(cudaFuncSetAttribute(k_sweep_async<R, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sweep_smem<R>()));
    WPF_CUDA(cudaFuncSetAttribute(k_sweep_async<R, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sweep_smem<R>()));
    WPF_CUDA(cudaFuncSetAttribute(k_sweep_async<R, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sweep_smem<R>()));
    return WPF_OK;
}

int solver_setup(wpf_handle* h) {
    int rc = h->opts.mode == WPF_SOLVER_MIXED ? set_sweep_smem<float>() : set_sweep_smem<double>();
    if (rc) return rc;
    if ((h->opts.flags & WPF_SOLVER_EXTRAPOLATE) && !h->ws[0]) {
        for (int q = 0; q < 3; ++q)
            if ((rc = dev_alloc(h, (void**)&h->ws[q], sizeof(float) * h->g.total))) return rc;
        h->ws_hist = 0;
    }
    if (!h->l0mark) {
        if ((rc = dev_alloc(h, (void**)&h->l0mark, (size_t)h->g.total))) return rc;
        WPF_CUDA(cudaMemsetAsync(h->l0mark, 0, (size_t)h->g.total, h->stream));
        h->l0_inc_ok = false;
    }
    if (h->opts.mode == WPF_SOLVER_MIXED) {
        rc = alloc_hierarchy(h, h->h32);
        if (rc) return rc;
        if (!h->dsum && (rc = dev_alloc(h, (void**)&h->dsum, sizeof(double) * h->g.total))) return rc;
        if ((h->opts.flags & WPF_SOLVER_EXTRAPOLATE) && !h->rkeep) {
            if ((rc = dev_alloc(h, (void**)&h->rkeep, sizeof(double) * h->g.total))) return rc;
            h->rkeep_ok = false;
        }
        return WPF_OK;
    }
    return alloc_hierarchy(h, h->h64);
}

void solver_drop_graphs(wpf_handle* h) {
    drop_cycles(h->h64);
    drop_cycles(h->h32);
    step_graphs_drop(h);
}

int solver_free(wpf_handle* h) {
    free_hierarchy(h->h64);
    free_hierarchy(h->h32);
    if (h->dsum) cudaFree(h->dsum);
    h->dsum = nullptr;
    if (h->rkeep) cudaFree(h->rkeep);
    h->rkeep = nullptr;
    h->rkeep_ok = false;
    if (h->l0mark) cudaFree(h->l0mark);
    h->l0mark = nullptr;
    h->l0_inc_ok = false;
    for (int q = 0; q < 3; ++q) {
        if (h->ws[q]) cudaFree(h->ws[q]);
        h->ws[q] = nullptr;
    }
    for (int q = 0; q < 3; ++q) {
        if (h->ws_e[q]) cudaFree(h->ws_e[q]);
        h->ws_e[q] = nullptr;
    }
    if (h->ws_in) cudaFree(h->ws_in);
    if (h->ws_out) cudaFree(h->ws_out);
    h->ws_in = nullptr;
    h->ws_out = nullptr;
    h->ws_hist = 0;
    return WPF_OK;
}

// Coefficients of e = a d1 + b d2: the Newton form of the quadratic through
// the last three pressures in time, evaluated one step hn ahead,
//   e = (hn/h1) d1 + hn (hn + h1) / (h1 + h2) (d1/h1 - d2/h2),
// (linear, e = (hn/h1) d1, with one increment; equal steps when a step size
// is unknown: 2 d1 - d2, d1).
void ws_coeffs(const wpf_handle* h, float* a, float* b) {
    *a = 0.f;
    *b = 0.f;
    if (h->ws_hist <= 0) return;
    const double hn = h->ws_hn, h1 = h->ws_h1, h2 = h->ws_h2;
    if (h->ws_hist == 1) {
        *a = (hn > 0 && h1 > 0) ? (float)(hn / h1) : 1.f;
        return;
    }
    if (!(hn > 0 && h1 > 0 && h2 > 0)) {
        *a = 2.f;
        *b = -1.f;
        return;
    }
    const double c = hn * (hn + h1) / (h1 + h2);
    *a = (float)(hn / h1 + c / h1);
    *b = (float)(-c / h2);
}

int ws_build_ext(wpf_handle* h, float a, float b, float* dnew) {
    const Grid& g = h->g;
    if (!h->ws_e[0]) {
        int rc = dev_alloc(h, (void**)&h->ws_e[0], sizeof(float) * g.total);
        if (rc) return rc;
    }
    WPF_CUDA(cudaMemsetAsync(h->dsc + S_WSS2, 0, 2 * sizeof(double), h->stream));   // WSS2, WSD2
    WPF_LAUNCH(h, KC_RESID64, k_ws_build_ext<<<row_blocks(h, g), RB, 0, h->stream>>>(
        g, h->ws[0], h->ws[1], a, b, h->ws_e[0], h->dsc, nullptr, dnew));
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

template <typename R>
static int solve_impl(wpf_handle* h, Hierarchy<R>& H, wpf_step_stats* st) {
    const Grid& g = h->g;
    cudaStream_t s = h->stream;
    const unsigned rb = row_blocks(h, g);
    const bool mixed = h->opts.mode == WPF_SOLVER_MIXED;
    int rc = build_hierarchy(h, H);
    if (rc) return rc;
    const int nu = h->opts.smooth_sweeps > 0 ? h->opts.smooth_sweeps : 2;
    int outer = 0, inner_total = 0, status = WPF_ERR_NOT_CONVERGED;
    double relres = 0.0, bnorm = 0.0, relres0 = 0.0;
    // extrapolated start: tried on pass 0 when two (or one) increments are
    // held; with an attached net, the net's correction on top of it too
    const bool ws_on = (h->opts.flags & WPF_SOLVER_EXTRAPOLATE) && h->ws[0];
    float* dnew = ws_on ? h->ws[2] : nullptr;
    const float* e1 = nullptr;   // the accepted start (added to p once): e_ext ...
    const float* e2 = nullptr;   // ... + alpha e_net
    float alpha = 0.f;
    const float* wc = nullptr;   // the learned coarse space of this solve's PCGs
    bool ws_tried = false;       // pass 0 evaluated r(p) beside the extrapolated start
    bool b_predicted = false;    // pass 0 took ||b|| from the last solve (least-squares prediction)
    bool ext_pending = false;    // a start accepted but not yet added to the pressure
    // the FP64 residual kept for the next solve (mixed form with the
    // extrapolated start): written by every plain pass, read by pass 0
    double* rk = mixed ? h->rkeep : nullptr;
    h->ws_used = 0;
    for (int pass = 0; pass <= h->opts.max_outer; ++pass) {
        WPF_CUDA(cudaMemsetAsync(h->dsc + S_RR64, 0, 5 * sizeof(double), s));   // RR64 BB64 RR0WS RW WW
        bool plain = true;
        if (pass == 0 && ws_on && h->ws_hist > 0) {
            ws_tried = true;
            float wa = 0.f, wb = 0.f;
            ws_coeffs(h, &wa, &wb);
            const double* rk_in = (rk && h->rkeep_ok) ? rk : nullptr;
            bool skip0 = false;   // pass 0's residual kernel replaced by the prediction
            if (rk_in && !(h->opts.flags & WPF_SOLVER_FIXED_START) &&
                ws_ls_wanted(h->ls_rp_rel, h->ls_bnorm, h->opts.rtol)) {   // the least-squares start
                const double sc = ws_ls_scale(h->ls_bnorm, h->opts.rtol, (long long)g.nx * g.ny * g.nz);
                WPF_CUDA(cudaMemsetAsync(h->dsc + S_LS0, 0, 6 * sizeof(double), s));
                WPF_LAUNCH(h, KC_RESID64, k_ws_ls_dots<R><<<row_blocks_for(h, g, k_ws_ls_dots<R>), RB, 0, s>>>(
                    g, H.lv[0].cx, H.lv[0].cy, H.lv[0].cz, H.lv[0].diag, h->flags, h->ws[0],
                    h->ws_hist >= 2 ? h->ws[1] : h->ws[0], rk_in, nullptr, sc, h->dsc));
                WPF_CUDA(cudaGetLastError());
                if ((rc = read_slot(h, S_LS0, 6))) return rc;
                ws_ls_solve(h->hsc + S_LS0, &wa, &wb);
                const double pred = fmax(ws_ls_predict(h->hsc + S_LS0, wa, wb), 0.0) / (sc * sc);
                // (the net, when it runs at every solve, needs pass 0's FP32 residual)
                if (!(h->opts.flags & WPF_SOLVER_NET_ALWAYS) &&
                    sqrt(pred) <= LS_SKIP * h->opts.rtol * h->ls_bnorm) {
                    skip0 = true;
                    b_predicted = true;
                    h->hsc[S_RR64] = pred;
                    h->hsc[S_RR0WS] = h->hsc[S_LS5] / (sc * sc);
                    h->hsc[S_BB64] = h->ls_bnorm * h->ls_bnorm;
                }
            }
            if ((rc = ws_build_ext(h, wa, wb, skip0 ? dnew : nullptr))) return rc;
            if (!skip0) {
                auto* kern = rk_in ? k_resid64_ws<R, true> : k_resid64_ws<R, false>;
                WPF_LAUNCH(h, KC_RESID64, kern<<<row_blocks_for(h, g, kern), RB, 0, s>>>(
                    g, h->pressure, h->T[0], h->T[1], h->T[2], h->flags, h->qterm, resid_dsum(h), H.lv[0].cx,
                    H.lv[0].cy, H.lv[0].cz, H.lv[0].diag, h->ws_e[0], H.r, dnew, h->dsc, rk_in, nullptr));
                WPF_CUDA(cudaGetLastError());
                rc = read_slot(h, S_RR64, 5);
                if (rc) return rc;
            }
            double rstart = h->hsc[S_RR64];
            const double r0 = h->hsc[S_RR0WS];
            double rw = 0.0, ww = 0.0;
            // the learned correction, tried when the extrapolation alone misses rtol
            // by at most NET_WINDOW (there it can save a refinement pass)
            const bool net = h->ws_net && h->ws_hist >= 2 &&
                             ((h->opts.flags & WPF_SOLVER_NET_ALWAYS) ||
                              net_gate(rstart, h->hsc[S_BB64], h->opts.rtol));
            if (net) {
                if ((rc = ws_net_correction(h))) return rc;
                WPF_CUDA(cudaMemsetAsync(h->dsc + S_RW, 0, 2 * sizeof(double), s));
                WPF_CUDA(cudaMemsetAsync(h->dsc + S_WAW, 0, sizeof(double), s));
                const bool coarse = (h->opts.flags & WPF_SOLVER_NET_COARSE) != 0;
                WPF_LAUNCH(h, KC_RESID64, k_net_dots<R><<<rb, RB, 0, s>>>(
                    g, H.lv[0].cx, H.lv[0].cy, H.lv[0].cz, H.lv[0].diag, h->flags, h->ws_e[1], H.r, h->dsc,
                    coarse ? h->ws_e[2] : nullptr));
                WPF_CUDA(cudaGetLastError());
                if ((rc = read_slot(h, S_RW, 2))) return rc;
                rw = h->hsc[S_RW];
                ww = h->hsc[S_WW];
                if (coarse) wc = h->ws_e[1];
            }
            // learned correction: the step that minimises the residual along it
            if (net && ww > 0.0 && rw > 0.0 && rw == rw) {
                alpha = (float)(rw / ww);
                rstart = fmax(rstart - rw * rw / ww, 0.0);
            }
            // the fallback rule: the start is kept only when its FP64-evaluated
            // residual is below that of p itself (the reference's start)
            if (rstart <= r0 && rstart == rstart) {
                plain = false;
                ext_pending = true;
                e1 = h->ws_e[0];
                h->ws_used = 1;
                if (alpha > 0.f) {
                    e2 = h->ws_e[1];
                    h->ws_used = 2;
                    WPF_LAUNCH(h, KC_RESID64, k_ws_take_net<R><<<rb, RB, 0, s>>>(
                        g, H.lv[0].cx, H.lv[0].cy, H.lv[0].cz, H.lv[0].diag, h->flags, alpha, e2, H.r, dnew));
                }
                h->hsc[S_RR64] = rstart;
            } else {
                h->ws_used = -1;
                ++h->ws_fallbacks;
                WPF_CUDA(cudaMemsetAsync(h->dsc + S_RR64, 0, 5 * sizeof(double), s));
            }
        }
        if (plain) {
            if (pass == 0 && ws_on) WPF_CUDA(cudaMemsetAsync(dnew, 0, sizeof(float) * g.total, s));
            // ||b|| on pass 0, and on the passes after a pass 0 whose residual
            // the least-squares prediction replaced (its ||b|| was the last step's)
            WPF_LAUNCH(h, KC_RESID64, k_resid64<R><<<row_blocks_for(h, g, k_resid64<R>), RB, 0, s>>>(g, h->pressure, h->T[0], h->T[1], h->T[2],
                                                              h->flags, h->qterm, resid_dsum(h), H.r, h->dsc,
                                                              pass == 0 || b_predicted, nullptr, nullptr, rk));
            WPF_CUDA(cudaGetLastError());
            h->rkeep_ok = rk != nullptr;
            rc = read_slot(h, S_RR64, 2);
            if (rc) return rc;
        }
        if (pass == 0 || h->hsc[S_BB64] > 0.0) bnorm = sqrt(h->hsc[S_BB64]);
        const double rnorm = sqrt(h->hsc[S_RR64]);
        relres = bnorm > 0.0 ? rnorm / bnorm : rnorm;
        h->ls_bnorm = bnorm;   // the next step's least-squares start: its scale
        if (pass == 0) {
            relres0 = relres;
            // and how close p itself was
            h->ls_rp_rel = ws_tried && bnorm > 0.0 ? sqrt(h->hsc[S_RR0WS]) / bnorm : relres;
        }
        if (!(relres == relres) || isinf(relres)) { status = WPF_ERR_NONFINITE; break; }
        if (relres <= h->opts.rtol) {
            // an extrapolated start whose (partly FP32-evaluated) residual
            // already meets rtol is added to p and verified by a plain FP64 pass
            if (ext_pending && pass < h->opts.max_outer) {
                WPF_LAUNCH(h, KC_VEC, k_add_correction_ws<R><<<rb, RB, 0, s>>>(
                    g, h->pressure, (const R*)nullptr, e1, e2, alpha, dnew));
                ext_pending = false;
                h->rkeep_ok = false;
                continue;
            }
            status = WPF_OK;
            break;
        }
        if (pass == h->opts.max_outer) break;
        outer = pass + 1;
        double want = 0.5 * h->opts.rtol / relres;
        double tol = mixed ? fmax(h->opts.inner_rtol, want) : want;
        int its = 0;
        double ratio = 1.0;
        rc = pcg<R>(h, H, tol, h->opts.max_inner, nu, &its, &ratio, wc, h->ws_e[2]);
        inner_total += its;
        if (rc == WPF_ERR_NONFINITE) { status = rc; break; }
        if (ws_on)
            WPF_LAUNCH(h, KC_VEC, k_add_correction_ws<R><<<rb, RB, 0, s>>>(
                g, h->pressure, H.x, ext_pending ? e1 : nullptr, e2, alpha, dnew));
        else
            WPF_LAUNCH(h, KC_VEC, k_add_correction<R><<<rb, RB, 0, s>>>(g, h->pressure, H.x));
        ext_pending = false;
        h->rkeep_ok = false;
        WPF_CUDA(cudaGetLastError());
    }
    if (ext_pending) {   // max_outer = 0: the start was accepted but never verified
        WPF_LAUNCH(h, KC_VEC, k_add_correction_ws<R><<<rb, RB, 0, s>>>(g, h->pressure, (const R*)nullptr,
                                                                       e1, e2, alpha, dnew));
        h->rkeep_ok = false;
    }
    if (status == WPF_ERR_NONFINITE) h->rkeep_ok = false;
    if (ws_on) {
        if (status == WPF_OK) {   // this increment becomes the newest of the history
            float* t = h->ws[1];
            h->ws[1] = h->ws[0];
            h->ws[0] = h->ws[2];
            h->ws[2] = t;
            h->ws_hist = h->ws_hist < 2 ? h->ws_hist + 1 : 2;
            h->ws_h2 = h->ws_h1;
            h->ws_h1 = h->ws_hn;
        } else {
            h->ws_hist = 0;
        }
    }
    if (st) {
        st->outer_iterations = outer;
        st->inner_iterations = inner_total;
        st->converged = status == WPF_OK;
        st->relres = relres;
        st->relres0 = relres0;
        st->warm_start = h->ws_used;
    }
    return status;
}

// ---------------------------------------------------------------------------
// Device-resident solve (WPF_SOLVER_STEP_GRAPH).  The same kernels as
// solve_impl / pcg and the fused update; the decisions those functions take
// on the host after each read-back are taken by one-thread control kernels,
// and the two loops are conditional WHILE nodes:
//   [Dirichlet, level-0 coefficients]
//   { pass-0 residual (extrapolated start + fallback), pass test  ||  coarse levels }
//   WHILE(passes) { [PCG prologue]  WHILE(iterations) { [cycle, apply, update, test] }
//                   [correction, next pass residual, pass test] }
//   [pressure halo, fused update]
// The "||" branches are independent graph branches (the coarse operators are
// not needed before the first cycle).  The PCG keeps r.z of the iteration in
// S_RZ1 and of the previous one in S_RZ0 (the test kernel moves it), and the
// two search-direction buffers swap roles on odd iterations inside k_apply_p /
// k_update_xr.
// ---------------------------------------------------------------------------

// Extrapolated start: kept when its residual is below that of p (solve_impl's
// fallback rule); else the slots are cleared for the plain pass-0 residual.
__global__ void k_ctl_accept(StepCtl* c, double* dsc) {
    if (threadIdx.x) return;
    const double rstart = dsc[S_RR64], r0 = dsc[S_RR0WS];
    if (dsc[S_BB64] > 0.0) c->rp_rel = sqrt(r0 / dsc[S_BB64]);   // for the next step's least-squares start
    if (rstart <= r0 && rstart == rstart) {
        c->accept = 1;
        c->used = 1;
    } else {
        c->accept = 0;
        c->used = -1;
        for (int q = 0; q < 5; ++q) dsc[S_RR64 + q] = 0.0;
    }
}

// Whether the learned correction is evaluated this step (net_gate on the
// extrapolated start's residual): the condition of the net's IF node.
__global__ void k_ctl_net_gate(StepCtl* c, const double* dsc, double rtol, int always,
                               cudaGraphConditionalHandle h_net) {
    if (threadIdx.x) return;
    const int run = (always || net_gate(dsc[S_RR64], dsc[S_BB64], rtol)) ? 1 : 0;
    c->net_runs = run;
    cudaGraphSetConditional(h_net, run);
}

// The same with a learned correction e_net (S_RW = r_ext.A'e_net, S_WW =
// |A'e_net|^2): the step alpha = RW / WW that minimises the residual along
// it, taken when positive; the start (extrapolation + alpha e_net) is kept when
// its residual is below that of p.  The arithmetic of solve_impl's pass 0.
__global__ void k_ctl_accept_net(StepCtl* c, double* dsc) {
    if (threadIdx.x) return;
    double rstart = dsc[S_RR64];
    const double r0 = dsc[S_RR0WS], rw = dsc[S_RW], ww = dsc[S_WW];
    if (dsc[S_BB64] > 0.0) c->rp_rel = sqrt(r0 / dsc[S_BB64]);
    float alpha = 0.f;
    if (ww > 0.0 && rw > 0.0 && rw == rw) {
        alpha = (float)(rw / ww);
        rstart = fmax(rstart - rw * rw / ww, 0.0);
    }
    if (rstart <= r0 && rstart == rstart) {
        c->accept = 1;
        c->used = alpha > 0.f ? 2 : 1;
        c->alpha = alpha > 0.f ? alpha : 0.f;
        dsc[S_RR64] = rstart;
    } else {
        c->accept = 0;
        c->used = -1;
        c->alpha = 0.f;
        for (int q = 0; q < 5; ++q) dsc[S_RR64 + q] = 0.0;
    }
}

// k_ws_take_net with the decision and the step read from the control block.
template <typename R>
__global__ void __launch_bounds__(RB) k_ws_take_net_dev(Grid g, const R* __restrict__ cx, const R* __restrict__ cy,
                                                        const R* __restrict__ cz, const R* __restrict__ diag,
                                                        const uint8_t* __restrict__ fl, const StepCtl* c,
                                                        const float* __restrict__ e2, R* __restrict__ r,
                                                        float* __restrict__ dnew) {
    __shared__ float salpha;
    if (threadIdx.x == 0) salpha = (c->accept && c->alpha > 0.f) ? c->alpha : 0.f;
    __syncthreads();
    const float alpha = salpha;
    if (!(alpha > 0.f)) return;
    const long long sy = g.P, sz = g.S;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        dnew[n] += alpha * e2[n];
        if (!(fl[n] & F_DIR)) r[n] -= (R)alpha * apply_l0(cx, cy, cz, diag, e2, n, sy, sz);
    }
}

// After a refinement pass's residual: the pass logic of solve_impl.
__global__ void k_ctl_pass(StepCtl* c, const double* dsc, double rtol, double inner_rtol, int max_outer,
                           int mixed, cudaGraphConditionalHandle h_pass) {
    if (threadIdx.x) return;
    const int pass = c->pass;
    int cont = 0, pcg = 0;
    if (c->status != WPF_ERR_NONFINITE) {   // else a PCG of the last pass broke down
        // ||b|| from pass 0, and from the verification pass after a pass 0
        // whose residual the least-squares prediction replaced (the exact one)
        if (pass == 0 || dsc[S_BB64] > 0.0) c->bnorm = sqrt(dsc[S_BB64]);
        const double bnorm = c->bnorm;
        const double rnorm = sqrt(dsc[S_RR64]);
        const double relres = bnorm > 0.0 ? rnorm / bnorm : rnorm;
        c->relres = relres;
        if (pass == 0) c->relres0 = relres;
        if (!(relres == relres) || isinf(relres)) {
            c->status = WPF_ERR_NONFINITE;
        } else if (relres <= rtol) {
            // an accepted start that already meets rtol: add it, verify by a plain pass
            if (c->accept && pass < max_outer) cont = 1;
            else c->status = WPF_OK;
        } else if (pass < max_outer) {
            c->outer = pass + 1;
            const double want = 0.5 * rtol / relres;
            c->tol = mixed ? fmax(inner_rtol, want) : want;
            cont = 1;
            pcg = 1;
        }
    }
    c->need_pcg = pcg;
    cudaGraphSetConditional(h_pass, cont);
}

// PCG prologue (r.r in S_RR): the iterations run when the pass needs a PCG
// and ||r_0|| > 0 (pcg's early return).
__global__ void k_ctl_pcg_start(StepCtl* c, const double* dsc, cudaGraphConditionalHandle h_it) {
    if (threadIdx.x) return;
    int run = 0;
    c->it = 0;
    if (c->need_pcg) {
        ++c->pcgs;
        const double r0 = sqrt(dsc[S_RR]);
        c->r0 = r0;
        if (r0 > 0.0) run = 1;
        else if (r0 != 0.0) c->status = WPF_ERR_NONFINITE;
    }
    cudaGraphSetConditional(h_it, run);
}

// After a PCG iteration: pcg's convergence test; this r.z becomes the previous.
__global__ void k_ctl_pcg_check(StepCtl* c, double* dsc, int maxit, cudaGraphConditionalHandle h_it) {
    if (threadIdx.x) return;
    const int it = ++c->it;
    ++c->inner;
    const double rn = sqrt(dsc[S_RR]);
    int cont = 0;
    if (!(rn == rn) || isinf(rn)) c->status = WPF_ERR_NONFINITE;
    else if (!(rn <= c->tol * c->r0) && it < maxit) cont = 1;
    dsc[S_RZ0] = dsc[S_RZ1];
    cudaGraphSetConditional(h_it, cont);
}

// Between passes: the start is consumed, the next pass's residual slots cleared.
__global__ void k_ctl_advance(StepCtl* c, double* dsc) {
    if (threadIdx.x) return;
    c->accept = 0;
    ++c->pass;
    for (int q = 0; q < 5; ++q) dsc[S_RR64 + q] = 0.0;
}

// p += x (when this pass ran PCG iterations) + e1 [+ alpha e2] (when the
// accepted start is pending; e2 the learned correction, taken when alpha > 0);
// dnew accumulates x.  The arithmetic of k_add_correction(_ws).
template <typename R>
__global__ void __launch_bounds__(RB) k_add_correction_dev(Grid g, double* __restrict__ pr,
                                                           const R* __restrict__ x,
                                                           const float* __restrict__ e1,
                                                           const float* __restrict__ e2,
                                                           float* __restrict__ dnew, const StepCtl* c) {
    __shared__ int suse;
    __shared__ float salpha;
    if (threadIdx.x == 0) {
        const bool ok = c->status != WPF_ERR_NONFINITE;
        suse = (ok && c->need_pcg && c->it > 0 ? 1 : 0) | (ok && e1 && c->accept ? 2 : 0);
        salpha = (e2 && c->alpha > 0.f) ? c->alpha : 0.f;
    }
    __syncthreads();
    const int use = suse;
    const float alpha = salpha;
    if (!use) return;
    ROW_LOOP_U4(g) {
        const long long n = g.at(i, j, k);
        double inc = (use & 1) ? to_f64<R>(x[n]) : 0.0;
        if (use & 2) inc += f32_to_f64(alpha > 0.f ? e1[n] + alpha * e2[n] : e1[n]);
        pr[n] += inc;
        if ((use & 1) && dnew) dnew[n] += to_f32<R>(x[n]);
    }
}

template <typename R>
static int solve_capture_impl(wpf_handle* h, Hierarchy<R>& H, GraphBuilder& b, StepCounts* cnt) {
    const Grid& g = h->g;
    cudaStream_t s = h->stream;
    const unsigned rb = row_blocks(h, g);
    const int mixed = h->opts.mode == WPF_SOLVER_MIXED;
    const bool ws_on = (h->opts.flags & WPF_SOLVER_EXTRAPOLATE) && h->ws[0] && h->ws_e[0];
    const bool net = ws_on && h->ws_net && h->ws_hist >= 2;
    // the learned coarse space in the PCG (active in the steps whose net ran)
    const float* wc = (net && (h->opts.flags & WPF_SOLVER_NET_COARSE)) ? h->ws_e[1] : nullptr;
    const int nu = h->opts.smooth_sweeps > 0 ? h->opts.smooth_sweeps : 2;
    StepCtl* c = h->gctl;
    double* d = h->dsc;
    Level<R>& L0 = H.lv[0];
    float* dnew = ws_on ? h->ws[2] : nullptr;
    // the kept FP64 residual: written by every plain pass, read by pass 0
    // when calcPermeability (captured just before) corrected it for this step
    double* rk = mixed ? h->rkeep : nullptr;
    const double* rk_in = (rk && h->rkeep_ok) ? rk : nullptr;
    cudaGraphConditionalHandle h_pass, h_it, h_net = 0;
    int rc;
    if ((rc = gb_handle(b, &h_pass)) || (rc = gb_handle(b, &h_it))) return rc;
    if (net && (rc = gb_handle(b, &h_net))) return rc;

    long long l0 = h->nlaunch;
    if ((rc = phys_set_dirichlet(h))) return rc;
    WPF_CUDA(cudaEventRecordWithFlags(h->ev[0], s, cudaEventRecordExternal));
    build_level0(h, H, s);
    if ((rc = gb_fork(h))) return rc;
    build_coarse(h, H, h->cap_side);
    if (ws_on) {
        const bool early = h->ws_early;
        if (early) {   // built beside calcPermeability
            WPF_CUDA(cudaEventRecord(h->cap_ws_join, h->cap_ws));
            WPF_CUDA(cudaStreamWaitEvent(s, h->cap_ws_join, 0));
            h->ws_early = false;
        }
        if (rk_in && !(h->opts.flags & WPF_SOLVER_FIXED_START)) {
            // the least-squares start: its coefficients need this step's
            // kept residual and level-0 operator, so it is built after them
            WPF_CUDA(cudaMemsetAsync(d + S_LS0, 0, 6 * sizeof(double), s));
            WPF_LAUNCH(h, KC_OTHER, k_ctl_ls_begin<<<1, 32, 0, s>>>(c, d, h->opts.rtol,
                                                                     (long long)g.nx * g.ny * g.nz));
            WPF_LAUNCH(h, KC_RESID64, k_ws_ls_dots<R><<<row_blocks_for(h, g, k_ws_ls_dots<R>), RB, 0, s>>>(g, L0.cx, L0.cy, L0.cz, L0.diag, h->flags,
                                                                        h->ws[0], h->ws[1], rk_in, c, 0.0, d));
            // (the net, when it runs at every solve, needs pass 0's FP32 residual)
            WPF_LAUNCH(h, KC_OTHER, k_ctl_ws_ls<<<1, 32, 0, s>>>(
                c, d, (h->opts.flags & WPF_SOLVER_NET_ALWAYS) ? -1.0 : h->opts.rtol));
            WPF_LAUNCH(h, KC_RESID64, k_ws_build_ext<<<rb, RB, 0, s>>>(g, h->ws[0], h->ws[1], 0.f, 0.f, h->ws_e[0],
                                                                       d, &c->wa, dnew));
        } else if (!early) {
            WPF_LAUNCH(h, KC_RESID64, k_ws_build_ext<<<rb, RB, 0, s>>>(g, h->ws[0], h->ws[1], 0.f, 0.f, h->ws_e[0],
                                                                       d, &c->wa));
        }
        auto* kern = rk_in ? k_resid64_ws<R, true> : k_resid64_ws<R, false>;
        const bool lsq = rk_in && !(h->opts.flags & WPF_SOLVER_FIXED_START);
        WPF_LAUNCH(h, KC_RESID64, kern<<<row_blocks_for(h, g, kern), RB, 0, s>>>(
            g, h->pressure, h->T[0], h->T[1], h->T[2], h->flags, h->qterm, resid_dsum(h), L0.cx, L0.cy, L0.cz, L0.diag,
            h->ws_e[0], H.r, dnew, d, rk_in, lsq ? &c->ls_skip : nullptr));
        if (net) {
            // the learned correction in an IF node, taken when the extrapolated
            // start misses rtol by at most NET_WINDOW (k_ctl_net_gate); the
            // coarse-level branch joins before it
            if ((rc = gb_join(h))) return rc;
            WPF_LAUNCH(h, KC_OTHER, k_ctl_net_gate<<<1, 32, 0, s>>>(
                c, d, h->opts.rtol, (h->opts.flags & WPF_SOLVER_NET_ALWAYS) ? 1 : 0, h_net));
            WPF_CUDA(cudaGetLastError());
            cnt->fixed += h->nlaunch - l0;
            if ((rc = gb_end(b))) return rc;
            GraphBuilder nb;
            if ((rc = gb_cond(b, cudaGraphCondTypeIf, h_net, &nb))) return rc;
            if ((rc = gb_begin(nb))) return rc;
            const long long ln = h->nlaunch;
            if ((rc = ws_net_capture(h, s))) return rc;   // e_net in ws_e[1]
            WPF_CUDA(cudaMemsetAsync(d + S_RW, 0, 2 * sizeof(double), s));
            WPF_CUDA(cudaMemsetAsync(d + S_WAW, 0, sizeof(double), s));
            WPF_LAUNCH(h, KC_RESID64, k_net_dots<R><<<rb, RB, 0, s>>>(g, L0.cx, L0.cy, L0.cz, L0.diag, h->flags,
                                                                    h->ws_e[1], H.r, d, wc ? h->ws_e[2] : nullptr));
            WPF_CUDA(cudaGetLastError());
            cnt->per_net = h->nlaunch - ln;
            if ((rc = gb_end(nb))) return rc;
            if ((rc = gb_begin(b))) return rc;
            l0 = h->nlaunch;
            WPF_LAUNCH(h, KC_OTHER, k_ctl_accept_net<<<1, 32, 0, s>>>(c, d));
            WPF_LAUNCH(h, KC_RESID64, k_ws_take_net_dev<R><<<rb, RB, 0, s>>>(
                g, L0.cx, L0.cy, L0.cz, L0.diag, h->flags, c, h->ws_e[1], H.r, dnew));
        } else {
            WPF_LAUNCH(h, KC_OTHER, k_ctl_accept<<<1, 32, 0, s>>>(c, d));
        }
        WPF_LAUNCH(h, KC_RESID64, k_resid64<R><<<row_blocks_for(h, g, k_resid64<R>), RB, 0, s>>>(g, h->pressure, h->T[0], h->T[1], h->T[2],
                                                                   h->flags, h->qterm, resid_dsum(h), H.r, d, 1, &c->accept,
                                                                   dnew, rk));
    } else {
        WPF_LAUNCH(h, KC_RESID64, k_resid64<R><<<row_blocks_for(h, g, k_resid64<R>), RB, 0, s>>>(g, h->pressure, h->T[0], h->T[1], h->T[2],
                                                                   h->flags, h->qterm, resid_dsum(h), H.r, d, 1,
                                                                   nullptr, nullptr, rk));
    }
    WPF_LAUNCH(h, KC_OTHER, k_ctl_pass<<<1, 32, 0, s>>>(c, d, h->opts.rtol, h->opts.inner_rtol, h->opts.max_outer,
                                                         mixed, h_pass));
    if (!net && (rc = gb_join(h))) return rc;   // (with the net it joined before the IF node)
    WPF_CUDA(cudaGetLastError());
    cnt->fixed += h->nlaunch - l0;
    if ((rc = gb_end(b))) return rc;

    GraphBuilder pass, iter;
    if ((rc = gb_cond(b, cudaGraphCondTypeWhile, h_pass, &pass))) return rc;
    if ((rc = gb_begin(pass))) return rc;
    l0 = h->nlaunch;
    WPF_CUDA(cudaMemsetAsync(d + S_PQ, 0, 4 * sizeof(double), s));   // PQ, RR, RZ0, RZ1
    WPF_LAUNCH(h, KC_VEC, k_dot<R><<<rb, RB, 0, s>>>(g, H.r, H.r, d + S_RR));
    if (wc) {
        WPF_CUDA(cudaMemsetAsync(d + S_WR, 0, sizeof(double), s));
        WPF_LAUNCH(h, KC_VEC, k_wdot<R><<<rb, RB, 0, s>>>(g, wc, H.r, c, d + S_WR));
        WPF_LAUNCH(h, KC_VEC, k_defl_start<R><<<rb, RB, 0, s>>>(g, wc, h->ws_e[2], c, d, H.x, H.r));
    }
    WPF_LAUNCH(h, KC_OTHER, k_ctl_pcg_start<<<1, 32, 0, s>>>(c, d, h_it));
    WPF_CUDA(cudaGetLastError());
    if ((rc = gb_end(pass))) return rc;
    if ((rc = gb_cond(pass, cudaGraphCondTypeWhile, h_it, &iter))) return rc;
    if ((rc = gb_begin(iter))) return rc;
    const long long l1 = h->nlaunch;
    WPF_CUDA(cudaMemsetAsync(d + S_RZ1, 0, sizeof(double), s));
    vcycle(h, H, nu, d + S_RZ1);
    if (wc) {
        WPF_CUDA(cudaMemsetAsync(d + S_WQ, 0, sizeof(double), s));
        WPF_LAUNCH(h, KC_VEC, k_wdot<R><<<rb, RB, 0, s>>>(g, h->ws_e[2], H.z, c, d + S_WQ));
        WPF_LAUNCH(h, KC_OTHER, k_cc_mu<<<1, 32, 0, s>>>(c, d));
    }
    WPF_CUDA(cudaMemsetAsync(d + S_PQ, 0, 2 * sizeof(double), s));   // PQ, RR
    WPF_LAUNCH(h, KC_APPLY, k_apply_p<R><<<row_blocks_for(h, g, k_apply_p<R>), RB, 0, s>>>(g, L0.cx, L0.cy, L0.cz, L0.diag, H.z, H.p2, H.p, H.q,
                                                             d + S_RZ1, d + S_RZ0, 0, &c->it, d + S_PQ, wc,
                                                             d + S_GAM));
    WPF_LAUNCH(h, KC_VEC, k_update_xr<R><<<rb, RB, 0, s>>>(g, H.x, H.r, H.p, H.p2, H.q, d + S_RZ1, d + S_PQ, 0,
                                                           &c->it, d + S_RR, wc != nullptr));
    WPF_LAUNCH(h, KC_OTHER, k_ctl_pcg_check<<<1, 32, 0, s>>>(c, d, h->opts.max_inner, h_it));
    WPF_CUDA(cudaGetLastError());
    cnt->per_iter = h->nlaunch - l1;
    if ((rc = gb_end(iter))) return rc;
    if ((rc = gb_begin(pass))) return rc;
    const long long l2 = h->nlaunch;
    WPF_LAUNCH(h, KC_VEC, k_add_correction_dev<R><<<rb, RB, 0, s>>>(g, h->pressure, H.x,
                                                                    ws_on ? h->ws_e[0] : nullptr,
                                                                    net ? h->ws_e[1] : nullptr, dnew, c));
    WPF_LAUNCH(h, KC_OTHER, k_ctl_advance<<<1, 32, 0, s>>>(c, d));
    // ||b|| again only after a pass 0 whose residual the least-squares
    // prediction replaced (its ||b|| was the last step's)
    WPF_LAUNCH(h, KC_RESID64, k_resid64<R><<<row_blocks_for(h, g, k_resid64<R>), RB, 0, s>>>(g, h->pressure, h->T[0], h->T[1], h->T[2],
                                                               h->flags, h->qterm, resid_dsum(h), H.r, d, 0,
                                                               nullptr, nullptr, rk, &c->ls_skip));
    WPF_LAUNCH(h, KC_OTHER, k_ctl_pass<<<1, 32, 0, s>>>(c, d, h->opts.rtol, h->opts.inner_rtol, h->opts.max_outer,
                                                         mixed, h_pass));
    WPF_CUDA(cudaGetLastError());
    cnt->per_pass = (l1 - l0) + (h->nlaunch - l2);
    if ((rc = gb_end(pass))) return rc;

    bool split_done = false;
    if ((rc = gb_add_split(h, b, &split_done))) return rc;
    if ((rc = gb_begin(b))) return rc;
    l0 = h->nlaunch;
    if ((rc = phys_halo(h, h->pressure))) return rc;   // updateHalo(pressure), :1050
    WPF_CUDA(cudaEventRecordWithFlags(h->ev[1], s, cudaEventRecordExternal));
    WPF_CUDA(cudaEventRecordWithFlags(h->ev[2], s, cudaEventRecordExternal));
    if ((rc = phys_capture_update(h, &c->dt, s, split_done))) return rc;
    WPF_CUDA(cudaEventRecordWithFlags(h->ev[3], s, cudaEventRecordExternal));
    cnt->fixed += h->nlaunch - l0;
    return WPF_OK;
}

int ws_capture_early(wpf_handle* h, bool* launched) {
    *launched = false;
    if (!((h->opts.flags & WPF_SOLVER_EXTRAPOLATE) && h->ws[0] && h->ws_e[0] && h->cap_ws)) return WPF_OK;
    // the least-squares start is built after calcPermeability (it needs the
    // kept residual corrected for this step)
    if (h->opts.mode == WPF_SOLVER_MIXED && h->rkeep_ok && !(h->opts.flags & WPF_SOLVER_FIXED_START)) return WPF_OK;
    const Grid& g = h->g;
    WPF_CUDA(cudaEventRecord(h->cap_ws_fork, h->stream));
    WPF_CUDA(cudaStreamWaitEvent(h->cap_ws, h->cap_ws_fork, 0));
    WPF_LAUNCH(h, KC_RESID64, k_ws_build_ext<<<row_blocks(h, g), RB, 0, h->cap_ws>>>(
        g, h->ws[0], h->ws[1], 0.f, 0.f, h->ws_e[0], h->dsc, &h->gctl->wa));
    WPF_CUDA(cudaGetLastError());
    *launched = true;
    return WPF_OK;
}

int solve_capture(wpf_handle* h, GraphBuilder& b, StepCounts* n) {
    if (h->ndir <= 0) return WPF_ERR_SINGULAR;
    if (h->opts.mode == WPF_SOLVER_MIXED) return solve_capture_impl(h, h->h32, b, n);
    return solve_capture_impl(h, h->h64, b, n);
}

int solve_pressure(wpf_handle* h, wpf_step_stats* st) {
    if (h->ndir <= 0) return WPF_ERR_SINGULAR;
    h->gctl_dirty = true;   // the increment history moves on the host
    int rc = solver_setup(h);
    if (rc) return rc;
    rc = phys_set_dirichlet(h);
    if (rc) return rc;
    WPF_CUDA(cudaEventRecord(h->ev[0], h->stream));
    if (h->opts.mode == WPF_SOLVER_MIXED) rc = solve_impl(h, h->h32, st);
    else rc = solve_impl(h, h->h64, st);
    int rc2 = phys_halo(h, h->pressure);   // updateHalo(pressure), :1050
    WPF_CUDA(cudaEventRecord(h->ev[1], h->stream));
    // a sweep whose bounded staging wait ran out left its flag
    WPF_CUDA(cudaMemcpyAsync(h->hsc + S_KERR, h->dsc + S_KERR, sizeof(double), cudaMemcpyDeviceToHost,
                             h->stream));
    WPF_CUDA(cudaEventSynchronize(h->ev[1]));
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    int kerr = 0;
    memcpy(&kerr, h->hsc + S_KERR, sizeof(int));
    if (kerr) {
        WPF_CUDA(cudaMemsetAsync(h->dsc + S_KERR, 0, sizeof(double), h->stream));
        rc = WPF_ERR_TIMEOUT;
    }
    if (st) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
        st->solve_ms = ms;
    }
    return rc ? rc : rc2;
}

}  // namespace wpf
