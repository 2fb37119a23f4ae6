// wpf_physics.cu -- FP64 field kernels of the wPFAW3D step on sm_103a.
//
// Per-cell physics follows wPFAW3D.f90 (calcPermeability :561-599,
// calcVelocity :1164-1193, calcPhaseDeriv :1197-1440, calcConcentDeriv
// :1554-1624, evolve* :1628-1640, updateHalo :1645-1657).  The trigonometric
// functions of calcPhaseDeriv are replaced by exact identities:
//   theta = atan(t), t = phiy/a, a = phix + 1e-20:
//     cos^2 = a^2/(a^2+phiy^2), sin^2 = phiy^2/(a^2+phiy^2),
//     cos = |a|/sqrt(a^2+phiy^2), sin = sign(a)*phiy/sqrt(a^2+phiy^2);
//   phi = acos(u), u = phiz/(|grad phi| + 1e-20):
//     cos 4phi = 8u^2(u^2-1)+1, sin 4phi = 4u sqrt(1-u^2)(2u^2-1),
//   cos 2theta = cos^2 - sin^2.
// and the angular-derivative terms f2, f4, f5, f6 are exactly zero unless one
// of the signed guards phix, phiy, phiz > 1/dx (:1333, :1342, :1355) holds,
// which needs a phase overshoot; the kernel evaluates them only then.
//
// FP64 on GB300 issues at a small fraction of the FP32 rate, so the kernels
// spend FP64 only where the result can differ from a known value:
//   * a cell whose 19-point phase neighbourhood is bitwise uniform (and
//     finite) has all nine derivatives exactly zero: the reference's early
//     exit (:1283) with tau = tau0 (|grad| = 0 -> v_s = 0 -> kxx = D);
//   * a non-well cell whose concentration and six neighbours are all zero has
//     zero diffusion and zero upwind fluxes: dc/dt = alpha dphi/dt;
//   * face velocities are formed only where one of the two needs them.
// Divisions by a parameter (dx, mu, tau0) become multiplications by its
// precomputed reciprocal; results differ from the literal Fortran arithmetic
// by a few ulp, well inside the parity tolerances.
#include "wpf_internal.cuh"

namespace wpf {

__device__ __forceinline__ long long bits(double v) { return __double_as_longlong(v); }
__device__ __forceinline__ bool zero_bits(double v) { return (bits(v) << 1) == 0; }
// Comparisons on the integer pipe (GB300 issues FP64 compares and min/max on
// its narrow FP64 pipe).  gt_bits(x, m) for m >= 0 is x > m for every x but a
// NaN of positive sign; every use below gives NaN for such an x either way.
__device__ __forceinline__ bool gt_bits(double x, double m) { return bits(x) > bits(m); }
// |x| > 1, false for NaN (as x > 1 || x < -1)
__device__ __forceinline__ bool abs_gt_one(double x) {
    const unsigned long long a = (unsigned long long)bits(x) & 0x7fffffffffffffffull;
    return a > 0x3ff0000000000000ull && a <= 0x7ff0000000000000ull;
}
// m := max(m, |x|) on the bit patterns, NaN ignored (as fmax(m, fabs(x)))
__device__ __forceinline__ void max_abs_bits(unsigned long long& m, double x) {
    const unsigned long long a = (unsigned long long)bits(x) & 0x7fffffffffffffffull;
    if (a <= 0x7ff0000000000000ull && a > m) m = a;
}

// All 18 neighbours (6 faces + 12 edges) equal to the finite centre, bitwise.
__device__ __forceinline__ bool phase_uniform(const double* __restrict__ ph, long long n,
                                              long long sy, long long sz) {
    const long long b0 = bits(ph[n]);
    if ((b0 & 0x7ff0000000000000LL) == 0x7ff0000000000000LL) return false;   // NaN / Inf
    if (bits(ph[n + 1]) != b0 || bits(ph[n - 1]) != b0 || bits(ph[n + sy]) != b0 ||
        bits(ph[n - sy]) != b0 || bits(ph[n + sz]) != b0 || bits(ph[n - sz]) != b0)
        return false;
    return bits(ph[n + 1 + sy]) == b0 && bits(ph[n + 1 - sy]) == b0 && bits(ph[n - 1 + sy]) == b0 &&
           bits(ph[n - 1 - sy]) == b0 && bits(ph[n + sy + sz]) == b0 && bits(ph[n - sy + sz]) == b0 &&
           bits(ph[n + sy - sz]) == b0 && bits(ph[n - sy - sz]) == b0 && bits(ph[n + 1 + sz]) == b0 &&
           bits(ph[n - 1 + sz]) == b0 && bits(ph[n + 1 - sz]) == b0 && bits(ph[n - 1 - sz]) == b0;
}

// The same two tests with every load issued before any comparison (no
// short circuit), so a thread keeps its 26 loads in flight together: the
// classification kernel touches every cell and is bound by memory latency.
__device__ __forceinline__ bool phase_uniform_eager(const double* __restrict__ ph, long long n,
                                                    long long sy, long long sz) {
    const long long o[18] = {1, -1, sy, -sy, sz, -sz, 1 + sy, 1 - sy, -1 + sy, -1 - sy, sy + sz, -sy + sz,
                             sy - sz, -sy - sz, 1 + sz, -1 + sz, 1 - sz, -1 - sz};
    long long v[18];
    const long long b0 = bits(ph[n]);
#pragma unroll
    for (int q = 0; q < 18; ++q) v[q] = bits(ph[n + o[q]]);
    long long diff = 0;
#pragma unroll
    for (int q = 0; q < 18; ++q) diff |= v[q] ^ b0;
    return diff == 0 && (b0 & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool concent_zero_eager(const double* __restrict__ C, long long n, long long sy,
                                                   long long sz) {
    const long long a = bits(C[n]) | bits(C[n + 1]) | bits(C[n - 1]) | bits(C[n + sy]) | bits(C[n - sy]) |
                        bits(C[n + sz]) | bits(C[n - sz]);
    return (a << 1) == 0;
}

// Face velocities around a cell: u_{x+}, u_{x-}, u_{y+}, u_{y-}, u_{z+}, u_{z-}.
struct FaceVel {
    double xp, xm, yp, ym, zp, zm;
};

// dphasedt and kxx of one interior cell (calcPhaseDeriv, wPFAW3D.f90:1231-1414).
// The relaxation time tau = tau_num / kxx (:1254) enters only the step's
// minimum; since a correctly rounded quotient falls as the divisor grows, that
// minimum is tau_num / (max kxx), taken once per block: one FP64 division
// per block instead of one per cell, and the same bits.
// vel() yields the six face velocities; it is called at most once, and only
// when |grad phi| > 1e-6 (the only use of the velocity in this routine).
template <typename VelF>
__device__ __forceinline__ void phase_cell(const double* __restrict__ ph, long long n, long long sy,
                                           long long sz, VelF&& vel, double conc, bool well,
                                           const Phys& P, double& rate, double& kxx_out, int& over) {
    rate = 0.0;
    over = 0;
    kxx_out = P.diffusion;
    if (phase_uniform(ph, n, sy, sz)) return;                            // :1283-1286
    const double c0 = ph[n];
    const double pe = ph[n + 1], pw = ph[n - 1], pn = ph[n + sy], ps = ph[n - sy];
    const double pt = ph[n + sz], pb = ph[n - sz];
    const double phix = (pe - pw) * P.inv_2dx;       // grad_phase, :1472-1474
    const double phiy = (pn - ps) * P.inv_2dx;
    const double phiz = (pt - pb) * P.inv_2dx;
    const double rxy2 = phix * phix + phiy * phiy;
    const double r2 = rxy2 + phiz * phiz;
    const double dpf = sqrt(r2);                                         // :1232
    double vs = 0.0;
    if (dpf > 1.0e-6) {                                                  // :1234-1244
        const FaceVel u = vel();
        const double vx = 0.5 * (u.xp + u.xm), vy = 0.5 * (u.yp + u.ym), vz = 0.5 * (u.zp + u.zm);
        vs = (vx * phix + vy * phiy + vz * phiz) / dpf;
    }
    double inv_tau = P.inv_tau0;                                         // :1246-1254
    if (!(vs >= 0.0)) {
        // ral vs^2 / sqrt(vs^2) of :1249 is ral |vs| (to a few ulp)
        const double kxx = P.diffusion + fabs(conc) * P.epsilon * (P.ral * fabs(vs));
        kxx_out = kxx;
        inv_tau = kxx * P.inv_tau_num;
    }
    if (well) return;                                                    // :1257-1261
    if (zero_bits(phix) && zero_bits(phiy) && zero_bits(phiz)) {         // :1283-1286
        const double pxx = pe - 2.0 * c0 + pw, pyy = pn - 2.0 * c0 + ps, pzz = pt - 2.0 * c0 + pb;
        const double pxy = ph[n + 1 + sy] - ph[n + 1 - sy] - ph[n - 1 + sy] + ph[n - 1 - sy];
        const double pyz = ph[n + sy + sz] - ph[n - sy + sz] - ph[n + sy - sz] + ph[n - sy - sz];
        const double pzx = ph[n + 1 + sz] - ph[n - 1 + sz] - ph[n + 1 - sz] + ph[n - 1 - sz];
        if (zero_bits(pxx) && zero_bits(pyy) && zero_bits(pzz) && zero_bits(pxy) && zero_bits(pyz) &&
            zero_bits(pzx))
            return;
    }
    const double lap = (pe + pw + pn + ps + pt + pb - 6.0 * c0) * P.inv_dx2;   // :1451-1460
    const double f1 = (1.0 - c0 * c0) * (c0 - P.lambda * conc);                // :1381
    const double a = phix + 1.0e-20;
    const double a2 = a * a, py2 = phiy * phiy;
    const double dd = dpf + 1.0e-20;
    const bool gth = gt_bits(phix, P.maxdphi) || gt_bits(phiy, P.maxdphi);       // :1333, :1355
    const bool gph = gth || gt_bits(phiz, P.maxdphi);                            // :1342
    if (!gph) {
        // f2 = f4 = f5 = f6 = 0: only W (:1309) is needed; one reciprocal
        // gives cos^2 theta, sin^2 theta and cos^2 phi.
        const double den = a2 + py2, dd2 = dd * dd;
        const double inv = 1.0 / (den * dd2);
        const double c2 = a2 * dd2 * inv, s2 = py2 * dd2 * inv;
        const double u2 = (phiz * phiz) * den * inv;
        const double c4phi = 8.0 * u2 * (u2 - 1.0) + 1.0;
        const double w = P.w0 * (1.0 + P.epsilon * (7.0 * (c2 * c2) - 6.0 * c2 + (s2 * s2) * c4phi));
        rate = (f1 + (w * w) * lap) * inv_tau;
    } else {
        const double rn = 1.0 / sqrt(a2 + py2);
        const double c = fabs(a) * rn;
        const double s = copysign(1.0, a) * phiy * rn;
        double u = phiz / dd;
        u = fmin(1.0, fmax(-1.0, u));
        const double u2 = u * u;
        const double sp = sqrt(fmax(0.0, 1.0 - u2));
        const double c4phi = 8.0 * u2 * (u2 - 1.0) + 1.0;
        const double s4phi = 4.0 * u * sp * (2.0 * u2 - 1.0);
        const double c2 = c * c, s2 = s * s, c4 = c2 * c2, s4 = s2 * s2;
        const double cos2t = c2 - s2;
        const double eps = P.epsilon, w0 = P.w0;
        const double w = w0 * (1.0 + eps * (7.0 * c4 - 6.0 * c2 + s4 * c4phi));                 // :1309
        const double dwdth = w0 * (4.0 * eps * s * c * (-7.0 * c2 + 3.0 + s2 * c4phi));        // :1312
        const double ddwdth = w0 * (4.0 * eps * (cos2t * (-7.0 * c2 + 3.0 + s2 * c4phi) +
                                                 2.0 * s2 * c2 * (7.0 + c4phi)));               // :1316
        const double dwdph = w0 * (-4.0 * eps * s4 * s4phi);                                    // :1320
        const double ddwdph = w0 * (-16.0 * eps * s4 * c4phi);                                  // :1323
        const double ddwdthph = w0 * (-16.0 * eps * (s2 * s) * c * s4phi);                      // :1326
        const double pxx = (pe - 2.0 * c0 + pw) * P.inv_dx2;
        const double pyy = (pn - 2.0 * c0 + ps) * P.inv_dx2;
        const double pzz = (pt - 2.0 * c0 + pb) * P.inv_dx2;
        const double pxy = (ph[n + 1 + sy] - ph[n + 1 - sy] - ph[n - 1 + sy] + ph[n - 1 - sy]) * P.inv_4dx2;
        const double pyz = (ph[n + sy + sz] - ph[n - sy + sz] - ph[n + sy - sz] + ph[n - sy - sz]) * P.inv_4dx2;
        const double pzx = (ph[n + 1 + sz] - ph[n - 1 + sz] - ph[n + 1 - sz] + ph[n - 1 - sz]) * P.inv_4dx2;
        double dthx = 0.0, dthy = 0.0, dthz = 0.0, dthpx = 0.0, dthpy = 0.0;
        if (gth) {                                                                              // :1333-1337
            const double den = 1.0 / (rxy2 + 1.0e-20);
            dthx = (pxy * phix - phiy * pxx) * den;
            dthy = (pyy * phix - phiy * pxy) * den;
            dthz = (pyz * phix - phiy * pzx) * den;
            dthpx = -phiy * r2 * den;                                                           // :1356
            dthpy = phix * r2 * den;                                                            // :1357
        }
        const double rxy = sqrt(rxy2);
        const double den2 = 1.0 / (r2 * rxy + 1.0e-20);                                         // :1344
        const double dphx = (phiz * (phix * pxx + phiy * pxy) - rxy2 * pzx) * den2;
        const double dphy = (phiz * (phix * pxy + phiy * pyy) - rxy2 * pyz) * den2;
        const double dphz = (phiz * (phix * pzx + phiy * pyz) - rxy2 * pzz) * den2;
        const double dphpx = phix * phiz / (rxy * dpf + 1.0e-20);                               // :1363
        const double dphpy = phiy * phiz / (rxy * dpf + 1.0e-20);                               // :1364
        const double dphpz = -rxy / dd;                                                         // :1365
        const double dwdx = dwdth * dthx + dwdph * dphx;                                        // :1367
        const double dwdy = dwdth * dthy + dwdph * dphy;
        const double dwdz = dwdth * dthz + dwdph * dphz;
        const double ddwthx = ddwdth * dthx + ddwdthph * dphx;                                  // :1371
        const double ddwthy = ddwdth * dthy + ddwdthph * dphy;
        const double ddwphx = ddwdph * dphx + ddwdthph * dthx;                                  // :1375
        const double ddwphy = ddwdph * dphy + ddwdthph * dthy;
        const double ddwphz = ddwdph * dphz + ddwdthph * dthz;
        const double d2 = dpf * dpf;
        const double f2 = 2.0 * w * (dwdx * phix + dwdy * phiy + dwdz * phiz);                  // :1386
        const double f3 = (w * w) * lap;                                                        // :1390
        const double f4 = dwdx * (dwdth * dthpx * d2 + dwdph * dphpx * d2) +
                          w * (ddwthx * dthpx * d2 + ddwphx * dphpx * d2);                      // :1395
        const double f5 = dwdy * (dwdth * dthpy * d2 + dwdph * dphpy * d2) +
                          w * (ddwthy * dthpy * d2 + ddwphy * dphpy * d2);                      // :1401
        const double f6 = dwdz * (dwdph * dphpz * d2) + w * (ddwphz * dphpz * d2);              // :1407
        rate = (f1 + f2 + f3 + f4 + f5 + f6) * inv_tau;                                         // :1414
    }
    over = abs_gt_one(c0) ? 1 : 0;                                                              // :1425
}

// The concentration and its six neighbours are all (signed) zero.
__device__ __forceinline__ bool concent_zero(const double* __restrict__ C, long long n, long long sy,
                                             long long sz) {
    return zero_bits(C[n]) && zero_bits(C[n + 1]) && zero_bits(C[n - 1]) && zero_bits(C[n + sy]) &&
           zero_bits(C[n - sy]) && zero_bits(C[n + sz]) && zero_bits(C[n - sz]);
}

// dconcentdt of one non-well interior cell (calcConcentDeriv, :1568-1606).
__device__ __forceinline__ double concent_cell(const double* __restrict__ C, long long n,
                                               long long sy, long long sz, const FaceVel& u,
                                               double dphidt, const Phys& P) {
    const double c0 = C[n];
    const double ce = C[n + 1], cw = C[n - 1], cn = C[n + sy], cs = C[n - sy];
    const double ct = C[n + sz], cb = C[n - sz];
    const double lap = (ce + cw + cn + cs + ct + cb - 6.0 * c0) * P.inv_dx2;
    const double fxp = u.xp * (gt_bits(u.xp, 0.0) ? c0 : ce), fxm = u.xm * (gt_bits(u.xm, 0.0) ? cw : c0);
    const double fyp = u.yp * (gt_bits(u.yp, 0.0) ? c0 : cn), fym = u.ym * (gt_bits(u.ym, 0.0) ? cs : c0);
    const double fzp = u.zp * (gt_bits(u.zp, 0.0) ? c0 : ct), fzm = u.zm * (gt_bits(u.zm, 0.0) ? cb : c0);
    const double div = ((fxp - fxm) + (fyp - fym) + (fzp - fzm)) * P.inv_dx;
    return P.diffusion * lap + P.alpha * dphidt - div;
}

// FP32 rates of the FP32-refined form.  Differences that cancel -- of the
// pressure across a face, of the phase across a cell -- are taken in FP64 from
// the FP64 state (neighbouring values agree in their leading digits); the
// rest -- face velocities, upwind fluxes, the Laplacians of c, the anisotropy
// function, the relaxation time -- in FP32, the conversions on the integer
// pipe.  A rate enters the FP64 state as x + dt * rate; its FP32 rounding
// (~1e-7 relative) is a 1e-7 part of one step's change.
struct LoConst {
    float diffusion, inv_dx, inv_dx2;
    float alpha, epsilon, ral, w0, inv_tau0, inv_tau_num;
};
__device__ __forceinline__ LoConst lo_const(const Phys& P) {
    return LoConst{f64_to_f32(P.diffusion), f64_to_f32(P.inv_dx),  f64_to_f32(P.inv_dx2),
                   f64_to_f32(P.alpha),     f64_to_f32(P.epsilon), f64_to_f32(P.ral),
                   f64_to_f32(P.w0),        f64_to_f32(P.inv_tau0), f64_to_f32(P.inv_tau_num)};
}
struct FaceVelF {
    float xp, xm, yp, ym, zp, zm;
};
// -K_f/mu (p_nb - p)/dx (:1169-1176) with 1/dx folded into Tv; p_nb - p in FP64
__device__ __forceinline__ FaceVelF face_vel_lo(const double* __restrict__ pr, const double* __restrict__ Tvx,
                                                const double* __restrict__ Tvy, const double* __restrict__ Tvz,
                                                long long n, long long sy, long long sz) {
    const double p0 = pr[n];
    FaceVelF u;
    u.xp = -(f64_to_f32(Tvx[n]) * f64_to_f32(pr[n + 1] - p0));
    u.xm = -(f64_to_f32(Tvx[n - 1]) * f64_to_f32(p0 - pr[n - 1]));
    u.yp = -(f64_to_f32(Tvy[n]) * f64_to_f32(pr[n + sy] - p0));
    u.ym = -(f64_to_f32(Tvy[n - sy]) * f64_to_f32(p0 - pr[n - sy]));
    u.zp = -(f64_to_f32(Tvz[n]) * f64_to_f32(pr[n + sz] - p0));
    u.zm = -(f64_to_f32(Tvz[n - sz]) * f64_to_f32(p0 - pr[n - sz]));
    return u;
}
__device__ __forceinline__ void fold_umax_lo(unsigned long long& umax, const FaceVelF& u) {
    max_abs_bits(umax, f32_to_f64(u.xp));
    max_abs_bits(umax, f32_to_f64(u.yp));
    max_abs_bits(umax, f32_to_f64(u.zp));
}
// D lap(c) - div(u c) of calcConcentDeriv (:1568-1606) in FP32, the Laplacian
// in difference form (no large value cancels); the caller adds alpha dphase/dt
__device__ __forceinline__ float concent_transport_lo(const double* __restrict__ C, long long n, long long sy,
                                                      long long sz, const FaceVelF& u, const LoConst& K,
                                                      float& diff) {
    const float c0 = f64_to_f32(C[n]);
    const float ce = f64_to_f32(C[n + 1]), cw = f64_to_f32(C[n - 1]), cn = f64_to_f32(C[n + sy]);
    const float cs = f64_to_f32(C[n - sy]), ct = f64_to_f32(C[n + sz]), cb = f64_to_f32(C[n - sz]);
    const float lap = (((ce - c0) + (cw - c0)) + ((cn - c0) + (cs - c0)) + ((ct - c0) + (cb - c0))) * K.inv_dx2;
    const float fxp = u.xp * (u.xp > 0.f ? c0 : ce), fxm = u.xm * (u.xm > 0.f ? cw : c0);   // strict > 0, :1593
    const float fyp = u.yp * (u.yp > 0.f ? c0 : cn), fym = u.ym * (u.ym > 0.f ? cs : c0);
    const float fzp = u.zp * (u.zp > 0.f ? c0 : ct), fzm = u.zm * (u.zm > 0.f ? cb : c0);
    diff = K.diffusion * lap;
    return ((fxp - fxm) + (fyp - fym) + (fzp - fzm)) * K.inv_dx;
}
// dconcentdt of a concentration-only cell (bitwise-uniform phase
// neighbourhood, so dphase/dt = 0 and the reaction term vanishes).  Folds |u|
// of the three + faces into umax.
__device__ __forceinline__ float concent_rate_lo(const double* __restrict__ C, const double* __restrict__ pr,
                                                 const double* __restrict__ Tvx, const double* __restrict__ Tvy,
                                                 const double* __restrict__ Tvz, long long n, long long sy,
                                                 long long sz, const LoConst& K, unsigned long long& umax) {
    const FaceVelF u = face_vel_lo(pr, Tvx, Tvy, Tvz, n, sy, sz);
    float diff;
    const float div = concent_transport_lo(C, n, sy, sz, u, K, diff);
    fold_umax_lo(umax, u);
    return diff - div;
}

// dphasedt and kxx of an interface cell on the guard-free path of phase_cell
// (f2 = f4 = f5 = f6 = 0), for the FP32-refined form.  In FP64: the three
// central differences (so the anisotropy guard and the zero tests see the same
// bits as phase_cell), the Laplacian's sum, the two factors of f1 and the
// pressure differences.  In FP32: the gradient, scaled by a power of two so
// that its largest component lies in [1, 2) (cos^2 theta, sin^2 theta,
// cos^2 phi and vs do not change under the scaling; the 1e-20 guards of
// :1232 and :1306 are scaled with it), W (:1309), vs and tau (:1234-1254), the
// rate (:1414).  Returns false, having written nothing, where phase_cell runs
// in FP64 instead: a uniform neighbourhood, the anisotropy guard, all three
// first derivatives zero (the second-derivative exit test of :1283-1286), or a
// gradient direction or size outside what the scaled FP32 form represents.
// u/have_u: the face velocities when vs needed them.
__device__ __forceinline__ bool phase_cell_lo(const double* __restrict__ ph, long long n, long long sy,
                                              long long sz, const double* __restrict__ pr,
                                              const double* __restrict__ Tvx, const double* __restrict__ Tvy,
                                              const double* __restrict__ Tvz, double conc, bool well,
                                              const Phys& P, const LoConst& K, float& rate, double& kxx_out,
                                              int& over, FaceVelF& u, bool& have_u) {
    if (phase_uniform(ph, n, sy, sz)) return false;
    const double c0 = ph[n];
    const double pe = ph[n + 1], pw = ph[n - 1], pn = ph[n + sy], ps = ph[n - sy];
    const double pt = ph[n + sz], pb = ph[n - sz];
    const double phix = (pe - pw) * P.inv_2dx;       // grad_phase, :1472-1474
    const double phiy = (pn - ps) * P.inv_2dx;
    const double phiz = (pt - pb) * P.inv_2dx;
    if (gt_bits(phix, P.maxdphi) || gt_bits(phiy, P.maxdphi) || gt_bits(phiz, P.maxdphi)) return false;
    if (zero_bits(phix) && zero_bits(phiy) && zero_bits(phiz)) return false;
    const float fx = f64_to_f32(phix), fy = f64_to_f32(phiy), fz = f64_to_f32(phiz);
    const unsigned mb = max(max(__float_as_uint(fx) & 0x7fffffffu, __float_as_uint(fy) & 0x7fffffffu),
                            __float_as_uint(fz) & 0x7fffffffu);
    const int e = (int)(mb >> 23) - 127;             // exponent of the largest component
    if (e < -100 || e > 100) return false;
    const float s = __uint_as_float((unsigned)(127 - e) << 23);   // 2^-e, exact scaling
    const float gx = fx * s, gy = fy * s, gz = fz * s, g20 = 1.0e-20f * s;
    const float rxy2 = gx * gx + gy * gy;
    const float dpf = sqrtf(rxy2 + gz * gz);         // s |grad phase|, :1232
    const float a = gx + g20, a2 = a * a, py2 = gy * gy;
    const float den = a2 + py2;
    if (den < 1.0e-30f) return false;                // gradient along z to FP32 precision
    float vs = 0.f;
    if (dpf > 1.0e-6f * s) {                         // :1234-1244
        u = face_vel_lo(pr, Tvx, Tvy, Tvz, n, sy, sz);
        have_u = true;
        const float vx = 0.5f * (u.xp + u.xm), vy = 0.5f * (u.yp + u.ym), vz = 0.5f * (u.zp + u.zm);
        vs = (vx * gx + vy * gy + vz * gz) / dpf;
    }
    float inv_tau = K.inv_tau0;                      // :1246-1254
    kxx_out = P.diffusion;
    if (!(vs >= 0.f)) {
        const float kxx = K.diffusion + fabsf(f64_to_f32(conc)) * K.epsilon * (K.ral * fabsf(vs));
        kxx_out = f32_to_f64(kxx);
        inv_tau = kxx * K.inv_tau_num;
    }
    over = 0;
    rate = 0.f;
    if (well) return true;                           // :1257-1261
    const float lap = f64_to_f32(pe + pw + pn + ps + pt + pb - 6.0 * c0) * K.inv_dx2;   // :1451-1460
    const float f1 = f64_to_f32(1.0 - c0 * c0) * f64_to_f32(c0 - P.lambda * conc);      // :1381
    const float dd = dpf + g20;
    const float rden = 1.0f / den;
    const float c2 = a2 * rden, s2 = py2 * rden;
    const float u2 = (gz * gz) / (dd * dd);
    const float c4phi = 8.0f * u2 * (u2 - 1.0f) + 1.0f;
    const float w = K.w0 * (1.0f + K.epsilon * (7.0f * (c2 * c2) - 6.0f * c2 + (s2 * s2) * c4phi));
    rate = (f1 + (w * w) * lap) * inv_tau;
    over = abs_gt_one(c0) ? 1 : 0;                   // :1425
    return true;
}

// kmax: the largest kxx of the block's cells (0 if none), so that the block's
// smallest relaxation time is tau_num / kmax
__device__ __forceinline__ void flush_step_reductions(double kmax, double tau_num, int over, double umax,
                                                      double* dsc) {
    __shared__ double sm[32];
    __shared__ int smi[32];
    const double kb = block_max(kmax, sm, 0.0);
    const int osum = block_sum(over, smi);
    const double um = block_max(umax, sm, 0.0);
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
        if (kb > 0.0) atomicMin(reinterpret_cast<unsigned long long*>(dsc + S_TAUMIN_KEY), dkey(tau_num / kb));
        if (osum) atomicAdd(reinterpret_cast<unsigned long long*>(dsc + S_OVERSHOOT),
                            (unsigned long long)osum);
        if (um > 0.0)
            atomicMax(reinterpret_cast<unsigned long long*>(dsc + S_UMAX_BITS),
                      (unsigned long long)__double_as_longlong(um));
    }
}

// ---------------------------------------------------------------------------
// calcPermeability (:561-599).  One thread per face-cell (i,j,k) in
// [0..nx]x[0..ny]x[0..nz]: the cell permeability K0 = kwh f + Krock (1-f) of
// the cell and its +x/+y/+z neighbours, and the three harmonic means
// 2ab/(a+b) (= 2/(1/a+1/b)).  T = K_f/mu with the global boundary faces set
// to zero (the merge guards of :843-848), and Tv = T/dx for the fused update's
// velocities (one FP64 multiply per face less there); Kf/K0 only when
// materialised.
// prev != null: skip a face-cell whose four cells have bitwise the same phase
// as in prev, the field T was last computed from (T is then unchanged).
// ---------------------------------------------------------------------------
// With rk (the FP64 outer residual of the current pressure under the old T):
// every recomputed face f between cells a and b whose T changed adds
// (T_new - T_old)(p_b - p_a) to the residual of a live cell a (and the mirror
// term to b), so that rk becomes the residual under the new T without a pass
// over the grid (the update changes the phase of a few per cent of the cells).
// Returns the owner cell a's share (summed by the caller into one atomic) and
// adds the neighbour's share to rk[b].
__device__ __forceinline__ double resid_face_delta(double* rk, const uint8_t* __restrict__ fl,
                                                   const double* __restrict__ pr, long long a, long long b,
                                                   double p_a, double dT) {
    if (zero_bits(dT)) return 0.0;   // dT == 0 on the integer pipe
    const double d = dT * (pr[b] - p_a);
    if (!(fl[b] & F_DIR)) atomicAdd(rk + b, -d);
    return d;
}

constexpr int PB_X = 32, PB_Y = 4, PB_Z = 2;   // k_permeability's block
__global__ void __launch_bounds__(PB_X * PB_Y * PB_Z) k_permeability(Grid g, Phys P, const double* __restrict__ ph,
                               const double* __restrict__ prev, const double* __restrict__ kr,
                               double* __restrict__ Tx, double* __restrict__ Ty,
                               double* __restrict__ Tz, double* __restrict__ Kx,
                               double* __restrict__ Ky, double* __restrict__ Kz, double inv_mu,
                               double* rk = nullptr, const uint8_t* __restrict__ fl = nullptr,
                               const double* __restrict__ pr = nullptr, uint8_t* __restrict__ mark = nullptr,
                               double* __restrict__ Tvx = nullptr, double* __restrict__ Tvy = nullptr,
                               double* __restrict__ Tvz = nullptr) {
    // A block of PB_X x PB_Y x PB_Z face-cells; the cell permeabilities its
    // faces need (its cells and the +x/+y/+z neighbours) are computed once
    // each into shared memory instead of once per adjacent face.
    constexpr int KX = PB_X + 1, KY = PB_Y + 1, KZ = PB_Z + 1, KN = KX * KY * KZ;
    __shared__ double sK[KN];
    __shared__ unsigned char need[KN];
    const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
    const int tid = tx + PB_X * (ty + PB_Y * tz);
    const int i0 = blockIdx.x * PB_X, j0 = blockIdx.y * PB_Y, k0 = blockIdx.z * PB_Z;
    const int i = i0 + tx, j = j0 + ty, k = k0 + tz;
    for (int q = tid; q < KN; q += PB_X * PB_Y * PB_Z) need[q] = 0;
    __syncthreads();
    const bool in = i <= g.nx && j <= g.ny && k <= g.nz;
    const long long n = in ? g.at(i, j, k) : 0;
    // with prev: a face is recomputed only when one of its two cells changed
    // phase (the harmonic means are FP64 divisions, the costliest work here)
    bool fx = in, fy = in, fz = in;
    if (in && prev) {
        const bool c0 = bits(ph[n]) != bits(prev[n]);
        fx = c0 || bits(ph[n + 1]) != bits(prev[n + 1]);
        fy = c0 || bits(ph[n + g.P]) != bits(prev[n + g.P]);
        fz = c0 || bits(ph[n + g.S]) != bits(prev[n + g.S]);
    }
    const int t0 = tx + KX * (ty + KY * tz);   // this face-cell in the K tile
    if (fx || fy || fz) {
        need[t0] = 1;
        if (fx) need[t0 + 1] = 1;
        if (fy) need[t0 + KX] = 1;
        if (fz) need[t0 + KX * KY] = 1;
    }
    if (!__syncthreads_or(fx || fy || fz)) return;   // block-uniform
    for (int q = tid; q < KN; q += PB_X * PB_Y * PB_Z) {
        if (!need[q]) continue;
        const int qx = q % KX, qy = (q / KX) % KY, qz = q / (KX * KY);
        const long long m = g.at(i0 + qx, j0 + qy, k0 + qz);
        const double f = 0.5 * (1.0 + ph[m]);
        sK[q] = P.kwh * f + kr[m] * (1.0 - f);   // K0 of :567-574
    }
    __syncthreads();
    if (!(fx || fy || fz)) return;   // no barrier below
    const double a = sK[t0];
    const double a2 = 2.0 * a;   // 2 a b = (2 a) b exactly: one multiply per face
    const bool in_j = j >= 1 && j <= g.ny, in_k = k >= 1 && k <= g.nz, in_i = i >= 1 && i <= g.nx;
    const double p_a = rk ? pr[n] : 0.0;
    double own = 0.0;
    // face towards m (owner n; its K0 at tile offset dm): T = 2 a b / (a + b)
    // / mu, 0 outside `inside`
    auto face = [&](long long m, int dm, bool inside, double* __restrict__ T, double* __restrict__ Kf,
                    double* __restrict__ Tv) {
        const double b = sK[t0 + dm];
        const double kf = (a2 * b) * rcp_nr(a + b);
        const double t = inside ? kf * inv_mu : 0.0;
        if (rk) own += resid_face_delta(rk, fl, pr, n, m, p_a, t - T[n]);
        T[n] = t;
        if (Tv) Tv[n] = t * P.inv_dx;
        if (mark) {   // both cells' level-0 rows use this face
            mark[n] = 1;
            mark[m] = 1;
        }
        if (Kf) Kf[n] = kf;
    };
    if (fx) face(n + 1, 1, i >= 1 && i < g.nx && in_j && in_k, Tx, Kx, Tvx);
    if (fy) face(n + g.P, KX, j >= 1 && j < g.ny && in_i && in_k, Ty, Ky, Tvy);
    if (fz) face(n + g.S, KX * KY, k >= 1 && k < g.nz && in_i && in_j, Tz, Kz, Tvz);
    // boundary faces stay 0 (dT = 0): only interior pairs change the residual
    if (rk && own != 0.0 && !(fl[n] & F_DIR)) atomicAdd(rk + n, own);
}

// K0 over every cell of the halo grid (:567-574), for downloads only.
__global__ void k_cell_K0(Grid g, Phys P, const double* __restrict__ ph,
                          const double* __restrict__ kr, double* __restrict__ K0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i > g.nx + 1 || j > g.ny + 1 || k > g.nz + 1) return;
    const long long n = g.at(i, j, k);
    const double f = 0.5 * (1.0 + ph[n]);
    K0[n] = P.kwh * f + kr[n] * (1.0 - f);
}

// calcVelocity (:1169-1176): faces 0..n in every direction, unmasked K_f.
__global__ void k_velocity(Grid g, Phys P, const double* __restrict__ pr,
                           const double* __restrict__ Kx, const double* __restrict__ Ky,
                           const double* __restrict__ Kz, double* __restrict__ vx,
                           double* __restrict__ vy, double* __restrict__ vz, double inv_mu) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    const long long n = g.at(i, j, k);
    const double p0 = pr[n];
    vx[n] = -(Kx[n] * inv_mu * ((pr[n + 1] - p0) * P.inv_dx));
    vy[n] = -(Ky[n] * inv_mu * ((pr[n + g.P] - p0) * P.inv_dx));
    vz[n] = -(Kz[n] * inv_mu * ((pr[n + g.S] - p0) * P.inv_dx));
}

// calcPhaseDeriv over the interior (:1227-1437) from the velocity arrays.
__global__ void __launch_bounds__(RB) k_phase_deriv(Grid g, Phys P, const double* __restrict__ ph,
                                                    const double* __restrict__ cc,
                                                    const double* __restrict__ vx,
                                                    const double* __restrict__ vy,
                                                    const double* __restrict__ vz,
                                                    const uint8_t* __restrict__ fl,
                                                    double* __restrict__ dph, double* dsc) {
    double kmax = 0.0;
    int overs = 0;
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        auto vel = [&]() {
            return FaceVel{vx[n], vx[n - 1], vy[n], vy[n - g.P], vz[n], vz[n - g.S]};
        };
        double rate, kxx;
        int over;
        phase_cell(ph, n, g.P, g.S, vel, cc[n], (fl[n] & F_WELL) != 0, P, rate, kxx, over);
        dph[n] = rate;
        kmax = fmax(kmax, kxx);
        overs += over;
    }
    flush_step_reductions(kmax, P.tau_num, overs, 0.0, dsc);
}

// calcConcentDeriv over the interior (:1559-1576).
__global__ void __launch_bounds__(RB) k_concent_deriv(Grid g, Phys P, const double* __restrict__ cc,
                                                      const double* __restrict__ vx,
                                                      const double* __restrict__ vy,
                                                      const double* __restrict__ vz,
                                                      const uint8_t* __restrict__ fl,
                                                      const double* __restrict__ dph,
                                                      double* __restrict__ dcc) {
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        if (fl[n] & F_WELL) {
            dcc[n] = 0.0;
        } else {
            const FaceVel u{vx[n], vx[n - 1], vy[n], vy[n - g.P], vz[n], vz[n - g.S]};
            dcc[n] = concent_cell(cc, n, g.P, g.S, u, dph[n], P);
        }
    }
}

// Euler update over the interior (the halo derivative is zero, :1629/:1637).
__global__ void __launch_bounds__(RB) k_evolve(Grid g, double* __restrict__ f,
                                               const double* __restrict__ d, double dt) {
    ROW_LOOP(g) {
        const long long n = g.at(i, j, k);
        f[n] = f[n] + d[n] * dt;
    }
}

// updateHalo (:1651-1656): the sequential x, y, z plane copies leave every
// halo cell equal to the interior cell at the clamped index; one thread per
// halo cell.  Index space: x faces (2*(ny+2)*(nz+2)), y faces (2*nx*(nz+2)),
// z faces (2*nx*ny).
__global__ void k_halo(Grid g, double* __restrict__ f) {
    const long long nxf = 2LL * (g.ny + 2) * (g.nz + 2);
    const long long nyf = 2LL * g.nx * (g.nz + 2);
    const long long nzf = 2LL * g.nx * g.ny;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int i, j, k;
    if (t < nxf) {
        const int side = (int)(t & 1); t >>= 1;
        j = (int)(t % (g.ny + 2)); k = (int)(t / (g.ny + 2));
        i = side ? g.nx + 1 : 0;
    } else if ((t -= nxf) < nyf) {
        const int side = (int)(t & 1); t >>= 1;
        i = 1 + (int)(t % g.nx); k = (int)(t / g.nx);
        j = side ? g.ny + 1 : 0;
    } else if ((t -= nyf) < nzf) {
        const int side = (int)(t & 1); t >>= 1;
        i = 1 + (int)(t % g.nx); j = 1 + (int)(t / g.nx);
        k = side ? g.nz + 1 : 0;
    } else {
        return;
    }
    const int si = min(max(i, 1), g.nx), sj = min(max(j, 1), g.ny), sk = min(max(k, 1), g.nz);
    f[g.at(i, j, k)] = f[g.at(si, sj, sk)];
}

// Write v to every halo cell whose clamped source is the boundary cell (i,j,k).
__device__ __forceinline__ void write_halo_of(const Grid& g, int i, int j, int k, double* __restrict__ f,
                                              double v) {
    const int i0 = i == 1 ? -1 : 0, i1 = i == g.nx ? 1 : 0;
    const int j0 = j == 1 ? -1 : 0, j1 = j == g.ny ? 1 : 0;
    const int k0 = k == 1 ? -1 : 0, k1 = k == g.nz ? 1 : 0;
    if (!(i0 | i1 | j0 | j1 | k0 | k1)) return;
    for (int dk = k0; dk <= k1; ++dk)
        for (int dj = j0; dj <= j1; ++dj)
            for (int di = i0; di <= i1; ++di)
                if (di | dj | dk) f[g.at(i + di, j + dj, k + dk)] = v;
}

// ---------------------------------------------------------------------------
// Fused update: calcVelocity + calcPhaseDeriv + calcConcentDeriv + evolvePhase
// + evolveConcent + updateHalo for the interior, in two kernels so that FP64
// is spent only on cells whose update can differ from a copy:
//   k_update_split  -- every cell: a cell with a bitwise-uniform phase
//       neighbourhood (dphi/dt = 0, tau = tau0) that is a well or has an
//       all-zero concentration neighbourhood (dc/dt = 0) is copied to the new
//       buffers; every other cell is appended to a work list (warp-aggregated):
//       interface cells (non-uniform phase) from the front, cells that only
//       need the concentration rate (uniform phase) from the back, so that no
//       warp mixes the long phase-rate path with the short one.
//   k_update_active -- the work list, densely packed into full warps: face
//       velocities from Tv = K_f/(mu dx) and the solved pressure (zero on the global
//       boundary faces, as the reference's halo copy makes them), the phase
//       and concentration rates, Euler, halo.
// max|u| (the advection CFL statistic) is taken over the faces of the cells
// where the velocity enters the update (interface or non-zero concentration).
//
// Quiescent bricks.  The split walks bricks of 32 x 4 x 2 cells (one block
// iteration each) and records per brick whether any of its cells went to a
// work list.  A brick that was all copies in the last update, with all 26
// neighbour bricks too, is skipped: none of the values within one cell of it
// changed in that update, so its classification is again all copies, and
// both ping-pong buffers already hold its values (the last update copied
// them, or skipped it under the same rule).  Most of the rock matrix (phase
// exactly -1, no acid) stays quiescent for the whole run.  bact_prev = null
// (after anything else changed the fields) processes every brick.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RB) k_update_split(Grid g, const double* __restrict__ ph,
                                                     const double* __restrict__ cc,
                                                     const uint8_t* __restrict__ fl,
                                                     double* __restrict__ ph_out,
                                                     double* __restrict__ cc_out,
                                                     int* __restrict__ work, int* nwork,
                                                     double tau0, double* dsc,
                                                     const uint8_t* __restrict__ bact_prev,
                                                     uint8_t* __restrict__ bact_cur) {
    const long long sy = g.P, sz = g.S;
    const long long cap = (long long)g.nx * g.ny * g.nz;   // work[] entries
    const int nbx = (g.nx + BRICK_X - 1) / BRICK_X, nby = (g.ny + BRICK_Y - 1) / BRICK_Y;
    const int nbz = (g.nz + BRICK_Z - 1) / BRICK_Z;
    const int nb = nbx * nby * nbz;
    const int lane = threadIdx.x & 31, wy = (threadIdx.x >> 5) & 3, wz = threadIdx.x >> 7;
    constexpr int SPLIT_WARPS = RB / 32;
    static_assert(SPLIT_WARPS == BRICK_Y * BRICK_Z, "one warp per brick row");
    __shared__ int s_cnt[2][SPLIT_WARPS], s_base[2], s_tot[2];
    int any_copy = 0;
    for (int t = blockIdx.x; t < nb; t += gridDim.x) {
        const int bx = t % nbx, r = t / nbx, by = r % nby, bz = r / nby;
        if (bact_prev) {
            int act = 0;
            if (threadIdx.x < 27) {
                const int x = bx + threadIdx.x % 3 - 1, y = by + (threadIdx.x / 3) % 3 - 1;
                const int z = bz + threadIdx.x / 9 - 1;
                if (x >= 0 && x < nbx && y >= 0 && y < nby && z >= 0 && z < nbz)
                    act = bact_prev[((long long)z * nby + y) * nbx + x];
            }
            if (!__syncthreads_or(act)) {   // quiescent: all copies, already in place
                any_copy = 1;
                if (threadIdx.x == 0) bact_cur[t] = 0;
                continue;
            }
        }
        const int i = 1 + bx * BRICK_X + lane, j = 1 + by * BRICK_Y + wy, k = 1 + bz * BRICK_Z + wz;
        bool uni = true, copy = true;
        long long n = 0;
        if (i <= g.nx && j <= g.ny && k <= g.nz) {
            n = g.at(i, j, k);
            const bool well = (fl[n] & F_WELL) != 0;
            uni = phase_uniform_eager(ph, n, sy, sz);
            const bool cz0 = concent_zero_eager(cc, n, sy, sz);
            copy = uni && (well || cz0);
            if (copy) {
                const double a = ph[n], c = cc[n];
                ph_out[n] = a;
                cc_out[n] = c;
                write_halo_of(g, i, j, k, ph_out, a);
                write_halo_of(g, i, j, k, cc_out, c);
                any_copy = 1;
            }
        }
        // one atomic per list and brick: the two counters are the same two
        // addresses for every block, and atomics on one address serialise
        const unsigned ma = __ballot_sync(0xffffffffu, !uni);          // interface cells
        const unsigned mb = __ballot_sync(0xffffffffu, uni && !copy);  // concentration-only cells
        const int warp = threadIdx.x >> 5;
        if (lane == 0) {
            s_cnt[0][warp] = __popc(ma);
            s_cnt[1][warp] = __popc(mb);
        }
        __syncthreads();
        if (threadIdx.x < 2) {
            int tot = 0;
            for (int w = 0; w < SPLIT_WARPS; ++w) tot += s_cnt[threadIdx.x][w];
            s_base[threadIdx.x] = tot ? atomicAdd(nwork + threadIdx.x, tot) : 0;
            s_tot[threadIdx.x] = tot;
        }
        __syncthreads();
        int offa = s_base[0], offb = s_base[1];
        for (int w = 0; w < warp; ++w) {
            offa += s_cnt[0][w];
            offb += s_cnt[1][w];
        }
        const unsigned below = (1u << lane) - 1;
        if (!uni) work[offa + __popc(ma & below)] = (int)n;
        if (uni && !copy) work[cap - 1 - (offb + __popc(mb & below))] = (int)n;
        if (threadIdx.x == 0 && bact_cur) bact_cur[t] = (uint8_t)((s_tot[0] + s_tot[1]) > 0);
        __syncthreads();   // s_cnt / s_tot are rewritten for the next brick
    }
    if (__syncthreads_or(any_copy) && threadIdx.x == 0)
        atomicMin(reinterpret_cast<unsigned long long*>(dsc + S_TAUMIN_KEY), dkey(tau0));
}

// LOWC (the FP32-refined form): the concentration-only cells take
// concent_rate_lo and the guard-free interface cells phase_cell_lo, at three
// blocks per SM (80 registers); the plain FP64 form keeps every rate in FP64.
// PART: 1 the interface cells (the front of the list), 2 the
// concentration-only cells (the back), 0 both.  The two lists run as two
// launches: the concentration-only kernel, without the phase-rate code, fits
// five blocks per SM (48 registers, no spills) to hide its gathers' latency.
template <bool LOWC, int PART>
__global__ void __launch_bounds__(RB, PART == 2 ? 5 : (LOWC ? 3 : 0)) k_update_active(Grid g, const Phys* __restrict__ Pp,
                                                      const double* __restrict__ ph,
                                                      const double* __restrict__ cc,
                                                      const double* __restrict__ pr,
                                                      const double* __restrict__ Tvx,
                                                      const double* __restrict__ Tvy,
                                                      const double* __restrict__ Tvz,
                                                      const uint8_t* __restrict__ fl,
                                                      const int* __restrict__ work,
                                                      const int* __restrict__ nwork,
                                                      double* __restrict__ ph_out,
                                                      double* __restrict__ cc_out, double dt,
                                                      double* dsc, const double* dtp = nullptr) {
    if (dtp) dt = *dtp;   // device-resident step: dt from the device dt law
    const Phys P = *Pp;
    LoConst K{};
    if (LOWC) K = lo_const(P);
    double kmax = 0.0;
    unsigned long long umax = 0;   // bits of the largest |u|
    int overs = 0;
    const long long sy = g.P, sz = g.S;
    const long long cap = (long long)g.nx * g.ny * g.nz;
    const int na = nwork[0], nw = na + nwork[1];
    const int qa = PART == 2 ? na : 0, qb = PART == 1 ? na : nw;
    for (int q = qa + blockIdx.x * RB + threadIdx.x; q < qb; q += gridDim.x * RB) {
        // from the back: uniform phase, concentration only
        const bool uni = PART == 2 ? true : (PART == 1 ? false : q >= na);
        const long long n = uni ? work[cap - 1 - (q - na)] : work[q];
        const long long r = n - XOFF;
        const int k = (int)(r / g.S);
        const long long r2 = r - (long long)k * g.S;
        const int j = (int)(r2 / g.P);
        const int i = (int)(r2 - (long long)j * g.P);
        bool have_u = false;
        FaceVel u{};
        auto vel = [&]() {
            if (!have_u) {
                const double p0 = pr[n];
                // -K_f/mu (p_nb - p)/dx (:1169-1176) with 1/dx folded into Tv
                u.xp = -(Tvx[n] * (pr[n + 1] - p0));
                u.xm = -(Tvx[n - 1] * (p0 - pr[n - 1]));
                u.yp = -(Tvy[n] * (pr[n + sy] - p0));
                u.ym = -(Tvy[n - sy] * (p0 - pr[n - sy]));
                u.zp = -(Tvz[n] * (pr[n + sz] - p0));
                u.zm = -(Tvz[n - sz] * (p0 - pr[n - sz]));
                have_u = true;
            }
            return u;
        };
        const bool well = (fl[n] & F_WELL) != 0;
        const double conc = cc[n];
        double rate = 0.0, kxx = P.diffusion;
        int over = 0;
        bool lo = false;           // the phase rate came from the FP32 path
        float rate_lo = 0.f;
        FaceVelF uf{};
        bool have_uf = false;
        if (!uni) {
            if (LOWC) lo = phase_cell_lo(ph, n, sy, sz, pr, Tvx, Tvy, Tvz, conc, well, P, K, rate_lo, kxx, over,
                                         uf, have_uf);
            if (lo) rate = f32_to_f64(rate_lo);
            else phase_cell(ph, n, sy, sz, vel, conc, well, P, rate, kxx, over);
        }
        double crate;
        if (well) crate = 0.0;
        else if (concent_zero(cc, n, sy, sz)) crate = P.alpha * rate;
        else if (LOWC && uni) crate = f32_to_f64(concent_rate_lo(cc, pr, Tvx, Tvy, Tvz, n, sy, sz, K, umax));
        else if (lo) {
            if (!have_uf) {
                uf = face_vel_lo(pr, Tvx, Tvy, Tvz, n, sy, sz);
                have_uf = true;
            }
            float diff;
            const float div = concent_transport_lo(cc, n, sy, sz, uf, K, diff);
            crate = f32_to_f64(diff + K.alpha * rate_lo - div);   // :1606
        } else crate = concent_cell(cc, n, sy, sz, vel(), rate, P);
        const double phn = ph[n] + rate * dt;
        const double ccn = conc + crate * dt;
        ph_out[n] = phn;
        cc_out[n] = ccn;
        write_halo_of(g, i, j, k, ph_out, phn);
        write_halo_of(g, i, j, k, cc_out, ccn);
        if (have_u) {
            max_abs_bits(umax, u.xp);
            max_abs_bits(umax, u.yp);
            max_abs_bits(umax, u.zp);
        }
        if (have_uf) fold_umax_lo(umax, uf);
        kmax = fmax(kmax, kxx);
        overs += over;
    }
    flush_step_reductions(kmax, P.tau_num, overs, __longlong_as_double((long long)umax), dsc);
}

// Pressure of the Dirichlet cells := well pressure (the identity rows of :840).
__global__ void k_set_dirichlet(double* __restrict__ pr, const long long* __restrict__ idx,
                                const double* __restrict__ val, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) pr[idx[t]] = val[t];
}

// ---------------------------------------------------------------------------
// The plane whose phase maximum signals breakthrough: ix = nx - ceil(2 w / dx)
// (at least 1).  The outlet wells pin phase = -1 on ix = nx (wPFAW3D.f90:474-483)
// and the diffuse interface, about 2w wide, cannot cross that pinned plane:
// once the dissolved region arrives, the phase settles into a steady profile
// that stays below 0 within ~2w of the outlet (measured at 64^3: -0.70, -0.41,
// -0.14 on ix = nx-1..nx-3, +0.11 on nx-4).  So the dissolved region reaching
// ix = nx - 2w/dx is the breakthrough event, where the criterion "phase > 0 on
// ix = nx - 1" of a free outlet never fires.
int breakthrough_plane(const wpf_params& p) {
    const double m = 2.0 * p.epsilon / p.dx;
    int k = (int)ceil(m - 1e-9);
    if (k < 1) k = 1;
    const int ix = p.nx - k;
    return ix >= 1 ? ix : 1;
}

// showProgress reductions (:1695, :1756-1810): per-block partials of
//   S0 = sum(1-phase), S1 = sum(1+phase)  (interior, compensated per thread)
//   M0 = max r^2 over phase > 0, max/min phase, max/min concent (over G)
//   S2 = inlet flux sum u_x(1->2) dx^2
// then one block folds the partials in a fixed order.
// ---------------------------------------------------------------------------
struct DiagPart {
    double s0, c0, s1, c1, s2, c2, r2max, pmax, pmin, cmax, cmin, omax;
};

__device__ __forceinline__ void two_sum(double& s, double& c, double v) {
    const double t = s + v;
    const double bp = t - s;
    c += (s - (t - bp)) + (v - bp);
    s = t;
}

__global__ void k_diag_partial(Grid g, Phys P, int ix_ref, int iy_ref, int iz_ref, int ix_bt,
                               const double* __restrict__ ph, const double* __restrict__ cc,
                               const double* __restrict__ pr, const double* __restrict__ Tx,
                               DiagPart* __restrict__ out) {
    // one block per plane k (0..nz+1), threads over rows j and x
    __shared__ double sm[32];
    const int k = blockIdx.x;
    double s0 = 0, c0 = 0, s1 = 0, c1 = 0, s2 = 0, c2 = 0, r2max = 0;
    double pmax = -1.0e308, pmin = 1.0e308, cmax = -1.0e308, cmin = 1.0e308, omax = -1.0e308;
    const double dx = P.dx;
    const double xref = dx * (ix_ref - 1) + 0.5 * dx, yref = dx * (iy_ref - 1) + 0.5 * dx,
                 zref = dx * (iz_ref - 1) + 0.5 * dx;
    for (int j = threadIdx.y; j <= g.ny + 1; j += blockDim.y)
        for (int i = threadIdx.x; i <= g.nx + 1; i += blockDim.x) {
            const long long n = g.at(i, j, k);
            const double f = ph[n], c = cc[n];
            pmax = fmax(pmax, f); pmin = fmin(pmin, f);
            cmax = fmax(cmax, c); cmin = fmin(cmin, c);
            const bool interior = i >= 1 && i <= g.nx && j >= 1 && j <= g.ny && k >= 1 && k <= g.nz;
            if (interior) {
                two_sum(s0, c0, 1.0 - f);
                two_sum(s1, c1, 1.0 + f);
                if (f > 0.0) {
                    const double x = dx * (i - 1) + 0.5 * dx - xref, y = dx * (j - 1) + 0.5 * dx - yref,
                                 z = dx * (k - 1) + 0.5 * dx - zref;
                    r2max = fmax(r2max, x * x + y * y + z * z);
                }
                if (i == 1 && g.nx >= 2) {
                    const double u = -(Tx[n] * ((pr[n + 1] - pr[n]) * P.inv_dx));
                    two_sum(s2, c2, u * dx * dx);
                }
                if (i == ix_bt) omax = fmax(omax, f);   // breakthrough plane
            }
        }
    DiagPart r;
    r.s0 = block_sum(s0, sm); r.c0 = block_sum(c0, sm);
    r.s1 = block_sum(s1, sm); r.c1 = block_sum(c1, sm);
    r.s2 = block_sum(s2, sm); r.c2 = block_sum(c2, sm);
    r.r2max = block_max(r2max, sm, 0.0);
    r.pmax = block_max(pmax, sm, -1.0e308); r.pmin = block_min(pmin, sm, 1.0e308);
    r.cmax = block_max(cmax, sm, -1.0e308); r.cmin = block_min(cmin, sm, 1.0e308);
    r.omax = block_max(omax, sm, -1.0e308);
    if (threadIdx.x == 0 && threadIdx.y == 0) out[k] = r;
}

__global__ void k_diag_final(const DiagPart* __restrict__ parts, int nparts, double* out) {
    if (threadIdx.x != 0) return;
    double s0 = 0, c0 = 0, s1 = 0, c1 = 0, s2 = 0, c2 = 0, r2 = 0;
    double pmax = -1.0e308, pmin = 1.0e308, cmax = -1.0e308, cmin = 1.0e308, omax = -1.0e308;
    for (int q = 0; q < nparts; ++q) {
        const DiagPart& p = parts[q];
        two_sum(s0, c0, p.s0); c0 += p.c0;
        two_sum(s1, c1, p.s1); c1 += p.c1;
        two_sum(s2, c2, p.s2); c2 += p.c2;
        r2 = fmax(r2, p.r2max);
        pmax = fmax(pmax, p.pmax); pmin = fmin(pmin, p.pmin);
        cmax = fmax(cmax, p.cmax); cmin = fmin(cmin, p.cmin);
        omax = fmax(omax, p.omax);
    }
    out[0] = s0 + c0; out[1] = s1 + c1; out[2] = s2 + c2; out[3] = r2;
    out[4] = pmax; out[5] = pmin; out[6] = cmax; out[7] = cmin; out[8] = omax;
}

// ---------------------------------------------------------------------------
// host wrappers
// ---------------------------------------------------------------------------
static void reset_step_slots(wpf_handle* h) {
    // taumin starts at 1e6 (:1223); overshoot and umax at zero.
    unsigned long long key = dkey_host(1.0e6);
    unsigned long long zero = 0;
    memcpy(&h->hsc[S_TAUMIN_KEY], &key, 8);
    memcpy(&h->hsc[S_OVERSHOOT], &zero, 8);
    memcpy(&h->hsc[S_UMAX_BITS], &zero, 8);
}

static int upload_step_slots(wpf_handle* h) {
    reset_step_slots(h);
    WPF_CUDA(cudaMemcpyAsync(h->dsc + S_TAUMIN_KEY, h->hsc + S_TAUMIN_KEY, 3 * sizeof(double),
                             cudaMemcpyHostToDevice, h->stream));
    return WPF_OK;
}

static int read_step_slots(wpf_handle* h, double* taumin, int32_t* overshoot, double* umax) {
    WPF_CUDA(cudaMemcpyAsync(h->hsc + S_TAUMIN_KEY, h->dsc + S_TAUMIN_KEY, 3 * sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream));
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    timer_flush(h);
    unsigned long long key, ov, um;
    memcpy(&key, &h->hsc[S_TAUMIN_KEY], 8);
    memcpy(&ov, &h->hsc[S_OVERSHOOT], 8);
    memcpy(&um, &h->hsc[S_UMAX_BITS], 8);
    const double tm = dkey_inv(key);
    h->taumin_last = tm;
    if (taumin) *taumin = tm;
    if (overshoot) *overshoot = (int32_t)ov;
    if (umax) { double v; memcpy(&v, &um, 8); *umax = v; }
    return WPF_OK;
}

static double inv_mu(const wpf_handle* h) { return 1.0 / h->prm.viscosity; }

int phys_permeability(wpf_handle* h, bool materialise) {
    const Grid& g = h->g;
    const dim3 b = cell_block();
    if (materialise) {
        int rc = ensure_per_routine_arrays(h);
        if (rc) return rc;
        WPF_LAUNCH(h, KC_PERM, k_cell_K0<<<cell_grid(g.nx + 2, g.ny + 2, g.nz + 2), b, 0, h->stream>>>(
            g, h->phys, h->phase, h->krock, h->K0));
    }
    // T is still valid for every face whose two cells kept their phase since
    // the fused update that produced the current phase (t_from_prev).
    const double* prev = (!materialise && h->t_from_prev) ? h->phase_n : nullptr;
    // the kept outer residual follows T only through the incremental form
    const bool keep = prev && h->rkeep && h->rkeep_ok;
    h->rkeep_ok = keep;
    // every face recomputed: the level-0 operator is rebuilt whole next time
    if (!prev) h->l0_inc_ok = false;
    const dim3 pb(PB_X, PB_Y, PB_Z);
    const dim3 pg((g.nx + 1 + PB_X - 1) / PB_X, (g.ny + 1 + PB_Y - 1) / PB_Y, (g.nz + 1 + PB_Z - 1) / PB_Z);
    WPF_LAUNCH(h, KC_PERM, k_permeability<<<pg, pb, 0, h->stream>>>(
        g, h->phys, h->phase, prev, h->krock, h->T[0], h->T[1], h->T[2],
        materialise ? h->Kf[0] : nullptr, materialise ? h->Kf[1] : nullptr,
        materialise ? h->Kf[2] : nullptr, inv_mu(h), keep ? h->rkeep : nullptr, h->flags, h->pressure,
        prev ? h->l0mark : nullptr, h->Tv[0], h->Tv[1], h->Tv[2]));
    WPF_CUDA(cudaGetLastError());
    h->kf_valid = materialise;
    h->t_current = true;
    h->t_from_prev = false;
    return WPF_OK;
}

int phys_velocity(wpf_handle* h) {
    int rc = ensure_per_routine_arrays(h);
    if (rc) return rc;
    if (!h->kf_valid) return WPF_ERR_ARG;   // calcPermeability must precede (:2249-2251)
    const Grid& g = h->g;
    WPF_LAUNCH(h, KC_OTHER, k_velocity<<<cell_grid(g.nx + 1, g.ny + 1, g.nz + 1), cell_block(), 0, h->stream>>>(
        g, h->phys, h->pressure, h->Kf[0], h->Kf[1], h->Kf[2], h->vel[0], h->vel[1], h->vel[2],
        inv_mu(h)));
    WPF_CUDA(cudaGetLastError());
    h->vel_valid = true;
    return WPF_OK;
}

int phys_phase_deriv(wpf_handle* h, double* taumin, int32_t* overshoot) {
    int rc = ensure_per_routine_arrays(h);
    if (rc) return rc;
    const Grid& g = h->g;
    if ((rc = upload_step_slots(h))) return rc;
    WPF_LAUNCH(h, KC_OTHER, k_phase_deriv<<<row_blocks(h, g, 4), RB, 0, h->stream>>>(
        g, h->phys, h->phase, h->concent, h->vel[0], h->vel[1], h->vel[2], h->flags, h->dphasedt,
        h->dsc));
    WPF_CUDA(cudaGetLastError());
    return read_step_slots(h, taumin, overshoot, nullptr);
}

int phys_concent_deriv(wpf_handle* h) {
    int rc = ensure_per_routine_arrays(h);
    if (rc) return rc;
    const Grid& g = h->g;
    WPF_LAUNCH(h, KC_OTHER, k_concent_deriv<<<row_blocks(h, g), RB, 0, h->stream>>>(
        g, h->phys, h->concent, h->vel[0], h->vel[1], h->vel[2], h->flags, h->dphasedt,
        h->dconcentdt));
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

int phys_halo(wpf_handle* h, double* f) {
    const Grid& g = h->g;
    const long long n = 2LL * (g.ny + 2) * (g.nz + 2) + 2LL * g.nx * (g.nz + 2) + 2LL * g.nx * g.ny;
    WPF_LAUNCH(h, KC_OTHER, k_halo<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(g, f));
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

int phys_evolve(wpf_handle* h, bool phase, double dtime) {
    int rc = ensure_per_routine_arrays(h);
    if (rc) return rc;
    const Grid& g = h->g;
    double* f = phase ? h->phase : h->concent;
    const double* d = phase ? h->dphasedt : h->dconcentdt;
    h->bact_ok = false;   // the fields change outside the fused update
    WPF_LAUNCH(h, KC_OTHER, k_evolve<<<row_blocks(h, g), RB, 0, h->stream>>>(g, f, d, dtime));
    if (phase) {
        h->kf_valid = false;
        h->t_current = false;
        h->t_from_prev = false;
    }
    WPF_CUDA(cudaGetLastError());
    return phys_halo(h, f);
}

// Work list and the two brick-activity arrays of the fused update.
int update_alloc(wpf_handle* h) {
    const Grid& g = h->g;
    int rc;
    if (!h->work && (rc = dev_alloc(h, (void**)&h->work, sizeof(int) * (size_t)g.nx * g.ny * g.nz))) return rc;
    const size_t nb = (size_t)((g.nx + BRICK_X - 1) / BRICK_X) * ((g.ny + BRICK_Y - 1) / BRICK_Y) *
                      ((g.nz + BRICK_Z - 1) / BRICK_Z);
    for (int q = 0; q < 2; ++q)
        if (!h->bact[q] && (rc = dev_alloc(h, (void**)&h->bact[q], nb))) return rc;
    return WPF_OK;
}

static unsigned split_blocks(const wpf_handle* h) {
    const Grid& g = h->g;
    const long long nb = (long long)((g.nx + BRICK_X - 1) / BRICK_X) * ((g.ny + BRICK_Y - 1) / BRICK_Y) *
                         ((g.nz + BRICK_Z - 1) / BRICK_Z);
    const long long cap = (long long)h->nsm * resident_blocks((const void*)k_update_split, RB, 0, 8);
    return (unsigned)(nb < cap ? nb : cap);
}

// After an update: the activity it recorded becomes the previous one.
void update_advance_bricks(wpf_handle* h) {
    uint8_t* t = h->bact[0];
    h->bact[0] = h->bact[1];
    h->bact[1] = t;
    h->bact_ok = true;
}

// The FP32-refined form takes the rates in FP32 unless WPF_SOLVER_FP64_UPDATE
// keeps them in FP64; the plain form always does.
static bool low_precision_rates(const wpf_handle* h) {
    return h->opts.mode == WPF_SOLVER_MIXED && !(h->opts.flags & WPF_SOLVER_FP64_UPDATE);
}

// k_update_active over both lists: the interface kernel in one wave of
// resident blocks (the FP32-rate form is built for three per SM, the FP64 form
// holds two; two per SM without spills measured 2 % slower for the FP32-rate
// form), then the concentration-only kernel in one wave of its own.
static int launch_update(wpf_handle* h, cudaStream_t s, double dt, const double* dtp) {
    const Grid& g = h->g;
    const int* nwork = reinterpret_cast<const int*>(h->dsc + S_NWORK);
    const bool low = low_precision_rates(h);
    auto* ui = low ? k_update_active<true, 1> : k_update_active<false, 1>;
    auto* uc = low ? k_update_active<true, 2> : k_update_active<false, 2>;
    const unsigned bi = (unsigned)h->nsm * (unsigned)resident_blocks((const void*)ui, RB, 0, 8);
    const unsigned bc = (unsigned)h->nsm * (unsigned)resident_blocks((const void*)uc, RB, 0, 8);
    WPF_LAUNCH(h, KC_FUSED, ui<<<bi, RB, 0, s>>>(g, h->dphys, h->phase, h->concent, h->pressure, h->Tv[0],
                                                 h->Tv[1], h->Tv[2], h->flags, h->work, nwork, h->phase_n,
                                                 h->concent_n, dt, h->dsc, dtp));
    WPF_LAUNCH(h, KC_FUSED, uc<<<bc, RB, 0, s>>>(g, h->dphys, h->phase, h->concent, h->pressure, h->Tv[0],
                                                 h->Tv[1], h->Tv[2], h->flags, h->work, nwork, h->phase_n,
                                                 h->concent_n, dt, h->dsc, dtp));
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}


int phys_fused_update(wpf_handle* h, double dtime, double* taumin, int32_t* overshoot,
                      double* umax) {
    const Grid& g = h->g;
    int rc = upload_step_slots(h);
    if (rc) return rc;
    if ((rc = update_alloc(h))) return rc;
    WPF_CUDA(cudaMemsetAsync(h->dsc + S_NWORK, 0, sizeof(double), h->stream));
    int* nwork = reinterpret_cast<int*>(h->dsc + S_NWORK);
    WPF_CUDA(cudaEventRecord(h->ev[2], h->stream));
    WPF_LAUNCH(h, KC_FUSED, k_update_split<<<split_blocks(h), RB, 0, h->stream>>>(
        g, h->phase, h->concent, h->flags, h->phase_n, h->concent_n, h->work, nwork, h->phys.tau0,
        h->dsc, h->bact_ok ? h->bact[0] : nullptr, h->bact[1]));
    if ((rc = launch_update(h, h->stream, dtime, nullptr))) return rc;
    WPF_CUDA(cudaEventRecord(h->ev[3], h->stream));
    double* t = h->phase; h->phase = h->phase_n; h->phase_n = t;
    t = h->concent; h->concent = h->concent_n; h->concent_n = t;
    update_advance_bricks(h);
    h->vel_valid = false;
    h->kf_valid = false;
    // T was computed from the phase now held in phase_n (wpf_step calls
    // calcPermeability right before the solve and this update).
    h->t_from_prev = h->t_current;
    h->t_current = false;
    WPF_CUDA(cudaMemcpyAsync(&h->hsc[S_NWORK], h->dsc + S_NWORK, sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream));
    rc = read_step_slots(h, taumin, overshoot, umax);
    int nw[2];   // interface cells, concentration-only cells (two ints in the slot)
    memcpy(nw, &h->hsc[S_NWORK], sizeof(nw));
    h->last_active = nw[0] + nw[1];
    h->last_interface = nw[0];
    return rc;
}

// The step slots' reset (upload_step_slots) and the work-list counters, on the
// device: the device-resident step has no host copy to upload from.
__global__ void k_step_slots_reset(double* dsc) {
    if (threadIdx.x) return;
    unsigned long long* u = reinterpret_cast<unsigned long long*>(dsc);
    u[S_TAUMIN_KEY] = dkey(1.0e6);
    u[S_OVERSHOOT] = 0ull;
    u[S_UMAX_BITS] = 0ull;
    u[S_NWORK] = 0ull;
}

int phys_capture_split(wpf_handle* h, cudaStream_t s) {
    const Grid& g = h->g;
    int* nwork = reinterpret_cast<int*>(h->dsc + S_NWORK);
    WPF_LAUNCH(h, KC_OTHER, k_step_slots_reset<<<1, 32, 0, s>>>(h->dsc));
    WPF_LAUNCH(h, KC_FUSED, k_update_split<<<split_blocks(h), RB, 0, s>>>(
        g, h->phase, h->concent, h->flags, h->phase_n, h->concent_n, h->work, nwork, h->phys.tau0,
        h->dsc, h->bact_ok ? h->bact[0] : nullptr, h->bact[1]));
    WPF_CUDA(cudaGetLastError());
    return WPF_OK;
}

int phys_capture_update(wpf_handle* h, const double* dtp, cudaStream_t s, bool split_done) {
    int rc;
    if (!split_done && (rc = phys_capture_split(h, s))) return rc;
    return launch_update(h, s, 0.0, dtp);
}

int phys_set_dirichlet(wpf_handle* h) {
    if (h->ndir > 0) {
        WPF_LAUNCH(h, KC_OTHER, k_set_dirichlet<<<(h->ndir + 255) / 256, 256, 0, h->stream>>>(
            h->pressure, h->dir_idx, h->dir_val, h->ndir));
        WPF_CUDA(cudaGetLastError());
    }
    return WPF_OK;
}

int phys_reduce(wpf_handle* h, wpf_diag* d) {
    const Grid& g = h->g;
    const int nparts = g.nz + 2;
    if (h->npartials < nparts) {
        if (h->partials) cudaFree(h->partials);
        h->partials = nullptr;
        int rc = dev_alloc(h, (void**)&h->partials, sizeof(DiagPart) * nparts + 64);
        if (rc) return rc;
        h->npartials = nparts;
    }
    DiagPart* parts = reinterpret_cast<DiagPart*>(h->partials);
    WPF_LAUNCH(h, KC_OTHER, k_diag_partial<<<nparts, dim3(32, 8), 0, h->stream>>>(
        g, h->phys, h->prm.ix_ref, h->prm.iy_ref, h->prm.iz_ref, breakthrough_plane(h->prm), h->phase,
        h->concent, h->pressure, h->T[0], parts));
    WPF_LAUNCH(h, KC_OTHER, k_diag_final<<<1, 32, 0, h->stream>>>(parts, nparts, h->dsc + S_SUM0));
    WPF_CUDA(cudaGetLastError());
    WPF_CUDA(cudaMemcpyAsync(h->hsc + S_SUM0, h->dsc + S_SUM0, 9 * sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream));
    double pref = 0.0;
    const wpf_params& p = h->prm;
    if (p.ix_ref >= 1 && p.ix_ref <= g.nx && p.iy_ref >= 1 && p.iy_ref <= g.ny && p.iz_ref >= 1 &&
        p.iz_ref <= g.nz) {
        WPF_CUDA(cudaMemcpyAsync(&pref, h->pressure + g.at(p.ix_ref, p.iy_ref, p.iz_ref),
                                 sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    WPF_CUDA(cudaStreamSynchronize(h->stream));
    const double* o = h->hsc + S_SUM0;
    const double dx = h->phys.dx;
    d->pv = dx * dx * dx * p.porosity * 0.5 * o[0];
    d->vcal = dx * dx * dx * (1.0 - p.porosity) * 0.5 * o[1];
    d->inlet_flux = o[2];
    d->rwhmax = sqrt(o[3]);
    d->phase_max = o[4]; d->phase_min = o[5];
    d->concent_max = o[6]; d->concent_min = o[7];
    d->phase_max_outlet = o[8];
    d->pressure_ref = pref;
    return WPF_OK;
}

}  // namespace wpf
