// FP64 Muskingum-Cunge secant solve of one segment for one time step, device side.
//
// Arithmetic follows the reference solver operation for operation
// (water-prediction/t-route/troute_mc_final.cu:42-139, the same algorithm as
// cpu_mc :181-248 and mc_solve_d in wavefront/wavefront_mc.cu:215-337):
//   - channel geometry at a depth: trapezoid + compound channel (:30-40);
//   - celerity Ck from Manning (R^(2/3), R^(5/3)), K = max(dt, dx/Ck), X, C1..C4;
//   - X clamped to [0, 0.5] at the lower point and [0.25, 0.5] at the upper
//     point, the upper X using the lower point's C1..C4 (:86 vs :105);
//   - C4 clamp only at the upper point (:109);
//   - up to `attempts` bracket-widening restarts (:121-122);
//   - outflow with the negative-flow fallbacks and trapezoid-only velocity
//     (:125-138).
// R^(2/3) and R^(5/3) come from pow23_53 (crpow.cuh), correctly rounded like
// the host pow() of the reference almost always is; with FMA contraction
// disabled for this code (the library builds it with -fmad=false) every other
// operation rounds exactly as the reference's C does.
// One change of evaluation, not of values: every quantity that depends only on
// the lower depth h_0 (geometry, Ck, K, Manning discharge) is carried over from
// the previous iteration's upper-depth evaluation, because each iteration sets
// h_0 = max(0, h) and h >= 0 always holds, so that evaluation is the same
// function of the same number. Only a restart (h_0 *= 0.67) re-evaluates it.
#pragma once

#include "crpow.cuh"
#include "troute_internal.h"

namespace tr {

__device__ __forceinline__ SegP load_seg(const NetDev& net, long long s)
{
    const SegRec* r = net.seg + s;
    const double2 a = __ldg(r->p + 0), b = __ldg(r->p + 1), c = __ldg(r->p + 2);
    const double2 e = __ldg(r->p + 3), f = __ldg(r->p + 4), g = __ldg(r->p + 5);
    SegP p;
    p.dx = a.x; p.bw = a.y; p.twcc = b.x; p.n_ch = b.y; p.ncc = c.x; p.s0 = c.y;
    p.z = e.x; p.bfd = e.y; p.sq_s0 = f.x; p.sq2 = f.y; p.ck_fac = g.x; p.z2 = g.y;
    return p;
}

// Everything at one depth that does not depend on the iteration's X.
struct DepthEval {
    double Ck, Km, twu, Qmn;
};


__device__ __forceinline__ DepthEval eval_depth(double h, const SegP& p, double dt)
{
    const double twl = p.bw + p.z2 * h;  // bw + 2 z h
    double above = fmax(h - p.bfd, 0.0);
    double below = fmin(p.bfd, h);
    if (above > 0.0 && p.twcc <= 0.0) {
        above = 0.0;
        below = h;
    }
    const double A = (p.bw + below * p.z) * below;
    const double WP = p.bw + below * p.sq2;  // bw + 2 below sqrt(1+z^2)
    const double AC = p.twcc * above;
    const double WPC = (above > 0.0) ? (p.twcc + 2.0 * above) : 0.0;
    const double P = WP + WPC;
    const double R = (P > 0.0) ? (A + AC) / P : 0.0;
    double r23, r53;
    pow23_53(R, &r23, &r53);
    DepthEval e;
    e.Ck = 0.0;
    if (h > 0.0) {
        // 2 sqrt(1+z^2) / (bw + 2 h z), the denominator being twl
        e.Ck = fmax(0.0, p.ck_fac * ((5.0 / 3.0) * r23 - (2.0 / 3.0) * r53 * (p.sq2 / twl)));
    }
    e.Km = (e.Ck > 0.0) ? fmax(dt, p.dx / e.Ck) : dt;
    e.twu = (h > p.bfd && p.twcc > 0.0) ? p.twcc : twl;
    e.Qmn = (P > 0.0) ? (1.0 / ((WP * p.n_ch + WPC * p.ncc) / P)) * (A + AC) * r23 * p.sq_s0 : 0.0;
    return e;
}

struct SolveOut {
    double q, depth, vel;
    int iters;
    int retried;
    int early;
};

__device__ __forceinline__ SolveOut mc_solve(double dt, double qup, double quc, double qdp,
                                             double ql, const SegP& p, double depthp,
                                             const Tol& tol)
{
    SolveOut o;
    o.iters = 0;
    o.retried = 0;
    o.early = 0;
    if (p.n_ch <= 0.0 || p.s0 <= 0.0 || p.z <= 0.0 || p.bw <= 0.0 ||
        (ql <= 0.0 && qup <= 0.0 && quc <= 0.0 && qdp <= 0.0)) {
        o.q = 0.0;
        o.depth = 0.0;
        o.vel = 0.0;
        o.early = 1;
        return o;
    }
    const double depth = fmax(depthp, 0.0);
    double h = depth * 1.33 + kMinDepth;
    double h_0 = depth * 0.67;
    double C1 = 0.0, C2 = 0.0, C3 = 0.0, C4 = 0.0, X;
    double Qj_0 = 0.0, Qj;
    int maxiter = tol.maxiter;
    int total = 0;
    DepthEval e0;
    bool have0 = false;
    for (int attempt = 0; attempt < tol.attempts; ++attempt) {
        double aerr = 0.01, rerr = 1.0;
        int iter = 0;
        bool first = true;
        while (first || (rerr > tol.rtol && aerr >= tol.atol && iter <= maxiter)) {
            first = false;
            if (!have0) {
                e0 = eval_depth(h_0, p, dt);
                have0 = true;
            }
            const double X0 = (e0.Ck > 0.0 && e0.twu * p.s0 * e0.Ck * p.dx > 0.0)
                                  ? fmin(0.5, fmax(0.0, 0.5 * (1.0 - Qj_0 / (2.0 * e0.twu * p.s0 * e0.Ck * p.dx))))
                                  : 0.5;
            double D0 = e0.Km * (1.0 - X0) + dt / 2.0;
            if (D0 == 0.0) D0 = 1.0;
            const double c1 = (e0.Km * X0 + dt / 2.0) / D0;
            const double c2 = (dt / 2.0 - e0.Km * X0) / D0;
            const double c3 = (e0.Km * (1.0 - X0) - dt / 2.0) / D0;
            const double c4 = (ql * dt) / D0;
            const double qmc0 = c1 * qup + c2 * quc + c3 * qdp + c4;
            Qj_0 = qmc0 - e0.Qmn;

            const DepthEval e1 = eval_depth(h, p, dt);
            X = (e1.Ck > 0.0 && e1.twu * p.s0 * e1.Ck * p.dx > 0.0)
                    ? fmin(0.5, fmax(0.25, 0.5 * (1.0 - qmc0 / (2.0 * e1.twu * p.s0 * e1.Ck * p.dx))))
                    : 0.5;
            double D1 = e1.Km * (1.0 - X) + dt / 2.0;
            if (D1 == 0.0) D1 = 1.0;
            C1 = (e1.Km * X + dt / 2.0) / D1;
            C2 = (dt / 2.0 - e1.Km * X) / D1;
            C3 = (e1.Km * (1.0 - X) - dt / 2.0) / D1;
            C4 = (ql * dt) / D1;
            if (C4 < 0.0 && fabs(C4) > C1 * qup + C2 * quc + C3 * qdp)
                C4 = -(C1 * qup + C2 * quc + C3 * qdp);
            Qj = (C1 * qup + C2 * quc + C3 * qdp + C4) - e1.Qmn;

            double h_1 = (Qj_0 - Qj != 0.0) ? h - (Qj * (h_0 - h)) / (Qj_0 - Qj) : h;
            if (h_1 < 0.0) h_1 = h;
            if (h > 0.0) {
                rerr = fabs((h_1 - h) / h);
                aerr = fabs(h_1 - h);
            } else {
                rerr = 0.0;
                aerr = 0.9;
            }
            h_0 = fmax(0.0, h);
            h = fmax(0.0, h_1);
            e0 = e1;
            ++iter;
            ++total;
            if (h < kMinDepth) break;
        }
        if (iter < maxiter) break;
        h *= 1.33;
        h_0 *= 0.67;
        maxiter += 25;
        have0 = false;
        o.retried = 1;
    }

    const double Qmc = C1 * qup + C2 * quc + C3 * qdp + C4;
    double qdc;
    if (Qmc < 0.0) {
        if (C4 < 0.0 && fabs(C4) > C1 * qup + C2 * quc + C3 * qdp)
            qdc = 0.0;
        else
            qdc = fmax(C1 * qup + C2 * quc + C4, C1 * qup + C3 * qdp + C4);
    } else {
        qdc = Qmc;
    }
    const double twl = p.bw + p.z2 * h;
    double Rv = (h * (p.bw + twl) / 2.0) /
                (p.bw + 2.0 * sqrt(((twl - p.bw) / 2.0) * ((twl - p.bw) / 2.0) + h * h));
    if (Rv < 0.0) Rv = 0.0;
    o.q = qdc;
    o.vel = (1.0 / p.n_ch) * pow23(Rv) * p.sq_s0;
    o.depth = h;
    o.iters = total;
    return o;
}

}  // namespace tr
