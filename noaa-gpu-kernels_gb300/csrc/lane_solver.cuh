// Per-lane secant solver shared by the persistent routing kernels that give
// every lane its own (reach, step): the lane state, the start of a segment
// solve and one "pass" (one depth evaluation plus its secant bookkeeping).
//
// A pass does, for every lane in SOLVE or VEL mode, exactly one evaluation of
// R^fl(2/3) and R^fl(5/3) (pow23_53), so the expensive part of the pass runs
// for all busy lanes of a warp together.
// The evaluation is at h_0 when a solve starts or restarts (need0), otherwise
// at h followed by the secant update and the stop test.
// When a solve stops, the segment's discharge and depth are stored and the next
// segment starts in the same pass; after the reach's last segment the lane goes
// to DONE and the kernel publishes the reach. The velocity, an output that no
// later solve reads, is computed once per run from the final depth
// (velocity_kernel), with the reference's formula (troute_mc_final.cu:132-136).
// The arithmetic is mc_solve's (mc_solve.cuh, the reference's
// troute_mc_final.cu:42-139) split at its evaluations, operation for
// operation.
#pragma once

#include "device_common.cuh"
#include "fpbits.cuh"

namespace tr {

// L_BEGIN: the lane's next segment (L.i) starts at the kernel's one
// begin_segment call site before the next evaluation pass; L_START: the lane
// holds an item (L.ri, L.tau) whose inputs are final, started at the kernel's
// one start_item call site. Modes from L_SOLVE up count as busy.
enum : int { L_IDLE = 0, L_WAIT = 1, L_SOLVE = 2, L_BEGIN = 3, L_DONE = 4, L_START = 5 };

// A lane's current segment parameters live in shared memory for the whole
// solve, read by every pass. (Re-reading them from global memory every pass
// misses L2 once a network's parameters outgrow it -- c1's are 260 MB -- and
// costs a DRAM round trip per pass.) Each lane has two buffers: while segment
// i is solved, segment i + 1's parameters, inflow column and scale and (warm
// start) learned starting depth are copied into the other buffer by cp.async,
// and its discharge and depth are prefetched into L2 -- all static during the
// launch or final since the reach's previous step completed -- so the next
// solve starts after one round trip (the inflow) instead of a chain of them.
// Buffer of segment i: i & 1. A buffer holds kParamPlanes parameter double2
// and one {inflow scale, inflow column | learned depth} double2.
// Layout [warp][buffer][plane][lane]: a warp's reads of one plane are 512
// contiguous bytes, free of bank conflicts, whatever the block size.
constexpr int kSegSmemStride = 32;
constexpr int kSegBufPlanes = kParamPlanes + 1;
constexpr int kSegBufStride = kSegBufPlanes * kSegSmemStride;   // double2 from buffer 0 to 1
// double2 of a block's staging array per thread
constexpr int kSegSmemPerThread = 2 * kSegBufPlanes;

// This thread's buffer 0 in a block's array of kSegSmemPerThread x blockDim
// double2.
__device__ __forceinline__ double2* seg_slot_of(double2* seg_sm)
{
    return seg_sm + (threadIdx.x >> 5) * (2 * kSegBufStride) + (threadIdx.x & 31);
}

// The buffer of the lane's segment i.
__device__ __forceinline__ double2* seg_buf(double2* slot, int i) { return slot + (i & 1) * kSegBufStride; }

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Asynchronous global -> shared copies of this thread; a thread waits only for
// its own (cp.async.wait_all).
__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Starts the copies of tile slot s's record (and learned depth for step tau)
// into buffer buf, and the L2 prefetch of its discharge and depth. Only data
// that no thread writes during the launch goes through the non-coherent
// cp.async path (the records; the prediction plane, written before the
// launch); the mutable discharge and depth are read later with ld.cg.
__device__ __forceinline__ void stage_seg_async(const NetDev& net, const RunDev& run, int tau, long long s,
                                                double2* buf)
{
    const SegRec* r = net.seg + s;
#pragma unroll
    for (int k = 0; k < kParamPlanes; ++k) cp_async16(buf + k * kSegSmemStride, r->p + k);
    double2* t = buf + kParamPlanes * kSegSmemStride;
    cp_async8(&t->x, &r->qscale);
    int* w = reinterpret_cast<int*>(&t->y);
    cp_async4(w, &r->qcol);
    if (run.warm) cp_async4(w + 1, run.start_pred + (size_t)tau * (size_t)net.n_seg_int + s);
    prefetch_l2(net.q + s);
    prefetch_l2(net.d + s);
}

__device__ __forceinline__ SegP staged_seg(const double2* slot)
{
    const double2 a = slot[0], b = slot[kSegSmemStride], c = slot[2 * kSegSmemStride];
    const double2 e = slot[3 * kSegSmemStride], f = slot[4 * kSegSmemStride], g = slot[5 * kSegSmemStride];
    SegP p;
    p.dx = a.x; p.bw = a.y; p.twcc = b.x; p.n_ch = b.y; p.ncc = c.x; p.s0 = c.y;
    p.z = e.x; p.bfd = e.y; p.sq_s0 = f.x; p.sq2 = f.y; p.ck_fac = g.x; p.z2 = g.y;
    return p;
}
// Warm-start phase of a solve: the plain bracket, or bracketing the learned
// depth (read from the launch's prediction plane when the solve begins).
enum : int { W_PLAIN = 0, W_ACTIVE = 2 };

// Everything a lane carries for one (reach, step) and the segment it solves.
struct Lane {
    int mode;
    int ri, tau, g, ns, i, ub, ue, dn;
    long long base;        // tile slot of segment 0
    long long wait_t0;
    unsigned long long wait_tail;  // queue tail seen when the current wait budget began
    double qup_head, quc_head, q_up_old, q_up_new, q_last;
    // current segment
    long long s;
    double qup, quc, qdp, ql;
    double h, h_0, Qj_0, qdc;
    double dpp;            // previous depth (clamped at 0): the plain bracket's centre
    DepthEval e0;
    int need0, iter, attempt, maxiter, total, retried, warm;
};

// The plain starting bracket from the previous depth (troute_mc_final.cu:193).
__device__ __forceinline__ void plain_bracket(Lane& L, const Tol& tol)
{
    L.h = L.dpp * 1.33 + kMinDepth;
    L.h_0 = L.dpp * 0.67;
    L.Qj_0 = 0.0;
    L.qdc = 0.0;
    L.maxiter = tol.maxiter;
    L.attempt = 0;
    L.iter = 0;
    L.need0 = 1;
}

// Starts segment L.i of the lane's reach; consecutive segments that exit early
// (invalid parameters or no flow at all, troute_mc_final.cu:54-63) are stored
// right away. Returns true when a secant solve is pending, false when the reach
// is complete.
__device__ __forceinline__ bool begin_segment(Lane& L, const NetDev& net, const RunDev& run,
                                              LocalStats& ls, unsigned int* hist_s, double2* slot)
{
    const double* qlat_row = run.qlat + (size_t)L.tau * (size_t)run.qlat_ld;
    while (L.i < L.ns) {
        L.s = L.base + (long long)L.i * kLanes;
        double2* const buf = seg_buf(slot, L.i);
        // segment 0 of an item is staged now; every later segment was staged
        // while the previous one was solved
        if (L.i == 0) stage_seg_async(net, run, L.tau, L.s, buf);
        cp_async_wait_all();
        if (L.i + 1 < L.ns) stage_seg_async(net, run, L.tau, L.s + kLanes, seg_buf(slot, L.i + 1));
        L.qdp = __ldcg(net.q + L.s);
        const double dpp = __ldcg(net.d + L.s);
        const double2 tail = buf[kParamPlanes * kSegSmemStride];
        const long long tw = __double_as_longlong(tail.y);
        L.ql = __ldg(qlat_row + (int)(unsigned)(tw & 0xffffffffll)) * tail.x;   // column: the low word
        const SegP p = staged_seg(buf);
        L.qup = (L.i == 0) ? L.qup_head : L.q_up_old;
        L.quc = (L.i == 0) ? L.quc_head : L.q_up_new;
        if (p.n_ch <= 0.0 || p.s0 <= 0.0 || p.z <= 0.0 || p.bw <= 0.0 ||
            (L.ql <= 0.0 && L.qup <= 0.0 && L.quc <= 0.0 && L.qdp <= 0.0)) {
            __stcg(net.q + L.s, 0.0);
            __stcg(net.d + L.s, 0.0);
            __stcg(net.v + L.s, 0.0);
            if (run.q_hist) __stcg(run.q_hist + (size_t)L.tau * (size_t)net.n_seg_int + L.s, 0.0);
            L.q_up_old = L.qdp;
            L.q_up_new = 0.0;
            L.q_last = 0.0;
            SolveOut o;
            o.iters = 0;
            o.retried = 0;
            o.early = 1;
            count_solve(ls, hist_s, o);
            ++L.i;
            continue;
        }
        L.dpp = fmax(dpp, 0.0);
        plain_bracket(L, run.tol);
        L.total = 0;
        L.retried = 0;
        L.warm = W_PLAIN;
        if (run.warm) {
            // the learned starting depth of this solve, predicted before the launch:
            // the bracket [p (1 - delta), p (1 + delta)] around a positive normal
            // float p below 1e4 m (0x461c4000), else the plain bracket
            const unsigned pb = (unsigned)((unsigned long long)tw >> 32);   // staged with the record
            if (pb >= 0x00800000u && pb < 0x461c4000u) {
                const double pr = __longlong_as_double(((long long)((pb >> 23) + 896) << 52) |
                                                       ((long long)(pb & 0x7fffff) << 29));  // exact widening
                L.h = pr * run.warm_hi;
                L.h_0 = pr * run.warm_lo;
                L.warm = W_ACTIVE;
                ls.warm_used++;
                if (run.start_hist) __stcg(run.start_hist + (size_t)L.tau * (size_t)net.n_seg_int + L.s, pr);
            }
        }
        return true;
    }
    return false;
}

// One evaluation pass of a lane in SOLVE or VEL mode (no-op otherwise).
__device__ __forceinline__ void lane_pass(Lane& L, const NetDev& net, const RunDev& run, LocalStats& ls,
                                          unsigned int* hist_s, double2* slot)
{
    const Tol& tol = run.tol;
    const double dt = run.dt;
    const double dt2 = run.dt_half;  // dt / 2 (exact), formed on the host
    if (L.mode == L_SOLVE) {
        // the segment's parameters, staged in shared memory
        const SegP p = staged_seg(seg_buf(slot, L.i));
        const double x = L.need0 ? L.h_0 : L.h;  // >= +0
        // Every comparison, minimum and maximum of the pass runs on the integer
        // pipes (fpbits.cuh: the IEEE results, bit for bit), leaving the FP64
        // pipe to the arithmetic.
        const bool twcc_pos = fp_gt0(p.twcc);
        const double twl = p.bw + p.z2 * x;  // bw + 2 z x
        double above = fp_max0(x - p.bfd);
        double below = fp_min_pos(p.bfd, x);
        if (fp_gt0(above) && (fp_lt0(p.twcc) || fp_eq0(p.twcc))) {
            above = 0.0;
            below = x;
        }
        const double A = (p.bw + below * p.z) * below;
        const double WP = p.bw + below * p.sq2;  // bw + 2 below sqrt(1+z^2)
        // the compound-channel terms: area A + AC, wetted perimeter P = WP + WPC,
        // conveyance weight WP n + WPC ncc
        double AAC, P, WPn;
        if (fp_gt0(above) || !fp_finite(p.twcc) || !fp_finite(p.ncc)) {
            const double AC = p.twcc * above;
            const double WPC = fp_gt0(above) ? (p.twcc + 2.0 * above) : 0.0;
            AAC = A + AC;
            P = WP + WPC;
            WPn = WP * p.n_ch + WPC * p.ncc;
        } else {
            // in bank (above = +0) with finite twcc, ncc: AC = +-0 and WPC = 0,
            // and adding a zero to A >= +0, WP > 0 or WP n > 0 returns it unchanged
            AAC = A;
            P = WP;
            WPn = WP * p.n_ch;
        }
        const bool P_pos = fp_gt0(P);
        // the two quotients by P share one correctly rounded reciprocal
        const SharedRcp rP = shared_rcp(P_pos ? P : 1.0);
        const double R = P_pos ? shared_div(AAC, rP) : 0.0;
        double r23, r53;
        pow23_53(R, &r23, &r53);
        {
            DepthEval e;
            e.Ck = 0.0;
            // 2 sqrt(1+z^2) / (bw + 2 x z): the denominator is twl
            if (fp_gt0(x)) e.Ck = fp_max0(p.ck_fac * ((5.0 / 3.0) * r23 - (2.0 / 3.0) * r53 * (p.sq2 / twl)));
            e.Km = fp_gt0(e.Ck) ? fp_max_pos(dt, p.dx / e.Ck) : dt;
            e.twu = (fp_gt_pos(x, p.bfd) && twcc_pos) ? p.twcc : twl;
            // 1.0 / t is the correctly rounded reciprocal of t
            e.Qmn = P_pos ? __drcp_rn(shared_div(WPn, rP)) * AAC * r23 * p.sq_s0 : 0.0;
            if (L.need0) {
                L.e0 = e;
                L.need0 = 0;
            } else {
                const double qup = L.qup, quc = L.quc, qdp = L.qdp, ql = L.ql;
                const DepthEval& e0 = L.e0;
                // X at the lower depth, clamped to [0, 0.5] (troute_mc_final.cu:86)
                double X0 = 0.5;
                {
                    const double g1 = e0.twu * p.s0, g2 = g1 * e0.Ck, g = g2 * p.dx;
                    if (fp_gt0(e0.Ck) && fp_gt0(g))
                        X0 = fp_min_pos(0.5, fp_max0(fp_half(1.0 - L.Qj_0 / twice_chain(g1, g2, g, e0.twu, p.s0, e0.Ck, p.dx))));
                }
                double D0 = e0.Km * (1.0 - X0) + dt2;
                if (fp_eq0(D0)) D0 = 1.0;
                const SharedRcp r0 = shared_rcp(D0);
                const double c1 = shared_div(e0.Km * X0 + dt2, r0);
                const double c2 = shared_div(dt2 - e0.Km * X0, r0);
                const double c3 = shared_div(e0.Km * (1.0 - X0) - dt2, r0);
                const double c4 = shared_div(ql * dt, r0);
                const double qmc0 = c1 * qup + c2 * quc + c3 * qdp + c4;
                L.Qj_0 = qmc0 - e0.Qmn;
                // X at the upper depth, clamped to [0.25, 0.5] (troute_mc_final.cu:105)
                double X = 0.5;
                {
                    const double g1 = e.twu * p.s0, g2 = g1 * e.Ck, g = g2 * p.dx;
                    if (fp_gt0(e.Ck) && fp_gt0(g))
                        X = fp_min_pos(0.5, fp_max_pos(0.25, fp_half(1.0 - qmc0 / twice_chain(g1, g2, g, e.twu, p.s0, e.Ck, p.dx))));
                }
                double D1 = e.Km * (1.0 - X) + dt2;
                if (fp_eq0(D1)) D1 = 1.0;
                const SharedRcp r1 = shared_rcp(D1);
                const double C1 = shared_div(e.Km * X + dt2, r1);
                const double C2 = shared_div(dt2 - e.Km * X, r1);
                const double C3 = shared_div(e.Km * (1.0 - X) - dt2, r1);
                double C4 = shared_div(ql * dt, r1);
                const double S3 = C1 * qup + C2 * quc + C3 * qdp;
                if (fp_lt0(C4) && fp_abs_gt(C4, S3)) C4 = -S3;
                const double Qj = (S3 + C4) - e.Qmn;
                // outflow of the last evaluated coefficients (troute_mc_final.cu:125-130)
                const double Qmc = S3 + C4;
                if (fp_lt0(Qmc)) {
                    if (fp_lt0(C4) && fp_abs_gt(C4, S3))
                        L.qdc = 0.0;
                    else
                        L.qdc = fmax(C1 * qup + C2 * quc + C4, C1 * qup + C3 * qdp + C4);
                } else {
                    L.qdc = Qmc;
                }
                const double h = L.h;
                const double dQ = L.Qj_0 - Qj;
                double h_1 = !fp_eq0(dQ) ? h - (Qj * (L.h_0 - h)) / dQ : h;
                if (fp_lt0(h_1)) h_1 = h;
                // the reference's test rerr > rtol && aerr >= atol with
                // rerr = |(h_1 - h) / h|, aerr = |h_1 - h| (rerr = 0, aerr = 0.9
                // for h <= 0); the relative error's quotient is only compared
                // with rtol, which quot_gt_pos does exactly without dividing
                bool more;
                if (fp_gt0(h)) {
                    const double aerr = fp_abs(h_1 - h);
                    more = fp_ge_nonneg(aerr, tol.atol) && quot_gt_pos(aerr, h, tol.rtol);
                } else {
                    more = fp_gt_pos(0.0, tol.rtol) && fp_ge_nonneg(0.9, tol.atol);
                }
                L.h_0 = fp_max0(h);
                L.h = fp_max0(h_1);
                L.e0 = e;
                ++L.iter;
                ++L.total;
                bool stop;
                if (L.warm == W_ACTIVE) {
                    // warm phase: accepted once the stop test passes at a depth of at
                    // least kMinDepth; otherwise, after warm_k passes (or below
                    // kMinDepth), the plain solve restarts from the previous depth
                    const bool below_min = fp_lt_pos(L.h, kMinDepth);
                    stop = !more && !below_min;
                    if (!stop && (below_min || L.iter >= run.warm_k)) {
                        L.warm = W_PLAIN;
                        ls.warm_fallback++;
                        plain_bracket(L, tol);
                    }
                } else {
                    stop = fp_lt_pos(L.h, kMinDepth) || !(more && L.iter <= L.maxiter);
                }
                if (stop) {
                    bool done = true;
                    if (L.warm == W_PLAIN && L.iter >= L.maxiter) {
                        // widen the bracket (also after the last attempt, as the reference does)
                        L.h *= 1.33;
                        L.h_0 *= 0.67;
                        L.maxiter += 25;
                        L.retried = 1;
                        if (++L.attempt < tol.attempts) {
                            L.iter = 0;
                            L.need0 = 1;
                            done = false;
                        }
                    }
                    if (done) {
                        // store the segment (its velocity is derived from the final depth
                        // once the run is over, see velocity_kernel) and start the next one
                        __stcg(net.q + L.s, L.qdc);
                        __stcg(net.d + L.s, L.h);
                        if (run.q_hist) __stcg(run.q_hist + (size_t)L.tau * (size_t)net.n_seg_int + L.s, L.qdc);
                        if (run.pairs) {
                            float* pr = run.pairs + ((size_t)L.tau * (size_t)net.n_seg_int + L.s) * 9;
                            pr[0] = (float)L.qup;
                            pr[1] = (float)L.quc;
                            pr[2] = (float)L.qdp;
                            pr[3] = (float)L.ql;
                            pr[4] = (float)p.dx;
                            pr[5] = (float)p.s0;
                            pr[6] = (float)p.n_ch;
                            pr[7] = (float)p.bw;
                            pr[8] = (float)L.h;
                        }
                        L.q_up_old = L.qdp;
                        L.q_up_new = L.qdc;
                        L.q_last = L.qdc;
                        SolveOut o;
                        o.iters = L.total;
                        o.retried = L.retried;
                        o.early = 0;
                        count_solve(ls, hist_s, o);
                        ++L.i;
                        L.mode = L.i < L.ns ? L_BEGIN : L_DONE;
                    }
                }
            }
        }
    }
}

}  // namespace tr
