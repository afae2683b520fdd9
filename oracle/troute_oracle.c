/*
 * CPU oracle for the t-route Muskingum-Cunge secant routing path.
 *
 * TEST INFRASTRUCTURE ONLY: the reference's algorithm that tests/,
 * __graft_entry__.smoke() and the CPU legs of bench.py compare the CUDA path
 * with. Nothing in the product calls it.
 *
 * This is a plain-C restatement of the reference's FP64 CPU routines:
 *   - oracle_mc_solve  follows cpu_mc's inlined solve,
 *       water-prediction/t-route/troute_mc_final.cu:181-248
 *       (device twin mc_solve/hgeo at :30-139);
 *   - oracle_cpu_mc    follows cpu_mc, troute_mc_final.cu:167-252;
 *   - oracle_route_tree follows cpu_wavefront_fp64,
 *       water-prediction/t-route/wavefront/wavefront_mc.cu:495-564,
 *       with FP64 inputs instead of the reference's float inputs.
 * The only change of algorithm is that the secant tolerances (rtol/atol,
 * maxiter, attempts) are parameters; at rtol = atol = 0.01, maxiter = 100,
 * attempts = 5 the arithmetic is operation-for-operation the reference's
 * (same association order, no FMA contraction: build with -ffp-contract=off),
 * which tests/test_oracle.py checks bit-for-bit against the compiled
 * reference.
 */
#include "troute_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define MINDEPTH 0.01 /* troute_mc_final.cu:58 */

/* ---------------------------------------------------------------------------
 * R^(2/3) and R^(5/3). Mode 0 calls the C library's pow() exactly as the
 * reference does. Mode 1 returns the correctly rounded values instead, from
 * this file's own evaluation of R^fl(2/3) and R^fl(5/3) (the exponents the
 * reference passes are the doubles nearest 2/3 and 5/3): split R = y 2^(3k)
 * with y in [1, 8) (frexp / ldexp, exact), z = cbrt(y)^2 to a few ulp, then
 * one Newton correction delta = -(z^3 - y^2) / (3 z^2) with the residual
 * formed from error-free products (a*b - fl(a*b) = fma(a, b, -fl(a*b))), the
 * exponent offset as the factor 1 + (fl(2/3) - 2/3) ln R, and round
 * z + (delta + z c2) and y z + (err(y z) + y delta + y z c5). Mode 1 is the platform-independent form of the
 * same arithmetic; the GPU library uses the same definition, so the two can be
 * compared bit for bit.
 * ------------------------------------------------------------------------- */
static int g_pow_mode = 0;
/* fl(2/3) - 2/3 = -(1/3) 2^-53 and fl(5/3) - 5/3 = (1/3) 2^-52 */
#define FL23_MINUS_23 (-3.700743415417188e-17)
#define FL53_MINUS_53 (7.401486830834377e-17)

void oracle_set_pow_mode(int mode) { g_pow_mode = mode; }

static void cr_pow23_53(double x, double* p23, double* p53)
{
    if (!(x > 0.0) || isinf(x)) {
        const double v = (x == 0.0 || isinf(x)) ? x : NAN;
        *p23 = v;
        *p53 = v;
        return;
    }
    int e;
    const double m = frexp(x, &e); /* x = m 2^e, m in [0.5, 1) */
    const int e1 = e - 1;          /* x = (2m) 2^e1 */
    const int k = (e1 >= 0) ? e1 / 3 : -((-e1 + 2) / 3);
    const int j = e1 - 3 * k;
    const double y = ldexp(2.0 * m, j); /* [1, 8) */
    const double c = cbrt(y);
    const double z = c * c;
    const double p = z * z, pe = fma(z, z, -p);
    const double q = z * p, qe = fma(z, p, -q);
    const double t = z * pe;
    const double s = y * y, se = fma(y, y, -s);
    const double d = (q - s) + ((qe + t) - se);
    const double delta = -d / (3.0 * p);
    const double w0 = y * z, we = fma(y, z, -w0);
    /* the reference's exponents are the doubles nearest 2/3 and 5/3, not the
     * rationals: x^fl(2/3) = x^(2/3) (1 + e2 ln x), e2 = fl(2/3) - 2/3 */
    const double L = log(x);
    const double c2 = FL23_MINUS_23 * L, c5 = FL53_MINUS_53 * L;
    *p23 = ldexp(z + (delta + z * c2), 2 * k);
    *p53 = ldexp(w0 + ((we + y * delta) + w0 * c5), 5 * k);
}

static double P23(double x)
{
    if (g_pow_mode == 0) return pow(x, 2.0 / 3.0);
    double a, b;
    cr_pow23_53(x, &a, &b);
    return a;
}

static double P53(double x)
{
    if (g_pow_mode == 0) return pow(x, 5.0 / 3.0);
    double a, b;
    cr_pow23_53(x, &a, &b);
    return b;
}

void oracle_pow23_53(double x, double* p23, double* p53)
{
    *p23 = P23(x);
    *p53 = P53(x);
}

typedef struct {
    const double* x;
    long long b, e;
    double *p23, *p53;
    int mode;
} pow_job;

static void* pow_rows(void* arg)
{
    const pow_job* J = (const pow_job*)arg;
    for (long long i = J->b; i < J->e; ++i) {
        if (J->mode == 0) {
            J->p23[i] = pow(J->x[i], 2.0 / 3.0);
            J->p53[i] = pow(J->x[i], 5.0 / 3.0);
        } else {
            cr_pow23_53(J->x[i], &J->p23[i], &J->p53[i]);
        }
    }
    return NULL;
}

int oracle_pow23_53_n(const double* x, long long n, double* p23, double* p53, int mode, int n_threads)
{
    if (n_threads < 1) n_threads = 1;
    pow_job* J = (pow_job*)calloc((size_t)n_threads, sizeof(pow_job));
    pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
    if (!J || !th) {
        free(J), free(th);
        return 2;
    }
    const long long per = (n + n_threads - 1) / n_threads;
    for (int i = 0; i < n_threads; ++i) {
        const long long b = i * per, e = (b + per < n) ? b + per : n;
        J[i] = (pow_job){x, b < n ? b : n, e, p23, p53, mode};
        if (i > 0) pthread_create(&th[i], NULL, pow_rows, &J[i]);
    }
    pow_rows(&J[0]);
    for (int i = 1; i < n_threads; ++i) pthread_join(th[i], NULL);
    free(J), free(th);
    return 0;
}

/* Channel geometry at depth h: trapezoid plus compound (floodplain) channel.
 * troute_mc_final.cu:30-40 (inlined at :200-205 and :216-221). */
typedef struct geo {
    double twl, R, A, AC, WP, WPC;
} geo;

static void channel_geometry(double h, double bfd, double bw, double twcc, double z,
                             geo* g)
{
    g->twl = bw + 2.0 * z * h;
    double above = fmax(h - bfd, 0.0);
    double below = fmin(bfd, h);
    if (above > 0.0 && twcc <= 0.0) {
        above = 0.0;
        below = h;
    }
    g->A = (bw + below * z) * below;
    g->WP = bw + 2.0 * below * sqrt(1.0 + z * z);
    g->AC = twcc * above;
    g->WPC = (above > 0.0) ? (twcc + 2.0 * above) : 0.0;
    g->R = (g->WP + g->WPC > 0.0) ? (g->A + g->AC) / (g->WP + g->WPC) : 0.0;
}

/* Kinematic celerity from Manning's equation, troute_mc_final.cu:78-82 / :97-101. */
static double celerity(double h, const geo* g, double s0, double n_ch, double bw, double z)
{
    if (!(h > 0.0)) return 0.0;
    double r23 = P23(g->R);
    double r53 = P53(g->R);
    return fmax(0.0, (sqrt(s0) / n_ch) *
                         ((5.0 / 3.0) * r23 -
                          (2.0 / 3.0) * r53 * (2.0 * sqrt(1.0 + z * z) / (bw + 2.0 * h * z))));
}

/* Manning discharge at the geometry g, troute_mc_final.cu:91 / :111. */
static double manning_q(const geo* g, double n_ch, double ncc, double s0)
{
    if (!(g->WP + g->WPC > 0.0)) return 0.0;
    return (1.0 / (((g->WP * n_ch) + (g->WPC * ncc)) / (g->WP + g->WPC))) * (g->A + g->AC) *
           P23(g->R) * sqrt(s0);
}

/* State of one secant solve between passes. */
typedef struct secant {
    double h, h_0, Qj_0, C1, C2, C3, C4, rerr, aerr;
} secant;

/* One pass of the secant loop body, troute_mc_final.cu:198-237: residuals at
 * h_0 and h, the secant update and the errors. */
static void secant_pass(secant* S, double dt, double qup, double quc, double qdp, double ql,
                        const oracle_chparams* p, double z, double bfd)
{
    const double bw = p->bw, twcc = p->twcc, n_ch = p->n_ch, ncc = p->ncc;
    const double s0 = p->s0, dx = p->dx;
    double h = S->h, h_0 = S->h_0;
    /* lower point h_0, :200-214 */
    geo g0;
    channel_geometry(h_0, bfd, bw, twcc, z, &g0);
    const double Ck0 = celerity(h_0, &g0, s0, n_ch, bw, z);
    const double Km0 = (Ck0 > 0.0) ? fmax(dt, dx / Ck0) : dt;
    const double twu0 = (h_0 > bfd && twcc > 0.0) ? twcc : g0.twl;
    const double X0 = (Ck0 > 0.0 && twu0 * s0 * Ck0 * dx > 0.0)
                          ? fmin(0.5, fmax(0.0, 0.5 * (1.0 - S->Qj_0 / (2.0 * twu0 * s0 * Ck0 * dx))))
                          : 0.5;
    double D0 = Km0 * (1.0 - X0) + dt / 2.0;
    if (D0 == 0.0) D0 = 1.0;
    const double c1 = (Km0 * X0 + dt / 2.0) / D0;
    const double c2 = (dt / 2.0 - Km0 * X0) / D0;
    const double c3 = (Km0 * (1.0 - X0) - dt / 2.0) / D0;
    const double c4 = (ql * dt) / D0;
    const double qmc0 = c1 * qup + c2 * quc + c3 * qdp + c4;
    const double Qj_0 = qmc0 - manning_q(&g0, n_ch, ncc, s0);

    /* upper point h, :216-231; X is clamped to [0.25, 0.5] here and uses the
     * h_0 coefficients in its numerator */
    geo g1;
    channel_geometry(h, bfd, bw, twcc, z, &g1);
    const double Ck1 = celerity(h, &g1, s0, n_ch, bw, z);
    const double Km1 = (Ck1 > 0.0) ? fmax(dt, dx / Ck1) : dt;
    const double twu1 = (h > bfd && twcc > 0.0) ? twcc : g1.twl;
    const double X = (Ck1 > 0.0 && twu1 * s0 * Ck1 * dx > 0.0)
                         ? fmin(0.5, fmax(0.25, 0.5 * (1.0 - qmc0 / (2.0 * twu1 * s0 * Ck1 * dx))))
                         : 0.5;
    double D1 = Km1 * (1.0 - X) + dt / 2.0;
    if (D1 == 0.0) D1 = 1.0;
    const double C1 = (Km1 * X + dt / 2.0) / D1;
    const double C2 = (dt / 2.0 - Km1 * X) / D1;
    const double C3 = (Km1 * (1.0 - X) - dt / 2.0) / D1;
    double C4 = (ql * dt) / D1;
    if (C4 < 0.0 && fabs(C4) > C1 * qup + C2 * quc + C3 * qdp)
        C4 = -(C1 * qup + C2 * quc + C3 * qdp);
    const double Qj = (C1 * qup + C2 * quc + C3 * qdp + C4) - manning_q(&g1, n_ch, ncc, s0);

    /* secant update, :233-237 */
    double h_1 = (Qj_0 - Qj != 0.0) ? h - (Qj * (h_0 - h)) / (Qj_0 - Qj) : h;
    if (h_1 < 0.0) h_1 = h;
    if (h > 0.0) {
        S->rerr = fabs((h_1 - h) / h);
        S->aerr = fabs(h_1 - h);
    } else {
        S->rerr = 0.0;
        S->aerr = 0.9;
    }
    S->h_0 = fmax(0.0, h);
    S->h = fmax(0.0, h_1);
    S->Qj_0 = Qj_0;
    S->C1 = C1;
    S->C2 = C2;
    S->C3 = C3;
    S->C4 = C4;
}

/* The solve with an optional learned starting depth. start > 0: the first
 * phase brackets [start (1 - delta), start (1 + delta)] and runs at most
 * warm_k passes; it is accepted when the stop test (rerr <= rtol or
 * aerr < atol) passes with h >= MINDEPTH, otherwise the solve restarts as the
 * plain solve from the previous depth (a fallback; its passes still count).
 * start <= 0: the plain solve. *warm_state: 0 plain, 1 warm start accepted,
 * 2 fallback. */
static double mc_solve_core(double dt, double qup, double quc, double qdp, double ql,
                            const oracle_chparams* p, double depthp, const oracle_tol* tol,
                            double start, double delta, int warm_k,
                            double* depthc, double* velc, int* iters, int* warm_state)
{
    const double bw = p->bw, tw = p->tw, n_ch = p->n_ch;
    const double s0 = p->s0;
    /* side slope and bankfull depth, :181-183 */
    const double z = (p->cs == 0.0) ? 1.0 : 1.0 / p->cs;
    const double bfd = (bw > tw) ? bw / 0.00001 : (bw == tw) ? bw / (2.0 * z) : (tw - bw) / (2.0 * z);
    *iters = 0;
    *warm_state = 0;

    /* invalid parameters or no flow at all: zero outputs, :187-190 */
    if (n_ch <= 0.0 || s0 <= 0.0 || z <= 0.0 || bw <= 0.0 ||
        (ql <= 0.0 && qup <= 0.0 && quc <= 0.0 && qdp <= 0.0)) {
        *depthc = 0.0;
        *velc = 0.0;
        return 0.0;
    }

    secant S;
    memset(&S, 0, sizeof S);
    int total = 0;
    int solved = 0;
    if (start > 0.0) {
        *warm_state = 1;
        S.h = start * (1.0 + delta);
        S.h_0 = start * (1.0 - delta);
        S.Qj_0 = 0.0;
        for (int iter = 0;;) {
            secant_pass(&S, dt, qup, quc, qdp, ql, p, z, bfd);
            iter++;
            total++;
            if (S.h < MINDEPTH) break;
            if (!(S.rerr > tol->rtol && S.aerr >= tol->atol)) {
                solved = 1;
                break;
            }
            if (iter >= warm_k) break;
        }
        if (!solved) *warm_state = 2;
    }
    if (!solved) {
        const double depth = fmax(depthp, 0.0);
        S.h = depth * 1.33 + MINDEPTH; /* upper secant start, :193 */
        S.h_0 = depth * 0.67;          /* lower secant start */
        S.Qj_0 = 0.0;
        int maxiter = tol->maxiter;
        for (int attempt = 0; attempt < tol->attempts; attempt++) {
            int iter = 0;
            S.aerr = 0.01;
            S.rerr = 1.0;
            int first = 1; /* the first pass of every attempt always runs */
            while (first || (S.rerr > tol->rtol && S.aerr >= tol->atol && iter <= maxiter)) {
                first = 0;
                secant_pass(&S, dt, qup, quc, qdp, ql, p, z, bfd);
                iter++;
                total++;
                if (S.h < MINDEPTH) break;
            }
            if (iter < maxiter) break;
            /* widen the bracket and allow more iterations, :240 */
            S.h *= 1.33;
            S.h_0 *= 0.67;
            maxiter += 25;
        }
    }

    /* outflow with the negative-flow fallbacks, :242-244 */
    const double C1 = S.C1, C2 = S.C2, C3 = S.C3, C4 = S.C4;
    double qdc;
    const double Qmc = C1 * qup + C2 * quc + C3 * qdp + C4;
    if (Qmc < 0.0) {
        if (C4 < 0.0 && fabs(C4) > C1 * qup + C2 * quc + C3 * qdp)
            qdc = 0.0;
        else
            qdc = fmax(C1 * qup + C2 * quc + C4, C1 * qup + C3 * qdp + C4);
    } else {
        qdc = Qmc;
    }

    /* velocity from the trapezoid-only hydraulic radius, :245-248 */
    const double h = S.h;
    const double twl = bw + 2.0 * z * h;
    double Rv = (h * (bw + twl) / 2.0) /
                (bw + 2.0 * sqrt(((twl - bw) / 2.0) * ((twl - bw) / 2.0) + h * h));
    if (Rv < 0.0) Rv = 0.0;
    *velc = (1.0 / n_ch) * P23(Rv) * sqrt(s0);
    *depthc = h;
    *iters = total;
    return qdc;
}

double oracle_mc_solve(double dt, double qup, double quc, double qdp, double ql,
                       const oracle_chparams* p, double depthp,
                       const oracle_tol* tol,
                       double* depthc, double* velc, int* iters)
{
    int ws;
    return mc_solve_core(dt, qup, quc, qdp, ql, p, depthp, tol, 0.0, 0.0, 0, depthc, velc, iters, &ws);
}

double oracle_mc_solve_warm(double dt, double qup, double quc, double qdp, double ql,
                            const oracle_chparams* p, double depthp, const oracle_tol* tol,
                            double start, double delta, int warm_k,
                            double* depthc, double* velc, int* iters, int* warm_state)
{
    return mc_solve_core(dt, qup, quc, qdp, ql, p, depthp, tol, start, delta, warm_k, depthc, velc, iters,
                         warm_state);
}

void oracle_cpu_mc(const oracle_chparams* p, const double* ql,
                   const int* rs, const int* rl,
                   const double* qu, const double* qd, const double* dp,
                   double* qo, double* vo, double* dpo,
                   double uq, double dt, int nr,
                   const oracle_tol* tol, long long* iters_total)
{
    long long total = 0;
    for (int r = 0; r < nr; r++) {
        double quc = uq; /* chained current-step inflow, seeded by uq: :175 */
        for (int i = 0; i < rl[r]; i++) {
            const int s = rs[r] + i;
            double dc, vc;
            int it;
            const double q = oracle_mc_solve(dt, qu[s], quc, qd[s], ql[s], &p[s], dp[s], tol,
                                             &dc, &vc, &it);
            qo[s] = q;
            vo[s] = vc;
            dpo[s] = dc;
            quc = q;
            total += it;
        }
    }
    if (iters_total) *iters_total = total;
}

/* ---------------------------------------------------------------------------
 * Tree routing (wavefront_mc.cu:495-564). State is double-buffered by step
 * parity instead of the reference's swap + refill; every reach and segment is
 * rewritten each step, so the values are the same.
 * ------------------------------------------------------------------------- */
typedef struct tree_job {
    const int *seg_start, *seg_len, *up_ptr, *up_idx, *level_ptr, *level_reach;
    int n_reaches, n_levels, n_segments;
    const oracle_chparams* params;
    const double* qlat_ts;
    int n_ts;
    double dt;
    const oracle_tol* tol;
    double *q[2], *d[2], *v, *rl[2];
    double* q_hist;
    double* d_hist;
    int* it_hist;
    const double* warm_start;
    double warm_delta;
    int warm_k;
    int n_threads;
    pthread_barrier_t barrier;
} tree_job;

typedef struct tree_worker {
    tree_job* job;
    int rank;
    long long iters, warm_used, warm_fallback;
} tree_worker;

static void route_reach(tree_job* J, int r, int t, tree_worker* W)
{
    const int prev = t & 1, cur = (t + 1) & 1;
    const double* qlat = J->qlat_ts + (size_t)t * (size_t)J->n_segments;
    /* upstream sums at the reach head, :525-531 */
    double qup_head = 0.0, quc_head = 0.0;
    for (int k = J->up_ptr[r]; k < J->up_ptr[r + 1]; ++k) {
        const int u = J->up_idx[k];
        qup_head += J->rl[prev][u];
        quc_head += J->rl[cur][u];
    }
    double quc_next = 0.0, q_last = 0.0;
    const int s0 = J->seg_start[r];
    for (int i = 0; i < J->seg_len[r]; ++i) {
        const int s = s0 + i;
        /* interior segments take the upstream segment's previous and current
         * discharge, :538-539 */
        const double qup = (i == 0) ? qup_head : J->q[prev][s - 1];
        const double quc = (i == 0) ? quc_head : quc_next;
        double dc, vc;
        int it, ws;
        const size_t ts = (size_t)t * (size_t)J->n_segments + s;
        const double start = J->warm_start ? J->warm_start[ts] : 0.0;
        const double q = mc_solve_core(J->dt, qup, quc, J->q[prev][s], qlat[s], &J->params[s],
                                       J->d[prev][s], J->tol, start, J->warm_delta, J->warm_k,
                                       &dc, &vc, &it, &ws);
        J->q[cur][s] = q;
        J->d[cur][s] = dc;
        J->v[s] = vc;
        if (J->q_hist) J->q_hist[ts] = q;
        if (J->d_hist) J->d_hist[ts] = dc;
        if (J->it_hist) J->it_hist[ts] = it;
        quc_next = q;
        q_last = q;
        W->iters += it;
        W->warm_used += (ws != 0);
        W->warm_fallback += (ws == 2);
    }
    J->rl[cur][r] = q_last;
}

static void* tree_worker_main(void* arg)
{
    tree_worker* W = (tree_worker*)arg;
    tree_job* J = W->job;
    for (int t = 0; t < J->n_ts; ++t) {
        for (int L = 0; L < J->n_levels; ++L) {
            const int lb = J->level_ptr[L], le = J->level_ptr[L + 1];
            const int n = le - lb;
            const int per = (n + J->n_threads - 1) / J->n_threads;
            const int b = lb + W->rank * per;
            const int e = (b + per < le) ? b + per : le;
            for (int ii = b; ii < e; ++ii) route_reach(J, J->level_reach[ii], t, W);
            if (J->n_threads > 1) pthread_barrier_wait(&J->barrier);
        }
    }
    return NULL;
}

int oracle_route_tree(const int* reach_seg_start, const int* reach_seg_len,
                      const int* reach_up_ptr, const int* reach_up_idx,
                      const int* level_ptr, const int* level_reach,
                      int n_reaches, int n_levels, int n_segments,
                      const oracle_chparams* params, const double* qlat_ts,
                      const double* qdp0, const double* dp0, const double* reach_last0,
                      int n_ts, double dt, const oracle_tol* tol,
                      double* q_out, double* d_out, double* v_out,
                      double* reach_last_out, double* q_hist,
                      long long* iters_total, int n_threads)
{
    return oracle_route_tree_it(reach_seg_start, reach_seg_len, reach_up_ptr, reach_up_idx, level_ptr,
                                level_reach, n_reaches, n_levels, n_segments, params, qlat_ts, qdp0, dp0,
                                reach_last0, n_ts, dt, tol, q_out, d_out, v_out, reach_last_out, q_hist,
                                NULL, iters_total, n_threads);
}

int oracle_route_tree_ex(const int* reach_seg_start, const int* reach_seg_len,
                         const int* reach_up_ptr, const int* reach_up_idx,
                         const int* level_ptr, const int* level_reach,
                         int n_reaches, int n_levels, int n_segments,
                         const oracle_chparams* params, const double* qlat_ts,
                         const double* qdp0, const double* dp0, const double* reach_last0,
                         int n_ts, double dt, const oracle_tol* tol,
                         double* q_out, double* d_out, double* v_out,
                         double* reach_last_out, oracle_tree_opts* opts)
{
    double* q_hist = opts->q_hist;
    int* it_hist = opts->it_hist;
    int n_threads = opts->n_threads;
    if (n_reaches < 0 || n_segments < 0 || n_levels < 0 || n_ts < 0) return 1;
    if (n_threads < 1) n_threads = 1;
    tree_job J;
    memset(&J, 0, sizeof J);
    J.seg_start = reach_seg_start;
    J.seg_len = reach_seg_len;
    J.up_ptr = reach_up_ptr;
    J.up_idx = reach_up_idx;
    J.level_ptr = level_ptr;
    J.level_reach = level_reach;
    J.n_reaches = n_reaches;
    J.n_levels = n_levels;
    J.n_segments = n_segments;
    J.params = params;
    J.qlat_ts = qlat_ts;
    J.n_ts = n_ts;
    J.dt = dt;
    J.tol = tol;
    J.q_hist = q_hist;
    J.it_hist = it_hist;
    J.d_hist = opts->d_hist;
    J.warm_start = opts->warm_start;
    J.warm_delta = opts->warm_delta;
    J.warm_k = opts->warm_k;
    J.n_threads = n_threads;
    const size_t S = (size_t)n_segments, R = (size_t)n_reaches;
    double* buf = (double*)calloc(4 * S + 2 * R + 1, sizeof(double));
    if (!buf) return 2;
    J.q[0] = buf;
    J.q[1] = buf + S;
    J.d[0] = buf + 2 * S;
    J.d[1] = buf + 3 * S;
    J.rl[0] = buf + 4 * S;
    J.rl[1] = buf + 4 * S + R;
    J.v = v_out;
    memcpy(J.q[0], qdp0, S * sizeof(double));
    memcpy(J.d[0], dp0, S * sizeof(double));
    memcpy(J.rl[0], reach_last0, R * sizeof(double));
    memset(v_out, 0, S * sizeof(double));

    long long total = 0, used = 0, fell = 0;
    if (n_threads == 1) {
        tree_worker W = {&J, 0, 0, 0, 0};
        tree_worker_main(&W);
        total = W.iters;
        used = W.warm_used;
        fell = W.warm_fallback;
    } else {
        pthread_barrier_init(&J.barrier, NULL, (unsigned)n_threads);
        tree_worker* W = (tree_worker*)calloc((size_t)n_threads, sizeof(tree_worker));
        pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
        for (int i = 0; i < n_threads; ++i) {
            W[i].job = &J;
            W[i].rank = i;
            if (i > 0) pthread_create(&th[i], NULL, tree_worker_main, &W[i]);
        }
        tree_worker_main(&W[0]);
        for (int i = 1; i < n_threads; ++i) pthread_join(th[i], NULL);
        for (int i = 0; i < n_threads; ++i) {
            total += W[i].iters;
            used += W[i].warm_used;
            fell += W[i].warm_fallback;
        }
        pthread_barrier_destroy(&J.barrier);
        free(W);
        free(th);
    }
    const int fin = n_ts & 1;
    memcpy(q_out, J.q[fin], S * sizeof(double));
    memcpy(d_out, J.d[fin], S * sizeof(double));
    memcpy(reach_last_out, J.rl[fin], R * sizeof(double));
    opts->iters_total = total;
    opts->warm_used = used;
    opts->warm_fallback = fell;
    free(buf);
    return 0;
}

int oracle_route_tree_it(const int* reach_seg_start, const int* reach_seg_len,
                         const int* reach_up_ptr, const int* reach_up_idx,
                         const int* level_ptr, const int* level_reach,
                         int n_reaches, int n_levels, int n_segments,
                         const oracle_chparams* params, const double* qlat_ts,
                         const double* qdp0, const double* dp0, const double* reach_last0,
                         int n_ts, double dt, const oracle_tol* tol,
                         double* q_out, double* d_out, double* v_out,
                         double* reach_last_out, double* q_hist, int* it_hist,
                         long long* iters_total, int n_threads)
{
    oracle_tree_opts o;
    memset(&o, 0, sizeof o);
    o.q_hist = q_hist;
    o.it_hist = it_hist;
    o.n_threads = n_threads;
    const int rc = oracle_route_tree_ex(reach_seg_start, reach_seg_len, reach_up_ptr, reach_up_idx, level_ptr,
                                        level_reach, n_reaches, n_levels, n_segments, params, qlat_ts, qdp0, dp0,
                                        reach_last0, n_ts, dt, tol, q_out, d_out, v_out, reach_last_out, &o);
    if (iters_total) *iters_total = o.iters_total;
    return rc;
}

/* ---------------------------------------------------------------------------
 * Linearised MC (water-prediction/t-route/wavefront/linear_mc.cu).
 * oracle_linear_coeffs follows compute_mc_coeffs (:57-100) in float with the
 * C library's powf/sqrtf (the reference evaluates it on the GPU with CUDA's;
 * the two differ in the last bits, so the GPU coefficients are compared with a
 * tolerance). oracle_linear_route follows cpu_linear_mc (:177-232): given the
 * same coefficients it is the reference's float arithmetic, operation for
 * operation (no contraction).
 * ------------------------------------------------------------------------- */
void oracle_linear_coeffs(const oracle_chparams_f32* params, int n, float dt, float* c1, float* c2, float* c3,
                          float* c4oq)
{
    for (int i = 0; i < n; ++i) {
        const oracle_chparams_f32 p = params[i];
        const float z = (p.cs == 0.0f) ? 1.0f : 1.0f / p.cs;
        float bfd;
        if (p.bw > p.tw) bfd = p.bw / 0.00001f;
        else if (p.bw == p.tw) bfd = p.bw / (2.0f * z);
        else bfd = (p.tw - p.bw) / (2.0f * z);
        const float h = fmaxf(0.5f * bfd, 0.1f);
        const float twl = p.bw + 2.0f * z * h;
        const float A = (p.bw + h * z) * h;
        const float WP = p.bw + 2.0f * h * sqrtf(1.0f + z * z);
        const float R = (WP > 0.0f) ? A / WP : 0.0f;
        const float r23 = powf(R, 2.0f / 3.0f);
        const float r53 = powf(R, 5.0f / 3.0f);
        const float Ck = fmaxf(1e-6f, (sqrtf(p.s0) / p.n_ch) *
                                          ((5.0f / 3.0f) * r23 -
                                           (2.0f / 3.0f) * r53 * (2.0f * sqrtf(1.0f + z * z) / (p.bw + 2.0f * h * z))));
        const float Km = fmaxf(dt, p.dx / Ck);
        const float tw_use = (h > bfd && p.twcc > 0.0f) ? p.twcc : twl;
        float X = 0.25f;
        if (Ck > 0.0f && tw_use * p.s0 * Ck * p.dx > 0.0f)
            X = fminf(0.5f, fmaxf(0.0f, 0.5f * (1.0f - 0.0f / (2.0f * tw_use * p.s0 * Ck * p.dx))));
        float D = Km * (1.0f - X) + dt / 2.0f;
        if (D == 0.0f) D = 1.0f;
        c1[i] = (Km * X + dt / 2.0f) / D;
        c2[i] = (dt / 2.0f - Km * X) / D;
        c3[i] = (Km * (1.0f - X) - dt / 2.0f) / D;
        c4oq[i] = dt / D;
    }
}

int oracle_linear_route(const float* c1, const float* c2, const float* c3, const float* c4oq,
                        const int* reach_seg_start, const int* reach_seg_len, const int* reach_up_ptr,
                        const int* reach_up_idx, const int* level_ptr, const int* level_reach, int n_reaches,
                        int n_levels, int n_segments, const float* qlat_ts, const float* q0, float* q_final,
                        int n_ts)
{
    (void)n_reaches;
    float* Qp = (float*)malloc((size_t)(n_segments ? n_segments : 1) * sizeof(float));
    float* Qn = (float*)calloc((size_t)(n_segments ? n_segments : 1), sizeof(float));
    if (!Qp || !Qn) {
        free(Qp);
        free(Qn);
        return 2;
    }
    memcpy(Qp, q0, (size_t)n_segments * sizeof(float));
    for (int t = 0; t < n_ts; ++t) {
        const float* qlat = qlat_ts + (size_t)t * (size_t)n_segments;
        for (int L = 0; L < n_levels; ++L) {
            for (int kk = level_ptr[L]; kk < level_ptr[L + 1]; ++kk) {
                const int r = level_reach[kk];
                const int s0 = reach_seg_start[r], sl = reach_seg_len[r];
                float sum_new = 0.f, sum_old = 0.f;
                for (int k = reach_up_ptr[r]; k < reach_up_ptr[r + 1]; ++k) {
                    const int u = reach_up_idx[k];
                    const int last_u = reach_seg_start[u] + reach_seg_len[u] - 1;
                    sum_new += Qn[last_u];
                    sum_old += Qp[last_u];
                }
                /* the first segment takes the upstream sums, the others the
                 * previous segment's new and old discharge */
                float pn = sum_new, po = sum_old;
                for (int i = 0; i < sl; ++i) {
                    const int idx = s0 + i;
                    Qn[idx] = c1[idx] * pn + c2[idx] * po + c3[idx] * Qp[idx] + c4oq[idx] * qlat[idx];
                    pn = Qn[idx];
                    po = Qp[idx];
                }
            }
        }
        float* tmp = Qp;
        Qp = Qn;
        Qn = tmp;
        memset(Qn, 0, (size_t)n_segments * sizeof(float));
    }
    memcpy(q_final, Qp, (size_t)n_segments * sizeof(float));
    free(Qp);
    free(Qn);
    return 0;
}

/* ---------------------------------------------------------------------------
 * Diffusive-wave tridiagonal step (water-prediction/owp_extended_kernels.cu:
 * 24-91, cpu_diffusive_tridiag): float, the reference's operation order.
 * Arrays [n_reaches][max_nodes]; nodes at or past ncomp untouched.
 * ------------------------------------------------------------------------- */
int oracle_diffusive_tridiag(const oracle_diff_reach* rp, const float* dx, const float* diffusivity,
                             const float* qp_prev, float* qp_out, int n_reaches, int max_nodes)
{
    float* eei = (float*)malloc((size_t)(max_nodes > 0 ? max_nodes : 1) * sizeof(float));
    float* ffi = (float*)malloc((size_t)(max_nodes > 0 ? max_nodes : 1) * sizeof(float));
    if (!eei || !ffi) {
        free(eei);
        free(ffi);
        return 2;
    }
    for (int j = 0; j < n_reaches; j++) {
        const int nc = rp[j].ncomp;
        const float theta = rp[j].theta, dtini = rp[j].dtini;
        const size_t base = (size_t)j * (size_t)max_nodes;
        if (nc < 1 || nc > max_nodes) {
            free(eei);
            free(ffi);
            return 1;
        }
        eei[0] = 1.0f;
        ffi[0] = 0.0f;
        for (int i = 1; i < nc; i++) {
            float dxi = dx[base + i - 1];
            if (dxi < 1.0f) dxi = 1.0f;
            const float alpha = 1.0f;
            float diff_i = diffusivity[base + i];
            if (diff_i < 0.01f) diff_i = 0.01f;
            const float ppi = -theta * diff_i * dtini / (dxi * dxi) * 2.0f / (alpha * (alpha + 1.0f)) * alpha;
            const float qqi = 1.0f - ppi * (alpha + 1.0f) / alpha;
            const float rri = ppi / alpha;
            const float qnext = (i < nc - 1) ? qp_prev[base + i + 1] : qp_prev[base + i];
            const float ssi = qp_prev[base + i] + dtini * diff_i * (1.0f - theta) *
                                                      (qp_prev[base + i - 1] - 2.0f * qp_prev[base + i] + qnext) /
                                                      (dxi * dxi);
            float denom = ppi * eei[i - 1] + qqi;
            if (fabsf(denom) < 1e-20f) denom = 1e-20f;
            eei[i] = -rri / denom;
            ffi[i] = (ssi - ppi * ffi[i - 1]) / denom;
        }
        /* downstream boundary: the ghost node takes the previous discharge */
        qp_out[base + nc - 1] = eei[nc - 1] * qp_prev[base + nc - 1] + ffi[nc - 1];
        for (int i = nc - 2; i >= 0; i--) qp_out[base + i] = eei[i] * qp_out[base + i + 1] + ffi[i];
    }
    free(eei);
    free(ffi);
    return 0;
}
