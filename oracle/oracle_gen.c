/*
 * Seeded synthetic inputs for the CPU legs, restated in C.
 *
 * TEST INFRASTRUCTURE ONLY (part of libtroute_oracle.so). The benchmark's CPU
 * legs (the reference arm and the one-core baseline) must build their inputs
 * without loading the product library, so this file restates the product's
 * seeded generator independently: the same counter-based hash, the same
 * +,-,*,/-only log, exp and sine series, the same draws in the same order.
 * tests/test_generator.py checks that every array it writes (tree topology,
 * channel parameters, lateral inflow, ensemble member factors) is byte for
 * byte the product generator's, and that its level schedule equals the
 * reference's level rule (water-prediction/t-route/wavefront/gen_network.py:
 * 219-231) as restated in troute_oracle.py.
 *
 * Distributions (the benchmark's): reach lengths 1..max_len segments from a
 * truncated geometric law with the requested mean; a uniformly random binary
 * tree (Remy's growth); dx ~ U(500, 5000) m, s0 ~ LogU(1e-5, 1e-2),
 * n ~ U(0.03, 0.08), ncc = 2n, bw ~ U(2, 50) m, tw = 3 bw, twcc = 5 tw,
 * cs ~ U(0.5, 2); lateral inflow Gamma(2, 0.05) m3/s times a diurnal sine with
 * a per-segment phase; ensemble members: inflow x LogN(0, 0.3) (Box-Muller),
 * Manning's n x U(0.8, 1.2).
 *
 * Compiled with -ffp-contract=off like the product generator, so both round
 * every operation alike on x86-64 and aarch64.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "troute_oracle.h"

static uint64_t og_mix(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t og_hash(uint64_t seed, uint64_t stream, uint64_t ctr)
{
    return og_mix(og_mix(seed ^ og_mix(stream * 0xD1B54A32D192ED03ull)) + ctr);
}

/* uniform in (0, 1) from the top 53 bits */
static double og_u01(uint64_t h) { return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

#define OG_LN2 0.69314718055994530942
#define OG_TWO_PI 6.28318530717958647692

/* log x, x > 0: x = m 2^e, m in [1/sqrt2, sqrt2), log m = 2 atanh((m-1)/(m+1)) */
static double og_log(double x)
{
    uint64_t b;
    memcpy(&b, &x, 8);
    int e = (int)((b >> 52) & 0x7FF) - 1023;
    b = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;
    double m;
    memcpy(&m, &b, 8);
    if (m > 1.4142135623730951) {
        m *= 0.5;
        e += 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    static const double c[12] = {1.0 / 1, 1.0 / 3, 1.0 / 5, 1.0 / 7, 1.0 / 9, 1.0 / 11,
                                 1.0 / 13, 1.0 / 15, 1.0 / 17, 1.0 / 19, 1.0 / 21, 1.0 / 23};
    double acc = c[11];
    for (int k = 10; k >= 0; --k) acc = acc * s2 + c[k];
    return 2.0 * s * acc + (double)e * OG_LN2;
}

/* e^x, |x| < 700: x = k ln2 + r, Taylor series of e^r to 22 terms */
static double og_exp(double x)
{
    const double kd = x / OG_LN2;
    const int k = (int)(kd < 0.0 ? kd - 0.5 : kd + 0.5);
    const double r = x - (double)k * OG_LN2;
    double term = 1.0, sum = 1.0;
    for (int n = 1; n <= 22; ++n) {
        term = term * r / (double)n;
        sum += term;
    }
    uint64_t b;
    memcpy(&b, &sum, 8);
    b += (uint64_t)((int64_t)k) << 52;
    double out;
    memcpy(&out, &b, 8);
    return out;
}

/* sin x: reduced by whole turns to [-pi, pi], Taylor series to r^31 */
static double og_sin(double x)
{
    const double turns = x / OG_TWO_PI;
    const double k = (double)(long long)(turns < 0.0 ? turns - 0.5 : turns + 0.5);
    const double r = x - k * OG_TWO_PI;
    const double r2 = r * r;
    double term = r, sum = 0.0;
    for (int i = 1; i <= 31; i += 2) {
        sum += term;
        term = -term * r2 / (double)((i + 1) * (i + 2));
    }
    return sum;
}

enum {
    OG_TREE = 1, OG_LEN = 2, OG_DX = 3, OG_S0 = 4, OG_N = 5, OG_BW = 6, OG_CS = 7,
    OG_Q1 = 8, OG_Q2 = 9, OG_PHASE = 10, OG_MQ1 = 11, OG_MQ2 = 12, OG_MN = 13
};

static double og_len_mean(double rho, int max_len)
{
    double w = 1.0, sw = 0.0, swk = 0.0;
    for (int k = 1; k <= max_len; ++k) {
        sw += w;
        swk += w * k;
        w *= rho;
    }
    return swk / sw;
}

int oracle_gen_tree(uint64_t seed, int n_leaves, int n_segments, int max_len, int* seg_start, int* seg_len,
                    int* up_ptr, int* up_idx)
{
    if (n_leaves < 1 || max_len < 1) return 1;
    const long long R = 2LL * n_leaves - 1;
    if (R > 0x3FFFFFFF || (long long)n_segments < R || (long long)n_segments > R * (long long)max_len) return 1;
    const int n = (int)R;
    int* parent = (int*)malloc(sizeof(int) * (size_t)n);
    int* c0 = (int*)malloc(sizeof(int) * (size_t)n);
    int* c1 = (int*)malloc(sizeof(int) * (size_t)n);
    int* order = (int*)malloc(sizeof(int) * (size_t)n);
    int* id = (int*)malloc(sizeof(int) * (size_t)n);
    double* cdf = (double*)malloc(sizeof(double) * (size_t)max_len);
    if (!parent || !c0 || !c1 || !order || !id || !cdf) {
        free(parent), free(c0), free(c1), free(order), free(id), free(cdf);
        return 2;
    }
    for (int i = 0; i < n; ++i) parent[i] = c0[i] = c1[i] = -1;

    /* Remy: each new leaf splits the edge above a uniformly chosen node */
    int root = 0, used = 1;
    uint64_t ctr = 0;
    for (int k = 1; k < n_leaves; ++k) {
        const uint64_t h = og_hash(seed, OG_TREE, ctr++);
        const int x = (int)(h % (uint64_t)used);
        const int inner = used, leaf = used + 1;
        used += 2;
        const int p = parent[x];
        if (p < 0) root = inner;
        else if (c0[p] == x) c0[p] = inner;
        else c1[p] = inner;
        parent[inner] = p;
        if ((h >> 63) & 1) { c0[inner] = x; c1[inner] = leaf; }
        else { c0[inner] = leaf; c1[inner] = x; }
        parent[x] = inner;
        parent[leaf] = inner;
    }

    /* ids: the reverse of the breadth-first order from the outlet */
    int tail = 0;
    order[tail++] = root;
    for (int i = 0; i < tail; ++i) {
        const int v = order[i];
        if (c0[v] >= 0) order[tail++] = c0[v];
        if (c1[v] >= 0) order[tail++] = c1[v];
    }
    for (int i = 0; i < n; ++i) id[order[n - 1 - i]] = i;

    up_ptr[0] = 0;
    {
        /* upstream counts by new id, then the CSR rows, ascending ids per row */
        int* cnt = parent; /* reuse: parent[] is no longer needed */
        for (int r = 0; r < n; ++r) cnt[r] = 0;
        for (int v = 0; v < n; ++v)
            if (c0[v] >= 0) cnt[id[v]] = 2;
        for (int r = 0; r < n; ++r) up_ptr[r + 1] = up_ptr[r] + cnt[r];
    }
    for (int v = 0; v < n; ++v) {
        if (c0[v] < 0) continue;
        int a = id[c0[v]], b = id[c1[v]];
        if (a > b) { const int t = a; a = b; b = t; }
        up_idx[up_ptr[id[v]]] = a;
        up_idx[up_ptr[id[v]] + 1] = b;
    }

    /* reach lengths: truncated geometric with the mean segments / reaches */
    const double target = (double)n_segments / (double)n;
    double lo = 1e-6, hi = 1e6;
    for (int it = 0; it < 200; ++it) {
        const double mid = (lo + hi) * 0.5;
        if (og_len_mean(mid, max_len) < target) lo = mid; else hi = mid;
    }
    const double rho = (lo + hi) * 0.5;
    {
        double w = 1.0, sw = 0.0;
        for (int k = 0; k < max_len; ++k) { sw += w; cdf[k] = sw; w *= rho; }
        for (int k = 0; k < max_len; ++k) cdf[k] /= sw;
    }
    long long total = 0;
    for (int r = 0; r < n; ++r) {
        const double u = og_u01(og_hash(seed, OG_LEN, (uint64_t)r));
        int k = 0;
        while (k < max_len - 1 && u > cdf[k]) ++k;
        seg_len[r] = k + 1;
        total += k + 1;
    }
    uint64_t c2 = (uint64_t)n;
    while (total != n_segments) {
        const int r = (int)(og_hash(seed, OG_LEN, c2++) % (uint64_t)n);
        if (total < n_segments && seg_len[r] < max_len) { seg_len[r]++; total++; }
        else if (total > n_segments && seg_len[r] > 1) { seg_len[r]--; total--; }
    }
    int s = 0;
    for (int r = 0; r < n; ++r) { seg_start[r] = s; s += seg_len[r]; }
    free(parent), free(c0), free(c1), free(order), free(id), free(cdf);
    return 0;
}

void oracle_gen_params(uint64_t seed, int n_segments, oracle_chparams* p)
{
    const double ls_lo = og_log(1e-5), ls_hi = og_log(1e-2);
    for (int s = 0; s < n_segments; ++s) {
        const uint64_t c = (uint64_t)s;
        oracle_chparams* q = &p[s];
        q->dx = 500.0 + 4500.0 * og_u01(og_hash(seed, OG_DX, c));
        q->s0 = og_exp(ls_lo + (ls_hi - ls_lo) * og_u01(og_hash(seed, OG_S0, c)));
        q->n_ch = 0.03 + 0.05 * og_u01(og_hash(seed, OG_N, c));
        q->ncc = 2.0 * q->n_ch;
        q->bw = 2.0 + 48.0 * og_u01(og_hash(seed, OG_BW, c));
        q->tw = 3.0 * q->bw;
        q->twcc = 5.0 * q->tw;
        q->cs = 0.5 + 1.5 * og_u01(og_hash(seed, OG_CS, c));
    }
}

typedef struct {
    uint64_t seed;
    int n_segments, t0, k_begin, k_end;
    double dt;
    const double *sphi, *cphi;
    double* qlat;
} og_qlat_job;

static void* og_qlat_rows(void* arg)
{
    const og_qlat_job* J = (const og_qlat_job*)arg;
    const double theta = 0.05;
    for (int k = J->k_begin; k < J->k_end; ++k) {
        const long long t = (long long)J->t0 + k;
        const double a = OG_TWO_PI * ((double)t * J->dt / 86400.0);
        const double sa = og_sin(a), ca = og_sin(a + 0.25 * OG_TWO_PI);
        double* row = J->qlat + (size_t)k * (size_t)J->n_segments;
        for (int s = 0; s < J->n_segments; ++s) {
            const uint64_t c = ((uint64_t)t << 32) | (uint64_t)(uint32_t)s;
            /* Gamma(2, theta) as -theta ln(u1 u2) */
            const double g = -theta * og_log(og_u01(og_hash(J->seed, OG_Q1, c)) * og_u01(og_hash(J->seed, OG_Q2, c)));
            row[s] = g * (1.0 + 0.5 * (sa * J->cphi[s] + ca * J->sphi[s]));
        }
    }
    return NULL;
}

int oracle_gen_qlat(uint64_t seed, int n_segments, int t0, int n_ts, double dt, double* qlat, int n_threads)
{
    if (n_segments <= 0 || n_ts <= 0) return 0;
    double* sphi = (double*)malloc(sizeof(double) * (size_t)n_segments);
    double* cphi = (double*)malloc(sizeof(double) * (size_t)n_segments);
    if (!sphi || !cphi) {
        free(sphi), free(cphi);
        return 2;
    }
    for (int s = 0; s < n_segments; ++s) {
        const double phi = OG_TWO_PI * og_u01(og_hash(seed, OG_PHASE, (uint64_t)s));
        sphi[s] = og_sin(phi);
        cphi[s] = og_sin(phi + 0.25 * OG_TWO_PI);
    }
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n_ts) n_threads = n_ts;
    og_qlat_job* J = (og_qlat_job*)calloc((size_t)n_threads, sizeof(og_qlat_job));
    pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
    if (!J || !th) {
        free(J), free(th), free(sphi), free(cphi);
        return 2;
    }
    const int per = (n_ts + n_threads - 1) / n_threads;
    for (int i = 0; i < n_threads; ++i) {
        J[i] = (og_qlat_job){seed, n_segments, t0, i * per, (i + 1) * per < n_ts ? (i + 1) * per : n_ts, dt,
                             sphi, cphi, qlat};
        if (i > 0 && J[i].k_begin < J[i].k_end) pthread_create(&th[i], NULL, og_qlat_rows, &J[i]);
    }
    og_qlat_rows(&J[0]);
    for (int i = 1; i < n_threads; ++i)
        if (J[i].k_begin < J[i].k_end) pthread_join(th[i], NULL);
    free(J), free(th), free(sphi), free(cphi);
    return 0;
}

void oracle_gen_member(uint64_t seed, int member, int n_segments, double* qfac, double* nfac)
{
    for (int s = 0; s < n_segments; ++s) {
        const uint64_t c = ((uint64_t)(uint32_t)member << 32) | (uint64_t)(uint32_t)s;
        if (qfac) {
            /* Box-Muller normal, then exp(0.3 N) */
            const double u1 = og_u01(og_hash(seed, OG_MQ1, c)), u2 = og_u01(og_hash(seed, OG_MQ2, c));
            const double rr = -2.0 * og_log(u1);
            const double rad = rr > 0.0 ? sqrt(rr) : 0.0;
            const double nrm = rad * og_sin(OG_TWO_PI * u2 + 0.25 * OG_TWO_PI);
            qfac[s] = og_exp(0.3 * nrm);
        }
        if (nfac) nfac[s] = 0.8 + 0.4 * og_u01(og_hash(seed, OG_MN, c));
    }
}

/* Level schedule by the reference's rule (gen_network.py:219-231): headwaters
 * level 0, every other reach 1 + the largest level upstream; reaches listed
 * by level, ascending reach id within a level (a stable sort). level_ptr has
 * room for n_reaches + 1 entries; returns the number of levels. */
int oracle_levels(int n_reaches, const int* up_ptr, const int* up_idx, int* level_ptr, int* level_reach)
{
    const int R = n_reaches;
    if (R <= 0) {
        level_ptr[0] = 0;
        return 0;
    }
    int* level = (int*)calloc((size_t)R, sizeof(int));
    int* down = (int*)malloc(sizeof(int) * (size_t)R);
    int* indeg = (int*)malloc(sizeof(int) * (size_t)R);
    int* queue = (int*)malloc(sizeof(int) * (size_t)R);
    if (!level || !down || !indeg || !queue) {
        free(level), free(down), free(indeg), free(queue);
        return -1;
    }
    for (int r = 0; r < R; ++r) down[r] = -1;
    for (int r = 0; r < R; ++r) {
        indeg[r] = up_ptr[r + 1] - up_ptr[r];
        for (int k = up_ptr[r]; k < up_ptr[r + 1]; ++k) down[up_idx[k]] = r;
    }
    int tail = 0;
    for (int r = 0; r < R; ++r)
        if (indeg[r] == 0) queue[tail++] = r;
    for (int i = 0; i < tail; ++i) {
        const int r = queue[i];
        int lv = 0;
        for (int k = up_ptr[r]; k < up_ptr[r + 1]; ++k)
            if (level[up_idx[k]] + 1 > lv) lv = level[up_idx[k]] + 1;
        level[r] = lv;
        const int d = down[r];
        if (d >= 0 && --indeg[d] == 0) queue[tail++] = d;
    }
    int L = 0;
    for (int r = 0; r < R; ++r)
        if (level[r] + 1 > L) L = level[r] + 1;
    for (int l = 0; l <= L; ++l) level_ptr[l] = 0;
    for (int r = 0; r < R; ++r) level_ptr[level[r] + 1]++;
    for (int l = 0; l < L; ++l) level_ptr[l + 1] += level_ptr[l];
    int* fill = indeg; /* reuse as per-level cursors */
    for (int l = 0; l < L; ++l) fill[l] = level_ptr[l];
    for (int r = 0; r < R; ++r) level_reach[fill[level[r]]++] = r;
    free(level), free(down), free(indeg), free(queue);
    return L;
}
