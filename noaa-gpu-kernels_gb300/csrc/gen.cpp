// Seeded synthetic river networks, channel parameters and lateral inflow.
//
// Every value is a function of (seed, stream, counter) through a counter-based
// hash, and the few transcendental functions needed (log, exp, sin) are
// evaluated here with series built from +,-,*,/ only, so the same seed yields
// the same bits on x86-64 and aarch64 (this file is compiled with
// -ffp-contract=off). The reference's generators are libc rand()
// (troute_mc_final.cu:254-274) and numpy default_rng (wavefront/gen_network.py:
// 66-289); their draws are platform- or library-specific, so the distributions
// here follow the benchmark definitions instead (see troute_gb300.h).
#include "troute_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace tr {

static inline uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t hash3(uint64_t seed, uint64_t stream, uint64_t ctr)
{
    return mix64(mix64(seed ^ mix64(stream * 0xD1B54A32D192ED03ull)) + ctr);
}

// uniform in (0, 1), never 0 or 1
double u01(uint64_t h) { return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

static const double LN2 = 0.69314718055994530942;
static const double TWO_PI = 6.28318530717958647692;

// natural log for x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)),
// log m = 2 atanh(s), s = (m-1)/(m+1), |s| < 0.172.
double det_log(double x)
{
    uint64_t b;
    std::memcpy(&b, &x, 8);
    int e = (int)((b >> 52) & 0x7FF) - 1023;
    b = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;
    double m;
    std::memcpy(&m, &b, 8);
    if (m > 1.4142135623730951) {
        m *= 0.5;
        e += 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    // atanh(s)/s = sum_k s^(2k) / (2k+1), k = 0..11 (|s|^25/25 < 1e-20), Horner
    static const double inv_odd[12] = {1.0 / 1, 1.0 / 3, 1.0 / 5, 1.0 / 7, 1.0 / 9, 1.0 / 11,
                                       1.0 / 13, 1.0 / 15, 1.0 / 17, 1.0 / 19, 1.0 / 21, 1.0 / 23};
    double poly = inv_odd[11];
    for (int k = 10; k >= 0; --k) poly = poly * s2 + inv_odd[k];
    return 2.0 * s * poly + (double)e * LN2;
}

// e^x for |x| < 700: x = k ln2 + r, |r| <= ln2/2, Taylor series of e^r.
double det_exp(double x)
{
    const double kd = x / LN2;
    const int k = (int)(kd < 0.0 ? kd - 0.5 : kd + 0.5);
    const double r = x - (double)k * LN2;
    double term = 1.0, sum = 1.0;
    for (int n = 1; n <= 22; ++n) {
        term = term * r / (double)n;
        sum += term;
    }
    uint64_t b;
    std::memcpy(&b, &sum, 8);
    b += (uint64_t)((int64_t)k) << 52;
    double out;
    std::memcpy(&out, &b, 8);
    return out;
}

// sine, reduced to [-pi, pi] then Taylor series.
double det_sin(double x)
{
    const double n = x / TWO_PI;
    const double k = (double)(long long)(n < 0.0 ? n - 0.5 : n + 0.5);
    const double r = x - k * TWO_PI;
    const double r2 = r * r;
    double term = r, sum = 0.0;
    for (int i = 1; i <= 31; i += 2) {
        sum += term;
        term = -term * r2 / (double)((i + 1) * (i + 2));
    }
    return sum;
}

enum Stream : uint64_t {
    S_TREE = 1, S_LEN = 2, S_DX = 3, S_S0 = 4, S_N = 5, S_BW = 6, S_CS = 7,
    S_Q1 = 8, S_Q2 = 9, S_PHASE = 10, S_MQ1 = 11, S_MQ2 = 12, S_MN = 13
};

}  // namespace tr

using namespace tr;

extern "C" int troute_gen_tree(uint64_t seed, int n_leaves, int n_segments, int max_len,
                               int* reach_seg_start, int* reach_seg_len,
                               int* reach_up_ptr, int* reach_up_idx)
{
    if (n_leaves < 1 || max_len < 1 || !reach_seg_start || !reach_seg_len || !reach_up_ptr ||
        (n_leaves > 1 && !reach_up_idx))
        return set_error(TROUTE_EINVAL, "gen_tree: bad arguments");
    const long long R = 2LL * n_leaves - 1;
    if (R > 0x3FFFFFFF) return set_error(TROUTE_EINVAL, "gen_tree: too many leaves");
    if ((long long)n_segments < R || (long long)n_segments > R * (long long)max_len)
        return set_error(TROUTE_EINVAL, "gen_tree: n_segments must lie in [reaches, reaches*max_len]");
    const int n = (int)R;

    // Remy's algorithm: grow a uniformly random binary tree one leaf at a time
    // by splitting a uniformly chosen node's incoming edge.
    std::vector<int> parent(n, -1), child0(n, -1), child1(n, -1);
    int root = 0, used = 1;
    uint64_t ctr = 0;
    for (int k = 1; k < n_leaves; ++k) {
        const uint64_t hx = hash3(seed, S_TREE, ctr++);
        const int x = (int)(hx % (uint64_t)used);
        const int I = used, L = used + 1;
        used += 2;
        const int p = parent[x];
        if (p < 0)
            root = I;
        else if (child0[p] == x)
            child0[p] = I;
        else
            child1[p] = I;
        parent[I] = p;
        if ((hx >> 63) & 1) {
            child0[I] = x;
            child1[I] = L;
        } else {
            child0[I] = L;
            child1[I] = x;
        }
        parent[x] = I;
        parent[L] = I;
    }

    // Number reaches upstream-first: reverse breadth-first order from the outlet.
    std::vector<int> bfs;
    bfs.reserve(n);
    bfs.push_back(root);
    for (size_t i = 0; i < bfs.size(); ++i) {
        const int v = bfs[i];
        if (child0[v] >= 0) bfs.push_back(child0[v]);
        if (child1[v] >= 0) bfs.push_back(child1[v]);
    }
    std::vector<int> id(n);
    for (int i = 0; i < n; ++i) id[bfs[n - 1 - i]] = i;

    // upstream CSR in the new numbering, ascending ids per reach
    std::vector<int> up_count(n, 0);
    for (int v = 0; v < n; ++v)
        if (child0[v] >= 0) up_count[id[v]] = 2;
    reach_up_ptr[0] = 0;
    for (int r = 0; r < n; ++r) reach_up_ptr[r + 1] = reach_up_ptr[r] + up_count[r];
    for (int v = 0; v < n; ++v) {
        if (child0[v] < 0) continue;
        int a = id[child0[v]], b = id[child1[v]];
        if (a > b) std::swap(a, b);
        reach_up_idx[reach_up_ptr[id[v]]] = a;
        reach_up_idx[reach_up_ptr[id[v]] + 1] = b;
    }

    // Segments per reach: truncated geometric on 1..max_len with the ratio
    // chosen (bisection) so the mean is n_segments / reaches, then adjusted to
    // the exact total.
    const double target = (double)n_segments / (double)n;
    auto mean_of = [&](double rho) {
        double w = 1.0, sw = 0.0, swk = 0.0;
        for (int k = 1; k <= max_len; ++k) {
            sw += w;
            swk += w * k;
            w *= rho;
        }
        return swk / sw;
    };
    double lo = 1e-6, hi = 1e6;
    for (int it = 0; it < 200; ++it) {
        const double mid = (lo + hi) * 0.5;
        if (mean_of(mid) < target) lo = mid; else hi = mid;
    }
    const double rho = (lo + hi) * 0.5;
    std::vector<double> cdf(max_len);
    {
        double w = 1.0, sw = 0.0;
        for (int k = 0; k < max_len; ++k) { sw += w; cdf[k] = sw; w *= rho; }
        for (int k = 0; k < max_len; ++k) cdf[k] /= sw;
    }
    long long total = 0;
    for (int r = 0; r < n; ++r) {
        const double u = u01(hash3(seed, S_LEN, (uint64_t)r));
        int k = 0;
        while (k < max_len - 1 && u > cdf[k]) ++k;
        reach_seg_len[r] = k + 1;
        total += k + 1;
    }
    uint64_t c2 = (uint64_t)n;
    while (total != n_segments) {
        const int r = (int)(hash3(seed, S_LEN, c2++) % (uint64_t)n);
        if (total < n_segments && reach_seg_len[r] < max_len) { reach_seg_len[r]++; total++; }
        else if (total > n_segments && reach_seg_len[r] > 1) { reach_seg_len[r]--; total--; }
    }
    int s = 0;
    for (int r = 0; r < n; ++r) { reach_seg_start[r] = s; s += reach_seg_len[r]; }
    return TROUTE_OK;
}

extern "C" int troute_gen_params(uint64_t seed, int n_segments, troute_chparams* p)
{
    if (n_segments < 0 || (n_segments > 0 && !p)) return set_error(TROUTE_EINVAL, "gen_params: bad arguments");
    const double ls_lo = det_log(1e-5), ls_hi = det_log(1e-2);
    for (int s = 0; s < n_segments; ++s) {
        const uint64_t c = (uint64_t)s;
        troute_chparams& q = p[s];
        q.dx = 500.0 + 4500.0 * u01(hash3(seed, S_DX, c));
        q.s0 = det_exp(ls_lo + (ls_hi - ls_lo) * u01(hash3(seed, S_S0, c)));
        q.n_ch = 0.03 + 0.05 * u01(hash3(seed, S_N, c));
        q.ncc = 2.0 * q.n_ch;
        q.bw = 2.0 + 48.0 * u01(hash3(seed, S_BW, c));
        q.tw = 3.0 * q.bw;
        q.twcc = 5.0 * q.tw;
        q.cs = 0.5 + 1.5 * u01(hash3(seed, S_CS, c));
    }
    return TROUTE_OK;
}

extern "C" int troute_gen_qlat(uint64_t seed, int n_segments, int t0, int n_ts, double dt,
                               double* qlat)
{
    if (n_segments < 0 || n_ts < 0 || t0 < 0 || (n_segments > 0 && n_ts > 0 && !qlat))
        return set_error(TROUTE_EINVAL, "gen_qlat: bad arguments");
    if (n_segments == 0 || n_ts == 0) return TROUTE_OK;
    // sin(a_t + phi_s) = sin a_t cos phi_s + cos a_t sin phi_s
    std::vector<double> sphi(n_segments), cphi(n_segments);
    for (int s = 0; s < n_segments; ++s) {
        const double phi = TWO_PI * u01(hash3(seed, S_PHASE, (uint64_t)s));
        sphi[s] = det_sin(phi);
        cphi[s] = det_sin(phi + 0.25 * TWO_PI);
    }
    const double theta = 0.05;
    auto work = [&](long long cell_begin, long long cell_end) {
        for (long long cell = cell_begin; cell < cell_end;) {
            const int k = (int)(cell / n_segments);
            const int s_begin = (int)(cell % n_segments);
            const int s_end = (int)std::min<long long>(n_segments, s_begin + (cell_end - cell));
            cell += s_end - s_begin;
            const long long t = (long long)t0 + k;
            const double a = TWO_PI * ((double)t * dt / 86400.0);
            const double sa = det_sin(a), ca = det_sin(a + 0.25 * TWO_PI);
            double* row = qlat + (size_t)k * (size_t)n_segments;
            for (int s = s_begin; s < s_end; ++s) {
                const uint64_t c = ((uint64_t)t << 32) | (uint64_t)(uint32_t)s;
                // Gamma(2, theta) = -theta ln(u1 u2), u1, u2 ~ U(0,1) independent
                const double g = -theta * det_log(u01(hash3(seed, S_Q1, c)) * u01(hash3(seed, S_Q2, c)));
                row[s] = g * (1.0 + 0.5 * (sa * cphi[s] + ca * sphi[s]));
            }
        }
    };
    const long long cells = (long long)n_segments * n_ts;
    const int nth = (int)std::min<long long>(std::max(1u, std::thread::hardware_concurrency()),
                                             std::max<long long>(1, cells / 200000));
    if (nth <= 1) {
        work(0, cells);
    } else {
        std::vector<std::thread> th;
        const long long per = (cells + nth - 1) / nth;
        for (int i = 0; i < nth; ++i) {
            const long long b = i * per, e = std::min(cells, b + per);
            if (b < e) th.emplace_back(work, b, e);
        }
        for (auto& x : th) x.join();
    }
    return TROUTE_OK;
}

extern "C" int troute_gen_member(uint64_t seed, int member, int n_segments, double* qfac,
                                 double* nfac)
{
    if (n_segments < 0 || member < 0) return set_error(TROUTE_EINVAL, "gen_member: bad arguments");
    for (int s = 0; s < n_segments; ++s) {
        const uint64_t c = ((uint64_t)(uint32_t)member << 32) | (uint64_t)(uint32_t)s;
        if (qfac) {
            // Box-Muller normal, then exp(0.3 N)
            const double u1 = u01(hash3(seed, S_MQ1, c)), u2 = u01(hash3(seed, S_MQ2, c));
            double rr = -2.0 * det_log(u1);
            const double rad = rr > 0.0 ? std::sqrt(rr) : 0.0;  // IEEE, correctly rounded
            const double nrm = rad * det_sin(TWO_PI * u2 + 0.25 * TWO_PI);
            qfac[s] = det_exp(0.3 * nrm);
        }
        if (nfac) nfac[s] = 0.8 + 0.4 * u01(hash3(seed, S_MN, c));
    }
    return TROUTE_OK;
}
