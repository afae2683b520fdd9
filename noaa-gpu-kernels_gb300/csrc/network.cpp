// Host side of the tree-routing path: topology checks, the device schedule
// (ALAP levels, level-blocks, segment tiles), the persistent handle and its
// run / state / checkpoint / graph entry points.
//
// Layout in HBM (internal order, built once per handle):
//   - reaches of one ALAP level are sorted by segment count (longest first)
//     and cut into level-blocks of 32; internal reach id = block*32 + lane, so
//     every per-reach array (segment count, upstream CSR row, readiness
//     counter, outflow ring) is read coalesced by a warp working on a block;
//   - segment i of lane k of block b lives at tile_off[b] + 32*i + k, so the
//     warp's loads of "segment i of every reach" are one 256-byte line per
//     double plane; a segment's parameters, inflow column and inflow scale
//     are one 128-byte record (SegRec: one L2 line per solve, whatever the
//     order in which the per-lane kernels take (reach, step) items);
//   - q, depth, velocity: one double plane each, updated in place each step;
//   - reach outflow: a [4][reaches] ring indexed by step % 4.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <array>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "troute_internal.h"

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

extern "C" const char* troute_last_error(void) { return g_last_error.c_str(); }

extern "C" void troute_cfg_default(troute_cfg* cfg)
{
    if (!cfg) return;
    std::memset(cfg, 0, sizeof *cfg);
    cfg->rtol = 0.01;
    cfg->atol = 0.01;
    cfg->maxiter = 100;
    cfg->attempts = 5;
    cfg->warm_k = 16;
}

namespace tr {

int check_cfg(const troute_cfg& c)
{
    if (!(c.rtol > 0.0 && c.rtol < 1.0)) return set_error(TROUTE_EINVAL, "cfg.rtol must be in (0, 1)");
    if (!(c.atol >= 0.0 && c.atol < 1.0)) return set_error(TROUTE_EINVAL, "cfg.atol must be in [0, 1)");
    if (c.maxiter < 1 || c.maxiter > 100000) return set_error(TROUTE_EINVAL, "cfg.maxiter out of range");
    if (c.attempts < 1 || c.attempts > 64) return set_error(TROUTE_EINVAL, "cfg.attempts out of range");
    if (c.threads_per_block != 0 && (c.threads_per_block % 32 != 0 || c.threads_per_block > 128))
        return set_error(TROUTE_EINVAL, "cfg.threads_per_block must be a multiple of 32, at most 128");
    if (c.blocks_per_sm < 0 || c.wait_cycles < 0) return set_error(TROUTE_EINVAL, "negative cfg field");
    if (c.mapping < 0 || c.mapping > 3) return set_error(TROUTE_EINVAL, "cfg.mapping must be 0..3");
    if (c.warm_start && c.mapping != 0 && c.mapping != 3)
        return set_error(TROUTE_EINVAL, "cfg.warm_start needs mapping 3 (the ready-queue kernel)");
    if (c.warm_start && (c.warm_k < 1 || c.warm_k > 100000)) return set_error(TROUTE_EINVAL, "cfg.warm_k out of range");
    return TROUTE_OK;
}

// atol + 0.0 turns a -0 tolerance into +0 (the same stop test; the device's
// integer-pipe comparison expects a non-negative tolerance of either sign bit 0)
Tol make_tol(const troute_cfg& c) { return Tol{c.rtol, c.atol + 0.0, c.maxiter, c.attempts}; }

int cuda_check(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return TROUTE_OK;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return set_error(TROUTE_ENODEV, "%s: %s", what, cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) return set_error(TROUTE_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
    return set_error(TROUTE_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Topology as the library sees it: a forest over all networks of a handle.
struct Forest {
    int R = 0, S = 0;
    std::vector<int> seg_start, seg_len, up_ptr, up_idx;
};

// Validates a forest; fills down[] (downstream reach or -1) and a
// topological order (upstream first).
int validate_forest(const Forest& f, std::vector<int>& down, std::vector<int>& order)
{
    const int R = f.R, S = f.S;
    if (R < 0 || S < 0) return set_error(TROUTE_ETOPO, "negative sizes");
    if ((int)f.up_ptr.size() != R + 1 || f.up_ptr[0] != 0)
        return set_error(TROUTE_ETOPO, "reach_up_ptr must have n_reaches+1 entries starting at 0");
    for (int r = 0; r < R; ++r)
        if (f.up_ptr[r + 1] < f.up_ptr[r]) return set_error(TROUTE_ETOPO, "reach_up_ptr not monotone at reach %d", r);
    if ((size_t)f.up_ptr[R] != f.up_idx.size()) return set_error(TROUTE_ETOPO, "reach_up_idx size mismatch");
    std::vector<unsigned char> covered((size_t)S, 0);
    for (int r = 0; r < R; ++r) {
        const long long a = f.seg_start[r], n = f.seg_len[r];
        if (n < 0 || a < 0 || a + n > S)
            return set_error(TROUTE_ETOPO, "reach %d segments [%lld, %lld) outside [0, %d)", r, a, a + n, S);
        for (long long s = a; s < a + n; ++s) {
            if (covered[s]) return set_error(TROUTE_ETOPO, "segment %lld belongs to two reaches", s);
            covered[s] = 1;
        }
    }
    down.assign(R, -1);
    for (int r = 0; r < R; ++r)
        for (int k = f.up_ptr[r]; k < f.up_ptr[r + 1]; ++k) {
            const int u = f.up_idx[k];
            if (u < 0 || u >= R) return set_error(TROUTE_ETOPO, "upstream index %d of reach %d out of range", u, r);
            if (u == r) return set_error(TROUTE_ETOPO, "reach %d drains into itself", r);
            if (down[u] >= 0)
                return set_error(TROUTE_ETOPO, "reach %d drains into two reaches (%d and %d)", u, down[u], r);
            down[u] = r;
        }
    // Kahn: in-degree = number of upstream reaches
    std::vector<int> indeg(R);
    for (int r = 0; r < R; ++r) indeg[r] = f.up_ptr[r + 1] - f.up_ptr[r];
    order.clear();
    order.reserve(R);
    for (int r = 0; r < R; ++r)
        if (indeg[r] == 0) order.push_back(r);
    for (size_t i = 0; i < order.size(); ++i) {
        const int d = down[order[i]];
        if (d >= 0 && --indeg[d] == 0) order.push_back(d);
    }
    if ((int)order.size() != R) return set_error(TROUTE_ETOPO, "topology has a cycle");
    return TROUTE_OK;
}

}  // namespace tr

using namespace tr;

// ---------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------
template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        if (count <= n && p) return TROUTE_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (count == 0) return TROUTE_OK;
        const int rc = cuda_check(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
        if (rc == TROUTE_OK) n = count;
        return rc;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct troute_handle {
    troute_cfg cfg;
    double dt = 300.0;
    int R_user = 0, S_user = 0, qlat_cols = 0;
    int n_levels = 0, n_blocks = 0, R_int = 0;
    long long S_int = 0;
    std::vector<int> lb_ptr;           // host copy
    std::vector<long long> seg_map;    // user segment -> internal slot (-1 none)
    std::vector<long long> reach_map;  // user reach -> internal reach
    std::vector<int> user_seg_start, user_seg_len;
    long long steps_done = 0;
    bool broken = false;

    DBuf<SegRec> seg;
    DBuf<int> nseg, block_level, lb_ptr_d, up_ptr, up_idx, down, done, step_base;
    DBuf<double> q, d, v, ring, tmp, qlat_buf, hist;
    DBuf<long long> tile_off, seg_map_d, reach_map_d;
    DBuf<unsigned long long> wave_ptr, wave_ptr_tail, ticket, rq_ctr;
    unsigned long long n_tickets = 0, n_tickets_tail = 0;
    size_t chunk_budget_bytes = 0;
    DBuf<int> df_cnt;
    DBuf<int2> df_rq, df_heads;
    DBuf<double> df_rh;
    int n_heads = 0, R_real = 0;
    DBuf<DevStats> stats;
    int hist_ts = 0;
    // learned warm start and its training data
    const troute_warm* warm_model = nullptr;
    double warm_delta = 0.05;
    DBuf<float> pairs;        // [n_ts][S_int][9]
    DBuf<double> start_hist;  // [n_ts][S_int]
    DBuf<float> pred;         // [chunk][S_int] learned starting depths of a warm-started launch
    int pairs_ts = 0, start_ts = 0;

    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int grid = 0, threads = 128, mapping = 2, n_sms = 1;
    int last_n_ts = 0;

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_n_ts = 0;

    NetDev net() const
    {
        NetDev n;
        n.n_blocks = n_blocks;
        n.n_levels = n_levels;
        n.n_reach_int = R_int;
        n.n_seg_int = S_int;
        n.seg = seg.p;
        n.nseg = nseg.p;
        n.tile_off = tile_off.p;
        n.block_level = block_level.p;
        n.lb_ptr = lb_ptr_d.p;
        n.up_ptr = up_ptr.p;
        n.up_idx = up_idx.p;
        n.down = down.p;
        n.q = q.p;
        n.d = d.p;
        n.v = v.p;
        n.ring = ring.p;
        n.done = done.p;
        return n;
    }

    ~troute_handle()
    {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (graph) cudaGraphDestroy(graph);
        seg.release();
        nseg.release(); block_level.release(); lb_ptr_d.release();
        up_ptr.release(); up_idx.release(); down.release(); done.release(); step_base.release();
        q.release(); d.release(); v.release(); ring.release(); tmp.release();
        qlat_buf.release(); hist.release(); tile_off.release(); seg_map_d.release();
        reach_map_d.release(); wave_ptr.release(); wave_ptr_tail.release(); ticket.release(); stats.release();
        rq_ctr.release(); df_cnt.release(); df_rq.release(); df_heads.release(); df_rh.release();
        pairs.release(); start_hist.release(); pred.release();
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
};

template <typename T>
static int upload(DBuf<T>& b, const std::vector<T>& h, cudaStream_t s)
{
    int rc = b.alloc(h.size());
    if (rc) return rc;
    if (h.empty()) return TROUTE_OK;
    return cuda_check(cudaMemcpyAsync(b.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s),
                      "upload");
}

// Persistent grid sized by occupancy: SMs x resident blocks per SM (capped by
// cfg.blocks_per_sm). Mapping 2 (per-lane refill) always runs 128-thread blocks.
static int launch_shape(troute_handle* H)
{
    int rc, dev = 0, sms = 0, bps = 0;
    if ((rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice"))) return rc;
    if ((rc = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr"))) return rc;
    H->mapping = H->cfg.mapping ? H->cfg.mapping : 3;
    if (H->mapping == 3) {
        H->threads = route_dataflow_threads();
        if ((rc = route_dataflow_occupancy(&bps, H->cfg.warm_start != 0))) return rc;
    } else if (H->mapping == 2) {
        H->threads = 128;
        if ((rc = route_pool_occupancy(&bps))) return rc;
    } else {
        H->threads = H->cfg.threads_per_block ? H->cfg.threads_per_block : 128;
        if ((rc = route_occupancy(H->threads, &bps))) return rc;
    }
    if (H->cfg.blocks_per_sm > 0) bps = std::min(bps, H->cfg.blocks_per_sm);
    H->n_sms = std::max(1, sms);
    H->grid = std::max(1, sms * std::max(1, bps));
    return TROUTE_OK;
}

// Host image of everything a handle uploads (internal order).
struct Layout {
    int R_user = 0, S_user = 0, n_levels = 0, NB = 0, R_int = 0, n_heads = 0, R_real = 0;
    long long S_int = 0;  // tiles + 1 trash slot
    std::vector<int> user_seg_start, user_seg_len;
    std::vector<int> lb_ptr, block_level, nseg, up_ptr, up_idx, down_i;
    std::vector<long long> tile_off, seg_map, reach_map;  // seg_map: -1 for uncovered segments
    std::vector<int2> heads;
    std::vector<SegRec> recs;    // parameters, inflow column and scale per tile slot
};

// A tile slot's record: derived parameters, inflow column, inflow scale.
static void put_params(Layout& Lt, long long t, const troute_chparams& c, int qcol, double qscale)
{
    const SegP p = derive_seg(c);
    SegRec& r = Lt.recs[(size_t)t];
    r.p[0] = double2{p.dx, p.bw};
    r.p[1] = double2{p.twcc, p.n_ch};
    r.p[2] = double2{p.ncc, p.s0};
    r.p[3] = double2{p.z, p.bfd};
    r.p[4] = double2{p.sq_s0, p.sq2};
    r.p[5] = double2{p.ck_fac, p.z2};
    r.qcol = qcol;
    r.qscale = qscale;
}

static SegRec empty_rec()
{
    SegRec r;
    std::memset(&r, 0, sizeof r);
    r.qscale = 1.0;
    r.reach = -1;
    return r;
}

// Schedule and layout of a forest (ALAP levels, level-blocks, tiles).
static int build_layout(const Forest& f, const std::vector<troute_chparams>& params,
                        const std::vector<int>& qcol_user, const std::vector<double>& qscale_user,
                        bool has_scale, Layout& Lt)
{
    std::vector<int> down, order;
    int rc = validate_forest(f, down, order);
    if (rc) return rc;
    const int R = f.R;
    Lt.R_user = R;
    Lt.S_user = f.S;
    Lt.R_real = R;
    Lt.user_seg_start = f.seg_start;
    Lt.user_seg_len = f.seg_len;

    // ALAP level: distance to the outlet, counted down from the deepest level.
    std::vector<int> dist(R, 0);
    int maxd = 0;
    for (int i = R - 1; i >= 0; --i) {
        const int r = order[i];
        dist[r] = (down[r] >= 0) ? dist[down[r]] + 1 : 0;
        maxd = std::max(maxd, dist[r]);
    }
    const int L = (R > 0) ? maxd + 1 : 0;
    Lt.n_levels = L;
    std::vector<std::vector<int>> by_level(L);
    for (int r = 0; r < R; ++r) by_level[L - 1 - dist[r]].push_back(r);
    Lt.lb_ptr.assign(L + 1, 0);
    std::vector<std::vector<int>> blocks;
    for (int l = 0; l < L; ++l) {
        auto& v = by_level[l];
        std::stable_sort(v.begin(), v.end(), [&](int a, int b) { return f.seg_len[a] > f.seg_len[b]; });
        for (size_t i = 0; i < v.size(); i += kLanes) {
            blocks.emplace_back(v.begin() + i, v.begin() + std::min(v.size(), i + kLanes));
            Lt.block_level.push_back(l);
        }
        Lt.lb_ptr[l + 1] = (int)blocks.size();
    }
    const int NB = (int)blocks.size();
    Lt.NB = NB;
    Lt.R_int = NB * kLanes;

    Lt.tile_off.assign(NB, 0);
    long long S_int = 0;
    Lt.reach_map.assign(R, -1);
    Lt.seg_map.assign(f.S, -1);
    Lt.nseg.assign(Lt.R_int, -1);
    for (int b = 0; b < NB; ++b) {
        Lt.tile_off[b] = S_int;
        int hmax = 0;
        for (size_t k = 0; k < blocks[b].size(); ++k) {
            const int r = blocks[b][k];
            const int ri = b * kLanes + (int)k;
            Lt.reach_map[r] = ri;
            Lt.nseg[ri] = f.seg_len[r];
            hmax = std::max(hmax, f.seg_len[r]);
            for (int i = 0; i < f.seg_len[r]; ++i)
                Lt.seg_map[f.seg_start[r] + i] = S_int + (long long)i * kLanes + (long long)k;
        }
        S_int += (long long)hmax * kLanes;
    }
    // one extra slot at the end: the target of segments no reach covers, so
    // scatter/gather through the segment map never leave the arrays
    Lt.S_int = S_int + 1;

    // upstream CSR over internal ids, keeping each reach's upstream order
    // (the order of the floating-point sum at the reach head)
    Lt.up_ptr.assign(Lt.R_int + 1, 0);
    Lt.down_i.assign(Lt.R_int, -1);
    Lt.up_idx.reserve(f.up_idx.size());
    {
        std::vector<int> user_of(Lt.R_int, -1);
        for (int r = 0; r < R; ++r) user_of[Lt.reach_map[r]] = r;
        for (int ri = 0; ri < Lt.R_int; ++ri) {
            const int r = user_of[ri];
            if (r >= 0) {
                for (int k = f.up_ptr[r]; k < f.up_ptr[r + 1]; ++k)
                    Lt.up_idx.push_back((int)Lt.reach_map[f.up_idx[k]]);
                if (down[r] >= 0) Lt.down_i[ri] = (int)Lt.reach_map[down[r]];
            }
            Lt.up_ptr[ri + 1] = (int)Lt.up_idx.size();
        }
    }
    // items ready at the start of a run: reaches without upstream reaches, step 0
    for (int ri = 0; ri < Lt.R_int; ++ri)
        if (Lt.nseg[ri] >= 0 && Lt.up_ptr[ri + 1] == Lt.up_ptr[ri]) Lt.heads.push_back(int2{ri, 0});
    Lt.n_heads = (int)Lt.heads.size();

    // parameters in tile order
    Lt.recs.assign((size_t)Lt.S_int, empty_rec());
    for (int s = 0; s < f.S; ++s) {
        const long long t = Lt.seg_map[s];
        if (t < 0) continue;
        put_params(Lt, t, params[s], qcol_user[s], has_scale ? qscale_user[s] : 1.0);
    }
    for (int r = 0; r < R; ++r)
        for (int i = 0; i < f.seg_len[r]; ++i) {
            const long long t = Lt.seg_map[f.seg_start[r] + i];
            Lt.recs[(size_t)t].reach = (int)Lt.reach_map[r];
            Lt.recs[(size_t)t].pos = i;
        }
    return TROUTE_OK;
}

// Layout of M copies of one network (ensemble members): same topology and
// schedule, member m's Manning's n (channel and floodplain) scaled by
// n_scale[m][s] and its lateral inflow by q_scale[m][s] (NULL: 1). Blocks are
// ordered level by level (members of one level together), tiles member-major.
static void replicate_layout(const Layout& B, const std::vector<troute_chparams>& params, int M,
                             const double* n_scale, const double* q_scale, Layout& E)
{
    const long long tiles = B.S_int - 1;
    const int S = B.S_user, R = B.R_user, L = B.n_levels;
    E.R_user = R * M;
    E.S_user = S * M;
    E.R_real = B.R_real * M;
    E.n_levels = L;
    E.NB = B.NB * M;
    E.R_int = E.NB * kLanes;
    E.S_int = tiles * M + 1;
    E.user_seg_start.resize((size_t)E.R_user);
    E.user_seg_len.resize((size_t)E.R_user);
    for (int m = 0; m < M; ++m)
        for (int r = 0; r < R; ++r) {
            E.user_seg_start[(size_t)m * R + r] = B.user_seg_start[r] + m * S;
            E.user_seg_len[(size_t)m * R + r] = B.user_seg_len[r];
        }
    // block b of level l, member m -> M*lb_ptr[l] + m*nb_l + (b - lb_ptr[l])
    std::vector<int> new_block((size_t)B.NB * M);
    E.lb_ptr.assign(L + 1, 0);
    E.block_level.resize((size_t)E.NB);
    for (int l = 0; l < L; ++l) {
        const int b0 = B.lb_ptr[l], nb = B.lb_ptr[l + 1] - b0;
        E.lb_ptr[l + 1] = M * B.lb_ptr[l + 1];
        for (int m = 0; m < M; ++m)
            for (int j = 0; j < nb; ++j) {
                const int nbk = M * b0 + m * nb + j;
                new_block[(size_t)m * B.NB + b0 + j] = nbk;
                E.block_level[nbk] = l;
            }
    }
    auto new_reach = [&](int m, int ri) { return new_block[(size_t)m * B.NB + ri / kLanes] * kLanes + ri % kLanes; };
    E.tile_off.assign((size_t)E.NB, 0);
    E.nseg.assign((size_t)E.R_int, -1);
    E.down_i.assign((size_t)E.R_int, -1);
    std::vector<int> up_cnt((size_t)E.R_int, 0);
    for (int m = 0; m < M; ++m)
        for (int b = 0; b < B.NB; ++b) {
            E.tile_off[new_block[(size_t)m * B.NB + b]] = B.tile_off[b] + (long long)m * tiles;
            for (int k = 0; k < kLanes; ++k) {
                const int ri = b * kLanes + k, ni = new_reach(m, ri);
                E.nseg[ni] = B.nseg[ri];
                E.down_i[ni] = B.down_i[ri] >= 0 ? new_reach(m, B.down_i[ri]) : -1;
                up_cnt[ni] = B.up_ptr[ri + 1] - B.up_ptr[ri];
            }
        }
    E.up_ptr.assign((size_t)E.R_int + 1, 0);
    for (int ri = 0; ri < E.R_int; ++ri) E.up_ptr[ri + 1] = E.up_ptr[ri] + up_cnt[ri];
    E.up_idx.assign((size_t)E.up_ptr[E.R_int], 0);
    for (int m = 0; m < M; ++m)
        for (int ri = 0; ri < B.R_int; ++ri) {
            const int ni = new_reach(m, ri);
            for (int k = B.up_ptr[ri]; k < B.up_ptr[ri + 1]; ++k)
                E.up_idx[E.up_ptr[ni] + (k - B.up_ptr[ri])] = new_reach(m, B.up_idx[k]);
        }
    for (int m = 0; m < M; ++m)
        for (const int2& h : B.heads) E.heads.push_back(int2{new_reach(m, h.x), 0});
    E.n_heads = (int)E.heads.size();
    E.reach_map.resize((size_t)E.R_user);
    E.seg_map.resize((size_t)E.S_user);
    for (int m = 0; m < M; ++m) {
        for (int r = 0; r < R; ++r) E.reach_map[(size_t)m * R + r] = new_reach(m, (int)B.reach_map[r]);
        for (int s = 0; s < S; ++s)
            E.seg_map[(size_t)m * S + s] = B.seg_map[s] < 0 ? -1 : B.seg_map[s] + (long long)m * tiles;
    }
    E.recs.assign((size_t)E.S_int, empty_rec());
    for (int m = 0; m < M; ++m)
        for (int s = 0; s < S; ++s) {
            const long long bt = B.seg_map[s];
            if (bt < 0) continue;
            const long long t = bt + (long long)m * tiles;
            troute_chparams c = params[s];
            if (n_scale) {
                const double f = n_scale[(size_t)m * S + s];
                c.n_ch *= f;
                c.ncc *= f;
            }
            put_params(E, t, c, B.recs[(size_t)bt].qcol, q_scale ? q_scale[(size_t)m * S + s] : B.recs[(size_t)bt].qscale);
            E.recs[(size_t)t].reach = B.recs[(size_t)bt].reach >= 0 ? new_reach(m, B.recs[(size_t)bt].reach) : -1;
            E.recs[(size_t)t].pos = B.recs[(size_t)bt].pos;
        }
}

// Uploads a layout into a handle and allocates its state.
static int upload_layout(troute_handle* H, Layout& Lt)
{
    int rc;
    H->R_user = Lt.R_user;
    H->S_user = Lt.S_user;
    H->R_real = Lt.R_real;
    H->user_seg_start = std::move(Lt.user_seg_start);
    H->user_seg_len = std::move(Lt.user_seg_len);
    H->n_levels = Lt.n_levels;
    H->n_blocks = Lt.NB;
    H->R_int = Lt.R_int;
    H->S_int = Lt.S_int;
    H->lb_ptr = Lt.lb_ptr;
    H->n_heads = Lt.n_heads;
    H->seg_map = Lt.seg_map;
    H->reach_map = Lt.reach_map;
    const long long trash = Lt.S_int - 1;
    std::vector<long long> seg_map_dev(std::move(Lt.seg_map));
    for (auto& m : seg_map_dev)
        if (m < 0) m = trash;

    cudaStream_t st = H->stream;
    if ((rc = upload(H->seg, Lt.recs, st))) return rc;
    if ((rc = cuda_check(cudaStreamSynchronize(st), "upload"))) return rc;
    std::vector<SegRec>().swap(Lt.recs);
    if ((rc = upload(H->nseg, Lt.nseg, st))) return rc;
    if ((rc = upload(H->tile_off, Lt.tile_off, st))) return rc;
    if ((rc = upload(H->block_level, Lt.block_level, st))) return rc;
    if ((rc = upload(H->lb_ptr_d, Lt.lb_ptr, st))) return rc;
    if ((rc = upload(H->up_ptr, Lt.up_ptr, st))) return rc;
    if ((rc = upload(H->up_idx, Lt.up_idx.empty() ? std::vector<int>{0} : Lt.up_idx, st))) return rc;
    if ((rc = upload(H->down, Lt.down_i, st))) return rc;
    if ((rc = upload(H->df_heads, Lt.heads.empty() ? std::vector<int2>{int2{0, 0}} : Lt.heads, st))) return rc;
    if ((rc = upload(H->seg_map_d, seg_map_dev.empty() ? std::vector<long long>{trash} : seg_map_dev, st))) return rc;
    if ((rc = upload(H->reach_map_d, H->reach_map.empty() ? std::vector<long long>{0} : H->reach_map, st))) return rc;
    if ((rc = cuda_check(cudaStreamSynchronize(st), "upload"))) return rc;
    if ((rc = H->q.alloc(H->S_int)) || (rc = H->d.alloc(H->S_int)) || (rc = H->v.alloc(H->S_int))) return rc;
    if ((rc = H->ring.alloc((size_t)kRing * std::max(1, H->R_int)))) return rc;
    if ((rc = H->done.alloc(std::max(1, H->R_int))) || (rc = H->step_base.alloc(1))) return rc;
    if ((rc = H->ticket.alloc(1)) || (rc = H->stats.alloc(1))) return rc;
    if ((rc = H->tmp.alloc(std::max<size_t>(std::max(H->S_user, H->R_user), 1)))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(H->q.p, 0, H->S_int * sizeof(double), st), "memset"))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(H->d.p, 0, H->S_int * sizeof(double), st), "memset"))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(H->v.p, 0, H->S_int * sizeof(double), st), "memset"))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(H->ring.p, 0, H->ring.n * sizeof(double), st), "memset"))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(H->done.p, 0, H->done.n * sizeof(int), st), "memset"))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(H->step_base.p, 0, sizeof(int), st), "memset"))) return rc;
    if ((rc = launch_shape(H))) return rc;
    return cuda_check(cudaStreamSynchronize(st), "build sync");
}

static int build_handle(troute_handle* H, const Forest& f, const std::vector<troute_chparams>& params,
                        const std::vector<int>& qcol_user, const std::vector<double>& qscale_user,
                        bool has_scale)
{
    Layout Lt;
    int rc = build_layout(f, params, qcol_user, qscale_user, has_scale, Lt);
    if (rc) return rc;
    return upload_layout(H, Lt);
}

static int new_handle(troute_handle** out, double dt, const troute_cfg* cfg)
{
    if (!out) return set_error(TROUTE_EINVAL, "null handle pointer");
    *out = nullptr;
    if (!(dt > 0.0)) return set_error(TROUTE_EINVAL, "dt must be positive");
    troute_cfg c;
    troute_cfg_default(&c);
    if (cfg) c = *cfg;
    int rc = check_cfg(c);
    if (rc) return rc;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device: %s", cudaGetErrorString(e));
    auto* H = new (std::nothrow) troute_handle();
    if (!H) return set_error(TROUTE_ENOMEM, "handle allocation");
    H->cfg = c;
    H->dt = dt;
    if ((rc = cuda_check(cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking), "stream"))) { delete H; return rc; }
    if ((rc = cuda_check(cudaEventCreate(&H->ev0), "event")) || (rc = cuda_check(cudaEventCreate(&H->ev1), "event"))) {
        delete H;
        return rc;
    }
    *out = H;
    return TROUTE_OK;
}

static bool append_topo(Forest& f, const troute_topo& t)
{
    if (t.n_reaches < 0 || t.n_segments < 0) return false;
    if (t.n_reaches > 0 && (!t.reach_seg_start || !t.reach_seg_len || !t.reach_up_ptr)) return false;
    const int r0 = f.R, s0 = f.S;
    if (f.up_ptr.empty()) f.up_ptr.push_back(0);
    const int base = f.up_ptr.back();
    const int nnz = t.n_reaches > 0 ? t.reach_up_ptr[t.n_reaches] - t.reach_up_ptr[0] : 0;
    if (nnz < 0 || (nnz > 0 && !t.reach_up_idx)) return false;
    for (int r = 0; r < t.n_reaches; ++r) {
        f.seg_start.push_back(t.reach_seg_start[r] + s0);
        f.seg_len.push_back(t.reach_seg_len[r]);
        f.up_ptr.push_back(base + t.reach_up_ptr[r + 1] - t.reach_up_ptr[0]);
    }
    for (int k = 0; k < nnz; ++k) {
        const int u = t.reach_up_idx[t.reach_up_ptr[0] + k];
        f.up_idx.push_back((u >= 0 && u < t.n_reaches) ? u + r0 : -1 - std::abs(u));
    }
    f.R += t.n_reaches;
    f.S += t.n_segments;
    return true;
}

extern "C" int troute_create_batch(troute_handle** h, int n_nets, const troute_topo* topos,
                                   const troute_chparams* const* params,
                                   const int* const* qlat_col, const double* const* qlat_scale,
                                   int qlat_cols, double dt, const troute_cfg* cfg)
{
    if (n_nets < 1 || !topos || !params) return set_error(TROUTE_EINVAL, "batch needs n_nets >= 1, topos and params");
    Forest f;
    f.up_ptr.push_back(0);
    for (int i = 0; i < n_nets; ++i) {
        if (!append_topo(f, topos[i])) return set_error(TROUTE_ETOPO, "network %d: malformed topology arrays", i);
        if (topos[i].n_segments > 0 && !params[i]) return set_error(TROUTE_EINVAL, "network %d: null params", i);
    }
    std::vector<troute_chparams> prm;
    prm.reserve(f.S);
    std::vector<int> qc;
    qc.reserve(f.S);
    std::vector<double> qs;
    bool has_scale = false;
    for (int i = 0; i < n_nets; ++i)
        if (qlat_scale && qlat_scale[i]) has_scale = true;
    long long col = 0;
    for (int i = 0; i < n_nets; ++i) {
        const int S = topos[i].n_segments;
        for (int s = 0; s < S; ++s) {
            prm.push_back(params[i][s]);
            const int c = (qlat_col && qlat_col[i]) ? qlat_col[i][s] : (int)(col + s);
            qc.push_back(c);
            if (has_scale) qs.push_back((qlat_scale && qlat_scale[i]) ? qlat_scale[i][s] : 1.0);
        }
        col += S;
    }
    int cols = qlat_cols > 0 ? qlat_cols : (int)col;
    for (int c : qc)
        if (c < 0 || c >= cols) return set_error(TROUTE_EINVAL, "lateral-inflow column %d outside [0, %d)", c, cols);
    troute_handle* H = nullptr;
    int rc = new_handle(&H, dt, cfg);
    if (rc) return rc;
    H->qlat_cols = cols;
    rc = build_handle(H, f, prm, qc, qs, has_scale);
    if (rc) {
        delete H;
        return rc;
    }
    // default state: zero flow, zero depth
    *h = H;
    return TROUTE_OK;
}

extern "C" int troute_create(troute_handle** h, const troute_topo* topo, const troute_chparams* params,
                             double dt, const troute_cfg* cfg)
{
    if (!topo) return set_error(TROUTE_EINVAL, "null topology");
    const troute_chparams* p[1] = {params};
    return troute_create_batch(h, 1, topo, p, nullptr, nullptr, 0, dt, cfg);
}

extern "C" int troute_create_ensemble(troute_handle** h, const troute_topo* topo,
                                      const troute_chparams* params, int n_members,
                                      const double* n_scale, const double* qlat_scale,
                                      double dt, const troute_cfg* cfg)
{
    if (!topo || n_members < 1) return set_error(TROUTE_EINVAL, "ensemble needs a topology and n_members >= 1");
    if (topo->n_segments > 0 && !params) return set_error(TROUTE_EINVAL, "null params");
    if ((long long)n_members * topo->n_segments > 0x7FFFFFFFLL || (long long)n_members * topo->n_reaches > 0x3FFFFFFFLL)
        return set_error(TROUTE_EINVAL, "ensemble too large for 32-bit segment/reach indices");
    Forest f;
    f.up_ptr.push_back(0);
    if (!append_topo(f, *topo)) return set_error(TROUTE_ETOPO, "malformed topology arrays");
    std::vector<troute_chparams> prm(params, params + f.S);
    std::vector<int> qc(f.S);
    for (int s = 0; s < f.S; ++s) qc[s] = s;
    Layout base, ens;
    int rc = build_layout(f, prm, qc, std::vector<double>(), false, base);
    if (rc) return rc;
    replicate_layout(base, prm, n_members, n_scale, qlat_scale, ens);
    troute_handle* H = nullptr;
    if ((rc = new_handle(&H, dt, cfg))) return rc;
    H->qlat_cols = f.S;
    if ((rc = upload_layout(H, ens))) {
        delete H;
        return rc;
    }
    *h = H;
    return TROUTE_OK;
}

extern "C" int troute_destroy(troute_handle* h)
{
    delete h;
    return TROUTE_OK;
}

extern "C" int troute_set_cfg(troute_handle* h, const troute_cfg* cfg)
{
    if (!h || !cfg) return set_error(TROUTE_EINVAL, "null argument");
    int rc = check_cfg(*cfg);
    if (rc) return rc;
    h->cfg = *cfg;
    return launch_shape(h);
}

extern "C" int troute_info(const troute_handle* h, int* n_reaches, int* n_segments, int* n_levels,
                           int* qlat_cols, long long* steps_done)
{
    if (!h) return set_error(TROUTE_EINVAL, "null handle");
    if (n_reaches) *n_reaches = h->R_user;
    if (n_segments) *n_segments = h->S_user;
    if (n_levels) *n_levels = h->n_levels;
    if (qlat_cols) *qlat_cols = h->qlat_cols;
    if (steps_done) *steps_done = h->steps_done;
    return TROUTE_OK;
}

// Writes user-order state into the device planes; v may be null (zeroed).
static int put_state(troute_handle* H, const double* q, const double* dd, const double* v,
                     const double* reach_last, long long steps)
{
    cudaStream_t st = H->stream;
    int rc;
    const size_t S = H->S_user, R = H->R_user;
    if ((rc = cuda_check(cudaMemsetAsync(H->q.p, 0, H->S_int * sizeof(double), st), "memset"))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(H->d.p, 0, H->S_int * sizeof(double), st), "memset"))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(H->v.p, 0, H->S_int * sizeof(double), st), "memset"))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(H->ring.p, 0, H->ring.n * sizeof(double), st), "memset"))) return rc;
    const double* srcs[3] = {q, dd, v};
    double* dsts[3] = {H->q.p, H->d.p, H->v.p};
    for (int i = 0; i < 3; ++i) {
        if (!srcs[i] || S == 0) continue;
        if ((rc = cuda_check(cudaMemcpyAsync(H->tmp.p, srcs[i], S * sizeof(double), cudaMemcpyHostToDevice, st), "state upload"))) return rc;
        if ((rc = launch_scatter(H->tmp.p, H->seg_map_d.p, (long long)S, dsts[i], st))) return rc;
        if ((rc = cuda_check(cudaStreamSynchronize(st), "state sync"))) return rc;
    }
    std::vector<double> rl(R, 0.0);
    if (reach_last) {
        std::memcpy(rl.data(), reach_last, R * sizeof(double));
    } else if (q) {
        // outflow of the previous step = discharge of the reach's last segment
        // (wavefront_mc.cu:675-680); a reach without segments sends nothing
        for (size_t r = 0; r < R; ++r)
            rl[r] = H->user_seg_len[r] > 0 ? q[H->user_seg_start[r] + H->user_seg_len[r] - 1] : 0.0;
    }
    const int slot = (int)(((steps - 1) % kRing + kRing) % kRing);
    if (R > 0) {
        if ((rc = cuda_check(cudaMemcpyAsync(H->tmp.p, rl.data(), R * sizeof(double), cudaMemcpyHostToDevice, st), "state upload"))) return rc;
        if ((rc = launch_scatter(H->tmp.p, H->reach_map_d.p, (long long)R, H->ring.p + (size_t)slot * H->R_int, st))) return rc;
    }
    if ((rc = launch_fill_int(H->done.p, H->R_int, nullptr, (int)steps, st))) return rc;
    if ((rc = launch_fill_int(H->step_base.p, 1, nullptr, (int)steps, st))) return rc;
    if ((rc = cuda_check(cudaStreamSynchronize(st), "state sync"))) return rc;
    H->steps_done = steps;
    H->broken = false;
    return TROUTE_OK;
}

extern "C" int troute_set_state(troute_handle* h, const double* qdp, const double* dp,
                                const double* reach_last)
{
    if (!h) return set_error(TROUTE_EINVAL, "null handle");
    return put_state(h, qdp, dp, nullptr, reach_last, 0);
}

extern "C" int troute_get_state(troute_handle* h, double* q, double* d, double* v, double* reach_last)
{
    if (!h) return set_error(TROUTE_EINVAL, "null handle");
    cudaStream_t st = h->stream;
    int rc;
    const size_t S = h->S_user, R = h->R_user;
    const double* srcs[3] = {h->q.p, h->d.p, h->v.p};
    double* dsts[3] = {q, d, v};
    // segments not covered by any reach carry zeros
    for (int i = 0; i < 3; ++i) {
        if (!dsts[i] || S == 0) continue;
        if ((rc = launch_gather(srcs[i], h->seg_map_d.p, (long long)S, h->tmp.p, st))) return rc;
        if ((rc = cuda_check(cudaMemcpyAsync(dsts[i], h->tmp.p, S * sizeof(double), cudaMemcpyDeviceToHost, st), "state download"))) return rc;
        if ((rc = cuda_check(cudaStreamSynchronize(st), "state sync"))) return rc;
        for (size_t s = 0; s < S; ++s)
            if (h->seg_map[s] < 0) dsts[i][s] = 0.0;
    }
    if (reach_last && R > 0) {
        const int slot = (int)(((h->steps_done - 1) % kRing + kRing) % kRing);
        if ((rc = launch_gather(h->ring.p + (size_t)slot * h->R_int, h->reach_map_d.p, (long long)R, h->tmp.p, st))) return rc;
        if ((rc = cuda_check(cudaMemcpyAsync(reach_last, h->tmp.p, R * sizeof(double), cudaMemcpyDeviceToHost, st), "state download"))) return rc;
        if ((rc = cuda_check(cudaStreamSynchronize(st), "state sync"))) return rc;
    }
    return TROUTE_OK;
}

// Ticket prefix per wave for a run of n_ts steps: wave w holds the blocks of
// levels max(0, w-n_ts+1) .. min(L-1, w), each at step w - level.
static void wave_prefix(const std::vector<int>& lb_ptr, int L, int n_ts, std::vector<unsigned long long>& wp)
{
    const int W = n_ts + L - 1;
    wp.assign(W + 1, 0);
    for (int w = 0; w < W; ++w) {
        const int lo = std::max(0, w - n_ts + 1), hi = std::min(L - 1, w);
        const unsigned long long c = hi >= lo ? (unsigned long long)(lb_ptr[hi + 1] - lb_ptr[lo]) : 0ull;
        wp[w + 1] = wp[w] + c;
    }
}

// A run of n_ts steps is routed in chunks whose per-step scratch (dependency
// counters, ready-queue entries and outflow history of the dataflow kernel,
// ~20 B per reach-step) fits a memory budget: cfg.max_chunk_steps if set,
// else a third of the free device memory at the first run.
struct RunPlan {
    int chunk = 0, n_full = 0, rem = 0;
};

static int plan_run(troute_handle* H, int n_ts, RunPlan* P)
{
    int chunk = n_ts;
    if (H->cfg.max_chunk_steps > 0) chunk = std::min(chunk, H->cfg.max_chunk_steps);
    if (H->mapping == 3) {
        const double per_step = (double)std::max(1, H->R_int) * (sizeof(int) + sizeof(double)) +
                                (double)std::max(1, H->R_real) * sizeof(int2) +
                                (H->cfg.warm_start ? (double)H->S_int * sizeof(float) : 0.0);
        if (H->chunk_budget_bytes == 0) {
            size_t fr = 0, tot = 0;
            if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) fr = (size_t)8 << 30;
            H->chunk_budget_bytes = fr / 3;
        }
        const long long fit = (long long)((double)H->chunk_budget_bytes / per_step);
        chunk = (int)std::max<long long>(1, std::min<long long>(chunk, fit));
    }
    P->chunk = chunk;
    P->n_full = n_ts / chunk;
    P->rem = n_ts % chunk;
    return TROUTE_OK;
}

// Enqueues one chunk of n_ts steps (wave table `wave` already on the device).
static int enqueue_chunk(troute_handle* H, const double* qlat_dev, int n_ts, const unsigned long long* wave,
                         unsigned long long n_tickets, double* q_hist, float* pairs, double* start_hist,
                         cudaStream_t st)
{
    int rc;
    RunDev run;
    run.step_base = H->step_base.p;
    run.n_ts = n_ts;
    run.dt = H->dt;
    run.dt_half = H->dt / 2.0;
    run.qlat = qlat_dev;
    run.qlat_ld = H->qlat_cols;
    run.wave_ptr = wave;
    run.n_waves = n_ts + H->n_levels - 1;
    run.n_tickets = n_tickets;
    run.ticket = H->ticket.p;
    run.stats = H->stats.p;
    run.wait_cycles = H->cfg.wait_cycles > 0 ? H->cfg.wait_cycles : 8000000000LL;
    run.tol = make_tol(H->cfg);
    run.q_hist = q_hist;
    run.pairs = pairs;
    run.start_hist = start_hist;
    run.warm = H->cfg.warm_start ? 1 : 0;
    run.warm_k = H->cfg.warm_k;
    run.warm_delta = H->warm_delta;
    run.warm_hi = 1.0 + H->warm_delta;
    run.warm_lo = 1.0 - H->warm_delta;
    run.start_pred = nullptr;
    if ((rc = cuda_check(cudaMemsetAsync(H->ticket.p, 0, sizeof(unsigned long long), st), "memset"))) return rc;
    if (H->mapping == 3) {
        DataflowDev df;
        df.cnt = H->df_cnt.p;
        df.rq = H->df_rq.p;
        df.rq_head = H->rq_ctr.p;
        df.rq_tail = H->rq_ctr.p + 1;
        df.n_done = H->rq_ctr.p + 2;
        df.rh = H->df_rh.p;
        df.heads = H->df_heads.p;
        df.n_heads = H->n_heads;
        df.continue_items = H->cfg.schedule_flags & 1;
        df.n_items = (unsigned long long)H->R_real * (unsigned long long)n_ts;
        if (run.warm) {
            // the launch's learned starting depths: one tcgen05 GEMM over every
            // (segment slot, step) from the state at the launch's start
            if (!warm_ready(H->warm_model))
                return set_error(TROUTE_ESTATE, "cfg.warm_start is set but no trained model is attached");
            int* err = reinterpret_cast<int*>(reinterpret_cast<char*>(H->stats.p) + offsetof(DevStats, error));
            if ((rc = launch_warm_plane(H->warm_model, H->net(), run, n_ts, H->pred.p, err, st)))
                return rc;
            run.start_pred = H->pred.p;
        }
        rc = launch_route_dataflow(H->net(), run, df, H->grid, st);
    } else if (H->mapping == 2) {
        rc = launch_route_pool(H->net(), run, H->grid, H->threads, st);
    } else {
        rc = launch_route(H->net(), run, H->grid, H->threads, st);
    }
    if (rc) return rc;
    return launch_bump_steps(H->step_base.p, n_ts, st);
}

// Enqueues a whole run as chunks; stats are zeroed once, the velocity of the
// final state derived once at the end.
static int enqueue_run(troute_handle* H, const double* qlat_dev, int n_ts, const RunPlan& P, cudaStream_t st,
                       bool timed)
{
    int rc;
    if ((rc = cuda_check(cudaMemsetAsync(H->stats.p, 0, sizeof(DevStats), st), "memset"))) return rc;
    const bool rec_pairs = H->cfg.record_pairs && H->pairs.p;
    const bool rec_start = H->cfg.record_start && H->start_hist.p;
    if (rec_pairs && (rc = cuda_check(cudaMemsetAsync(H->pairs.p, 0, (size_t)n_ts * H->S_int * 9 * sizeof(float), st),
                                      "memset")))
        return rc;
    if (rec_start &&
        (rc = cuda_check(cudaMemsetAsync(H->start_hist.p, 0, (size_t)n_ts * H->S_int * sizeof(double), st), "memset")))
        return rc;
    if (timed && (rc = cuda_check(cudaEventRecord(H->ev0, st), "event"))) return rc;
    const int n_chunks = P.n_full + (P.rem ? 1 : 0);
    for (int c = 0; c < n_chunks; ++c) {
        const int t0 = c * P.chunk;
        const int len = (c < P.n_full) ? P.chunk : P.rem;
        const bool tail = (c >= P.n_full);
        const unsigned long long* wave = tail ? H->wave_ptr_tail.p : H->wave_ptr.p;
        const unsigned long long nt = tail ? H->n_tickets_tail : H->n_tickets;
        double* qh = (H->cfg.record_history && H->hist.p) ? H->hist.p + (size_t)t0 * H->S_int : nullptr;
        float* pr = rec_pairs ? H->pairs.p + (size_t)t0 * H->S_int * 9 : nullptr;
        double* sh = rec_start ? H->start_hist.p + (size_t)t0 * H->S_int : nullptr;
        if ((rc = enqueue_chunk(H, qlat_dev + (size_t)t0 * (size_t)H->qlat_cols, len, wave, nt, qh, pr, sh, st)))
            return rc;
    }
    if (H->mapping >= 2 && (rc = launch_velocity(H->net(), st))) return rc;
    if (timed && (rc = cuda_check(cudaEventRecord(H->ev1, st), "event"))) return rc;
    return TROUTE_OK;
}

static int upload_waves(troute_handle* H, int len, DBuf<unsigned long long>& buf, unsigned long long* n_tickets)
{
    std::vector<unsigned long long> wp;
    wave_prefix(H->lb_ptr, H->n_levels, len, wp);
    *n_tickets = wp.back();
    int rc = buf.alloc(wp.size());
    if (rc) return rc;
    rc = cuda_check(cudaMemcpyAsync(buf.p, wp.data(), wp.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                                    H->stream), "wave upload");
    if (rc) return rc;
    return cuda_check(cudaStreamSynchronize(H->stream), "wave sync");
}

static int prepare_run(troute_handle* H, int n_ts, RunPlan* P)
{
    if (H->cfg.warm_start && !warm_ready(H->warm_model))
        return set_error(TROUTE_ESTATE, "cfg.warm_start is set but no trained model is attached (troute_set_warm_start)");
    int rc = plan_run(H, n_ts, P);
    if (rc) return rc;
    if (H->mapping != 3) {
        if ((rc = upload_waves(H, P->chunk, H->wave_ptr, &H->n_tickets))) return rc;
        if (P->rem && (rc = upload_waves(H, P->rem, H->wave_ptr_tail, &H->n_tickets_tail))) return rc;
    }
    if (H->cfg.record_history) {
        if ((rc = H->hist.alloc((size_t)n_ts * H->S_int))) return rc;
        H->hist_ts = n_ts;
    }
    if (H->cfg.record_pairs) {
        if ((rc = H->pairs.alloc((size_t)n_ts * H->S_int * 9))) return rc;
        H->pairs_ts = n_ts;
    }
    if (H->cfg.record_start) {
        if ((rc = H->start_hist.alloc((size_t)n_ts * H->S_int))) return rc;
        H->start_ts = n_ts;
    }
    if (H->cfg.warm_start && (rc = H->pred.alloc((size_t)P->chunk * H->S_int))) return rc;
    if (H->mapping == 3) {
        const size_t R = (size_t)std::max(1, H->R_int);
        const size_t T = (size_t)P->chunk;
        if ((rc = H->df_cnt.alloc(T * R)) || (rc = H->df_rh.alloc((T + 1) * R)) ||
            (rc = H->df_rq.alloc(std::max<size_t>(1, (size_t)H->R_real * T))) || (rc = H->rq_ctr.alloc(3)))
            return rc;
    }
    return TROUTE_OK;
}

static int collect(troute_handle* H, troute_stats* stats, bool timed)
{
    DevStats ds;
    int rc = cuda_check(cudaMemcpy(&ds, H->stats.p, sizeof ds, cudaMemcpyDeviceToHost), "stats download");
    if (rc) return rc;
    if (stats) {
        std::memset(stats, 0, sizeof *stats);
        stats->solves = ds.solves;
        stats->iterations = ds.iterations;
        stats->retries = ds.retries;
        stats->early_exits = ds.early_exits;
        stats->warm_used = ds.warm_used;
        stats->warm_fallback = ds.warm_fallback;
        for (int i = 0; i < 16; ++i) stats->iter_hist[i] = ds.hist[i];
        stats->warp_passes = ds.warp_passes;
        stats->lane_busy = ds.lane_busy;
        stats->lane_wait = ds.lane_wait;
        stats->lane_idle = ds.lane_idle;
        stats->solve_passes = ds.solve_passes;
        stats->timeout = ds.error == TROUTE_ETIMEOUT;
        if (timed) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, H->ev0, H->ev1);
            stats->kernel_ms = ms;
        }
    }
    if (ds.error == TROUTE_ETIMEOUT) {
        H->broken = true;
        return set_error(TROUTE_ETIMEOUT, "device wait ran out (internal reach %d, step %d, wait kind %d)",
                         ds.err_reach, ds.err_step, ds.err_where);
    }
    if (ds.error) {
        H->broken = true;
        return set_error(ds.error, "device reported error %d", ds.error);
    }
    return TROUTE_OK;
}

extern "C" int troute_run_device(troute_handle* h, const double* qlat_ts_device, int n_ts, void* stream)
{
    if (!h) return set_error(TROUTE_EINVAL, "null handle");
    if (h->broken) return set_error(TROUTE_ESTATE, "handle unusable after an earlier device failure; restore or set state");
    if (n_ts < 0) return set_error(TROUTE_EINVAL, "n_ts < 0");
    if (n_ts == 0 || h->R_user == 0) return TROUTE_OK;
    if (!qlat_ts_device) return set_error(TROUTE_EINVAL, "null lateral inflow");
    RunPlan P;
    int rc = prepare_run(h, n_ts, &P);
    if (rc) return rc;
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    if (stream) {
        // order our stream's prior work (uploads) before the caller's stream
        cudaEvent_t e;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        cudaEventRecord(e, h->stream);
        cudaStreamWaitEvent(st, e, 0);
        cudaEventDestroy(e);
    }
    if ((rc = enqueue_run(h, qlat_ts_device, n_ts, P, st, true))) return rc;
    h->steps_done += n_ts;
    h->last_n_ts = n_ts;
    return TROUTE_OK;
}

extern "C" int troute_sync(troute_handle* h, troute_stats* stats)
{
    if (!h) return set_error(TROUTE_EINVAL, "null handle");
    int rc = cuda_check(cudaDeviceSynchronize(), "run");
    if (rc) return rc;
    return collect(h, stats, h->last_n_ts > 0);
}

extern "C" int troute_run(troute_handle* h, const double* qlat_ts, int n_ts, troute_stats* stats)
{
    if (!h) return set_error(TROUTE_EINVAL, "null handle");
    if (h->broken) return set_error(TROUTE_ESTATE, "handle unusable after an earlier device failure; restore or set state");
    if (n_ts < 0) return set_error(TROUTE_EINVAL, "n_ts < 0");
    if (stats) std::memset(stats, 0, sizeof *stats);
    if (n_ts == 0 || h->R_user == 0) return TROUTE_OK;
    if (!qlat_ts) return set_error(TROUTE_EINVAL, "null lateral inflow");
    const size_t n = (size_t)n_ts * (size_t)h->qlat_cols;
    int rc = h->qlat_buf.alloc(std::max<size_t>(n, 1));
    if (rc) return rc;
    if ((rc = cuda_check(cudaMemcpyAsync(h->qlat_buf.p, qlat_ts, n * sizeof(double), cudaMemcpyHostToDevice, h->stream),
                         "qlat upload")))
        return rc;
    if ((rc = troute_run_device(h, h->qlat_buf.p, n_ts, nullptr))) return rc;
    rc = cuda_check(cudaStreamSynchronize(h->stream), "run");
    if (rc) return rc;
    return collect(h, stats, true);
}

extern "C" int troute_graph_capture(troute_handle* h, const double* qlat_ts_device, int n_ts)
{
    if (!h || !qlat_ts_device || n_ts <= 0) return set_error(TROUTE_EINVAL, "bad graph arguments");
    RunPlan P;
    int rc = prepare_run(h, n_ts, &P);
    if (rc) return rc;
    if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
    if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
    if ((rc = cuda_check(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture"))) return rc;
    rc = enqueue_run(h, qlat_ts_device, n_ts, P, h->stream, false);
    cudaGraph_t g = nullptr;
    const int rc2 = cuda_check(cudaStreamEndCapture(h->stream, &g), "end capture");
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (rc2) return rc2;
    h->graph = g;
    if ((rc = cuda_check(cudaGraphInstantiate(&h->graph_exec, g, 0), "graph instantiate"))) return rc;
    h->graph_n_ts = n_ts;
    return TROUTE_OK;
}

extern "C" int troute_graph_launch(troute_handle* h, void* stream)
{
    if (!h || !h->graph_exec) return set_error(TROUTE_EINVAL, "no captured graph");
    if (h->broken) return set_error(TROUTE_ESTATE, "handle unusable after an earlier device failure");
    int rc = cuda_check(cudaGraphLaunch(h->graph_exec, stream ? (cudaStream_t)stream : h->stream), "graph launch");
    if (rc) return rc;
    h->steps_done += h->graph_n_ts;
    h->last_n_ts = 0;
    return TROUTE_OK;
}

extern "C" int troute_set_warm_start(troute_handle* h, const troute_warm* model, double delta)
{
    if (!h) return set_error(TROUTE_EINVAL, "null handle");
    if (model && !warm_ready(model)) return set_error(TROUTE_ESTATE, "model has no trained weights");
    if (model && !(delta > 0.0 && delta < 1.0)) return set_error(TROUTE_EINVAL, "delta must be in (0, 1)");
    h->warm_model = model;
    if (model) h->warm_delta = delta;
    return TROUTE_OK;
}

extern "C" int troute_get_pairs(troute_handle* h, float* pairs_device, long long capacity, long long* n_pairs)
{
    if (!h || !n_pairs) return set_error(TROUTE_EINVAL, "null argument");
    *n_pairs = 0;
    if (!h->cfg.record_pairs || !h->pairs.p || h->pairs_ts == 0)
        return set_error(TROUTE_ESTATE, "no pairs recorded (set cfg.record_pairs before the run)");
    if (capacity > 0 && !pairs_device) return set_error(TROUTE_EINVAL, "null pair buffer");
    return compact_pairs(h->pairs.p, (long long)h->pairs_ts * h->S_int, pairs_device, capacity, n_pairs, h->stream);
}

extern "C" int troute_get_start_history(troute_handle* h, double* start_hist, int n_ts)
{
    if (!h || !start_hist) return set_error(TROUTE_EINVAL, "null argument");
    if (!h->cfg.record_start || !h->start_hist.p || n_ts != h->start_ts)
        return set_error(TROUTE_ESTATE, "no starting depths of %d steps recorded (set cfg.record_start)", n_ts);
    const size_t S = (size_t)h->S_user;
    int rc;
    for (int t = 0; t < n_ts; ++t) {
        if ((rc = launch_gather(h->start_hist.p + (size_t)t * h->S_int, h->seg_map_d.p, (long long)S, h->tmp.p, h->stream)))
            return rc;
        if ((rc = cuda_check(cudaMemcpyAsync(start_hist + (size_t)t * S, h->tmp.p, S * sizeof(double),
                                             cudaMemcpyDeviceToHost, h->stream), "start history download")))
            return rc;
        if ((rc = cuda_check(cudaStreamSynchronize(h->stream), "start history sync"))) return rc;
    }
    return TROUTE_OK;
}

extern "C" int troute_get_history(troute_handle* h, double* q_hist, int n_ts)
{
    if (!h || !q_hist) return set_error(TROUTE_EINVAL, "null argument");
    if (!h->cfg.record_history || !h->hist.p || n_ts != h->hist_ts)
        return set_error(TROUTE_ESTATE, "no history of %d steps recorded (set cfg.record_history)", n_ts);
    const size_t S = h->S_user;
    int rc;
    for (int t = 0; t < n_ts; ++t) {
        if ((rc = launch_gather(h->hist.p + (size_t)t * h->S_int, h->seg_map_d.p, (long long)S, h->tmp.p, h->stream))) return rc;
        if ((rc = cuda_check(cudaMemcpyAsync(q_hist + (size_t)t * S, h->tmp.p, S * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "history download"))) return rc;
    }
    return cuda_check(cudaStreamSynchronize(h->stream), "history sync");
}

// checkpoint: header + q, d, v [S_user] + reach_last [R_user], user order
struct CkptHeader {
    char magic[8];
    int version, R, S, pad;
    long long steps;
};

// ---- autotuner -----------------------------------------------------------
// The routing state a run changes, copied device-to-device so every trial of
// the tuner starts from the same state and the handle's state is untouched by
// tuning.
struct DevSnapshot {
    DBuf<double> q, d, v, ring;
    DBuf<int> done, step_base;
    long long steps = 0;
};

static int snapshot_copy(troute_handle* H, DevSnapshot& S, bool save)
{
    int rc;
    if (save && ((rc = S.q.alloc(H->q.n)) || (rc = S.d.alloc(H->d.n)) || (rc = S.v.alloc(H->v.n)) ||
                 (rc = S.ring.alloc(H->ring.n)) || (rc = S.done.alloc(H->done.n)) ||
                 (rc = S.step_base.alloc(H->step_base.n))))
        return rc;
    const cudaStream_t st = H->stream;
    auto cp = [&](void* dst, const void* src, size_t bytes) {
        return bytes ? cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st), "snapshot") : 0;
    };
    if (save) {
        if ((rc = cp(S.q.p, H->q.p, H->q.n * 8)) || (rc = cp(S.d.p, H->d.p, H->d.n * 8)) ||
            (rc = cp(S.v.p, H->v.p, H->v.n * 8)) || (rc = cp(S.ring.p, H->ring.p, H->ring.n * 8)) ||
            (rc = cp(S.done.p, H->done.p, H->done.n * 4)) || (rc = cp(S.step_base.p, H->step_base.p, H->step_base.n * 4)))
            return rc;
        S.steps = H->steps_done;
    } else {
        if ((rc = cp(H->q.p, S.q.p, H->q.n * 8)) || (rc = cp(H->d.p, S.d.p, H->d.n * 8)) ||
            (rc = cp(H->v.p, S.v.p, H->v.n * 8)) || (rc = cp(H->ring.p, S.ring.p, H->ring.n * 8)) ||
            (rc = cp(H->done.p, S.done.p, H->done.n * 4)) || (rc = cp(H->step_base.p, S.step_base.p, H->step_base.n * 4)))
            return rc;
        H->steps_done = S.steps;
        H->broken = false;
    }
    return cuda_check(cudaStreamSynchronize(st), "snapshot sync");
}

static int occupancy_of(int mapping, int threads, bool warm, int* bps)
{
    if (mapping == 3) return route_dataflow_occupancy(bps, warm);
    if (mapping == 2) return route_pool_occupancy(bps);
    return route_occupancy(threads, bps);
}

extern "C" int troute_autotune(troute_handle* h, const double* qlat_ts_device, int n_ts, int repeats, int flags,
                               troute_tune_result* res)
{
    if (!h || !qlat_ts_device || !res) return set_error(TROUTE_EINVAL, "null argument");
    if (n_ts < 1 || repeats < 1) return set_error(TROUTE_EINVAL, "n_ts and repeats must be positive");
    if (h->broken) return set_error(TROUTE_ESTATE, "handle unusable after an earlier device failure");
    std::memset(res, 0, sizeof *res);
    const troute_cfg base = h->cfg;
    const bool warm = base.warm_start != 0;
    // candidate launch configurations: {mapping, blocks_per_sm, threads_per_block, schedule_flags}
    std::vector<std::array<int, 4>> cand;
    int rc, occ = 0;
    if ((rc = occupancy_of(3, 128, warm, &occ))) return rc;
    const int occ3 = std::max(1, occ);
    for (int b = 1; b <= std::max(1, occ); ++b)
        for (int f = 0; f < 2; ++f) cand.push_back({3, b, 128, f});
    if (!warm && (flags & TROUTE_TUNE_ALL_MAPPINGS)) {
        if ((rc = occupancy_of(2, 128, false, &occ))) return rc;
        for (int b = 1; b <= std::max(1, occ); ++b) cand.push_back({2, b, 128, 0});
        for (int t : {32, 64, 128}) cand.push_back({1, 0, t, 0});
    }
    if ((int)cand.size() > TROUTE_TUNE_MAX_TRIALS) cand.resize(TROUTE_TUNE_MAX_TRIALS);
    // the tuner's own graph-free runs; a captured graph no longer matches the shape
    if (h->graph_exec) {
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
    }
    if (h->graph) {
        cudaGraphDestroy(h->graph);
        h->graph = nullptr;
    }
    DevSnapshot snap;
    if ((rc = snapshot_copy(h, snap, true))) return rc;
    int best = -1;
    double best_ms = 0.0;
    for (size_t i = 0; i < cand.size(); ++i) {
        troute_cfg c = base;
        c.mapping = cand[i][0];
        c.blocks_per_sm = cand[i][1];
        c.threads_per_block = cand[i][0] == 1 ? cand[i][2] : 0;
        c.schedule_flags = (base.schedule_flags & ~1) | cand[i][3];
        c.record_history = c.record_pairs = c.record_start = 0;
        h->cfg = c;
        double ms = -1.0;
        if ((rc = launch_shape(h)) == TROUTE_OK) {
            for (int r = 0; r < repeats; ++r) {
                if ((rc = snapshot_copy(h, snap, false))) break;
                troute_stats st;
                if ((rc = troute_run_device(h, qlat_ts_device, n_ts, nullptr))) break;
                if ((rc = troute_sync(h, &st))) break;
                if (ms < 0.0 || st.kernel_ms < ms) ms = st.kernel_ms;
            }
        }
        res->trial_cfg[i][0] = cand[i][0];
        res->trial_cfg[i][1] = h->grid / std::max(1, h->n_sms);
        res->trial_cfg[i][2] = h->threads;
        res->trial_cfg[i][3] = cand[i][3];
        res->trial_ms[i] = rc == TROUTE_OK ? ms : -1.0;
        res->n_trials = (int)i + 1;
        if (rc != TROUTE_OK) continue;  // a failing shape (e.g. a wait that ran out) is skipped
        if (best < 0 || ms < best_ms) {
            best = (int)i;
            best_ms = ms;
        }
        if (cand[i][0] == 3 && cand[i][1] == occ3 && cand[i][3] == 0) res->default_ms = ms;
    }
    h->cfg = base;
    if (best >= 0) {
        h->cfg.mapping = cand[best][0];
        h->cfg.blocks_per_sm = cand[best][1];
        h->cfg.threads_per_block = cand[best][0] == 1 ? cand[best][2] : 0;
        h->cfg.schedule_flags = (base.schedule_flags & ~1) | cand[best][3];
    }
    if ((rc = launch_shape(h))) return rc;
    if ((rc = snapshot_copy(h, snap, false))) return rc;
    if (best < 0) return set_error(TROUTE_ECUDA, "no launch configuration completed a trial run");
    res->mapping = h->cfg.mapping;
    res->blocks_per_sm = h->grid / std::max(1, h->n_sms);
    res->threads_per_block = h->threads;
    res->schedule_flags = h->cfg.schedule_flags;
    res->best_ms = best_ms;
    return TROUTE_OK;
}

extern "C" int troute_checkpoint(troute_handle* h, void* buf, size_t* nbytes)
{
    if (!h || !nbytes) return set_error(TROUTE_EINVAL, "null argument");
    const size_t need = sizeof(CkptHeader) + (3 * (size_t)h->S_user + (size_t)h->R_user) * sizeof(double);
    if (!buf) { *nbytes = need; return TROUTE_OK; }
    if (*nbytes < need) { *nbytes = need; return set_error(TROUTE_EINVAL, "checkpoint buffer too small"); }
    if (h->broken) return set_error(TROUTE_ESTATE, "handle state invalid after a device failure");
    CkptHeader hd;
    std::memset(&hd, 0, sizeof hd);
    std::memcpy(hd.magic, "TRGB300", 8);
    hd.version = 1;
    hd.R = h->R_user;
    hd.S = h->S_user;
    hd.steps = h->steps_done;
    char* p = static_cast<char*>(buf);
    std::memcpy(p, &hd, sizeof hd);
    double* x = reinterpret_cast<double*>(p + sizeof hd);
    const size_t S = h->S_user;
    int rc = troute_get_state(h, x, x + S, x + 2 * S, x + 3 * S);
    if (rc) return rc;
    *nbytes = need;
    return TROUTE_OK;
}

extern "C" int troute_restore(troute_handle* h, const void* buf, size_t nbytes)
{
    if (!h || !buf) return set_error(TROUTE_EINVAL, "null argument");
    CkptHeader hd;
    if (nbytes < sizeof hd) return set_error(TROUTE_ESTATE, "checkpoint truncated");
    std::memcpy(&hd, buf, sizeof hd);
    if (std::memcmp(hd.magic, "TRGB300", 8) != 0 || hd.version != 1) return set_error(TROUTE_ESTATE, "not a checkpoint");
    if (hd.R != h->R_user || hd.S != h->S_user) return set_error(TROUTE_ESTATE, "checkpoint is for another network");
    const size_t S = h->S_user;
    if (nbytes < sizeof hd + (3 * S + (size_t)hd.R) * sizeof(double)) return set_error(TROUTE_ESTATE, "checkpoint truncated");
    std::vector<double> x(3 * S + hd.R);
    std::memcpy(x.data(), static_cast<const char*>(buf) + sizeof hd, x.size() * sizeof(double));
    return put_state(h, x.data(), x.data() + S, x.data() + 2 * S, x.data() + 3 * S, hd.steps);
}
