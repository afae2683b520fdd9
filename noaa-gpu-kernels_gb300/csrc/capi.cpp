// C-ABI entry points that wrap the handle API or the reach-parallel kernel:
// the cpu_mc drop-in, the cpu_wavefront_fp64 drop-in, the one-shot FP64 tree
// routing call, topology helpers and device info.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "troute_internal.h"

namespace tr {
int check_cfg(const troute_cfg& c);
Tol make_tol(const troute_cfg& c);
int cuda_check(cudaError_t e, const char* what);
}  // namespace tr
using namespace tr;

extern "C" int troute_device_info(int* sm_count, int* cc_major, int* cc_minor, size_t* free_bytes)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return set_error(TROUTE_ENODEV, "no CUDA device: %s", cudaGetErrorString(e));
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp p;
    int rc = cuda_check(cudaGetDeviceProperties(&p, dev), "device properties");
    if (rc) return rc;
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    if (free_bytes) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        *free_bytes = fr;
    }
    return TROUTE_OK;
}

// ---------------------------------------------------------------------------
// reach-parallel (cpu_mc / kernel_mc_gpu)
// ---------------------------------------------------------------------------
namespace {
struct DevPtr {
    void* p = nullptr;
    ~DevPtr() { if (p) cudaFree(p); }
};

// Counter buffers of troute_mc_reach_parallel_device: one per (host thread,
// device), so a thread that switches devices never hands a kernel another
// GPU's memory, and two threads never share one. Freed when the thread exits
// (errors ignored: at process exit the runtime may already be unloading).
constexpr int kMaxDevices = 64;
struct ThreadDevStats {
    DevStats* p[kMaxDevices] = {};
    ~ThreadDevStats()
    {
        int cur = -1;
        bool any = false;
        for (int d = 0; d < kMaxDevices; ++d) {
            if (!p[d]) continue;
            if (!any) {
                any = true;
                if (cudaGetDevice(&cur) != cudaSuccess) cur = -1;
            }
            if (cudaSetDevice(d) == cudaSuccess) cudaFree(p[d]);
        }
        if (any && cur >= 0) cudaSetDevice(cur);
        cudaGetLastError();
    }
};
thread_local ThreadDevStats t_stats;

int device_stats(DevStats** out)
{
    int dev = 0;
    int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= kMaxDevices) return set_error(TROUTE_EINVAL, "device %d beyond the supported range", dev);
    if (!t_stats.p[dev] && (rc = cuda_check(cudaMalloc(&t_stats.p[dev], sizeof(DevStats)), "cudaMalloc"))) {
        t_stats.p[dev] = nullptr;
        return rc;
    }
    *out = t_stats.p[dev];
    return TROUTE_OK;
}
}  // namespace

namespace tr {
// An error left pending by earlier CUDA work of the calling thread is reported
// (and left pending) rather than consumed by this library's own launch check.
int pending_cuda_error(const char* entry)
{
    const cudaError_t e = cudaPeekAtLastError();
    if (e == cudaSuccess) return TROUTE_OK;
    return set_error(TROUTE_ECUDA, "%s: a CUDA error was pending before the call (%s); nothing was launched", entry,
                     cudaGetErrorString(e));
}
}  // namespace tr

extern "C" int troute_mc_reach_parallel_device(const troute_chparams* p, const double* ql,
                                               const int* rs, const int* rl,
                                               const double* qu, const double* qd, const double* dp,
                                               double* qo, double* vo, double* dpo,
                                               double uq, double dt, int nr, int n_segments,
                                               const troute_cfg* cfg, void* stream)
{
    if (nr < 0 || n_segments < 0) return set_error(TROUTE_EINVAL, "negative size");
    if (nr == 0) return TROUTE_OK;
    if (!p || !ql || !rs || !rl || !qu || !qd || !dp || !qo || !vo || !dpo)
        return set_error(TROUTE_EINVAL, "null array");
    troute_cfg c;
    troute_cfg_default(&c);
    if (cfg) c = *cfg;
    int rc = check_cfg(c);
    if (rc) return rc;
    if ((rc = pending_cuda_error("troute_mc_reach_parallel_device"))) return rc;
    DevStats* stats = nullptr;
    if ((rc = device_stats(&stats))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(stats, 0, sizeof(DevStats), (cudaStream_t)stream), "memset"))) return rc;
    return launch_reach_parallel(p, ql, rs, rl, qu, qd, dp, qo, vo, dpo, uq, dt, nr, n_segments, make_tol(c),
                                 stats, c.threads_per_block, stream);
}

extern "C" int troute_mc_reach_parallel_cfg(const troute_chparams* p, const double* ql,
                                            const int* rs, const int* rl,
                                            const double* qu, const double* qd, const double* dp,
                                            double* qo, double* vo, double* dpo,
                                            double uq, double dt, int nr,
                                            const troute_cfg* cfg, troute_stats* stats)
{
    if (stats) std::memset(stats, 0, sizeof *stats);
    if (nr < 0) return set_error(TROUTE_EINVAL, "nr < 0");
    if (nr == 0) return TROUTE_OK;
    if (!p || !ql || !rs || !rl || !qu || !qd || !dp || !qo || !vo || !dpo)
        return set_error(TROUTE_EINVAL, "null array");
    troute_cfg c;
    troute_cfg_default(&c);
    if (cfg) c = *cfg;
    int rc = check_cfg(c);
    if (rc) return rc;
    // segment count = end of the furthest reach (cpu_mc indexes rs[r]+i directly)
    long long S = 0;
    for (int r = 0; r < nr; ++r) {
        if (rs[r] < 0 || rl[r] < 0) return set_error(TROUTE_EINVAL, "reach %d: negative start or length", r);
        S = std::max<long long>(S, (long long)rs[r] + rl[r]);
    }
    if (S > 0x7FFFFFFF) return set_error(TROUTE_EINVAL, "too many segments");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");

    const size_t bs = (size_t)std::max<long long>(S, 1);
    // one device block: params | ql qu qd dp qo vo dpo | rs rl | stats
    const size_t off_d = bs * sizeof(troute_chparams);
    const size_t off_i = off_d + 7 * bs * sizeof(double);
    const size_t off_s = off_i + 2 * (size_t)nr * sizeof(int) + 256;
    DevPtr mem;
    if ((rc = cuda_check(cudaMalloc(&mem.p, off_s + sizeof(DevStats)), "cudaMalloc"))) return rc;
    char* base = static_cast<char*>(mem.p);
    auto* dpar = reinterpret_cast<troute_chparams*>(base);
    double* dd = reinterpret_cast<double*>(base + off_d);
    int* di = reinterpret_cast<int*>(base + off_i);
    DevStats* dst = reinterpret_cast<DevStats*>(base + off_s);
    cudaStream_t st = nullptr;
    if ((rc = cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream"))) return rc;
    auto fail = [&](int code) { cudaStreamDestroy(st); return code; };
    const size_t Sd = (size_t)S * sizeof(double);
    if ((rc = cuda_check(cudaMemcpyAsync(dpar, p, (size_t)S * sizeof(troute_chparams), cudaMemcpyHostToDevice, st), "H2D")) ||
        (rc = cuda_check(cudaMemcpyAsync(dd + 0 * bs, ql, Sd, cudaMemcpyHostToDevice, st), "H2D")) ||
        (rc = cuda_check(cudaMemcpyAsync(dd + 1 * bs, qu, Sd, cudaMemcpyHostToDevice, st), "H2D")) ||
        (rc = cuda_check(cudaMemcpyAsync(dd + 2 * bs, qd, Sd, cudaMemcpyHostToDevice, st), "H2D")) ||
        (rc = cuda_check(cudaMemcpyAsync(dd + 3 * bs, dp, Sd, cudaMemcpyHostToDevice, st), "H2D")) ||
        (rc = cuda_check(cudaMemcpyAsync(di, rs, (size_t)nr * sizeof(int), cudaMemcpyHostToDevice, st), "H2D")) ||
        (rc = cuda_check(cudaMemcpyAsync(di + nr, rl, (size_t)nr * sizeof(int), cudaMemcpyHostToDevice, st), "H2D")) ||
        (rc = cuda_check(cudaMemsetAsync(dst, 0, sizeof(DevStats), st), "memset")))
        return fail(rc);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    rc = launch_reach_parallel(dpar, dd, di, di + nr, dd + bs, dd + 2 * bs, dd + 3 * bs, dd + 4 * bs, dd + 5 * bs,
                               dd + 6 * bs, uq, dt, nr, (int)S, make_tol(c), dst, c.threads_per_block, st);
    cudaEventRecord(e1, st);
    if (!rc) rc = cuda_check(cudaMemcpyAsync(qo, dd + 4 * bs, Sd, cudaMemcpyDeviceToHost, st), "D2H");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(vo, dd + 5 * bs, Sd, cudaMemcpyDeviceToHost, st), "D2H");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(dpo, dd + 6 * bs, Sd, cudaMemcpyDeviceToHost, st), "D2H");
    DevStats ds;
    std::memset(&ds, 0, sizeof ds);
    if (!rc) rc = cuda_check(cudaMemcpyAsync(&ds, dst, sizeof ds, cudaMemcpyDeviceToHost, st), "D2H");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(st), "reach-parallel run");
    float ms = 0.f;
    if (!rc) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return fail(rc);
    cudaStreamDestroy(st);
    if (stats) {
        stats->solves = ds.solves;
        stats->iterations = ds.iterations;
        stats->retries = ds.retries;
        stats->early_exits = ds.early_exits;
        for (int i = 0; i < 16; ++i) stats->iter_hist[i] = ds.hist[i];
        stats->kernel_ms = ms;
    }
    if (ds.error) return set_error(ds.error, "reach-parallel kernel reported error %d at reach %d", ds.error, ds.err_reach);
    return TROUTE_OK;
}

extern "C" int troute_mc_reach_parallel(const troute_chparams* p, const double* ql,
                                        const int* rs, const int* rl,
                                        const double* qu, const double* qd, const double* dp,
                                        double* qo, double* vo, double* dpo,
                                        double uq, double dt, int nr)
{
    return troute_mc_reach_parallel_cfg(p, ql, rs, rl, qu, qd, dp, qo, vo, dpo, uq, dt, nr, nullptr, nullptr);
}

extern "C" int troute_debug_timeout_probe(long long wait_cycles)
{
    if (wait_cycles < 0) return set_error(TROUTE_EINVAL, "negative wait");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");
    DevStats* st = nullptr;
    int rc = cuda_check(cudaMalloc(&st, sizeof(DevStats)), "cudaMalloc");
    if (rc) return rc;
    DevStats h;
    std::memset(&h, 0, sizeof h);
    rc = cuda_check(cudaMemset(st, 0, sizeof(DevStats)), "memset");
    if (!rc) rc = launch_timeout_probe(st, wait_cycles, nullptr);
    if (!rc) rc = cuda_check(cudaMemcpy(&h, st, sizeof h, cudaMemcpyDeviceToHost), "probe");
    cudaFree(st);
    if (rc) return rc;
    if (h.error == TROUTE_ETIMEOUT) return set_error(TROUTE_ETIMEOUT, "bounded wait gave up as intended");
    return set_error(TROUTE_ESTATE, "probe did not report a timeout");
}

extern "C" int troute_measure_fp64_rate(double* warp_instr_per_s, double* ms)
{
    if (!warp_instr_per_s) return set_error(TROUTE_EINVAL, "null output");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");
    int dev = 0, sms = 0;
    int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (!rc) rc = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr");
    if (rc) return rc;
    const int blocks = 4 * sms;   // 32 warps per SM
    DevPtr sink;
    if ((rc = cuda_check(cudaMalloc(&sink.p, (size_t)blocks * sizeof(double)), "cudaMalloc"))) return rc;
    cudaEvent_t e0, e1;
    if ((rc = cuda_check(cudaEventCreate(&e0), "event"))) return rc;
    if ((rc = cuda_check(cudaEventCreate(&e1), "event"))) { cudaEventDestroy(e0); return rc; }
    double best = 0.0, best_ms = 0.0, wi = 0.0;
    int iters = 2048;
    for (int rep = 0; rep < 6 && !rc; ++rep) {
        cudaEventRecord(e0, nullptr);
        rc = launch_fp64_rate(blocks, iters, static_cast<double*>(sink.p), nullptr, &wi);
        cudaEventRecord(e1, nullptr);
        if (!rc) rc = cuda_check(cudaEventSynchronize(e1), "fp64 rate");
        float t = 0.f;
        if (!rc) cudaEventElapsedTime(&t, e0, e1);
        if (!rc && t > 0.f) {
            if (t < 20.f && iters < (1 << 24)) {   // grow to a launch of >= 20 ms, then keep the best
                iters *= 2;
                --rep;
                continue;
            }
            const double r = wi / (t * 1e-3);
            if (r > best) { best = r; best_ms = t; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    *warp_instr_per_s = best;
    if (ms) *ms = best_ms;
    return TROUTE_OK;
}

extern "C" int troute_debug_pow(const double* x, int n, double* out)
{
    if (n < 0 || (n > 0 && (!x || !out))) return set_error(TROUTE_EINVAL, "bad arguments");
    if (n == 0) return TROUTE_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");
    DevPtr dx, dout;
    int rc;
    if ((rc = cuda_check(cudaMalloc(&dx.p, (size_t)n * sizeof(double)), "cudaMalloc")) ||
        (rc = cuda_check(cudaMalloc(&dout.p, (size_t)4 * n * sizeof(double)), "cudaMalloc")) ||
        (rc = cuda_check(cudaMemcpy(dx.p, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice), "H2D")))
        return rc;
    if ((rc = launch_debug_pow(static_cast<double*>(dx.p), n, static_cast<double*>(dout.p), nullptr))) return rc;
    return cuda_check(cudaMemcpy(out, dout.p, (size_t)4 * n * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
}

// Device evaluation of a binary operation of the solver on n host pairs:
// `cols` result columns of n doubles each (launch writes them).
template <class L>
static int debug_binary(const double* a, const double* b, int n, double* out, int cols, L launch)
{
    if (n < 0 || (n > 0 && (!a || !b || !out))) return set_error(TROUTE_EINVAL, "bad arguments");
    if (n == 0) return TROUTE_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");
    DevPtr da, db, dout;
    int rc;
    const size_t bytes = (size_t)n * sizeof(double);
    if ((rc = cuda_check(cudaMalloc(&da.p, bytes), "cudaMalloc")) || (rc = cuda_check(cudaMalloc(&db.p, bytes), "cudaMalloc")) ||
        (rc = cuda_check(cudaMalloc(&dout.p, cols * bytes), "cudaMalloc")) ||
        (rc = cuda_check(cudaMemcpy(da.p, a, bytes, cudaMemcpyHostToDevice), "H2D")) ||
        (rc = cuda_check(cudaMemcpy(db.p, b, bytes, cudaMemcpyHostToDevice), "H2D")))
        return rc;
    if ((rc = launch(static_cast<double*>(da.p), static_cast<double*>(db.p), n, static_cast<double*>(dout.p))))
        return rc;
    return cuda_check(cudaMemcpy(out, dout.p, cols * bytes, cudaMemcpyDeviceToHost), "D2H");
}

extern "C" int troute_debug_div(const double* a, const double* b, int n, double* out)
{
    return debug_binary(a, b, n, out, 1, [](const double* da, const double* db, int m, double* o) {
        return launch_debug_div(da, db, m, o, nullptr);
    });
}

extern "C" int troute_debug_quot_gt(const double* a, const double* b, double c, int n, int* out)
{
    if (n < 0 || (n > 0 && (!a || !b || !out))) return set_error(TROUTE_EINVAL, "bad arguments");
    if (!(c > 0.0)) return set_error(TROUTE_EINVAL, "c must be > 0");
    if (n == 0) return TROUTE_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");
    DevPtr da, db, dout;
    int rc;
    const size_t bytes = (size_t)n * sizeof(double);
    if ((rc = cuda_check(cudaMalloc(&da.p, bytes), "cudaMalloc")) || (rc = cuda_check(cudaMalloc(&db.p, bytes), "cudaMalloc")) ||
        (rc = cuda_check(cudaMalloc(&dout.p, (size_t)n * sizeof(int)), "cudaMalloc")) ||
        (rc = cuda_check(cudaMemcpy(da.p, a, bytes, cudaMemcpyHostToDevice), "H2D")) ||
        (rc = cuda_check(cudaMemcpy(db.p, b, bytes, cudaMemcpyHostToDevice), "H2D")))
        return rc;
    if ((rc = launch_debug_quot_gt(static_cast<double*>(da.p), static_cast<double*>(db.p), c, n,
                                   static_cast<int*>(dout.p), nullptr)))
        return rc;
    return cuda_check(cudaMemcpy(out, dout.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost), "D2H");
}

// ---------------------------------------------------------------------------
// topology helpers
// ---------------------------------------------------------------------------
extern "C" int troute_levels(int n_reaches, const int* up_ptr, const int* up_idx, int* reach_level,
                             int* level_ptr, int* level_reach, int* n_levels)
{
    if (n_reaches < 0 || (n_reaches > 0 && (!up_ptr || !reach_level || !level_ptr || !level_reach || !n_levels)))
        return set_error(TROUTE_EINVAL, "bad arguments");
    const int R = n_reaches;
    // levels need upstream reaches first; find an order with Kahn's algorithm
    std::vector<int> down(R, -1), indeg(R), order;
    for (int r = 0; r < R; ++r) {
        if (up_ptr[r + 1] < up_ptr[r]) return set_error(TROUTE_ETOPO, "reach_up_ptr not monotone");
        indeg[r] = up_ptr[r + 1] - up_ptr[r];
        for (int k = up_ptr[r]; k < up_ptr[r + 1]; ++k) {
            const int u = up_idx[k];
            if (u < 0 || u >= R || u == r) return set_error(TROUTE_ETOPO, "bad upstream index %d", u);
            if (down[u] >= 0) return set_error(TROUTE_ETOPO, "reach %d drains into two reaches", u);
            down[u] = r;
        }
    }
    for (int r = 0; r < R; ++r)
        if (indeg[r] == 0) order.push_back(r);
    for (size_t i = 0; i < order.size(); ++i) {
        const int d = down[order[i]];
        if (d >= 0 && --indeg[d] == 0) order.push_back(d);
    }
    if ((int)order.size() != R) return set_error(TROUTE_ETOPO, "topology has a cycle");
    int L = 0;
    for (int r : order) {
        int lv = 0;
        for (int k = up_ptr[r]; k < up_ptr[r + 1]; ++k) lv = std::max(lv, reach_level[up_idx[k]] + 1);
        reach_level[r] = lv;
        L = std::max(L, lv + 1);
    }
    // stable grouping by level (numpy argsort(kind="stable") in the reference)
    std::vector<int> cnt(L + 1, 0);
    for (int r = 0; r < R; ++r) cnt[reach_level[r] + 1]++;
    for (int l = 0; l < L; ++l) cnt[l + 1] += cnt[l];
    for (int l = 0; l <= L; ++l) level_ptr[l] = cnt[l];
    std::vector<int> pos(cnt.begin(), cnt.end() - 1);
    for (int r = 0; r < R; ++r) level_reach[pos[reach_level[r]]++] = r;
    *n_levels = L;
    return TROUTE_OK;
}

extern "C" int troute_validate(const troute_topo* topo)
{
    if (!topo) return set_error(TROUTE_EINVAL, "null topology");
    if (topo->n_reaches < 0 || topo->n_segments < 0) return set_error(TROUTE_ETOPO, "negative sizes");
    const int R = topo->n_reaches, S = topo->n_segments;
    if (R == 0) return TROUTE_OK;
    if (!topo->reach_seg_start || !topo->reach_seg_len || !topo->reach_up_ptr)
        return set_error(TROUTE_ETOPO, "null topology array");
    if (topo->reach_up_ptr[0] != 0) return set_error(TROUTE_ETOPO, "reach_up_ptr[0] must be 0");
    if (topo->reach_up_ptr[R] > 0 && !topo->reach_up_idx) return set_error(TROUTE_ETOPO, "null reach_up_idx");
    std::vector<unsigned char> covered((size_t)S, 0);
    for (int r = 0; r < R; ++r) {
        const long long a = topo->reach_seg_start[r], n = topo->reach_seg_len[r];
        if (n < 0 || a < 0 || a + n > S) return set_error(TROUTE_ETOPO, "reach %d segments out of range", r);
        for (long long s = a; s < a + n; ++s) {
            if (covered[s]) return set_error(TROUTE_ETOPO, "segment %lld belongs to two reaches", s);
            covered[s] = 1;
        }
    }
    std::vector<int> lv(R), lp(R + 1), lr(R);
    int L = 0;
    return troute_levels(R, topo->reach_up_ptr, topo->reach_up_idx, lv.data(), lp.data(), lr.data(), &L);
}

// Longest chain of segment solves in the (reach, step) dependency graph of an
// n_ts-step run: item (r, t) follows (r, t - 1) and every (u, t) with u
// upstream of r, and takes seg_len[r] solves in order. Dynamic programme over
// the steps, reaches in level order within a step:
//   L[r] <- seg_len[r] + max(L[r] of step t - 1, max over upstream u of L[u] of step t).
extern "C" int troute_critical_path(const troute_topo* topo, int n_ts, long long* solves)
{
    if (!solves) return set_error(TROUTE_EINVAL, "null argument");
    *solves = 0;
    if (n_ts < 0) return set_error(TROUTE_EINVAL, "negative n_ts");
    int rc = troute_validate(topo);
    if (rc) return rc;
    const int R = topo->n_reaches;
    if (R == 0 || n_ts == 0) return TROUTE_OK;
    std::vector<int> lv(R), lp(R + 1), lr(R);
    int L = 0;
    if ((rc = troute_levels(R, topo->reach_up_ptr, topo->reach_up_idx, lv.data(), lp.data(), lr.data(), &L)))
        return rc;
    std::vector<long long> chain(R, 0);  // longest chain ending with reach r's item of the current step
    long long best = 0;
    for (int t = 0; t < n_ts; ++t) {
        for (int i = 0; i < R; ++i) {  // level order: upstream reaches of this step come first
            const int r = lr[i];
            long long m = chain[r];     // the same reach, previous step
            for (int k = topo->reach_up_ptr[r]; k < topo->reach_up_ptr[r + 1]; ++k)
                m = std::max(m, chain[topo->reach_up_idx[k]]);
            chain[r] = m + topo->reach_seg_len[r];
            best = std::max(best, chain[r]);
        }
    }
    *solves = best;
    return TROUTE_OK;
}

// ---------------------------------------------------------------------------
// one-shot tree routing
// ---------------------------------------------------------------------------
extern "C" int troute_route_tree(const troute_topo* topo, const troute_chparams* params,
                                 const double* qlat_ts, const double* qdp0, const double* dp0,
                                 const double* reach_last0, int n_ts, double dt,
                                 const troute_cfg* cfg,
                                 double* q_out, double* d_out, double* v_out,
                                 double* reach_last_out, troute_stats* stats)
{
    if (!topo || (topo->n_segments > 0 && (!params || !qdp0 || !dp0)))
        return set_error(TROUTE_EINVAL, "null argument");
    troute_handle* h = nullptr;
    int rc = troute_create(&h, topo, params, dt, cfg);
    if (rc) return rc;
    rc = troute_set_state(h, qdp0, dp0, reach_last0);
    if (!rc) rc = troute_run(h, qlat_ts, n_ts, stats);
    if (!rc) rc = troute_get_state(h, q_out, d_out, v_out, reach_last_out);
    troute_destroy(h);
    return rc;
}

extern "C" int troute_mc_route_tree(const troute_topo* topo, const troute_chparams* params,
                                    const double* qlat_ts, const double* qdp0, const double* dp0,
                                    const double* reach_last0, int n_ts, double dt,
                                    const troute_cfg* cfg,
                                    double* q_out, double* d_out, double* v_out,
                                    double* reach_last_out, troute_stats* stats)
{
    return troute_route_tree(topo, params, qlat_ts, qdp0, dp0, reach_last0, n_ts, dt, cfg, q_out, d_out, v_out,
                             reach_last_out, stats);
}

extern "C" int troute_wavefront_fp64(const troute_chparams_f32* params,
                                     const int* reach_seg_start, const int* reach_seg_len,
                                     const int* reach_up_ptr, const int* reach_up_idx,
                                     const int* level_ptr, const int* level_reach,
                                     int n_reaches, int n_levels, int n_segments,
                                     const float* qlat_ts, const float* qdp0_seg,
                                     const float* dp0_seg, const float* reach_last0,
                                     double* qdc_seg_out_d, double* reach_last_out_d,
                                     int n_timesteps, double dt)
{
    if (n_reaches < 0 || n_segments < 0 || n_levels < 0 || n_timesteps < 0)
        return set_error(TROUTE_EINVAL, "negative size");
    if (n_reaches > 0 && (!level_ptr || !level_reach)) return set_error(TROUTE_EINVAL, "null level arrays");
    // The caller's level schedule must be a valid one: every reach listed once,
    // each after all of its upstream reaches (otherwise the reference's
    // single-pass loop would read stale inflows, which this library does not
    // reproduce).
    std::vector<int> lvl_of(n_reaches, -1);
    if (n_reaches > 0) {
        if (level_ptr[0] != 0 || level_ptr[n_levels] != n_reaches)
            return set_error(TROUTE_ETOPO, "level_ptr must span all reaches");
        for (int l = 0; l < n_levels; ++l)
            for (int k = level_ptr[l]; k < level_ptr[l + 1]; ++k) {
                const int r = level_reach[k];
                if (r < 0 || r >= n_reaches || lvl_of[r] >= 0) return set_error(TROUTE_ETOPO, "level_reach is not a permutation");
                lvl_of[r] = l;
            }
        for (int r = 0; r < n_reaches; ++r)
            for (int k = reach_up_ptr[r]; k < reach_up_ptr[r + 1]; ++k) {
                const int u = reach_up_idx[k];
                if (u < 0 || u >= n_reaches || lvl_of[u] >= lvl_of[r])
                    return set_error(TROUTE_ETOPO, "reach %d is scheduled no later than its upstream reach %d", r, u);
            }
    }
    const size_t S = n_segments, R = n_reaches, T = n_timesteps;
    std::vector<troute_chparams> p(S);
    for (size_t s = 0; s < S; ++s) {
        const troute_chparams_f32& a = params[s];
        p[s] = troute_chparams{a.dx, a.bw, a.tw, a.twcc, a.n_ch, a.ncc, a.cs, a.s0};
    }
    std::vector<double> ql(S * T), q0(S), d0(S), rl0(R);
    for (size_t i = 0; i < S * T; ++i) ql[i] = qlat_ts[i];
    for (size_t i = 0; i < S; ++i) { q0[i] = qdp0_seg[i]; d0[i] = dp0_seg[i]; }
    for (size_t i = 0; i < R; ++i) rl0[i] = reach_last0[i];
    troute_topo t{n_reaches, n_segments, reach_seg_start, reach_seg_len, reach_up_ptr, reach_up_idx};
    return troute_route_tree(&t, p.data(), ql.data(), q0.data(), d0.data(), rl0.data(), n_timesteps, dt, nullptr,
                             qdc_seg_out_d, nullptr, nullptr, reach_last_out_d, nullptr);
}
