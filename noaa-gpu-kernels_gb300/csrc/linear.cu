// Linearised Muskingum-Cunge: the reference's fast approximate mode
// (water-prediction/t-route/wavefront/linear_mc.cu), with the secant path as
// the yardstick of its error.
//
// Per segment, once: C1..C3 and C4/ql from the channel at a reference depth
// of half bankfull (at least 0.1 m) with X from the Cunge formula at zero
// residual (linear_mc.cu:57-100), FP32. Per step, in topological order:
//   Q_new[i] = C1 Q_up_new + C2 Q_up_old + C3 Q_old[i] + (C4/ql) qlat[i]
// where Q_up is the sum of the upstream reaches' last segments for a reach's
// first segment and the previous segment otherwise (linear_mc.cu:129-165,
// cpu_linear_mc :177-232), FP32 like the reference.
//
// On the GPU the (reach, step) items of a whole run form the same DAG as the
// secant path's; one persistent kernel runs them from a ready queue: a lane
// takes a ready item, routes the reach's segments, publishes the reach
// outflow and queues the items it completes. Each item is a few dozen FP32
// operations, so the queue's atomics set the pace; there are no per-level
// launches (the reference launches one kernel per level per step).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "troute_internal.h"

namespace tr {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// Coefficients of one segment (linear_mc.cu:57-100), FP32 with the reference's
// operation order; powf / sqrtf are CUDA's.
__device__ __forceinline__ float4 lin_coeffs(const troute_chparams_f32& p, float dt)
{
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
    return make_float4((Km * X + dt / 2.0f) / D, (dt / 2.0f - Km * X) / D, (Km * (1.0f - X) - dt / 2.0f) / D, dt / D);
}

__global__ void lin_coeff_kernel(const troute_chparams_f32* __restrict__ p, int n, float dt, float4* __restrict__ c)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) c[i] = lin_coeffs(p[i], dt);
}

struct LinRun {
    int R;
    long long S;
    int T;                          // steps of this launch
    const int* seg_start;
    const int* seg_len;
    const int* up_ptr;
    const int* up_idx;
    const int* down;
    const float4* coef;             // [S] {C1, C2, C3, C4/ql}
    float* Q;                       // [S] discharge, updated in place step by step
    const float* qlat;              // [T][S]
    float* rh;                      // [T+1][R] reach outflow: row 0 before the launch, row t+1 after step t
    int* cnt;                       // [T][R] completed dependencies
    long long* rq;                  // [n_items] packed (step << 32 | reach), -1 = not written
    unsigned long long* rq_head;    // claimed
    unsigned long long* rq_tail;    // reserved
    unsigned long long* n_done;     // completed items
    unsigned long long n_items;
    int* error;                     // 0 ok, TROUTE_ETIMEOUT, TROUTE_EINVAL
    long long wait_cycles;
};

__device__ __forceinline__ unsigned long long ld_vol_ull(const unsigned long long* p)
{
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}

// One (reach, step) item: the reach's segments in order (cpu_linear_mc's
// inner loops, linear_mc.cu:206-224); returns the reach outflow.
__device__ __forceinline__ float lin_item(const LinRun& d, int r, int t)
{
    const float* rprev = d.rh + (size_t)t * d.R;
    const float* rcur = rprev + d.R;
    float sum_new = 0.f, sum_old = 0.f;
    for (int k = __ldg(d.up_ptr + r); k < __ldg(d.up_ptr + r + 1); ++k) {
        const int u = __ldg(d.up_idx + k);
        sum_new += __ldcg(rcur + u);
        sum_old += __ldcg(rprev + u);
    }
    const int s0 = __ldg(d.seg_start + r), sl = __ldg(d.seg_len + r);
    const float* ql = d.qlat + (size_t)t * (size_t)d.S;
    float pn = sum_new, po = sum_old, last = 0.f;
    for (int i = 0; i < sl; ++i) {
        const long long idx = s0 + i;
        const float4 c = __ldg(d.coef + idx);
        const float qo = __ldcg(d.Q + idx);
        const float qn = c.x * pn + c.y * po + c.z * qo + c.w * __ldg(ql + idx);
        __stcg(d.Q + idx, qn);
        pn = qn;
        po = qo;
        last = qn;
    }
    return last;
}

__global__ void __launch_bounds__(128) lin_dataflow_kernel(LinRun d)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    // A lane holds at most one claimed queue slot. Claims are taken only for
    // slots that are (or are about to be) written; a lane whose slot is not
    // yet written keeps it and looks again in the next round, while the other
    // lanes of its warp go on working -- a warp never blocks on one slot.
    unsigned long long slot = 0;
    bool holding = false;
    long long t0 = 0;
    unsigned long long seen = 0;
    unsigned sleep_ns = 64;
    unsigned long long idle_seen = ~0ull;  // warp-uniform: n_done when this warp last saw progress
    long long idle_t0 = clock64();
    while (true) {
        // ---- idle lanes claim queued slots (one atomic per warp) ----
        const unsigned idle = __ballot_sync(kFull, !holding);
        unsigned n = 0;
        unsigned long long base = 0, nd = 0;
        int err = 0;
        if (lane == 0) {
            const unsigned long long tail = ld_vol_ull(d.rq_tail), head = ld_vol_ull(d.rq_head);
            nd = ld_vol_ull(d.n_done);
            err = *reinterpret_cast<volatile int*>(d.error);
            if (idle && tail > head && nd < d.n_items && !err) {
                n = (unsigned)min((unsigned long long)__popc(idle), tail - head);
                base = atomicAdd(d.rq_head, (unsigned long long)n);
            }
        }
        n = __shfl_sync(kFull, n, 0);
        base = __shfl_sync(kFull, base, 0);
        nd = __shfl_sync(kFull, nd, 0);
        err = __shfl_sync(kFull, err, 0);
        // the run is over once every item has completed (claims past the last
        // item are never written and are dropped)
        if (err || nd >= d.n_items) break;
        if (!holding && n) {
            const unsigned rank = __popc(idle & lt);
            if (rank < n && base + rank < d.n_items) {
                slot = base + rank;
                holding = true;
                t0 = clock64();
                seen = nd;
            }
        }
        // ---- lanes whose slot is written take the item ----
        bool have = false;
        int r = -1, t = -1;
        if (holding) {
            const long long v = *reinterpret_cast<const volatile long long*>(d.rq + slot);
            if (v >= 0) {
                r = (int)(v & 0xffffffffll);
                t = (int)(v >> 32);
                holding = false;
                have = true;
                if (r < 0 || r >= d.R || t < 0 || t >= d.T) {
                    atomicCAS(d.error, 0, TROUTE_EINVAL);  // an entry that names no item: never index with it
                    have = false;
                }
            } else if (clock64() - t0 > d.wait_cycles) {
                // a slot may stay empty for long while the run advances; give up
                // only if no item completed during a whole wait budget
                const unsigned long long now_done = ld_vol_ull(d.n_done);
                if (now_done == seen) atomicCAS(d.error, 0, TROUTE_ETIMEOUT);
                seen = now_done;
                t0 = clock64();
            }
        }
        // ---- route the items, publish, count dependencies ----
        int npush = 0;
        long long push0 = -1, push1 = -1;
        if (have) {
            __threadfence();  // the item's inputs were published before it was queued
            const float out = lin_item(d, r, t);
            __stcg(d.rh + (size_t)(t + 1) * d.R + r, out);
            __threadfence();
            const int nup = __ldg(d.up_ptr + r + 1) - __ldg(d.up_ptr + r);
            if (t + 1 < d.T && atomicAdd(d.cnt + (size_t)(t + 1) * d.R + r, 1) + 1 == nup + 1)
                push0 = ((long long)(t + 1) << 32) | (unsigned)r, npush = 1;
            const int dn = __ldg(d.down + r);
            if (dn >= 0) {
                const int need = (__ldg(d.up_ptr + dn + 1) - __ldg(d.up_ptr + dn)) + (t > 0 ? 1 : 0);
                if (atomicAdd(d.cnt + (size_t)t * d.R + dn, 1) + 1 == need) {
                    const long long v = ((long long)t << 32) | (unsigned)dn;
                    if (npush == 0) push0 = v;
                    else push1 = v;
                    ++npush;
                }
            }
        }
        const unsigned done_mask = __ballot_sync(kFull, have);
        // ---- warp-aggregated append of the newly ready items ----
        unsigned total = npush;
        for (int off = 16; off > 0; off >>= 1) total += __shfl_xor_sync(kFull, total, off);
        if (total) {
            unsigned incl = npush;
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned v = __shfl_up_sync(kFull, incl, off);
                if (lane >= off) incl += v;
            }
            unsigned long long pb = 0;
            if (lane == 31) pb = atomicAdd(d.rq_tail, (unsigned long long)total);
            pb = __shfl_sync(kFull, pb, 31);
            const unsigned long long pos = pb + (incl - npush);
            if (npush && pos + npush > d.n_items) {
                atomicCAS(d.error, 0, TROUTE_EINVAL);  // more items than the run has
                npush = 0;
            }
            if (npush >= 1) *reinterpret_cast<volatile long long*>(d.rq + pos) = push0;
            if (npush >= 2) *reinterpret_cast<volatile long long*>(d.rq + pos + 1) = push1;
        }
        if (done_mask && lane == 0) atomicAdd(d.n_done, (unsigned long long)__popc(done_mask));
        // a warp that did nothing this round backs off before polling again;
        // one that has seen no item complete anywhere for a whole wait budget
        // reports a timeout (the run would otherwise never end)
        if (done_mask == 0) {
            if (nd != idle_seen) {
                idle_seen = nd;
                idle_t0 = clock64();
            } else if (clock64() - idle_t0 > d.wait_cycles) {
                if (lane == 0) atomicCAS(d.error, 0, TROUTE_ETIMEOUT);
            }
            __nanosleep(sleep_ns);
            sleep_ns = sleep_ns < 2048 ? 2 * sleep_ns : 2048;
        } else {
            sleep_ns = 64;
            idle_t0 = clock64();
        }
    }
}

// rh[0][r] = discharge of the reach's last segment before the launch.
__global__ void lin_init_kernel(LinRun d)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < d.R; r += gridDim.x * blockDim.x)
        d.rh[r] = d.Q[d.seg_start[r] + d.seg_len[r] - 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *d.rq_head = 0;
        *d.n_done = 0;
    }
}

template <typename T>
struct DArr {
    T* p = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        if (count <= n && p) return TROUTE_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        const cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e != cudaSuccess) return set_error(TROUTE_ENOMEM, "cudaMalloc: %s", cudaGetErrorString(e));
        n = count;
        return TROUTE_OK;
    }
    ~DArr()
    {
        if (p) cudaFree(p);
    }
};

int lin_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return TROUTE_OK;
    return set_error(e == cudaErrorMemoryAllocation ? TROUTE_ENOMEM : TROUTE_ECUDA, "%s: %s", what,
                     cudaGetErrorString(e));
}

}  // namespace
}  // namespace tr

using namespace tr;

struct troute_linear {
    int R = 0;
    long long S = 0;
    std::vector<int> heads;  // reaches without upstream reaches
    DArr<int> seg_start, seg_len, up_ptr, up_idx, down, cnt, err;
    DArr<float4> coef;
    DArr<float> rh, qlat;
    DArr<long long> rq;
    DArr<unsigned long long> ctr;  // head, tail, done
    int grid = 0;
    cudaStream_t stream = nullptr;
    ~troute_linear()
    {
        if (stream) cudaStreamDestroy(stream);
    }
};

extern "C" int troute_linear_coeffs(const troute_chparams_f32* params, int n_segments, double dt, float* c1,
                                    float* c2, float* c3, float* c4oq)
{
    if (n_segments < 0 || !(dt > 0.0)) return set_error(TROUTE_EINVAL, "bad arguments");
    if (n_segments == 0) return TROUTE_OK;
    if (!params || !c1 || !c2 || !c3 || !c4oq) return set_error(TROUTE_EINVAL, "null array");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");
    DArr<troute_chparams_f32> p;
    DArr<float4> c;
    int rc;
    if ((rc = p.alloc(n_segments)) || (rc = c.alloc(n_segments))) return rc;
    if ((rc = lin_cuda(cudaMemcpy(p.p, params, (size_t)n_segments * sizeof *params, cudaMemcpyHostToDevice), "H2D")))
        return rc;
    lin_coeff_kernel<<<std::min(4096, (n_segments + 255) / 256), 256>>>(p.p, n_segments, (float)dt, c.p);
    std::vector<float4> h(n_segments);
    if ((rc = lin_cuda(cudaMemcpy(h.data(), c.p, (size_t)n_segments * sizeof(float4), cudaMemcpyDeviceToHost), "D2H")))
        return rc;
    for (int i = 0; i < n_segments; ++i) {
        c1[i] = h[i].x;
        c2[i] = h[i].y;
        c3[i] = h[i].z;
        c4oq[i] = h[i].w;
    }
    return TROUTE_OK;
}

extern "C" int troute_linear_create(troute_linear** out, const troute_topo* topo, const float* c1, const float* c2,
                                    const float* c3, const float* c4oq)
{
    if (!out || !topo) return set_error(TROUTE_EINVAL, "null argument");
    *out = nullptr;
    int rc = troute_validate(topo);
    if (rc) return rc;
    const int R = topo->n_reaches;
    const long long S = topo->n_segments;
    for (int r = 0; r < R; ++r)
        if (topo->reach_seg_len[r] < 1)
            return set_error(TROUTE_ETOPO, "reach %d has no segments (the linear form needs at least one)", r);
    if (S > 0 && (!c1 || !c2 || !c3 || !c4oq)) return set_error(TROUTE_EINVAL, "null coefficient array");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");
    auto* L = new (std::nothrow) troute_linear();
    if (!L) return set_error(TROUTE_ENOMEM, "handle");
    L->R = R;
    L->S = S;
    std::vector<int> down(R, -1);
    const int nnz = R ? topo->reach_up_ptr[R] - topo->reach_up_ptr[0] : 0;
    for (int r = 0; r < R; ++r) {
        for (int k = topo->reach_up_ptr[r]; k < topo->reach_up_ptr[r + 1]; ++k) down[topo->reach_up_idx[k]] = r;
        if (topo->reach_up_ptr[r + 1] == topo->reach_up_ptr[r]) L->heads.push_back(r);
    }
    std::vector<float4> coef(S);
    for (long long i = 0; i < S; ++i) coef[i] = make_float4(c1[i], c2[i], c3[i], c4oq[i]);
    auto up = [&](auto& arr, const void* src, size_t count, size_t elem) {
        int r2 = arr.alloc(count);
        if (r2) return r2;
        return count ? lin_cuda(cudaMemcpy(arr.p, src, count * elem, cudaMemcpyHostToDevice), "upload") : 0;
    };
    std::vector<int> up_ptr0(R + 1);
    for (int r = 0; r <= R; ++r) up_ptr0[r] = topo->reach_up_ptr[r] - topo->reach_up_ptr[0];
    if ((rc = up(L->seg_start, topo->reach_seg_start, R, 4)) || (rc = up(L->seg_len, topo->reach_seg_len, R, 4)) ||
        (rc = up(L->up_ptr, up_ptr0.data(), R + 1, 4)) ||
        (rc = up(L->up_idx, topo->reach_up_idx + topo->reach_up_ptr[0], nnz, 4)) ||
        (rc = up(L->down, down.data(), R, 4)) || (rc = up(L->coef, coef.data(), S, sizeof(float4))) ||
        (rc = L->ctr.alloc(3)) || (rc = L->err.alloc(1)) ||
        (rc = lin_cuda(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking), "stream"))) {
        delete L;
        return rc;
    }
    int dev = 0, sms = 0, bps = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, lin_dataflow_kernel, 128, 0);
    L->grid = std::max(1, sms * std::max(1, bps));
    *out = L;
    return TROUTE_OK;
}

extern "C" int troute_linear_destroy(troute_linear* L)
{
    delete L;
    return TROUTE_OK;
}

// Steps per launch: the per-step scratch (counters, queue, outflow history,
// ~16 B per reach-step) within a quarter of the free memory, at most 1024.
static int lin_chunk(const troute_linear* L, int n_ts)
{
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) fr = (size_t)4 << 30;
    const double per = 16.0 * std::max(1, L->R);
    const long long fit = (long long)((double)(fr / 4) / per);
    return (int)std::max<long long>(1, std::min<long long>({(long long)n_ts, fit, 1024}));
}

extern "C" int troute_linear_run_device(troute_linear* L, const float* qlat_dev, int n_ts, float* q_dev,
                                        long long wait_cycles, void* stream)
{
    if (!L) return set_error(TROUTE_EINVAL, "null handle");
    if (n_ts < 0) return set_error(TROUTE_EINVAL, "n_ts < 0");
    if (n_ts == 0 || L->R == 0) return TROUTE_OK;
    if (!qlat_dev || !q_dev) return set_error(TROUTE_EINVAL, "null device array");
    const cudaStream_t st = stream ? (cudaStream_t)stream : L->stream;
    const int chunk = lin_chunk(L, n_ts);
    const size_t R = (size_t)L->R;
    int rc;
    if ((rc = L->cnt.alloc(chunk * R)) || (rc = L->rh.alloc((chunk + 1) * R)) || (rc = L->rq.alloc(chunk * R)))
        return rc;
    if ((rc = lin_cuda(cudaMemsetAsync(L->err.p, 0, sizeof(int), st), "memset"))) return rc;
    for (int t0 = 0; t0 < n_ts; t0 += chunk) {
        const int T = std::min(chunk, n_ts - t0);
        LinRun d;
        d.R = L->R;
        d.S = L->S;
        d.T = T;
        d.seg_start = L->seg_start.p;
        d.seg_len = L->seg_len.p;
        d.up_ptr = L->up_ptr.p;
        d.up_idx = L->up_idx.p;
        d.down = L->down.p;
        d.coef = L->coef.p;
        d.Q = q_dev;
        d.qlat = qlat_dev + (size_t)t0 * (size_t)L->S;
        d.rh = L->rh.p;
        d.cnt = L->cnt.p;
        d.rq = L->rq.p;
        d.rq_head = L->ctr.p;
        d.rq_tail = L->ctr.p + 1;
        d.n_done = L->ctr.p + 2;
        d.n_items = (unsigned long long)R * (unsigned long long)T;
        d.error = L->err.p;
        d.wait_cycles = wait_cycles > 0 ? wait_cycles : 8000000000LL;
        const unsigned long long tail0 = L->heads.size();
        cudaError_t e;
        if ((e = cudaMemsetAsync(L->cnt.p, 0, (size_t)T * R * sizeof(int), st)) != cudaSuccess ||
            (e = cudaMemsetAsync(L->rq.p, 0xff, (size_t)T * R * sizeof(long long), st)) != cudaSuccess)
            return lin_cuda(e, "linear set-up");
        // headwater items of step 0 at the queue front (host-built, pageable copy)
        std::vector<long long> hq(L->heads.begin(), L->heads.end());
        if (!hq.empty() &&
            (e = cudaMemcpyAsync(L->rq.p, hq.data(), hq.size() * sizeof(long long), cudaMemcpyHostToDevice, st)) !=
                cudaSuccess)
            return lin_cuda(e, "linear set-up");
        if ((e = cudaMemcpyAsync(L->ctr.p + 1, &tail0, sizeof tail0, cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return lin_cuda(e, "linear set-up");
        lin_init_kernel<<<std::min<int>(4096, (int)((R + 255) / 256)), 256, 0, st>>>(d);
        lin_dataflow_kernel<<<L->grid, 128, 0, st>>>(d);
        if ((e = cudaGetLastError()) != cudaSuccess) return lin_cuda(e, "linear launch");
        // the pageable copies above complete before this call returns; keep hq alive until then
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return lin_cuda(e, "linear run");
    }
    int err = 0;
    if ((rc = lin_cuda(cudaMemcpy(&err, L->err.p, sizeof err, cudaMemcpyDeviceToHost), "status"))) return rc;
    if (err == TROUTE_ETIMEOUT) return set_error(TROUTE_ETIMEOUT, "linear routing: a device wait ran out");
    if (err) return set_error(err, "linear routing: device reported error %d", err);
    return TROUTE_OK;
}

extern "C" int troute_linear_route(const troute_topo* topo, const float* c1, const float* c2, const float* c3,
                                   const float* c4oq, const float* qlat_ts, const float* q0, int n_ts, float* q_out)
{
    if (!topo || n_ts < 0) return set_error(TROUTE_EINVAL, "bad arguments");
    const long long S = topo->n_segments;
    if (S > 0 && (!q0 || !q_out || (n_ts > 0 && !qlat_ts))) return set_error(TROUTE_EINVAL, "null array");
    troute_linear* L = nullptr;
    int rc = troute_linear_create(&L, topo, c1, c2, c3, c4oq);
    if (rc) return rc;
    DArr<float> q, ql;
    if ((rc = q.alloc(S)) || (rc = ql.alloc((size_t)n_ts * S)) ||
        (rc = lin_cuda(cudaMemcpy(q.p, q0, S * sizeof(float), cudaMemcpyHostToDevice), "H2D")) ||
        (rc = lin_cuda(cudaMemcpy(ql.p, qlat_ts, (size_t)n_ts * S * sizeof(float), cudaMemcpyHostToDevice), "H2D")) ||
        (rc = troute_linear_run_device(L, ql.p, n_ts, q.p, 0, nullptr)) ||
        (rc = lin_cuda(cudaMemcpy(q_out, q.p, S * sizeof(float), cudaMemcpyDeviceToHost), "D2H"))) {
        troute_linear_destroy(L);
        return rc;
    }
    troute_linear_destroy(L);
    return TROUTE_OK;
}
