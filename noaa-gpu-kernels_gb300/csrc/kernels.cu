// CUDA kernels of the MC routing path (sm_103a).
//
// route_kernel: the whole multi-step run of a river network (or a batch of
// networks) in ONE persistent launch. The work items are (level-block, step)
// pairs; a level-block is up to 32 reaches of one schedule level, one reach per
// lane. Items are handed out through a global ticket counter in "wave" order
// w = step + level, where the level is the reach's ALAP level (distance from
// its outlet, counted down from the deepest level). That order is a
// topological order of the (reach, step) dependency graph:
//   (r, t) needs (u, t) for every upstream reach u   [current inflow, quc]
//             and (r, t-1)                            [own previous state]
// so a warp only ever waits for items handed out before its own, and the run
// needs no grid-wide barrier: reach r at step t starts as soon as its own
// inputs are ready (time-skewed dataflow, the critical path is ~levels + steps
// instead of levels x steps as in the reference's per-level launches,
// wavefront/wavefront_mc.cu:737-755, or grid.sync per level,
// wavefront/wavefront_persistent.cu:155-189).
// Readiness is a per-reach counter of completed steps (release/acquire at GPU
// scope). Each reach publishes its outflow for step t into a 4-deep ring; a
// reach may overwrite slot t%4 only once its downstream reach has consumed step
// t-3, which with ALAP levels is a wait that is already satisfied in practice.
// Every wait is bounded by RunDev::wait_cycles; on expiry the kernel records
// TROUTE_ETIMEOUT and every warp returns.
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "fpbits.cuh"

namespace tr {

// ---------------------------------------------------------------------------
// Reach-parallel single step: the drop-in for kernel_mc_gpu / cpu_mc
// (troute_mc_final.cu:141-164, :167-252). One thread per reach, segments in
// sequence, the first segment's current inflow seeded by uq. Parameters are
// read in the caller's AoS layout (64-byte records).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) reach_parallel_kernel(
    const troute_chparams* __restrict__ p, const double* __restrict__ ql,
    const int* __restrict__ rs, const int* __restrict__ rl,
    const double* __restrict__ qu, const double* __restrict__ qd,
    const double* __restrict__ dp, double* __restrict__ qo, double* __restrict__ vo,
    double* __restrict__ dpo, double uq, double dt, int nr, int n_segments, Tol tol,
    DevStats* stats)
{
    __shared__ unsigned int hist_s[16];
    if (threadIdx.x < 16) hist_s[threadIdx.x] = 0;
    __syncthreads();
    LocalStats ls = {0, 0, 0, 0};
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nr; r += gridDim.x * blockDim.x) {
        const int start = rs[r], ns = rl[r];
        if (start < 0 || ns < 0 || (long long)start + ns > (long long)n_segments) {
            record_error(stats, TROUTE_EINVAL, r, 0, 4);
            continue;
        }
        double quc = uq;
        for (int i = 0; i < ns; ++i) {
            const int s = start + i;
            const SegP sp = derive_seg(p[s]);
            const SolveOut o = mc_solve(dt, qu[s], quc, qd[s], ql[s], sp, dp[s], tol);
            qo[s] = o.q;
            vo[s] = o.vel;
            dpo[s] = o.depth;
            quc = o.q;
            count_solve(ls, hist_s, o);
        }
    }
    flush_stats(ls, hist_s, stats);
}

// ---------------------------------------------------------------------------
// Persistent time-skewed tree routing.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) route_kernel(NetDev net, RunDev run)
{
    __shared__ unsigned int hist_s[16];
    if (threadIdx.x < 16) hist_s[threadIdx.x] = 0;
    __syncthreads();
    LocalStats ls = {0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    const int t_base = __ldg(run.step_base);
    const int T = run.n_ts;

    while (true) {
        unsigned long long k = 0;
        if (lane == 0) k = atomicAdd(run.ticket, 1ull);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= run.n_tickets) break;
        int failed = (lane == 0) ? ld_volatile_int(&run.stats->error) : 0;
        if (__shfl_sync(0xffffffffu, failed, 0) != 0) break;

        const int w = find_wave(run.wave_ptr, run.n_waves, k);
        const int lo_level = max(0, w - T + 1);
        const int b = __ldg(net.lb_ptr + lo_level) + (int)(k - __ldg(run.wave_ptr + w));
        const int level = __ldg(net.block_level + b);
        const int tau = w - level;            // step within this run
        const int g = t_base + tau;            // cumulative step index
        const int ri = b * kLanes + lane;
        const int ns = __ldg(net.nseg + ri);
        bool ok = true;

        if (ns >= 0) {
            // ---- wait for inputs ----
            if (!wait_at_least(net.done + ri, g, run.wait_cycles, run.stats)) {
                record_error(run.stats, TROUTE_ETIMEOUT, ri, g, 1);
                ok = false;
            }
            const int ub = __ldg(net.up_ptr + ri), ue = __ldg(net.up_ptr + ri + 1);
            for (int j = ub; ok && j < ue; ++j) {
                const int u = __ldg(net.up_idx + j);
                if (!wait_at_least(net.done + u, g + 1, run.wait_cycles, run.stats)) {
                    record_error(run.stats, TROUTE_ETIMEOUT, ri, g, 2);
                    ok = false;
                }
            }
            const int dn = __ldg(net.down + ri);
            if (ok && dn >= 0 && !wait_at_least(net.done + dn, g - kRing + 2, run.wait_cycles, run.stats)) {
                record_error(run.stats, TROUTE_ETIMEOUT, ri, g, 3);
                ok = false;
            }
            if (ok) {
                // ---- reach head inflow: sums over upstream reaches of the
                // previous- and current-step outflow (wavefront_mc.cu:525-531) ----
                const double* ring_prev = net.ring + (size_t)((g + kRing - 1) % kRing) * net.n_reach_int;
                const double* ring_cur = net.ring + (size_t)(g % kRing) * net.n_reach_int;
                double qup_head = 0.0, quc_head = 0.0;
                for (int j = ub; j < ue; ++j) {
                    const int u = __ldg(net.up_idx + j);
                    qup_head += __ldcg(ring_prev + u);
                    quc_head += __ldcg(ring_cur + u);
                }
                const long long base = __ldg(net.tile_off + b) + lane;
                const double* qlat_row = run.qlat + (size_t)tau * (size_t)run.qlat_ld;
                double q_up_old = 0.0;   // previous-step discharge of segment i-1
                double q_up_new = 0.0;   // this step's discharge of segment i-1
                double q_last = 0.0;
                for (int i = 0; i < ns; ++i) {
                    const long long s = base + (long long)i * kLanes;
                    const double qdp = __ldcg(net.q + s);
                    const double dpp = __ldcg(net.d + s);
                    const double ql = __ldg(qlat_row + __ldg(&net.seg[s].qcol)) * __ldg(&net.seg[s].qscale);
                    const SegP sp = load_seg(net, s);
                    const double qup = (i == 0) ? qup_head : q_up_old;
                    const double quc = (i == 0) ? quc_head : q_up_new;
                    const SolveOut o = mc_solve(run.dt, qup, quc, qdp, ql, sp, dpp, run.tol);
                    __stcg(net.q + s, o.q);
                    __stcg(net.d + s, o.depth);
                    __stcg(net.v + s, o.vel);
                    if (run.q_hist) __stcg(run.q_hist + (size_t)tau * (size_t)net.n_seg_int + s, o.q);
                    q_up_old = qdp;
                    q_up_new = o.q;
                    q_last = o.q;
                    count_solve(ls, hist_s, o);
                }
                __stcg(net.ring + (size_t)(g % kRing) * net.n_reach_int + ri, q_last);
                __threadfence();
                st_release(net.done + ri, g + 1);
            }
        }
        if (__any_sync(0xffffffffu, !ok)) break;
    }
    flush_stats(ls, hist_s, run.stats);
}

__global__ void bump_steps_kernel(int* step_base, int n_ts) { *step_base += n_ts; }

__global__ void fill_int_kernel(int* p, long long n, const int* value_dev, int value_host)
{
    const int v = value_dev ? *value_dev : value_host;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void scatter_kernel(const double* __restrict__ src, const long long* __restrict__ map,
                               long long n, double* __restrict__ dst)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dst[map[i]] = src[i];
}

__global__ void gather_kernel(const double* __restrict__ src, const long long* __restrict__ map,
                              long long n, double* __restrict__ dst)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[map[i]];
}

// A wait on a flag that nothing sets: exercises the bounded-wait path (the
// kernel must come back with TROUTE_ETIMEOUT, the context must stay usable).
__global__ void timeout_probe_kernel(DevStats* st, long long wait_cycles)
{
    __shared__ int never;
    if (threadIdx.x == 0) never = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        const long long t0 = clock64();
        while (*reinterpret_cast<volatile int*>(&never) == 0) {
            __nanosleep(256);
            if (clock64() - t0 > wait_cycles) {
                record_error(st, TROUTE_ETIMEOUT, -1, -1, 5);
                break;
            }
        }
    }
}

// Velocity of every segment from its final depth, the reference's formula
// (troute_mc_final.cu:132-136; zero for the invalid-parameter exit, :54-56).
// The per-lane kernels store discharge and depth only; velocity feeds no later
// solve, so it is derived once per run here.
__global__ void velocity_kernel(NetDev net)
{
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < net.n_seg_int;
         s += (long long)gridDim.x * blockDim.x) {
        const SegP p = load_seg(net, s);
        double vel = 0.0;
        if (!(p.n_ch <= 0.0 || p.s0 <= 0.0 || p.z <= 0.0 || p.bw <= 0.0)) {
            const double h = __ldcg(net.d + s);
            const double twl = p.bw + p.z2 * h;
            double Rv = (h * (p.bw + twl) / 2.0) /
                        (p.bw + 2.0 * sqrt(((twl - p.bw) / 2.0) * ((twl - p.bw) / 2.0) + h * h));
            if (Rv < 0.0) Rv = 0.0;
            vel = (1.0 / p.n_ch) * pow23(Rv) * p.sq_s0;
        }
        __stcg(net.v + s, vel);
    }
}

__global__ void debug_div_kernel(const double* __restrict__ a, const double* __restrict__ b, int n,
                                 double* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = shared_div(a[i], shared_rcp(b[i]));
}

__global__ void debug_quot_gt_kernel(const double* __restrict__ a, const double* __restrict__ b, double c, int n,
                                     int* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = quot_gt_pos(a[i], b[i], c) ? 1 : 0;
}

__global__ void debug_pow_kernel(const double* __restrict__ x, int n, double* __restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double a, b;
        pow23_53(x[i], &a, &b);
        out[i] = a;
        out[n + i] = b;
        out[2 * n + i] = pow(x[i], 2.0 / 3.0);
        out[3 * n + i] = pow(x[i], 5.0 / 3.0);
    }
}

static int cuda_status(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return TROUTE_OK;
    return set_error(TROUTE_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

static int grid_for(long long n, int threads)
{
    long long g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > 65535LL * 8) g = 65535LL * 8;
    return (int)g;
}

int launch_reach_parallel(const troute_chparams* p, const double* ql, const int* rs,
                          const int* rl, const double* qu, const double* qd, const double* dp,
                          double* qo, double* vo, double* dpo, double uq, double dt, int nr,
                          int n_segments, const Tol& tol, DevStats* stats, int threads,
                          void* stream)
{
    if (nr <= 0) return TROUTE_OK;
    if (threads <= 0) threads = 128;
    reach_parallel_kernel<<<grid_for(nr, threads), threads, 0, (cudaStream_t)stream>>>(
        p, ql, rs, rl, qu, qd, dp, qo, vo, dpo, uq, dt, nr, n_segments, tol, stats);
    return cuda_status(cudaGetLastError(), "reach_parallel_kernel launch");
}

int route_occupancy(int threads, int* blocks_per_sm)
{
    return cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, route_kernel, threads, 0),
                       "occupancy query");
}

int launch_route(const NetDev& net, const RunDev& run, int grid, int threads, void* stream)
{
    if (run.n_tickets == 0) return TROUTE_OK;
    route_kernel<<<grid, threads, 0, (cudaStream_t)stream>>>(net, run);
    return cuda_status(cudaGetLastError(), "route_kernel launch");
}

int launch_bump_steps(int* step_base, int n_ts, void* stream)
{
    bump_steps_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(step_base, n_ts);
    return cuda_status(cudaGetLastError(), "bump_steps launch");
}

int launch_fill_int(int* p, long long n, const int* value_dev, int value_host, void* stream)
{
    if (n <= 0) return TROUTE_OK;
    fill_int_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(p, n, value_dev, value_host);
    return cuda_status(cudaGetLastError(), "fill launch");
}

int launch_scatter(const double* src, const long long* map, long long n, double* dst, void* stream)
{
    if (n <= 0) return TROUTE_OK;
    scatter_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(src, map, n, dst);
    return cuda_status(cudaGetLastError(), "scatter launch");
}

int launch_gather(const double* src, const long long* map, long long n, double* dst, void* stream)
{
    if (n <= 0) return TROUTE_OK;
    gather_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(src, map, n, dst);
    return cuda_status(cudaGetLastError(), "gather launch");
}

int launch_velocity(const NetDev& net, void* stream)
{
    if (net.n_seg_int <= 0) return TROUTE_OK;
    velocity_kernel<<<grid_for(net.n_seg_int, 256), 256, 0, (cudaStream_t)stream>>>(net);
    return cuda_status(cudaGetLastError(), "velocity launch");
}

int launch_debug_div(const double* a, const double* b, int n, double* out, void* stream)
{
    if (n <= 0) return TROUTE_OK;
    debug_div_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(a, b, n, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(TROUTE_ECUDA, "debug_div_kernel: %s", cudaGetErrorString(e));
    return TROUTE_OK;
}

int launch_debug_quot_gt(const double* a, const double* b, double c, int n, int* out, void* stream)
{
    if (n <= 0) return TROUTE_OK;
    debug_quot_gt_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(a, b, c, n, out);
    return cuda_status(cudaGetLastError(), "debug quotient comparison launch");
}

int launch_debug_pow(const double* x, int n, double* out, void* stream)
{
    if (n <= 0) return TROUTE_OK;
    debug_pow_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(x, n, out);
    return cuda_status(cudaGetLastError(), "debug pow launch");
}

// FP64 issue-rate probe: every thread runs kFp64Chains independent chains of
// multiplications by a and 1/a in turn (the values stay near their start, no
// overflow, no denormals); each chain step is one DMUL warp instruction per
// warp. The sum is stored so nothing is optimised away.
constexpr int kFp64Chains = 8;
__global__ void __launch_bounds__(256) fp64_rate_kernel(double a, double ainv, int iters, double* sink)
{
    double x[kFp64Chains];
#pragma unroll
    for (int c = 0; c < kFp64Chains; ++c) x[c] = 1.0 + 1e-3 * (double)(threadIdx.x * kFp64Chains + c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kFp64Chains; ++c) x[c] = x[c] * a;
#pragma unroll
        for (int c = 0; c < kFp64Chains; ++c) x[c] = x[c] * ainv;
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kFp64Chains; ++c) s += x[c];
    if (s == 12345.678) sink[blockIdx.x] = s;   // never true; keeps the chains live
}

int launch_fp64_rate(int blocks, int iters, double* sink, void* stream, double* warp_instr)
{
    fp64_rate_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(1.0000001, 1.0 / 1.0000001, iters, sink);
    *warp_instr = (double)blocks * (256 / 32) * (double)iters * 2.0 * kFp64Chains;
    return cuda_status(cudaGetLastError(), "fp64 rate launch");
}

int launch_timeout_probe(DevStats* stats, long long wait_cycles, void* stream)
{
    timeout_probe_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(stats, wait_cycles);
    return cuda_status(cudaGetLastError(), "timeout probe launch");
}

}  // namespace tr
