// Persistent tree routing driven by a ready queue (reach-to-warp mapping 3).
//
// The (reach, step) items of a run form a DAG: (r, t) needs (u, t) for every
// upstream reach u (its current-step outflow, the reach head's quc) and
// (r, t-1) (its own previous state). Instead of handing items out in a fixed
// order and letting lanes wait on them, each item carries a counter of
// completed dependencies; the lane that completes the last dependency of an
// item appends the item to a global ready queue, and idle lanes pop only from
// that queue. Lanes therefore only ever hold items whose inputs are final, so
// the warps' FP64 work goes to lanes that are actually solving (a warp issues
// every FP64 instruction at full cost however few of its lanes are busy).
//
//   cnt[t][r]   dependencies of (r, t) completed so far; (r, t) is ready at
//               n_up(r) + (t > 0)
//   rq[i]       ready items in the order they became ready; slot i is claimed
//               by an idle lane (atomic head) before or after it is written
//               (atomic tail); -1 = not yet written
//   rh[t+1][r]  outflow of reach r at step t of this run, rh[0][r] the
//               outflow of the step before the run (from the 4-slot ring of
//               the handle's state); a whole run is kept, so upstream reaches
//               never wait for downstream ones to consume a value.
// Every item is pushed exactly once, so the queue ends with exactly n_items
// entries and a claimed slot is always filled eventually. The head sums at a
// reach use the upstream order of the reference (wavefront_mc.cu:525-531),
// and the solve is lane_solver.cuh's, i.e. the reference's arithmetic.
#include "lane_solver.cuh"

namespace tr {

namespace {
constexpr unsigned kFullMask = 0xffffffffu;
constexpr int L_FETCH = L_WAIT;  // claimed a queue slot, waiting for it to be written

__device__ __forceinline__ unsigned lanemask_lt_df()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ long long ld_volatile_ll(const long long* p)
{
    return *reinterpret_cast<const volatile long long*>(p);
}
}  // namespace

__global__ void __launch_bounds__(128) route_dataflow_kernel(NetDev net, RunDev run, DataflowDev df)
{
    __shared__ unsigned int hist_s[16];
    if (threadIdx.x < 16) hist_s[threadIdx.x] = 0;
    __syncthreads();
    LocalStats ls = {0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt_df();
    const int t_base = __ldg(run.step_base);
    const int T = run.n_ts;
    const int R = net.n_reach_int;
    bool exhausted = false;
    bool failed = false;
    unsigned long long slot = 0;
    Lane L;
    L.mode = L_IDLE;
    unsigned long long n_pass = 0, n_busy = 0, n_wait = 0, n_idle = 0;

    while (true) {
        // ---- idle lanes claim queue slots (one atomic per warp) ----
        const unsigned idle = __ballot_sync(kFullMask, L.mode == L_IDLE);
        if (idle && !exhausted) {
            const unsigned n = __popc(idle);
            unsigned long long base = 0;
            int err = 0;
            if (lane == 0) {
                base = atomicAdd(df.rq_head, (unsigned long long)n);
                err = ld_volatile_int(&run.stats->error);
            }
            base = __shfl_sync(kFullMask, base, 0);
            err = __shfl_sync(kFullMask, err, 0);
            if (err) break;
            if (base + n >= df.n_items) exhausted = true;
            if (L.mode == L_IDLE) {
                const unsigned long long my = base + __popc(idle & lt);
                if (my < df.n_items) {
                    slot = my;
                    L.mode = L_FETCH;
                    L.wait_t0 = clock64();
                }
            }
        }
        if (__ballot_sync(kFullMask, L.mode != L_IDLE) == 0 && exhausted) break;
        {
            const unsigned wmask = __ballot_sync(kFullMask, L.mode == L_FETCH);
            const unsigned bmask = __ballot_sync(kFullMask, L.mode >= L_SOLVE);
            n_pass++;
            n_wait += __popc(wmask);
            n_busy += __popc(bmask);
            n_idle += 32 - __popc(wmask | bmask);
        }

        // ---- lanes with a claimed slot: start the item once it is written ----
        if (L.mode == L_FETCH) {
            const long long raw = ld_volatile_ll(reinterpret_cast<const long long*>(df.rq + slot));
            const int ri = (int)(raw & 0xffffffffll);
            if (ri >= 0) {
                __threadfence();  // the item's inputs were published before it was queued
                L.ri = ri;
                L.tau = (int)(raw >> 32);
                L.g = t_base + L.tau;
                L.ns = __ldg(net.nseg + L.ri);
                L.ub = __ldg(net.up_ptr + L.ri);
                L.ue = __ldg(net.up_ptr + L.ri + 1);
                L.dn = __ldg(net.down + L.ri);
                L.base = __ldg(net.tile_off + L.ri / kLanes) + (L.ri % kLanes);
                const double* rprev = df.rh + (size_t)L.tau * R;
                const double* rcur = df.rh + (size_t)(L.tau + 1) * R;
                L.qup_head = 0.0;
                L.quc_head = 0.0;
                for (int j = L.ub; j < L.ue; ++j) {
                    const int u = __ldg(net.up_idx + j);
                    L.qup_head += __ldcg(rprev + u);
                    L.quc_head += __ldcg(rcur + u);
                }
                L.q_up_old = 0.0;
                L.q_up_new = 0.0;
                L.q_last = 0.0;
                L.i = 0;
                L.mode = begin_segment(L, net, run, ls, hist_s) ? L_SOLVE : L_DONE;
            } else if (clock64() - L.wait_t0 > run.wait_cycles) {
                record_error(run.stats, TROUTE_ETIMEOUT, -1, (int)(slot & 0x7fffffff), 6);
                failed = true;
            }
        }

        // ---- one depth evaluation per solving lane ----
        if (__any_sync(kFullMask, L.mode >= L_SOLVE)) lane_pass(L, net, run, ls, hist_s);

        // ---- completed reaches: publish, count dependencies, queue ready items ----
        int npush = 0;
        int2 push0 = make_int2(-1, -1), push1 = make_int2(-1, -1);
        if (L.mode == L_DONE) {
            __stcg(df.rh + (size_t)(L.tau + 1) * R + L.ri, L.q_last);
            __stcg(net.ring + (size_t)(L.g % kRing) * R + L.ri, L.q_last);
            __threadfence();
            st_release(net.done + L.ri, L.g + 1);
            const int nup = L.ue - L.ub;
            if (L.tau + 1 < T) {
                // own next step: needs its upstream reaches too
                const int old = atomicAdd(df.cnt + (size_t)(L.tau + 1) * R + L.ri, 1);
                if (old + 1 == nup + 1) push0 = make_int2(L.ri, L.tau + 1), npush = 1;
            }
            if (L.dn >= 0) {
                const int need = (__ldg(net.up_ptr + L.dn + 1) - __ldg(net.up_ptr + L.dn)) + (L.tau > 0 ? 1 : 0);
                const int old = atomicAdd(df.cnt + (size_t)L.tau * R + L.dn, 1);
                if (old + 1 == need) {
                    if (npush == 0) push0 = make_int2(L.dn, L.tau);
                    else push1 = make_int2(L.dn, L.tau);
                    ++npush;
                }
            }
            L.mode = L_IDLE;
        }
        // warp-aggregated append to the ready queue
        unsigned total = npush;
        for (int off = 16; off > 0; off >>= 1) total += __shfl_xor_sync(kFullMask, total, off);
        if (total) {
            unsigned incl = npush;
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned v = __shfl_up_sync(kFullMask, incl, off);
                if (lane >= off) incl += v;
            }
            unsigned long long base = 0;
            if (lane == 31) base = atomicAdd(df.rq_tail, (unsigned long long)total);
            base = __shfl_sync(kFullMask, base, 31);
            const unsigned long long pos = base + (incl - npush);
            if (npush) __threadfence();  // every dependency's writes before the item is visible
            if (npush >= 1) {
                const long long v = ((long long)push0.y << 32) | (unsigned)push0.x;
                *reinterpret_cast<volatile long long*>(df.rq + pos) = v;
            }
            if (npush >= 2) {
                const long long v = ((long long)push1.y << 32) | (unsigned)push1.x;
                *reinterpret_cast<volatile long long*>(df.rq + pos + 1) = v;
            }
        }
        if (__any_sync(kFullMask, failed)) break;
        if (__ballot_sync(kFullMask, L.mode >= L_SOLVE) == 0) __nanosleep(64);
    }
    if (lane == 0) {
        atomicAdd(&run.stats->warp_passes, n_pass);
        atomicAdd(&run.stats->lane_busy, n_busy);
        atomicAdd(&run.stats->lane_wait, n_wait);
        atomicAdd(&run.stats->lane_idle, n_idle);
    }
    flush_stats(ls, hist_s, run.stats);
}

// Run set-up on the device: queue tail = number of headwater items (already
// copied to the queue front), rh[0] = outflow of the step before the run.
__global__ void dataflow_init_kernel(NetDev net, RunDev run, DataflowDev df)
{
    const int t_base = *run.step_base;
    const int slot = ((t_base - 1) % kRing + kRing) % kRing;
    const double* src = net.ring + (size_t)slot * net.n_reach_int;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < net.n_reach_int; r += gridDim.x * blockDim.x)
        df.rh[r] = src[r];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *df.rq_head = 0;
        *df.rq_tail = (unsigned long long)df.n_heads;
    }
}

int launch_route_dataflow(const NetDev& net, const RunDev& run, const DataflowDev& df, int grid, void* stream)
{
    if (df.n_items == 0) return TROUTE_OK;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    if ((e = cudaMemsetAsync(df.cnt, 0, (size_t)run.n_ts * net.n_reach_int * sizeof(int), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(df.rq, 0xff, (size_t)df.n_items * sizeof(int2), st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(df.rq, df.heads, (size_t)df.n_heads * sizeof(int2), cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return set_error(TROUTE_ECUDA, "dataflow set-up: %s", cudaGetErrorString(e));
    int ig = (net.n_reach_int + 255) / 256;
    if (ig > 4096) ig = 4096;
    if (ig < 1) ig = 1;
    dataflow_init_kernel<<<ig, 256, 0, st>>>(net, run, df);
    route_dataflow_kernel<<<grid, 128, 0, st>>>(net, run, df);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(TROUTE_ECUDA, "route_dataflow_kernel launch: %s", cudaGetErrorString(e));
    return TROUTE_OK;
}

int route_dataflow_occupancy(int* blocks_per_sm)
{
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, route_dataflow_kernel, 128, 0);
    if (e != cudaSuccess) return set_error(TROUTE_ECUDA, "occupancy query: %s", cudaGetErrorString(e));
    return TROUTE_OK;
}

}  // namespace tr
