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
//   rq[i]       ready items in the order they became ready (atomic tail);
//               idle lanes claim slots (atomic head); -1 = not yet written
//   rh[t+1][r]  outflow of reach r at step t of this run, rh[0][r] the
//               outflow of the step before the run (from the 4-slot ring of
//               the handle's state); a whole run is kept, so upstream reaches
//               never wait for downstream ones to consume a value.
// The lane that makes an item ready continues with it itself when it has no
// other work (the downstream item when two became ready), so busy lanes stay
// in their warps and the queue carries only the rest. A warp claims only
// slots that are already written (or that a racing warp is about to see
// written); the run ends when the count of completed items reaches n_items.
// The head sums at a reach use the upstream order of the reference
// (wavefront_mc.cu:525-531), and the solve is lane_solver.cuh's, i.e. the
// reference's arithmetic.
#include "lane_solver.cuh"

namespace tr {

namespace {
constexpr unsigned kFullMask = 0xffffffffu;
constexpr int L_FETCH = L_WAIT;  // claimed a queue slot, waiting for it to be written
constexpr unsigned long long kWakeItems = 16;  // queued items that wake an idle warp
constexpr long long kWakeCycles = 8000;        // ... or this long unclaimed (~4 us)
#ifndef TROUTE_SLEEP_MAX_NS
#define TROUTE_SLEEP_MAX_NS 3200
#endif
constexpr unsigned kSleepMinNs = 200, kSleepMaxNs = TROUTE_SLEEP_MAX_NS;  // idle-warp polling back-off

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

__device__ __forceinline__ unsigned long long ld_volatile_ull(const unsigned long long* p)
{
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}
}  // namespace

// Loads the reach head inflows of (ri, tau) (all its dependencies are
// complete) and starts its first segment.
__device__ __forceinline__ void start_item(Lane& L, int ri, int tau, int t_base, const NetDev& net,
                                           const RunDev& run, const DataflowDev& df, LocalStats& ls,
                                           unsigned int* hist_s, double2* slot)
{
    const int R = net.n_reach_int;
#ifdef TROUTE_CHECK
    // self-check build (the outflow history is NaN-filled before the run):
    // every value (ri, tau) reads must already be written, and its own output
    // slot must not be
    {
        bool ok = !isnan(__ldcg(df.rh + (size_t)tau * R + ri)) && isnan(__ldcg(df.rh + (size_t)(tau + 1) * R + ri));
        for (int j = __ldg(net.up_ptr + ri); j < __ldg(net.up_ptr + ri + 1); ++j) {
            const int u = __ldg(net.up_idx + j);
            ok = ok && !isnan(__ldcg(df.rh + (size_t)tau * R + u)) && !isnan(__ldcg(df.rh + (size_t)(tau + 1) * R + u));
        }
        if (!ok) record_error(run.stats, TROUTE_EINVAL, ri, t_base + tau, 7);
    }
#endif
    L.ri = ri;
    L.tau = tau;
    L.g = t_base + tau;
    L.ns = __ldg(net.nseg + ri);
    L.ub = __ldg(net.up_ptr + ri);
    L.ue = __ldg(net.up_ptr + ri + 1);
    L.dn = __ldg(net.down + ri);
    L.base = __ldg(net.tile_off + ri / kLanes) + (ri % kLanes);
    const double* rprev = df.rh + (size_t)tau * R;
    const double* rcur = df.rh + (size_t)(tau + 1) * R;
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
    L.mode = L_BEGIN;
}

// Threads per block, and the register budget: resident blocks per SM the
// allocation is sized for, or (TROUTE_DF_MAXNREG) a register cap.
#ifndef TROUTE_DF_THREADS
#define TROUTE_DF_THREADS 128
#endif
#ifndef TROUTE_DF_MINB
#define TROUTE_DF_MINB 1
#endif
#ifdef TROUTE_DF_MAXNREG
#define TROUTE_DF_BOUNDS __maxnreg__(TROUTE_DF_MAXNREG)
#else
#define TROUTE_DF_BOUNDS __launch_bounds__(TROUTE_DF_THREADS, TROUTE_DF_MINB)
#endif
constexpr int kDfThreads = TROUTE_DF_THREADS;
static_assert(kDfThreads % 32 == 0 && kDfThreads >= 32 && kDfThreads <= 1024, "whole warps per block");

// Warm-started runs read each solve's learned starting depth from the
// prediction plane the launch's GEMM filled (warm_gemm.cu) when the solve
// begins (lane_solver.cuh, begin_segment): the same kernel serves plain and
// warm-started runs.
__global__ void TROUTE_DF_BOUNDS route_dataflow_kernel(NetDev net, RunDev run, DataflowDev df)
{
    __shared__ unsigned int hist_s[16];
    __shared__ double2 seg_sm[kSegSmemPerThread * kDfThreads];
    double2* const seg_slot = seg_slot_of(seg_sm);
    if (threadIdx.x < 16) hist_s[threadIdx.x] = 0;
    __syncthreads();
    LocalStats ls = {0, 0, 0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt_df();
    const int t_base = __ldg(run.step_base);
    const int T = run.n_ts;
    const int R = net.n_reach_int;
    bool failed = false;
    unsigned long long slot = 0;
    long long queued_since = -1;  // lane 0: when this idle warp first saw unclaimed items
    Lane L;
    L.mode = L_IDLE;
    unsigned long long n_pass = 0, n_busy = 0, n_wait = 0, n_idle = 0, n_solve = 0;
    unsigned idle_ns = kSleepMinNs;  // warp-uniform
    unsigned long long idle_seen = ~0ull;  // warp-uniform: n_done when this warp last saw progress
    long long idle_t0 = clock64();

    while (true) {
        // ---- idle lanes claim queue slots (one atomic per warp) ----
        // A warp claims only as many slots as there are queued items it could
        // take (tail - head), so the ready work lands on few, full warps instead
        // of one lane in each of many warps (a warp pays for every FP64
        // instruction whatever the number of its busy lanes). Two warps can
        // race past the tail; their extra lanes wait for the next items.
        const unsigned idle = __ballot_sync(kFullMask, L.mode == L_IDLE);
        if (idle) {
            // a warp with busy lanes tops itself up with whatever is queued; a
            // warp with none waits until enough is queued to fill a good part
            // of it, or until queued items have not been taken for a while
            const bool has_busy = idle != kFullMask;
            unsigned n = 0;
            unsigned long long base = 0;
            int err = 0;
            if (lane == 0) {
                const unsigned long long tail = ld_volatile_ull(df.rq_tail);
                const unsigned long long head = ld_volatile_ull(df.rq_head);
                err = ld_volatile_int(&run.stats->error);
                if (tail > head) {
                    const unsigned long long avail = tail - head;
                    bool take = has_busy || avail >= kWakeItems;
                    if (!take) {
                        const long long now = clock64();
                        if (queued_since < 0) queued_since = now;
                        take = now - queued_since > kWakeCycles;
                    }
                    if (take) {
                        queued_since = -1;
                        n = (unsigned)min((unsigned long long)__popc(idle), avail);
                        base = atomicAdd(df.rq_head, (unsigned long long)n);
                    }
                } else {
                    queued_since = -1;
                }
            }
            n = __shfl_sync(kFullMask, n, 0);
            base = __shfl_sync(kFullMask, base, 0);
            err = __shfl_sync(kFullMask, err, 0);
            if (err) break;
            if (n && L.mode == L_IDLE) {
                const unsigned rank = __popc(idle & lt);
                // racing warps can push the head past the end of the queue;
                // such slots do not exist and are never read
                if (rank < n && base + rank < df.n_items) {
                    slot = base + rank;
                    L.mode = L_FETCH;
                    L.wait_t0 = clock64();
                    L.wait_tail = 0;
                }
            }
        }
        // the run is over once every (reach, step) item has completed; lanes
        // still holding a claimed slot then leave it (it will not be written)
        if (__ballot_sync(kFullMask, L.mode >= L_SOLVE) == 0) {
            unsigned long long nd = 0;
            if (lane == 0) nd = ld_volatile_ull(df.n_done);
            nd = __shfl_sync(kFullMask, nd, 0);
            if (nd >= df.n_items) break;
            // a warp without work that sees no item complete anywhere for a
            // whole wait budget reports a timeout instead of polling forever
            if (nd != idle_seen) {
                idle_seen = nd;
                idle_t0 = clock64();
            } else if (clock64() - idle_t0 > run.wait_cycles) {
                if (lane == 0) record_error(run.stats, TROUTE_ETIMEOUT, -1, -1, 10);
                break;
            }
        } else {
            idle_t0 = clock64();
        }
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
            const int tau = (int)(raw >> 32);
            if (ri >= 0 && (ri >= R || tau < 0 || tau >= T)) {
                // an entry that names no item of this run: report, never index with it
                record_error(run.stats, TROUTE_EINVAL, ri, tau, 8);
                failed = true;
            } else if (ri >= 0) {
                __threadfence();  // the item's inputs were published before it was queued
                L.ri = ri;
                L.tau = tau;
                L.mode = L_START;
            } else if (clock64() - L.wait_t0 > run.wait_cycles) {
                // a slot can legitimately stay empty for long while the run
                // advances; give up only if no item completed during a whole
                // wait budget
                const unsigned long long nd = ld_volatile_ull(df.n_done);
                if (nd != L.wait_tail) {
                    L.wait_tail = nd;
                    L.wait_t0 = clock64();
                } else {
                    record_error(run.stats, TROUTE_ETIMEOUT, -1, (int)(slot & 0x7fffffff), 6);
                    failed = true;
                }
            }
        }

        // ---- lanes starting an item, then a segment (the one inlined
        // start_item and begin_segment) ----
        if (L.mode == L_START) start_item(L, L.ri, L.tau, t_base, net, run, df, ls, hist_s, seg_slot);
        if (L.mode == L_BEGIN) L.mode = begin_segment(L, net, run, ls, hist_s, seg_slot) ? L_SOLVE : L_DONE;

        // ---- one depth evaluation per solving lane ----
        if (__any_sync(kFullMask, L.mode >= L_SOLVE)) {
            n_solve++;
            lane_pass(L, net, run, ls, hist_s, seg_slot);
        }

        // ---- completed reaches: publish, count dependencies, queue ready items ----
        int npush = 0;
        int2 push0 = make_int2(-1, -1), push1 = make_int2(-1, -1);
        const unsigned dmask = __ballot_sync(kFullMask, L.mode == L_DONE);
        if (dmask && lane == 0) atomicAdd(df.n_done, (unsigned long long)__popc(dmask));
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
            if (npush && df.continue_items) {
                // continue with one newly ready item here (the downstream one when
                // there are two: it lies toward the outlet); queue the other
                __threadfence();  // other dependencies' writes, seen through the counters
                const int2 mine = (npush == 2) ? push1 : push0;
                if (npush == 2) push1 = make_int2(-1, -1);
                --npush;
                // started in the next pass, before its evaluation
                L.ri = mine.x;
                L.tau = mine.y;
                L.mode = L_START;
            }
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
            if (npush && pos + npush > df.n_items) {
                // more items than the run has: an accounting error, never write past the queue
                record_error(run.stats, TROUTE_EINVAL, push0.x, push0.y, 9);
                failed = true;
                npush = 0;
            }
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
        // a warp without solving lanes sleeps before polling again: briefly when
        // it holds claimed slots (their items are about to be written), with a
        // doubling back-off while it finds nothing at all, so that idle warps
        // do not crowd the queue counters' L2 lines while others solve
        if (__ballot_sync(kFullMask, L.mode >= L_SOLVE) == 0) {
            if (__any_sync(kFullMask, L.mode == L_FETCH)) {
                __nanosleep(kSleepMinNs);
            } else {
                __nanosleep(idle_ns);
                idle_ns = idle_ns < kSleepMaxNs ? 2 * idle_ns : kSleepMaxNs;
            }
        } else {
            idle_ns = kSleepMinNs;
        }
    }
    if (lane == 0) {
        atomicAdd(&run.stats->warp_passes, n_pass);
        atomicAdd(&run.stats->lane_busy, n_busy);
        atomicAdd(&run.stats->lane_wait, n_wait);
        atomicAdd(&run.stats->lane_idle, n_idle);
        atomicAdd(&run.stats->solve_passes, n_solve);
    }
    cp_async_wait_all();   // a lane that left an item early may still have its next segment in flight
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
        *df.n_done = 0;
    }
}

int launch_route_dataflow(const NetDev& net, const RunDev& run, const DataflowDev& df, int grid, void* stream)
{
    if (run.warm && !run.start_pred) return set_error(TROUTE_ESTATE, "warm start requested without a prediction plane");
    if (df.n_items == 0) return TROUTE_OK;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
#ifdef TROUTE_CHECK
    if ((e = cudaMemsetAsync(df.rh, 0xff, (size_t)(run.n_ts + 1) * net.n_reach_int * sizeof(double), st)) != cudaSuccess)
        return set_error(TROUTE_ECUDA, "dataflow set-up: %s", cudaGetErrorString(e));
#endif
    if ((e = cudaMemsetAsync(df.cnt, 0, (size_t)run.n_ts * net.n_reach_int * sizeof(int), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(df.rq, 0xff, (size_t)df.n_items * sizeof(int2), st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(df.rq, df.heads, (size_t)df.n_heads * sizeof(int2), cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return set_error(TROUTE_ECUDA, "dataflow set-up: %s", cudaGetErrorString(e));
    int ig = (net.n_reach_int + 255) / 256;
    if (ig > 4096) ig = 4096;
    if (ig < 1) ig = 1;
    dataflow_init_kernel<<<ig, 256, 0, st>>>(net, run, df);
    route_dataflow_kernel<<<grid, kDfThreads, 0, st>>>(net, run, df);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(TROUTE_ECUDA, "route_dataflow_kernel launch: %s", cudaGetErrorString(e));
    return TROUTE_OK;
}

int route_dataflow_threads() { return kDfThreads; }

int route_dataflow_occupancy(int* blocks_per_sm, bool)
{
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, route_dataflow_kernel, kDfThreads, 0);
    if (e != cudaSuccess) return set_error(TROUTE_ECUDA, "occupancy query: %s", cudaGetErrorString(e));
    return TROUTE_OK;
}

}  // namespace tr
