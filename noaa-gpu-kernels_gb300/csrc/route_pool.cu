// Persistent time-skewed tree routing with per-lane work refill.
//
// Same schedule, dependencies, flags and outflow ring as route_kernel
// (kernels.cu), but a warp no longer works on one 32-reach item until its
// slowest lane is done. The secant iteration count of a segment solve is
// heavy-tailed (a few solves restart with a widened bracket and run hundreds
// of iterations), so a warp bound to one item idles most of its lanes. Here
// every lane runs a small state machine and each pass of the warp's loop does,
// for every busy lane, exactly one depth evaluation (channel geometry and the
// R^(2/3), R^(5/3) powers) plus the secant bookkeeping around it:
//   WAIT   poll the readiness counters of the reach's inputs (non-blocking)
//   SOLVE  one evaluation: at h_0 when starting or restarting a solve,
//          otherwise at h followed by the secant update and stop test
//   VEL    the R^(2/3) of the trapezoid radius for the velocity, then store
//          the segment and start the next one (or publish the reach)
// Lanes that finish take the next (reach, step) from a per-warp queue in shared
// memory, which the warp refills one ticket (one level-block) at a time in the
// global wave order. The arithmetic of a solve is exactly mc_solve's
// (mc_solve.cuh), split at its evaluations.
//
// Progress: a lane only waits for (reach, step) items whose tickets are
// smaller than its own; those were handed to lanes that are running, and a
// waiting lane never stops the rest of its warp, so the smallest outstanding
// ticket always advances. Every wait is bounded by RunDev::wait_cycles.
#include "lane_solver.cuh"

namespace tr {

namespace {

constexpr int kQCap = 64;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace

__device__ __forceinline__ void publish(Lane& L, const NetDev& net)
{
    __stcg(net.ring + (size_t)(L.g % kRing) * net.n_reach_int + L.ri, L.q_last);
    __threadfence();
    st_release(net.done + L.ri, L.g + 1);
}

__global__ void __launch_bounds__(128) route_pool_kernel(NetDev net, RunDev run)
{
    __shared__ unsigned int hist_s[16];
    __shared__ double2 seg_sm[kSegSmemPerThread * 128];
    double2* const slot = seg_slot_of(seg_sm);
    __shared__ int2 queue[4][kQCap];
    if (threadIdx.x < 16) hist_s[threadIdx.x] = 0;
    __syncthreads();
    LocalStats ls = {0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    int2* Q = queue[threadIdx.x >> 5];
    const unsigned lt = lanemask_lt();
    const int t_base = __ldg(run.step_base);
    const int T = run.n_ts;
    unsigned q_head = 0, q_tail = 0;  // warp-uniform
    bool exhausted = false;
    bool failed = false;
    Lane L;
    L.mode = L_IDLE;
    unsigned long long n_pass = 0, n_busy = 0, n_wait = 0, n_idle = 0, n_solve = 0;  // lane 0's tallies

    while (true) {
        // ---- refill the warp queue with one level-block when lanes are idle ----
        const unsigned idle = __ballot_sync(kFull, L.mode == L_IDLE);
        unsigned pending = q_tail - q_head;
        if (idle && !exhausted && pending < (unsigned)__popc(idle) && pending + kLanes <= kQCap) {
            unsigned long long k = 0;
            int err = 0;
            if (lane == 0) {
                k = atomicAdd(run.ticket, 1ull);
                err = ld_volatile_int(&run.stats->error);
            }
            k = __shfl_sync(kFull, k, 0);
            err = __shfl_sync(kFull, err, 0);
            if (err) break;
            if (k >= run.n_tickets) {
                exhausted = true;
            } else {
                const int w = find_wave(run.wave_ptr, run.n_waves, k);
                const int lo_level = max(0, w - T + 1);
                const int b = __ldg(net.lb_ptr + lo_level) + (int)(k - __ldg(run.wave_ptr + w));
                const int tau = w - __ldg(net.block_level + b);
                const int rj = b * kLanes + lane;
                const bool real = __ldg(net.nseg + rj) >= 0;
                const unsigned rmask = __ballot_sync(kFull, real);
                if (real) Q[(q_tail + __popc(rmask & lt)) % kQCap] = make_int2(rj, tau);
                q_tail += __popc(rmask);
                __syncwarp();
            }
        }
        pending = q_tail - q_head;
        if (idle && pending) {
            const unsigned rank = __popc(idle & lt);
            if (L.mode == L_IDLE && rank < pending) {
                const int2 e = Q[(q_head + rank) % kQCap];
                L.ri = e.x;
                L.tau = e.y;
                L.g = t_base + L.tau;
                L.ns = __ldg(net.nseg + L.ri);
                L.ub = __ldg(net.up_ptr + L.ri);
                L.ue = __ldg(net.up_ptr + L.ri + 1);
                L.dn = __ldg(net.down + L.ri);
                L.base = __ldg(net.tile_off + L.ri / kLanes) + (L.ri % kLanes);
                L.wait_t0 = clock64();
                L.mode = L_WAIT;
            }
            q_head += min(pending, (unsigned)__popc(idle));
        }
        __syncwarp();
        if (__ballot_sync(kFull, L.mode != L_IDLE) == 0 && exhausted) break;

        {
            const unsigned wmask = __ballot_sync(kFull, L.mode == L_WAIT);
            const unsigned bmask = __ballot_sync(kFull, L.mode >= L_SOLVE);
            n_pass++;
            n_wait += __popc(wmask);
            n_busy += __popc(bmask);
            n_idle += 32 - __popc(wmask | bmask);
        }
        // ---- waiting lanes: inputs ready? ----
        if (L.mode == L_WAIT) {
            bool ready = ld_acquire(net.done + L.ri) >= L.g;
            for (int j = L.ub; ready && j < L.ue; ++j) ready = ld_acquire(net.done + __ldg(net.up_idx + j)) >= L.g + 1;
            if (ready && L.dn >= 0) ready = ld_acquire(net.done + L.dn) >= L.g - kRing + 2;
            if (ready) {
                const double* ring_prev = net.ring + (size_t)((L.g + kRing - 1) % kRing) * net.n_reach_int;
                const double* ring_cur = net.ring + (size_t)(L.g % kRing) * net.n_reach_int;
                L.qup_head = 0.0;
                L.quc_head = 0.0;
                for (int j = L.ub; j < L.ue; ++j) {
                    const int u = __ldg(net.up_idx + j);
                    L.qup_head += __ldcg(ring_prev + u);
                    L.quc_head += __ldcg(ring_cur + u);
                }
                L.q_up_old = 0.0;
                L.q_up_new = 0.0;
                L.q_last = 0.0;
                L.i = 0;
                L.mode = L_BEGIN;
            } else if (clock64() - L.wait_t0 > run.wait_cycles) {
                record_error(run.stats, TROUTE_ETIMEOUT, L.ri, L.g, 1);
                failed = true;
            }
        }

        // ---- lanes starting a segment (the one inlined begin_segment) ----
        if (L.mode == L_BEGIN) {
            if (begin_segment(L, net, run, ls, hist_s, slot)) {
                L.mode = L_SOLVE;
            } else {
                publish(L, net);
                L.mode = L_IDLE;
            }
        }

        // ---- one evaluation per busy lane ----
        const unsigned active = __ballot_sync(kFull, L.mode >= L_SOLVE);
        if (active == 0) {
            if (__any_sync(kFull, failed)) break;
            __nanosleep(128);
            continue;
        }
        n_solve++;
        lane_pass(L, net, run, ls, hist_s, slot);
        if (L.mode == L_DONE) {
            publish(L, net);
            L.mode = L_IDLE;
        }
        if (__any_sync(kFull, failed)) break;
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

int launch_route_pool(const NetDev& net, const RunDev& run, int grid, int threads, void* stream)
{
    if (run.n_tickets == 0) return TROUTE_OK;
    if (threads != 128) threads = 128;  // the per-warp queues assume 4 warps per block
    route_pool_kernel<<<grid, threads, 0, (cudaStream_t)stream>>>(net, run);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(TROUTE_ECUDA, "route_pool_kernel launch: %s", cudaGetErrorString(e));
    return TROUTE_OK;
}

int route_pool_occupancy(int* blocks_per_sm)
{
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, route_pool_kernel, 128, 0);
    if (e != cudaSuccess) return set_error(TROUTE_ECUDA, "occupancy query: %s", cudaGetErrorString(e));
    return TROUTE_OK;
}

}  // namespace tr
