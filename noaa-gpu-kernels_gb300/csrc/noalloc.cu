// Reach-parallel MC step that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the point where they route: a host
// model driver or framework that owns every device buffer through its own
// pool (a stray cudaMalloc would sit outside its accounting and could fail
// when the pool has reserved the device's memory), or a hot path where an
// allocation would synchronise the device. For them this entry point runs the
// same per-reach solve as troute_mc_reach_parallel_device but keeps its only
// scratch memory, the per-block solve counters, in a fixed array compiled
// into the library. Every GPU that loads the library holds that array (about
// 1.7 MB) until the process exits. The caller still passes every input and
// output array.
//
// Limits and behaviour:
//  - at most kNoAllocMaxBlocks blocks of kNoAllocThreads reaches, i.e.
//    2,097,152 reaches per call; larger calls are rejected with TROUTE_EINVAL;
//  - the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current;
//  - all calls share the array and it keeps the last call's contents: calls
//    whose kernels overlap on the GPU (other streams, other host threads)
//    race on it. Every counter a call reads is written by that call first, so
//    nothing left from an earlier call leaks in;
//  - a reach whose segment range falls outside [0, n_segments) is skipped and
//    its outputs are left unwritten. Only a call given `stats` waits for the
//    GPU and can report that (TROUTE_EINVAL); without `stats` the call returns
//    as soon as the kernels are queued and cannot see it.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "mc_solve.cuh"

namespace tr {

int check_cfg(const troute_cfg& c);
Tol make_tol(const troute_cfg& c);
int pending_cuda_error(const char* entry);

namespace {

constexpr int kNoAllocThreads = 128;
constexpr int kNoAllocMaxBlocks = 16384;
constexpr int kNoAllocMaxDevices = 64;

// Solve counters of one block (or, in the last slot, of the whole call).
struct NoAllocPartial {
    unsigned long long solves, iterations, retries, early;
    unsigned int hist[16];
    int error, err_reach;
};

static __device__ __align__(256) NoAllocPartial g_noalloc_scratch[kNoAllocMaxBlocks + 1];

std::mutex g_noalloc_mutex;
NoAllocPartial* g_noalloc_ptr[kNoAllocMaxDevices] = {};

__global__ void __launch_bounds__(kNoAllocThreads) noalloc_reach_kernel(
    const troute_chparams* __restrict__ p, const double* __restrict__ ql, const int* __restrict__ rs,
    const int* __restrict__ rl, const double* __restrict__ qu, const double* __restrict__ qd,
    const double* __restrict__ dp, double* __restrict__ qo, double* __restrict__ vo, double* __restrict__ dpo,
    double uq, double dt, int nr, int n_segments, Tol tol, NoAllocPartial* __restrict__ part)
{
    __shared__ unsigned long long s_cnt[4];
    __shared__ unsigned int s_hist[16];
    __shared__ int s_err, s_err_reach;
    if (threadIdx.x < 4) s_cnt[threadIdx.x] = 0;
    if (threadIdx.x < 16) s_hist[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        s_err = 0;
        s_err_reach = -1;
    }
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long solves = 0, iters = 0, retries = 0, early = 0;
    if (r < nr) {
        const int start = rs[r], ns = rl[r];
        if (start < 0 || ns < 0 || (long long)start + ns > (long long)n_segments) {
            if (atomicCAS(&s_err, 0, TROUTE_EINVAL) == 0) s_err_reach = r;
        } else {
            double quc = uq;  // troute_mc_final.cu:153
            for (int i = 0; i < ns; ++i) {
                const int s = start + i;
                const SegP sp = derive_seg(p[s]);
                const SolveOut o = mc_solve(dt, qu[s], quc, qd[s], ql[s], sp, dp[s], tol);
                qo[s] = o.q;
                vo[s] = o.vel;
                dpo[s] = o.depth;
                quc = o.q;
                ++solves;
                iters += (unsigned)o.iters;
                retries += (unsigned)o.retried;
                early += (unsigned)o.early;
                atomicAdd(&s_hist[o.iters < 15 ? o.iters : 15], 1u);
            }
        }
    }
    atomicAdd(&s_cnt[0], solves);
    atomicAdd(&s_cnt[1], iters);
    atomicAdd(&s_cnt[2], retries);
    atomicAdd(&s_cnt[3], early);
    __syncthreads();
    if (threadIdx.x == 0) {
        NoAllocPartial& o = part[blockIdx.x];
        o.solves = s_cnt[0];
        o.iterations = s_cnt[1];
        o.retries = s_cnt[2];
        o.early = s_cnt[3];
        for (int k = 0; k < 16; ++k) o.hist[k] = s_hist[k];
        o.error = s_err;
        o.err_reach = s_err_reach;
    }
}

// Sums the per-block counters into the last slot (one block).
__global__ void noalloc_reduce_kernel(NoAllocPartial* part, int nblocks)
{
    __shared__ unsigned long long s[4];
    __shared__ unsigned int h[16];
    __shared__ int err, err_reach;
    if (threadIdx.x < 4) s[threadIdx.x] = 0;
    if (threadIdx.x < 16) h[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        err = 0;
        err_reach = -1;
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        const NoAllocPartial& q = part[b];
        atomicAdd(&s[0], q.solves);
        atomicAdd(&s[1], q.iterations);
        atomicAdd(&s[2], q.retries);
        atomicAdd(&s[3], q.early);
        for (int k = 0; k < 16; ++k)
            if (q.hist[k]) atomicAdd(&h[k], q.hist[k]);
        if (q.error && atomicCAS(&err, 0, q.error) == 0) err_reach = q.err_reach;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        NoAllocPartial& o = part[kNoAllocMaxBlocks];
        o.solves = s[0];
        o.iterations = s[1];
        o.retries = s[2];
        o.early = s[3];
        for (int k = 0; k < 16; ++k) o.hist[k] = h[k];
        o.error = err;
        o.err_reach = err_reach;
    }
}

// Device address of the scratch array on the current device (looked up once).
int noalloc_scratch(NoAllocPartial** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(TROUTE_ENODEV, "no CUDA device: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return set_error(TROUTE_EINVAL, "device %d beyond the supported range", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return set_error(TROUTE_ECUDA, "cudaGetSymbolAddress of the no-alloc scratch: %s", cudaGetErrorString(e));
        g_noalloc_ptr[dev] = static_cast<NoAllocPartial*>(ptr);
    }
    *out = g_noalloc_ptr[dev];
    return TROUTE_OK;
}

}  // namespace
}  // namespace tr

using namespace tr;

extern "C" int troute_mc_reach_parallel_device_noalloc(const troute_chparams* p, const double* ql,
                                                       const int* rs, const int* rl,
                                                       const double* qu, const double* qd, const double* dp,
                                                       double* qo, double* vo, double* dpo,
                                                       double uq, double dt, int nr, int n_segments,
                                                       const troute_cfg* cfg, void* stream,
                                                       troute_stats* stats)
{
    if (stats) std::memset(stats, 0, sizeof *stats);
    if (nr < 0 || n_segments < 0) return set_error(TROUTE_EINVAL, "negative size");
    if (nr > kNoAllocMaxBlocks * kNoAllocThreads)
        return set_error(TROUTE_EINVAL, "%d reaches exceed the no-alloc limit of %d reaches per call", nr,
                         kNoAllocMaxBlocks * kNoAllocThreads);
    if (nr == 0) return TROUTE_OK;
    if (!p || !ql || !rs || !rl || !qu || !qd || !dp || !qo || !vo || !dpo)
        return set_error(TROUTE_EINVAL, "null array");
    troute_cfg c;
    troute_cfg_default(&c);
    if (cfg) c = *cfg;
    int rc = check_cfg(c);
    if (rc) return rc;
    if ((rc = pending_cuda_error("troute_mc_reach_parallel_device_noalloc"))) return rc;
    NoAllocPartial* part = nullptr;
    if ((rc = noalloc_scratch(&part))) return rc;
    const int nblocks = (nr + kNoAllocThreads - 1) / kNoAllocThreads;
    cudaStream_t st = (cudaStream_t)stream;
    noalloc_reach_kernel<<<nblocks, kNoAllocThreads, 0, st>>>(p, ql, rs, rl, qu, qd, dp, qo, vo, dpo, uq, dt, nr,
                                                              n_segments, make_tol(c), part);
    noalloc_reduce_kernel<<<1, 256, 0, st>>>(part, nblocks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(TROUTE_ECUDA, "no-alloc launch: %s", cudaGetErrorString(e));
    if (!stats) return TROUTE_OK;
    NoAllocPartial tot;
    e = cudaMemcpyAsync(&tot, part + kNoAllocMaxBlocks, sizeof tot, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_error(TROUTE_ECUDA, "no-alloc counters: %s", cudaGetErrorString(e));
    stats->solves = tot.solves;
    stats->iterations = tot.iterations;
    stats->retries = tot.retries;
    stats->early_exits = tot.early;
    for (int k = 0; k < 16; ++k) stats->iter_hist[k] = tot.hist[k];
    if (tot.error) return set_error(tot.error, "reach %d: segment range outside [0, n_segments)", tot.err_reach);
    return TROUTE_OK;
}
