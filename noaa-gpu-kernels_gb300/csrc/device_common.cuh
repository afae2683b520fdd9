// Device helpers shared by the routing kernels: GPU-scope acquire/release
// flags, bounded waits, error recording, solve counters, ticket decoding.
#pragma once

#include <cuda_runtime.h>

#include "mc_solve.cuh"

namespace tr {

__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile_int(const int* p)
{
    return *reinterpret_cast<const volatile int*>(p);
}

__device__ inline void record_error(DevStats* st, int code, int reach, int step, int where)
{
    if (atomicCAS(&st->error, 0, code) == 0) {
        st->err_reach = reach;
        st->err_step = step;
        st->err_where = where;
    }
}

// Per-thread counters, folded into the block's shared copy at the end.
struct LocalStats {
    unsigned long long solves, iterations, retries, early, warm_used, warm_fallback;
};

__device__ __forceinline__ void count_solve(LocalStats& ls, unsigned int* hist_s, const SolveOut& o)
{
    ls.solves++;
    ls.iterations += (unsigned)o.iters;
    ls.retries += (unsigned)o.retried;
    ls.early += (unsigned)o.early;
    atomicAdd(&hist_s[o.iters < 15 ? o.iters : 15], 1u);
}

__device__ inline void flush_stats(LocalStats& ls, unsigned int* hist_s, DevStats* st)
{
    // warp reduce, one atomic per warp
    for (int off = 16; off > 0; off >>= 1) {
        ls.solves += __shfl_down_sync(0xffffffffu, ls.solves, off);
        ls.iterations += __shfl_down_sync(0xffffffffu, ls.iterations, off);
        ls.retries += __shfl_down_sync(0xffffffffu, ls.retries, off);
        ls.early += __shfl_down_sync(0xffffffffu, ls.early, off);
        ls.warm_used += __shfl_down_sync(0xffffffffu, ls.warm_used, off);
        ls.warm_fallback += __shfl_down_sync(0xffffffffu, ls.warm_fallback, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&st->solves, ls.solves);
        atomicAdd(&st->iterations, ls.iterations);
        atomicAdd(&st->retries, ls.retries);
        atomicAdd(&st->early_exits, ls.early);
        if (ls.warm_used) atomicAdd(&st->warm_used, ls.warm_used);
        if (ls.warm_fallback) atomicAdd(&st->warm_fallback, ls.warm_fallback);
    }
    __syncthreads();
    if (threadIdx.x < 16 && hist_s[threadIdx.x]) atomicAdd(&st->hist[threadIdx.x], (unsigned long long)hist_s[threadIdx.x]);
}

__device__ __forceinline__ int find_wave(const unsigned long long* __restrict__ wave_ptr,
                                         int n_waves, unsigned long long k)
{
    // largest w with wave_ptr[w] <= k
    int lo = 0, hi = n_waves - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(wave_ptr + mid) <= k) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Waits until *flag >= want; false on timeout or when another warp failed.
__device__ __forceinline__ bool wait_at_least(const int* flag, int want, long long budget,
                                              DevStats* st)
{
    if (ld_acquire(flag) >= want) return true;
    const long long t0 = clock64();
    unsigned ns = 32;
    while (true) {
        __nanosleep(ns);
        if (ld_acquire(flag) >= want) return true;
        if (ns < 1024) ns <<= 1;
        if (clock64() - t0 > budget) return false;
        if (ld_volatile_int(&st->error) != 0) return false;
    }
}

}  // namespace tr
