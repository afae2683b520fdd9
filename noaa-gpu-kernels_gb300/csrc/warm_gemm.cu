// Learned warm start as one dense GEMM per launch, on the 5th-generation
// tensor cores (tcgen05, TMEM accumulators).
//
// Before a routing launch of T steps, the starting depth of every solve of
// the launch -- every (segment slot, step) -- is predicted by the
// 8 -> 64 -> 64 -> 1 SiLU MLP and written to a plane [T][slots] the routing
// kernel reads when a solve begins. The features a solve would see that are
// not known before the launch (its upstream inflows and its own previous
// discharge, which the time-skewed sweep produces during the launch) are
// taken from the state at the launch's start: the previous segment's discharge
// (or, at a reach head, the sum of the upstream reaches' outflow) for qup and
// quc, the segment's own discharge for qdp. The step's own lateral inflow and
// the segment's static parameters are exact. (Measured on the 64-member c4w
// ensemble with 32-step launches: 6.557 secant iterations per solve with
// these launch-start features against 6.542 with the exact ones.) Any
// prediction only places the secant's starting bracket; the solve, its
// fallback and the oracle's replay from the recorded starting depths are
// unchanged.
//
// The GEMM: one CTA of 128 threads holds a 128-row tile (row r = thread r =
// TMEM lane r) and walks the launch's steps for it, so the static and lagged
// features are formed once per slot and only the inflow feature per step.
//   layer 1: D1[128 x 64] = A1[128 x 16] . W1^T   (one tcgen05.mma, K = 16:
//            the 8 features zero-padded)
//   layer 2: D2[128 x 64] = A2[128 x 64] . W2^T   (four tcgen05.mma, K = 16
//            each, accumulating), A2 = SiLU(D1 + b1) in bf16x2 arithmetic
//   layer 3: y = b3 + w3 . SiLU(D2 + b2) on the CUDA cores (one output column)
// BF16 operands from shared memory (no-swizzle K-major canonical layout: 8-row
// x 16-byte core matrices of 128 contiguous bytes), FP32 accumulation in TMEM
// (128 columns), read back with tcgen05.ld (each warp its 32 lanes). One
// thread issues the MMAs; their completion is signalled on an mbarrier by
// tcgen05.commit. Every wait is bounded: on expiry the CTA records an error,
// stops, frees its TMEM and returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "warm.cuh"

namespace tr {
namespace {

constexpr int kGRows = 128;        // rows per tile = threads per CTA = TMEM lanes
constexpr int kTmemCols = 128;     // D1 in columns 0-63, D2 in 64-127
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz per MMA completion wait

// bf16 tiles in the canonical no-swizzle K-major layout: [8-row group][8-element
// K group][row in group][element] -- a core matrix is 8 rows x 16 bytes.
struct __align__(128) GemmSmem {
    __nv_bfloat16 a1[kGRows / 8][2][8][8];    // 128 x 16   (4 KB)
    __nv_bfloat16 a2[kGRows / 8][8][8][8];    // 128 x 64   (16 KB)
    __nv_bfloat16 w1[kWHid / 8][2][8][8];     // W1 (n x k), 64 x 16
    __nv_bfloat16 w2[kWHid / 8][8][8][8];     // W2 (n x k), 64 x 64
    float b1[kWHid], b2[kWHid], w3[kWHid];
    unsigned long long mbar;
    uint32_t tmem_base;
    int fail;
};
// at most 4 CTAs per SM (4 x 128 TMEM columns = the SM's 512): the launch asks
// for this much dynamic shared memory per CTA
constexpr size_t kGemmSmemBytes = 56 * 1024;
static_assert(sizeof(GemmSmem) <= kGemmSmemBytes, "shared layout");

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading byte offset (between
// core matrices along K), stride byte offset (between 8-row groups), the
// descriptor version 1 at bits 46-47, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(const void* p, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((smem_u32(p) & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 64, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kWHid >> 3) << 17) |
                            ((uint32_t)(kGRows >> 4) << 24);

__device__ __forceinline__ void mma_bf16_ss(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// A waiting thread is suspended by the hardware until the phase completes (or
// this long) instead of spinning, leaving the issue slots to the other CTAs'
// epilogues.
constexpr uint32_t kSuspendNs = 100000;

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred P1;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2, %3;\n\t"
        "selp.b32 %0, 1, 0, P1;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity), "r"(kSuspendNs)
        : "memory");
    return done != 0;
}

// Waits for the mbarrier phase with the given parity, at most kWaitCycles.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity)
{
    const long long t0 = clock64();
    while (!mbar_try(mbar, parity))
        if (clock64() - t0 > kWaitCycles) return false;
    return true;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 64 consecutive FP32 columns of this thread's TMEM lane, one load and one wait.
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float (&v)[64])
{
    uint32_t r[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
        "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
        "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
          "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
          "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
          "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
          "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

// SiLU of two values as a packed bf16 pair: z rounded to bf16, then t (1 +
// tanh t) with t = z / 2 in bf16x2 arithmetic (the result feeds a BF16 MMA).
__device__ __forceinline__ unsigned silu2_bf16(float lo, float hi)
{
    const unsigned z = pack_bf16(lo, hi);
    unsigned t, th, r;
    asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(t) : "r"(z), "r"(0x3f003f00u));  // z * 0.5
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(th) : "r"(t));
    asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(r) : "r"(t), "r"(th), "r"(t));  // t + t tanh(t)
    return r;
}

// Rows of the GEMM from caller-provided raw inputs [n][8] (one step).
struct RawRows {
    const float* raw;
    long long n;
    double* out;
    __device__ bool valid(long long row) const { return row < n; }
    __device__ void static_features(const WarmDev& m, long long row, float (&f)[kWIn]) const
    {
#pragma unroll
        for (int k = 0; k < kWIn; ++k) f[k] = warm_feature(raw[row * kWIn + k], k < 4, m.mu[k], m.inv_sd[k]);
    }
    __device__ float step_feature(const WarmDev& m, long long row, int t, float f3) const { return f3; }
    __device__ void store(long long row, int t, float pred) const { out[row] = (double)pred; }
};

// Rows of the GEMM from a routing launch: segment slot `row` at step t of the
// launch, features from the state at the launch's start.
struct PlaneRows {
    NetDev net;
    const double* qlat;
    long long qlat_ld;
    const int* step_base;
    float* out;       // [T][n_seg_int]
    __device__ bool valid(long long row) const { return row < net.n_seg_int; }
    __device__ void static_features(const WarmDev& m, long long row, float (&f)[kWIn]) const
    {
        const SegRec* r = net.seg + row;
        const int ri = __ldg(&r->reach);      // internal reach (-1: an unused slot)
        const int i = __ldg(&r->pos);         // position in the reach
        double qdp = 0.0, quc = 0.0;
        if (ri >= 0) {
            qdp = __ldcg(net.q + row);
            if (i > 0) {
                quc = __ldcg(net.q + row - kLanes);
            } else {
                // outflow of the upstream reaches in the step before the launch
                const int tb = __ldg(step_base);
                const double* ring = net.ring + (size_t)(((tb - 1) % kRing + kRing) % kRing) * net.n_reach_int;
                for (int j = __ldg(net.up_ptr + ri); j < __ldg(net.up_ptr + ri + 1); ++j)
                    quc += __ldcg(ring + __ldg(net.up_idx + j));
            }
        }
        const double2 p0 = __ldg(r->p + 0), p1 = __ldg(r->p + 1), p2 = __ldg(r->p + 2);
        f[0] = warm_feature(pos_to_float(quc), true, m.mu[0], m.inv_sd[0]);   // qup: the same launch-start value
        f[1] = warm_feature(pos_to_float(quc), true, m.mu[1], m.inv_sd[1]);   // quc
        f[2] = warm_feature(pos_to_float(qdp), true, m.mu[2], m.inv_sd[2]);   // qdp
        f[3] = 0.0f;
        f[4] = warm_feature(pos_to_float(p0.x), false, m.mu[4], m.inv_sd[4]);   // dx
        f[5] = warm_feature(pos_to_float(p2.y), false, m.mu[5], m.inv_sd[5]);   // s0
        f[6] = warm_feature(pos_to_float(p1.y), false, m.mu[6], m.inv_sd[6]);   // n
        f[7] = warm_feature(pos_to_float(p0.y), false, m.mu[7], m.inv_sd[7]);   // bw
    }
    __device__ float step_feature(const WarmDev& m, long long row, int t, float) const
    {
        const double2 qs = __ldg(reinterpret_cast<const double2*>(&net.seg[row].qscale));
        const int col = (int)(unsigned)(__double_as_longlong(qs.y) & 0xffffffffll);
        const double ql = __ldg(qlat + (size_t)t * (size_t)qlat_ld + col) * qs.x;
        return warm_feature(pos_to_float(ql), true, m.mu[3], m.inv_sd[3]);
    }
    __device__ void store(long long row, int t, float pred) const { out[(size_t)t * (size_t)net.n_seg_int + row] = pred; }
};

template <class Rows>
__global__ void __launch_bounds__(kGRows) warm_gemm_kernel(WarmDev m, Rows rows, long long n_rows, int T, int* error)
{
    extern __shared__ __align__(1024) unsigned char gemm_smem_raw[];
    GemmSmem& S = *reinterpret_cast<GemmSmem*>(gemm_smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;

    // weights into the canonical layouts (W1 padded to K = 16 in the source)
    for (int i = tid; i < kWHid * kWK1; i += kGRows) {
        const int n = i / kWK1, k = i % kWK1;
        S.w1[n / 8][k / 8][n % 8][k % 8] = m.w1t[i];
    }
    for (int i = tid; i < kWHid * kWHid; i += kGRows) {
        const int n = i / kWHid, k = i % kWHid;
        S.w2[n / 8][k / 8][n % 8][k % 8] = m.w2t[i];
    }
    for (int i = tid; i < kWHid; i += kGRows) {
        S.b1[i] = m.b1[i];
        S.b2[i] = m.b2[i];
        S.w3[i] = __bfloat162float(m.w3t[i]);
    }
    const uint32_t mbar = smem_u32(&S.mbar);
    if (tid == 0) {
        S.fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(1u) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                     "r"((uint32_t)kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = S.tmem_base;
    const uint32_t d1 = tmem, d2 = tmem + kWHid;
    const uint32_t lane_off = (uint32_t)(warp * 32) << 16;   // this warp's 32 TMEM lanes

    const uint64_t w1d = smem_desc(&S.w1[0][0][0][0], 128, 256);
    uint32_t parity = 0;
    bool ok = true;
    const long long n_tiles = (n_rows + kGRows - 1) / kGRows;
    for (long long tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const long long row = tile * kGRows + tid;
        const bool live = rows.valid(row);
        float f[kWIn];
        if (live) rows.static_features(m, row, f);
        else
            for (int k = 0; k < kWIn; ++k) f[k] = 0.0f;
        for (int t = 0; t < T && ok; ++t) {
            // ---- layer 1 ----
            const float f3 = live ? rows.step_feature(m, row, t, f[3]) : 0.0f;
            {
                uint4 lo, hi;
                lo.x = pack_bf16(f[0], f[1]);
                lo.y = pack_bf16(f[2], f3);
                lo.z = pack_bf16(f[4], f[5]);
                lo.w = pack_bf16(f[6], f[7]);
                hi = make_uint4(0u, 0u, 0u, 0u);
                *reinterpret_cast<uint4*>(&S.a1[tid / 8][0][tid % 8][0]) = lo;
                *reinterpret_cast<uint4*>(&S.a1[tid / 8][1][tid % 8][0]) = hi;
            }
            fence_async_smem();
            __syncthreads();
            if (tid == 0) {
                tc_after_sync();
                mma_bf16_ss(d1, smem_desc(&S.a1[0][0][0][0], 128, 256), w1d, 0u);
                mma_commit(mbar);
            }
            if (!mbar_wait(mbar, parity)) S.fail = 1;
            parity ^= 1u;
            tc_after_sync();
            // ---- SiLU(D1 + b1) -> A2 (bf16) ----
            {
                float v[64];
                tmem_ld64(d1 + lane_off, v);
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    uint4 q;
                    q.x = silu2_bf16(v[8 * c + 0] + S.b1[8 * c + 0], v[8 * c + 1] + S.b1[8 * c + 1]);
                    q.y = silu2_bf16(v[8 * c + 2] + S.b1[8 * c + 2], v[8 * c + 3] + S.b1[8 * c + 3]);
                    q.z = silu2_bf16(v[8 * c + 4] + S.b1[8 * c + 4], v[8 * c + 5] + S.b1[8 * c + 5]);
                    q.w = silu2_bf16(v[8 * c + 6] + S.b1[8 * c + 6], v[8 * c + 7] + S.b1[8 * c + 7]);
                    *reinterpret_cast<uint4*>(&S.a2[tid / 8][c][tid % 8][0]) = q;
                }
            }
            fence_async_smem();
            tc_before_sync();
            __syncthreads();
            // ---- layer 2: four K = 16 chunks accumulated in D2 ----
            if (tid == 0 && !S.fail) {
                tc_after_sync();
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    mma_bf16_ss(d2, smem_desc(&S.a2[0][2 * q][0][0], 128, 1024), smem_desc(&S.w2[0][2 * q][0][0], 128, 1024),
                                q > 0 ? 1u : 0u);
                mma_commit(mbar);
            }
            __syncthreads();
            if (S.fail) {
                ok = false;
                break;
            }
            if (!mbar_wait(mbar, parity)) S.fail = 1;
            parity ^= 1u;
            tc_after_sync();
            // ---- layer 3 on the CUDA cores ----
            float y = m.b3;
            {
                float v[64];
                tmem_ld64(d2 + lane_off, v);
#pragma unroll
                for (int j = 0; j < 64; ++j) y += S.w3[j] * silu(v[j] + S.b2[j]);
            }
            if (live) rows.store(row, t, __expf(y * m.sd_y + m.mu_y));
            tc_before_sync();
            __syncthreads();
            if (S.fail) ok = false;
        }
    }
    if (!ok) {
        // an MMA that has not signalled may still be running: give it one more
        // bounded wait before its TMEM is released
        mbar_wait(mbar, parity ^ 1u);
        if (tid == 0) atomicExch(error, TROUTE_ETIMEOUT);
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)kTmemCols)
                     : "memory");
}

int gemm_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return TROUTE_OK;
    return set_error(e == cudaErrorMemoryAllocation ? TROUTE_ENOMEM : TROUTE_ECUDA, "%s: %s", what,
                     cudaGetErrorString(e));
}

template <class Rows>
int launch_gemm(const WarmDev& m, const Rows& rows, long long n_rows, int T, int* error, cudaStream_t st)
{
    if (n_rows <= 0 || T <= 0) return TROUTE_OK;
    int rc = gemm_cuda(cudaFuncSetAttribute(warm_gemm_kernel<Rows>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)kGemmSmemBytes),
                       "warm GEMM smem attribute");
    if (rc) return rc;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long n_tiles = (n_rows + kGRows - 1) / kGRows;
    const int grid = (int)std::min<long long>(n_tiles, 4LL * sms);
    warm_gemm_kernel<Rows><<<grid, kGRows, kGemmSmemBytes, st>>>(m, rows, n_rows, T, error);
    return gemm_cuda(cudaGetLastError(), "warm GEMM launch");
}

}  // namespace

// Predictions of a routing launch (plane [T][n_seg_int] of starting depths).
int launch_warm_plane(const troute_warm* w, const NetDev& net, const RunDev& run, int T, float* plane, int* error,
                      void* stream)
{
    PlaneRows rows;
    rows.net = net;
    rows.qlat = run.qlat;
    rows.qlat_ld = run.qlat_ld;
    rows.step_base = run.step_base;
    rows.out = plane;
    return launch_gemm(warm_device_view(w, run.warm_delta, run.warm_k), rows, net.n_seg_int, T, error,
                       (cudaStream_t)stream);
}

// Predictions for raw inputs [n][8] through the same GEMM (device arrays).
int launch_warm_gemm_raw(const troute_warm* w, const float* raw, long long n, double* depth, int* error, void* stream)
{
    RawRows rows{raw, n, depth};
    return launch_gemm(warm_device_view(w, 0.0, 0), rows, n, 1, error, (cudaStream_t)stream);
}

}  // namespace tr
