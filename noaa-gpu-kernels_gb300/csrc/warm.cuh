// Learned warm start of the secant depth solve: an 8 -> 64 -> 64 -> 1 MLP
// (SiLU) that predicts a segment's converged flow depth from its normalised
// inflows, geometry, slope and Manning's n. Device-side inference with BF16
// tensor cores (mma.sync m16n8k16, FP32 accumulate), one warp evaluating the
// rows of its lanes; training kernels live in warm.cu.
#pragma once

#include <cuda_bf16.h>

#include "troute_internal.h"

namespace tr {

constexpr int kWIn = 8;      // inputs
constexpr int kWHid = 64;    // hidden width
constexpr int kWK1 = 16;     // first layer K padded to the MMA's 16
constexpr int kWLd = 72;     // padded row (bf16) of the transposed weights in shared memory
constexpr int kWOut = 8;     // last layer N padded to the MMA's 8 (column 0 is the output)

// Raw input -> feature: log of the value (flows offset by kFlowFloor m3/s, which
// may be zero), then standardised with the training set's mean / std.
constexpr float kFlowFloor = 1e-3f;

// Parameters of a trained model as the routing kernels read them.
struct WarmDev {
    const __nv_bfloat16* w1t;  // [64][16]   W1 transposed (n-major, k contiguous; k >= 8 zero)
    const __nv_bfloat16* w2t;  // [64][64]
    const __nv_bfloat16* w3t;  // [8][64]    row 0 = w3, rows 1..7 zero
    const float* b1;           // [64]
    const float* b2;           // [64]
    float b3;
    float mu[kWIn], sd[kWIn], inv_sd[kWIn];
    float mu_y, sd_y;
    double delta;              // half-width of the starting bracket around the prediction (relative)
    int k;                     // iterations a warm-started solve gets before the plain restart
};

// Device view of a trained model (host side, warm.cu).
WarmDev warm_device_view(const troute_warm* w, double delta, int k);

// Shared-memory copy of the weights for the MMA fragments.
struct __align__(16) WarmSmem {
    __nv_bfloat16 w1t[kWHid][kWK1 + 8];
    __nv_bfloat16 w2t[kWHid][kWLd];
    __nv_bfloat16 w3t[kWOut][kWLd];
    float b1[kWHid], b2[kWHid];
    unsigned int xin[4][32][4];  // per warp: 32 rows x 8 bf16 features (packed pairs)
};

__device__ __forceinline__ void warm_stage(WarmSmem& s, const WarmDev& m)
{
    for (int i = threadIdx.x; i < kWHid * kWK1; i += blockDim.x) s.w1t[i / kWK1][i % kWK1] = m.w1t[i];
    for (int i = threadIdx.x; i < kWHid * kWHid; i += blockDim.x) s.w2t[i / kWHid][i % kWHid] = m.w2t[i];
    for (int i = threadIdx.x; i < kWOut * kWHid; i += blockDim.x) s.w3t[i / kWHid][i % kWHid] = m.w3t[i];
    for (int i = threadIdx.x; i < kWHid; i += blockDim.x) {
        s.b1[i] = m.b1[i];
        s.b2[i] = m.b2[i];
    }
}

// A positive double as a float, truncated, on the integer pipe (the FP64
// pipe, shared with the secant's arithmetic, is kept free): exponent rebias
// and the top 23 mantissa bits. Non-positive values give 0, values outside
// float's normal range are clamped to it. The features only need a
// deterministic monotone map, not correct rounding.
__device__ __forceinline__ float pos_to_float(double v)
{
    const long long b = __double_as_longlong(v);
    if (b <= 0) return 0.0f;
    const int e = (int)(b >> 52);  // biased exponent; the sign bit is 0
    if (e > 1150) return 3.4e38f;
    if (e < 897) return 1.18e-38f;
    return __int_as_float(((e - 896) << 23) | (int)((b >> 29) & 0x7fffff));
}

// A positive normal float as the equal double, on the integer pipe.
__device__ __forceinline__ double widen_pos(float f)
{
    const unsigned fb = __float_as_uint(f);
    return __longlong_as_double(((long long)((fb >> 23) + 896) << 52) | ((long long)(fb & 0x7fffff) << 29));
}

// Raw input -> feature: log of the value (flows offset by kFlowFloor m3/s, which
// may be zero), standardised with the training set's mean / standard deviation.
__device__ __forceinline__ float warm_feature(float x, bool flow, float mu, float inv_sd)
{
    if (flow) x += kFlowFloor;
    return (__logf(fmaxf(x, 1e-30f)) - mu) * inv_sd;
}

__device__ __forceinline__ unsigned int pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const unsigned int*>(&v);
}

// SiLU through the hardware tanh approximation: z sigmoid(z) = z (1 + tanh(z/2)) / 2
// (the training kernels use the exact form; the difference is far below the
// BF16 rounding of the activations).
__device__ __forceinline__ float tanh_approx(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float silu(float z) { return 0.5f * z * (1.0f + tanh_approx(0.5f * z)); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned ld_pair(const __nv_bfloat16* p) { return *reinterpret_cast<const unsigned*>(p); }

// SiLU of two accumulator values, returned as the bf16x2 A-fragment register
// of the next layer: z rounded to bf16, then z/2 (1 + tanh(z/2)) in bf16x2
// arithmetic (three instructions for the pair; the values are rounded to
// bf16 for the next MMA in any case).
__device__ __forceinline__ unsigned silu_bf16x2(float lo, float hi)
{
    const unsigned z = pack_bf16(lo, hi);
    unsigned t, th, r;
    asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(t) : "r"(z), "r"(0x3f003f00u));  // z * 0.5
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(th) : "r"(t));
    asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(r) : "r"(t), "r"(th), "r"(t));  // t + t tanh(t)
    return r;
}

// Four 8x8 bf16 matrices from shared memory (one row address per lane: lanes
// 8m..8m+7 give the rows of matrix m); register m holds the fragment of matrix
// m that mma.sync's col-major B operand expects when the rows are the output
// columns n and the 8 columns are consecutive k.
__device__ __forceinline__ void ldsm_x4(unsigned (&d)[4], const __nv_bfloat16* row)
{
    const unsigned addr = (unsigned)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3])
                 : "r"(addr));
}

// Two 8x8 matrices (lanes 0-7 and 8-15 give the row addresses; the others'
// addresses are not used).
__device__ __forceinline__ void ldsm_x2(unsigned& d0, unsigned& d1, const __nv_bfloat16* row)
{
    const unsigned addr = (unsigned)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];" : "=r"(d0), "=r"(d1) : "r"(addr));
}

// One 16-row tile of the MLP (rows mt*16 .. mt*16+15 of the warp's staging
// area). Returns the C fragment of the output column: rows g (o0) and g + 8
// (o2) on the lanes with t == 0.
__device__ __forceinline__ void warm_mlp_tile(const WarmSmem& s, int w, int mt, int lane, float b3, float& o0,
                                              float& o2)
{
    const int g = lane >> 2, t = lane & 3;
    const int lm = lane >> 3, lr = lane & 7;  // ldmatrix: matrix and row this lane addresses
    // ---- layer 1: [16 x 16(8)] x [16 x 64] ----
    unsigned a[4];
    a[0] = s.xin[w][mt * 16 + g][t];
    a[1] = s.xin[w][mt * 16 + g + 8][t];
    a[2] = 0u;
    a[3] = 0u;
    unsigned a2[4][4];  // SiLU(h1) as the A fragments of layer 2 (C -> A in registers)
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        // B fragments of n-blocks j = 2kk, 2kk+1: matrices (j, k 0-7), (j, k 8-15), (j+1, ...), (j+1, ...)
        unsigned bw[4];
        ldsm_x4(bw, &s.w1t[8 * (2 * kk + (lm >> 1)) + lr][8 * (lm & 1)]);
        float h[2][4];
#pragma unroll
        for (int jj = 0; jj < 2; ++jj) {
            const int n = 8 * (2 * kk + jj) + 2 * t;
            const float2 bias = *reinterpret_cast<const float2*>(&s.b1[n]);
            h[jj][0] = bias.x;
            h[jj][1] = bias.y;
            h[jj][2] = bias.x;
            h[jj][3] = bias.y;
            mma_bf16(h[jj], a, bw[2 * jj], bw[2 * jj + 1]);
        }
        a2[kk][0] = silu_bf16x2(h[0][0], h[0][1]);
        a2[kk][1] = silu_bf16x2(h[0][2], h[0][3]);
        a2[kk][2] = silu_bf16x2(h[1][0], h[1][1]);
        a2[kk][3] = silu_bf16x2(h[1][2], h[1][3]);
    }
    // ---- layers 2 and 3, one 16-column chunk of the hidden layer at a time ----
    float o[4] = {b3, b3, b3, b3};
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        float h[2][4];
#pragma unroll
        for (int jj = 0; jj < 2; ++jj) {
            const int j = 2 * kk + jj, n = 8 * j + 2 * t;
            const float2 bias = *reinterpret_cast<const float2*>(&s.b2[n]);
            h[jj][0] = bias.x;
            h[jj][1] = bias.y;
            h[jj][2] = bias.x;
            h[jj][3] = bias.y;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                // B fragment of n-block j, k-chunk q: matrices (j, k 16q..+7), (j, k 16q+8..+15)
                unsigned b0, b1;
                ldsm_x2(b0, b1, &s.w2t[8 * j + lr][16 * q + 8 * (lm & 1)]);
                mma_bf16(h[jj], a2[q], b0, b1);
            }
        }
        unsigned a3[4];
        a3[0] = silu_bf16x2(h[0][0], h[0][1]);
        a3[1] = silu_bf16x2(h[0][2], h[0][3]);
        a3[2] = silu_bf16x2(h[1][0], h[1][1]);
        a3[3] = silu_bf16x2(h[1][2], h[1][3]);
        unsigned c0, c1;  // layer-3 B fragment (row 0 = w3, rows 1-7 zero), k-chunk kk
        ldsm_x2(c0, c1, &s.w3t[lr][16 * kk + 8 * (lm & 1)]);
        mma_bf16(o, a3, c0, c1);
    }
    o0 = o[0];
    o2 = o[2];
}

// Evaluates the MLP for the lanes of a warp that ask for it (`want`). Every
// lane of the warp must call it (warp-synchronous MMA). The asking lanes'
// feature rows are packed into the first rows of the warp's staging area, so
// up to 16 requests cost one 16-row tile and more cost two. Each output row
// depends on its own input row only. Returns the prediction (normalised
// units) on the asking lanes.
#ifdef TROUTE_MLP_INLINE
#define TR_MLP_ATTR __forceinline__
#else
#define TR_MLP_ATTR __noinline__
#endif
static __device__ TR_MLP_ATTR float warm_mlp_warp(WarmSmem& s, const float (&feat)[kWIn], bool want, float b3)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    const int rank = __popc(mask & ((1u << lane) - 1u));
    if (want) {
        unsigned int* xin = s.xin[w][rank];
        xin[0] = pack_bf16(feat[0], feat[1]);
        xin[1] = pack_bf16(feat[2], feat[3]);
        xin[2] = pack_bf16(feat[4], feat[5]);
        xin[3] = pack_bf16(feat[6], feat[7]);
    }
    __syncwarp();
    const int n_tiles = __popc(mask) > 16 ? 2 : 1;
    float r[2][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
    warm_mlp_tile(s, w, 0, lane, b3, r[0][0], r[0][1]);
    if (n_tiles == 2) warm_mlp_tile(s, w, 1, lane, b3, r[1][0], r[1][1]);
    // row `rank`: tile rank/16, row-in-tile rr = rank%16, held by lane (rr%8)*4, half rr/8
    const int rr = rank & 15, src = (rr & 7) * 4, half = rr >> 3, mt = rank >> 4;
    const float v00 = __shfl_sync(0xffffffffu, r[0][0], src);
    const float v01 = __shfl_sync(0xffffffffu, r[0][1], src);
    const float v10 = __shfl_sync(0xffffffffu, r[1][0], src);
    const float v11 = __shfl_sync(0xffffffffu, r[1][1], src);
    __syncwarp();
    return mt == 0 ? (half ? v01 : v00) : (half ? v11 : v10);
}

}  // namespace tr
