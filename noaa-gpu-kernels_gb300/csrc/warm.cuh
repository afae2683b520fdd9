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
    float mu[kWIn], sd[kWIn];
    float mu_y, sd_y;
    double delta;              // half-width of the starting bracket around the prediction (relative)
    int k;                     // iterations a warm-started solve gets before the plain restart
};

// Device view of a trained model (host side, warm.cu).
WarmDev warm_device_view(const troute_warm* w, double delta, int k);

// Shared-memory copy of the weights for the MMA fragments.
struct WarmSmem {
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

__device__ __forceinline__ float warm_feature(double v, bool flow, float mu, float sd)
{
    const float x = flow ? (float)v + kFlowFloor : (float)v;
    return (__logf(fmaxf(x, 1e-30f)) - mu) / sd;
}

__device__ __forceinline__ unsigned int pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const unsigned int*>(&v);
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned ld_pair(const __nv_bfloat16* p) { return *reinterpret_cast<const unsigned*>(p); }

// Evaluates the MLP for the 32 rows of a warp (row = lane). Every lane of the
// warp must call it (it uses warp-synchronous MMA); `feat` is the lane's 8
// normalised features (ignored for lanes whose prediction is not used).
// Returns the prediction of the lane's own row in normalised units.
static __device__ __noinline__ float warm_mlp_warp(WarmSmem& s, const float (&feat)[kWIn], float b3)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
    unsigned int* xin = s.xin[w][lane];
    xin[0] = pack_bf16(feat[0], feat[1]);
    xin[1] = pack_bf16(feat[2], feat[3]);
    xin[2] = pack_bf16(feat[4], feat[5]);
    xin[3] = pack_bf16(feat[6], feat[7]);
    __syncwarp();
    float out_rows[2][2];  // [m-tile][half]: prediction of rows g, g+8 (valid on lanes with t == 0)
    for (int mt = 0; mt < 2; ++mt) {
        // ---- layer 1: [16 x 16(8)] x [16 x 64] ----
        unsigned a[4];
        a[0] = s.xin[w][mt * 16 + g][t];
        a[1] = s.xin[w][mt * 16 + g + 8][t];
        a[2] = 0u;
        a[3] = 0u;
        float h1[8][4];
        for (int j = 0; j < 8; ++j) {
            const int n = 8 * j + 2 * t;
            h1[j][0] = s.b1[n];
            h1[j][1] = s.b1[n + 1];
            h1[j][2] = s.b1[n];
            h1[j][3] = s.b1[n + 1];
            mma_bf16(h1[j], a, ld_pair(&s.w1t[8 * j + g][2 * t]), ld_pair(&s.w1t[8 * j + g][8 + 2 * t]));
        }
        // ---- layer 2: SiLU(h1) [16 x 64] x [64 x 64]; C fragments become A fragments ----
        unsigned a2[4][4];
        for (int kk = 0; kk < 4; ++kk) {
            a2[kk][0] = pack_bf16(silu(h1[2 * kk][0]), silu(h1[2 * kk][1]));
            a2[kk][1] = pack_bf16(silu(h1[2 * kk][2]), silu(h1[2 * kk][3]));
            a2[kk][2] = pack_bf16(silu(h1[2 * kk + 1][0]), silu(h1[2 * kk + 1][1]));
            a2[kk][3] = pack_bf16(silu(h1[2 * kk + 1][2]), silu(h1[2 * kk + 1][3]));
        }
        float h2[8][4];
        for (int j = 0; j < 8; ++j) {
            const int n = 8 * j + 2 * t;
            h2[j][0] = s.b2[n];
            h2[j][1] = s.b2[n + 1];
            h2[j][2] = s.b2[n];
            h2[j][3] = s.b2[n + 1];
            for (int kk = 0; kk < 4; ++kk)
                mma_bf16(h2[j], a2[kk], ld_pair(&s.w2t[8 * j + g][16 * kk + 2 * t]),
                         ld_pair(&s.w2t[8 * j + g][16 * kk + 8 + 2 * t]));
        }
        // ---- layer 3: SiLU(h2) [16 x 64] x [64 x 8(1)] ----
        float o[4] = {b3, b3, b3, b3};
        for (int kk = 0; kk < 4; ++kk) {
            unsigned a3[4];
            a3[0] = pack_bf16(silu(h2[2 * kk][0]), silu(h2[2 * kk][1]));
            a3[1] = pack_bf16(silu(h2[2 * kk][2]), silu(h2[2 * kk][3]));
            a3[2] = pack_bf16(silu(h2[2 * kk + 1][0]), silu(h2[2 * kk + 1][1]));
            a3[3] = pack_bf16(silu(h2[2 * kk + 1][2]), silu(h2[2 * kk + 1][3]));
            mma_bf16(o, a3, ld_pair(&s.w3t[g][16 * kk + 2 * t]), ld_pair(&s.w3t[g][16 * kk + 8 + 2 * t]));
        }
        out_rows[mt][0] = o[0];  // row g, column 2t (column 0 on t == 0)
        out_rows[mt][1] = o[2];  // row g + 8
    }
    // row r = lane: m-tile r/16, row-in-tile rr = r%16 -> held by lane (rr%8)*4, half rr/8
    const int rr = lane & 15, src = (rr & 7) * 4, half = rr >> 3, mt = lane >> 4;
    const float v00 = __shfl_sync(0xffffffffu, out_rows[0][0], src);
    const float v01 = __shfl_sync(0xffffffffu, out_rows[0][1], src);
    const float v10 = __shfl_sync(0xffffffffu, out_rows[1][0], src);
    const float v11 = __shfl_sync(0xffffffffu, out_rows[1][1], src);
    __syncwarp();
    return mt == 0 ? (half ? v01 : v00) : (half ? v11 : v10);
}

}  // namespace tr
