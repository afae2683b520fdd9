// Learned warm start of the secant depth solve: an 8 -> 64 -> 64 -> 1 MLP
// (SiLU) that predicts a segment's converged flow depth from its normalised
// inflows, geometry, slope and Manning's n. The model's device view and the
// feature and activation functions; the training kernels live in warm.cu, the
// tcgen05 inference GEMM in warm_gemm.cu.
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

}  // namespace tr
