// Learned warm start: model object, training kernels (forward / backward /
// AdamW, hand-written, FP32) and the C ABI around them.
//
// Training pairs are what the plain routing solves: for every segment solve
// (qup, quc, qdp, ql, dx, s0, n, bw) and the depth the secant converged to
// (recorded by the routing kernel, see troute_record_pairs). The network maps
// standardised logarithms of the eight inputs to the standardised logarithm of
// the depth; the loss is the mean squared error in those units.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "warm.cuh"

namespace tr {

// Flat parameter vector: W1 [64][8] (out x in), b1 [64], W2 [64][64], b2 [64],
// w3 [64], b3.
constexpr int kP_W1 = 0, kP_B1 = kP_W1 + kWHid * kWIn, kP_W2 = kP_B1 + kWHid, kP_B2 = kP_W2 + kWHid * kWHid,
              kP_W3 = kP_B2 + kWHid, kP_B3 = kP_W3 + kWHid, kNParams = kP_B3 + 1;
constexpr int kPairW = 9;  // qup quc qdp ql dx s0 n bw depth
constexpr int kTrainRows = 64;

struct Norm {
    float mu[kWIn], sd[kWIn], mu_y, sd_y;
};

__device__ __forceinline__ bool pair_features(const float* pr, const Norm& nm, float (&x)[kWIn], float* y)
{
    const float h = pr[8];
    if (!(h > 0.0f) || !isfinite(h)) return false;
    for (int k = 0; k < kWIn; ++k) {
        const float v = (k < 4) ? pr[k] + kFlowFloor : pr[k];
        if (!(v > 0.0f) || !isfinite(v)) return false;
        x[k] = (logf(v) - nm.mu[k]) / nm.sd[k];
    }
    *y = (logf(h) - nm.mu_y) / nm.sd_y;
    return true;
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float dsilu_f(float z)
{
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// Per-block sums of the log features and log depth (and their squares) over
// the valid pairs, for the standardisation. Fixed-order reductions: the
// result does not depend on scheduling.
constexpr int kMomThreads = 256;
constexpr int kMomBlocks = 1024;
constexpr int kMomW = 2 * kPairW + 1;

__global__ void __launch_bounds__(kMomThreads) warm_moments_kernel(const float* __restrict__ pairs, long long n,
                                                                   long long stride, double* __restrict__ part)
{
    __shared__ double red[kMomThreads];
    double acc[kMomW] = {};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i * stride < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float* pr = pairs + (i * stride) * kPairW;
        bool ok = true;
        double v[kPairW];
        for (int k = 0; k < kPairW; ++k) {
            const float raw = (k < 4) ? pr[k] + kFlowFloor : pr[k];
            if (!(raw > 0.0f) || !isfinite(raw)) ok = false;
            v[k] = ok ? log((double)raw) : 0.0;
        }
        if (!ok) continue;
        for (int k = 0; k < kPairW; ++k) {
            acc[k] += v[k];
            acc[kPairW + k] += v[k] * v[k];
        }
        acc[2 * kPairW] += 1.0;
    }
    for (int k = 0; k < kMomW; ++k) {
        red[threadIdx.x] = acc[k];
        __syncthreads();
        for (int w = kMomThreads / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[(size_t)blockIdx.x * kMomW + k] = red[0];
        __syncthreads();
    }
}

// One mini-batch block of kTrainRows samples: forward, backward, and the
// block's gradient (part[block][kNParams]) and loss sum (loss_part[block]).
// Sample i of the batch is pair (perm_a * i + perm_b) mod n, a permutation of
// the pairs when gcd(perm_a, n) = 1. Every sum runs in a fixed order, so a
// training run is reproducible bit for bit.
__global__ void __launch_bounds__(kTrainRows) warm_fb_kernel(const float* __restrict__ pairs, long long n,
                                                             long long offset, int batch, unsigned long long perm_a,
                                                             unsigned long long perm_b, const float* __restrict__ prm,
                                                             Norm nm, float* __restrict__ part,
                                                             double* __restrict__ loss_part, float inv_batch)
{
    extern __shared__ float sm[];
    float* W1 = sm;                          // 512
    float* B1 = W1 + kWHid * kWIn;           // 64
    float* W2 = B1 + kWHid;                  // 4096
    float* B2 = W2 + kWHid * kWHid;          // 64
    float* W3 = B2 + kWHid;                  // 64
    float* G = W3 + kWHid;                   // [64] d(loss)/d(out) per sample
    float* E = G + kTrainRows;               // [64] (err^2)/2 per sample
    float* X = E + kTrainRows;               // [64][8]
    float* Z1 = X + kTrainRows * kWIn;       // [64][65] pre-activations, then dZ1
    float* A1 = Z1 + kTrainRows * 65;        // [64][65]
    float* Z2 = A1 + kTrainRows * 65;        // [64][65] pre-activations, then dZ2
    const int tid = threadIdx.x;
    for (int i = tid; i < kP_B3; i += blockDim.x) W1[i] = prm[i];
    __syncthreads();
    const float b3 = prm[kP_B3];
    const long long i = offset + (long long)blockIdx.x * kTrainRows + tid;
    float x[kWIn] = {};
    float y = 0.0f;
    bool valid = false;
    if (i < offset + batch) {
        const unsigned long long p = (perm_a * (unsigned long long)i + perm_b) % (unsigned long long)n;
        valid = pair_features(pairs + p * kPairW, nm, x, &y);
        if (!valid)
            for (int k = 0; k < kWIn; ++k) x[k] = 0.0f;
    }
    for (int k = 0; k < kWIn; ++k) X[tid * kWIn + k] = x[k];
    // forward
    for (int j = 0; j < kWHid; ++j) {
        float z = B1[j];
        for (int k = 0; k < kWIn; ++k) z += W1[j * kWIn + k] * x[k];
        Z1[tid * 65 + j] = z;
        A1[tid * 65 + j] = silu_f(z);
    }
    float out = b3;
    for (int j = 0; j < kWHid; ++j) {
        float z = B2[j];
        for (int k = 0; k < kWHid; ++k) z += W2[j * kWHid + k] * A1[tid * 65 + k];
        Z2[tid * 65 + j] = z;
        out += W3[j] * silu_f(z);
    }
    const float err = valid ? (out - y) : 0.0f;
    G[tid] = err * inv_batch;  // loss = sum(err^2) / (2 batch)
    E[tid] = 0.5f * err * err;
    __syncthreads();
    float* gp = part + (size_t)blockIdx.x * kNParams;
    {
        // dw3[j] = sum_s G[s] silu(Z2[s][j]) (thread j); db3, loss (thread 0)
        const int j = tid;
        float acc = 0.0f;
        for (int s = 0; s < kTrainRows; ++s) acc += G[s] * silu_f(Z2[s * 65 + j]);
        gp[kP_W3 + j] = acc;
        if (tid == 0) {
            float gb = 0.0f;
            double ls = 0.0;
            for (int s = 0; s < kTrainRows; ++s) {
                gb += G[s];
                ls += (double)E[s];
            }
            gp[kP_B3] = gb;
            loss_part[blockIdx.x] = ls;
        }
    }
    __syncthreads();
    // dZ2 (own row, in place)
    for (int j = 0; j < kWHid; ++j) Z2[tid * 65 + j] = G[tid] * W3[j] * dsilu_f(Z2[tid * 65 + j]);
    __syncthreads();
    // dW2[j][k] = sum_s dZ2[s][j] A1[s][k], db2[j] (thread j)
    {
        const int j = tid;
        float db = 0.0f;
        for (int s = 0; s < kTrainRows; ++s) db += Z2[s * 65 + j];
        gp[kP_B2 + j] = db;
        for (int k = 0; k < kWHid; ++k) {
            float acc = 0.0f;
            for (int s = 0; s < kTrainRows; ++s) acc += Z2[s * 65 + j] * A1[s * 65 + k];
            gp[kP_W2 + j * kWHid + k] = acc;
        }
    }
    // dZ1 (own row, in place): dA1[k] = sum_j W2[j][k] dZ2[j]
    for (int k = 0; k < kWHid; ++k) {
        float da = 0.0f;
        for (int j = 0; j < kWHid; ++j) da += W2[j * kWHid + k] * Z2[tid * 65 + j];
        Z1[tid * 65 + k] = da * dsilu_f(Z1[tid * 65 + k]);
    }
    __syncthreads();
    {
        const int j = tid;
        float db = 0.0f;
        float acc[kWIn] = {};
        for (int s = 0; s < kTrainRows; ++s) {
            const float d = Z1[s * 65 + j];
            db += d;
            for (int k = 0; k < kWIn; ++k) acc[k] += d * X[s * kWIn + k];
        }
        gp[kP_B1 + j] = db;
        for (int k = 0; k < kWIn; ++k) gp[kP_W1 + j * kWIn + k] = acc[k];
    }
}

// grad[i] = sum over blocks of part[b][i], blocks in order; loss likewise.
__global__ void warm_reduce_kernel(const float* __restrict__ part, int nblocks, float* __restrict__ grad,
                                   const double* __restrict__ loss_part, double* __restrict__ loss_acc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kNParams) {
        float g = 0.0f;
        for (int b = 0; b < nblocks; ++b) g += part[(size_t)b * kNParams + i];
        grad[i] = g;
    }
    if (i == 0) {
        double l = 0.0;
        for (int b = 0; b < nblocks; ++b) l += loss_part[b];
        *loss_acc += l;
    }
}

__global__ void warm_adamw_kernel(float* __restrict__ prm, const float* __restrict__ grad, float* __restrict__ m,
                                  float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float wd,
                                  float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float g = grad[i];
        const float mi = b1 * m[i] + (1.0f - b1) * g;
        const float vi = b2 * v[i] + (1.0f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        const bool is_weight = (i < kP_B1) || (i >= kP_W2 && i < kP_B2) || (i >= kP_W3 && i < kP_B3);
        float p = prm[i];
        if (is_weight) p -= lr * wd * p;
        p -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        prm[i] = p;
    }
}

// Pair compaction: valid rows (depth > 0) per 1024-row block, then their
// scatter to the block's offset in row order.
constexpr int kCompactRows = 1024;

__global__ void __launch_bounds__(kCompactRows) pair_count_kernel(const float* __restrict__ dense, long long n,
                                                                  int* __restrict__ counts)
{
    const long long i = (long long)blockIdx.x * kCompactRows + threadIdx.x;
    const bool ok = i < n && dense[i * kPairW + 8] > 0.0f;
    const int c = __syncthreads_count(ok);
    if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

__global__ void __launch_bounds__(kCompactRows) pair_scatter_kernel(const float* __restrict__ dense, long long n,
                                                                    const long long* __restrict__ offsets,
                                                                    float* __restrict__ out, long long capacity)
{
    __shared__ int warp_cnt[kCompactRows / 32];
    const long long i = (long long)blockIdx.x * kCompactRows + threadIdx.x;
    const bool ok = i < n && dense[i * kPairW + 8] > 0.0f;
    const unsigned b = __ballot_sync(0xffffffffu, ok);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) warp_cnt[w] = __popc(b);
    __syncthreads();
    int before = 0;
    for (int k = 0; k < w; ++k) before += warp_cnt[k];
    before += __popc(b & ((1u << lane) - 1u));
    const long long dst = offsets[blockIdx.x] + before;
    if (ok && dst < capacity)
        for (int k = 0; k < kPairW; ++k) out[dst * kPairW + k] = dense[i * kPairW + k];
}

int compact_pairs(const float* dense, long long n_rows, float* out, long long capacity, long long* n_valid,
                  void* stream)
{
    *n_valid = 0;
    if (n_rows <= 0) return TROUTE_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const long long nb = (n_rows + kCompactRows - 1) / kCompactRows;
    if (nb > 0x7fffffffLL) return set_error(TROUTE_EINVAL, "too many pair rows");
    int* d_counts = nullptr;
    long long* d_off = nullptr;
    cudaError_t e = cudaMalloc(&d_counts, nb * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&d_off, nb * sizeof(long long));
    std::vector<int> counts(nb);
    std::vector<long long> off(nb);
    if (e == cudaSuccess) {
        pair_count_kernel<<<(unsigned)nb, kCompactRows, 0, st>>>(dense, n_rows, d_counts);
        e = cudaMemcpyAsync(counts.data(), d_counts, nb * sizeof(int), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    long long tot = 0;
    for (long long b = 0; b < nb; ++b) {
        off[b] = tot;
        tot += counts[b];
    }
    if (e == cudaSuccess && out && capacity > 0) {
        e = cudaMemcpyAsync(d_off, off.data(), nb * sizeof(long long), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            pair_scatter_kernel<<<(unsigned)nb, kCompactRows, 0, st>>>(dense, n_rows, d_off, out, capacity);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFree(d_counts);
    cudaFree(d_off);
    if (e != cudaSuccess) return set_error(TROUTE_ECUDA, "pair compaction: %s", cudaGetErrorString(e));
    *n_valid = tot;
    return TROUTE_OK;
}

}  // namespace tr

using namespace tr;

struct troute_warm {
    float prm[kNParams];
    Norm nm;
    bool trained = false;
    // device: fp32 master copy, AdamW moments, gradient; bf16 inference layout;
    // per-block partial gradients / losses / moments of the training kernels
    float *d_prm = nullptr, *d_m = nullptr, *d_v = nullptr, *d_g = nullptr;
    __nv_bfloat16 *d_w1t = nullptr, *d_w2t = nullptr, *d_w3t = nullptr;
    float *d_b1 = nullptr, *d_b2 = nullptr;
    double *d_loss = nullptr, *d_mom = nullptr;
    float* d_part = nullptr;
    double* d_lpart = nullptr;
    int part_blocks = 0;

    ~troute_warm()
    {
        for (void* p : {(void*)d_prm, (void*)d_m, (void*)d_v, (void*)d_g, (void*)d_w1t, (void*)d_w2t, (void*)d_w3t,
                        (void*)d_b1, (void*)d_b2, (void*)d_loss, (void*)d_mom, (void*)d_part, (void*)d_lpart})
            if (p) cudaFree(p);
    }
};

static int warm_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return TROUTE_OK;
    return set_error(e == cudaErrorMemoryAllocation ? TROUTE_ENOMEM : TROUTE_ECUDA, "%s: %s", what,
                     cudaGetErrorString(e));
}

static int warm_alloc(troute_warm* w)
{
    if (w->d_prm) return TROUTE_OK;
    int rc;
    if ((rc = warm_cuda(cudaMalloc(&w->d_prm, kNParams * sizeof(float)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_m, kNParams * sizeof(float)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_v, kNParams * sizeof(float)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_g, kNParams * sizeof(float)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_w1t, kWHid * kWK1 * sizeof(__nv_bfloat16)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_w2t, kWHid * kWHid * sizeof(__nv_bfloat16)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_w3t, kWOut * kWHid * sizeof(__nv_bfloat16)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_b1, kWHid * sizeof(float)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_b2, kWHid * sizeof(float)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_loss, sizeof(double)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_mom, (size_t)kMomBlocks * kMomW * sizeof(double)), "cudaMalloc")))
        return rc;
    return TROUTE_OK;
}

// Room for the per-block partials of a mini-batch of nblocks blocks.
static int warm_parts(troute_warm* w, int nblocks)
{
    if (nblocks <= w->part_blocks) return TROUTE_OK;
    if (w->d_part) cudaFree(w->d_part);
    if (w->d_lpart) cudaFree(w->d_lpart);
    w->d_part = nullptr;
    w->d_lpart = nullptr;
    w->part_blocks = 0;
    int rc;
    if ((rc = warm_cuda(cudaMalloc(&w->d_part, (size_t)nblocks * kNParams * sizeof(float)), "cudaMalloc")) ||
        (rc = warm_cuda(cudaMalloc(&w->d_lpart, (size_t)nblocks * sizeof(double)), "cudaMalloc")))
        return rc;
    w->part_blocks = nblocks;
    return TROUTE_OK;
}

constexpr size_t kFbSmem = (size_t)(kP_B3 + 2 * kTrainRows + kTrainRows * kWIn + 3 * kTrainRows * 65) * sizeof(float);

// Gradient (into d_g) and loss sum (added to *d_loss) of one mini-batch.
static int warm_fb(troute_warm* w, const float* pairs, long long n, long long off, int b, unsigned long long pa,
                   unsigned long long pb, float inv_batch)
{
    const int nblocks = (b + kTrainRows - 1) / kTrainRows;
    int rc = warm_parts(w, nblocks);
    if (rc) return rc;
    warm_fb_kernel<<<nblocks, kTrainRows, kFbSmem>>>(pairs, n, off, b, pa, pb, w->d_prm, w->nm, w->d_part, w->d_lpart,
                                                     inv_batch);
    warm_reduce_kernel<<<(kNParams + 255) / 256, 256>>>(w->d_part, nblocks, w->d_g, w->d_lpart, w->d_loss);
    return TROUTE_OK;
}

// Rounds the fp32 weights to the bf16, transposed, padded layout of the MMA path.
static int warm_publish(troute_warm* w)
{
    std::vector<__nv_bfloat16> w1t(kWHid * kWK1), w2t(kWHid * kWHid), w3t(kWOut * kWHid);
    for (int n = 0; n < kWHid; ++n)
        for (int k = 0; k < kWK1; ++k)
            w1t[n * kWK1 + k] = __float2bfloat16_rn(k < kWIn ? w->prm[kP_W1 + n * kWIn + k] : 0.0f);
    for (int n = 0; n < kWHid; ++n)
        for (int k = 0; k < kWHid; ++k) w2t[n * kWHid + k] = __float2bfloat16_rn(w->prm[kP_W2 + n * kWHid + k]);
    for (int n = 0; n < kWOut; ++n)
        for (int k = 0; k < kWHid; ++k) w3t[n * kWHid + k] = __float2bfloat16_rn(n == 0 ? w->prm[kP_W3 + k] : 0.0f);
    int rc;
    if ((rc = warm_cuda(cudaMemcpy(w->d_w1t, w1t.data(), w1t.size() * 2, cudaMemcpyHostToDevice), "H2D")) ||
        (rc = warm_cuda(cudaMemcpy(w->d_w2t, w2t.data(), w2t.size() * 2, cudaMemcpyHostToDevice), "H2D")) ||
        (rc = warm_cuda(cudaMemcpy(w->d_w3t, w3t.data(), w3t.size() * 2, cudaMemcpyHostToDevice), "H2D")) ||
        (rc = warm_cuda(cudaMemcpy(w->d_b1, w->prm + kP_B1, kWHid * 4, cudaMemcpyHostToDevice), "H2D")) ||
        (rc = warm_cuda(cudaMemcpy(w->d_b2, w->prm + kP_B2, kWHid * 4, cudaMemcpyHostToDevice), "H2D")))
        return rc;
    return TROUTE_OK;
}

namespace tr {
WarmDev warm_device_view(const troute_warm* w, double delta, int k)
{
    WarmDev m;
    m.w1t = w->d_w1t;
    m.w2t = w->d_w2t;
    m.w3t = w->d_w3t;
    m.b1 = w->d_b1;
    m.b2 = w->d_b2;
    m.b3 = w->prm[kP_B3];
    for (int i = 0; i < kWIn; ++i) {
        m.mu[i] = w->nm.mu[i];
        m.sd[i] = w->nm.sd[i];
        m.inv_sd[i] = 1.0f / w->nm.sd[i];
    }
    m.mu_y = w->nm.mu_y;
    m.sd_y = w->nm.sd_y;
    m.delta = delta;
    m.k = k;
    return m;
}
bool warm_ready(const troute_warm* w) { return w && w->d_w1t && w->trained; }
}  // namespace tr

extern "C" int troute_warm_create(troute_warm** out, uint64_t seed)
{
    if (!out) return set_error(TROUTE_EINVAL, "null pointer");
    auto* w = new (std::nothrow) troute_warm();
    if (!w) return set_error(TROUTE_ENOMEM, "model allocation");
    // He-style initialisation from the seed (counter-based, platform independent)
    for (int i = 0; i < kNParams; ++i) {
        const double u = u01(hash3(seed, 777, (uint64_t)i)) * 2.0 - 1.0;
        double scale = 0.0;
        if (i < kP_B1) scale = std::sqrt(6.0 / kWIn);
        else if (i >= kP_W2 && i < kP_B2) scale = std::sqrt(6.0 / kWHid);
        else if (i >= kP_W3 && i < kP_B3) scale = std::sqrt(6.0 / kWHid);
        w->prm[i] = (float)(u * scale * 0.5);
    }
    for (int k = 0; k < kWIn; ++k) {
        w->nm.mu[k] = 0.0f;
        w->nm.sd[k] = 1.0f;
    }
    w->nm.mu_y = 0.0f;
    w->nm.sd_y = 1.0f;
    *out = w;
    return TROUTE_OK;
}

extern "C" int troute_warm_destroy(troute_warm* w)
{
    delete w;
    return TROUTE_OK;
}

// params: [kNParams] then mu[8], sd[8], mu_y, sd_y
extern "C" int troute_warm_get(const troute_warm* w, float* params, int n)
{
    if (!w || !params || n < kNParams + 2 * kWIn + 2) return set_error(TROUTE_EINVAL, "need %d floats", kNParams + 2 * kWIn + 2);
    std::memcpy(params, w->prm, sizeof w->prm);
    std::memcpy(params + kNParams, w->nm.mu, sizeof w->nm.mu);
    std::memcpy(params + kNParams + kWIn, w->nm.sd, sizeof w->nm.sd);
    params[kNParams + 2 * kWIn] = w->nm.mu_y;
    params[kNParams + 2 * kWIn + 1] = w->nm.sd_y;
    return TROUTE_OK;
}

extern "C" int troute_warm_set(troute_warm* w, const float* params, int n)
{
    if (!w || !params || n < kNParams + 2 * kWIn + 2) return set_error(TROUTE_EINVAL, "need %d floats", kNParams + 2 * kWIn + 2);
    std::memcpy(w->prm, params, sizeof w->prm);
    std::memcpy(w->nm.mu, params + kNParams, sizeof w->nm.mu);
    std::memcpy(w->nm.sd, params + kNParams + kWIn, sizeof w->nm.sd);
    w->nm.mu_y = params[kNParams + 2 * kWIn];
    w->nm.sd_y = params[kNParams + 2 * kWIn + 1];
    int rc = warm_alloc(w);
    if (rc) return rc;
    if ((rc = warm_publish(w))) return rc;
    w->trained = true;
    return TROUTE_OK;
}

// Standardisation constants from the pairs (every stride-th pair).
static int warm_normalise(troute_warm* w, const float* pairs_dev, long long n, long long stride)
{
    int rc;
    warm_moments_kernel<<<kMomBlocks, kMomThreads>>>(pairs_dev, n, stride, w->d_mom);
    std::vector<double> part((size_t)kMomBlocks * kMomW);
    if ((rc = warm_cuda(cudaMemcpy(part.data(), w->d_mom, part.size() * sizeof(double), cudaMemcpyDeviceToHost),
                        "moments")))
        return rc;
    double acc[kMomW] = {};
    for (int b = 0; b < kMomBlocks; ++b)
        for (int k = 0; k < kMomW; ++k) acc[k] += part[(size_t)b * kMomW + k];
    const double cnt = acc[2 * kPairW];
    if (cnt < 2) return set_error(TROUTE_EINVAL, "no valid training pairs");
    float mu[kPairW], sd[kPairW];
    for (int k = 0; k < kPairW; ++k) {
        const double m = acc[k] / cnt;
        const double var = acc[kPairW + k] / cnt - m * m;
        mu[k] = (float)m;
        sd[k] = (float)std::sqrt(var > 1e-12 ? var : 1e-12);
    }
    for (int k = 0; k < kWIn; ++k) {
        w->nm.mu[k] = mu[k];
        w->nm.sd[k] = sd[k];
    }
    w->nm.mu_y = mu[8];
    w->nm.sd_y = sd[8];
    return TROUTE_OK;
}

static unsigned long long coprime_near(unsigned long long n, unsigned long long want)
{
    auto gcd = [](unsigned long long a, unsigned long long b) {
        while (b) { const unsigned long long t = a % b; a = b; b = t; }
        return a;
    };
    unsigned long long a = want % n;
    if (a == 0) a = 1;
    while (gcd(a, n) != 1) a = (a + 1) % n ? (a + 1) % n : 1;
    return a;
}

extern "C" int troute_warm_fit(troute_warm* w, const float* pairs_dev, long long n_pairs, int epochs, int batch,
                               float lr, float weight_decay, uint64_t seed, float* loss_per_epoch)
{
    if (!w || !pairs_dev || n_pairs < 2 || epochs < 1 || batch < kTrainRows || lr <= 0.0f)
        return set_error(TROUTE_EINVAL, "bad training arguments");
    int rc = warm_alloc(w);
    if (rc) return rc;
    if ((rc = warm_normalise(w, pairs_dev, n_pairs, n_pairs > 4000000 ? n_pairs / 4000000 : 1))) return rc;
    batch = (batch / kTrainRows) * kTrainRows;
    if ((rc = warm_cuda(cudaMemcpy(w->d_prm, w->prm, sizeof w->prm, cudaMemcpyHostToDevice), "H2D")) ||
        (rc = warm_cuda(cudaMemset(w->d_m, 0, kNParams * sizeof(float)), "memset")) ||
        (rc = warm_cuda(cudaMemset(w->d_v, 0, kNParams * sizeof(float)), "memset")))
        return rc;
    if ((rc = warm_cuda(cudaFuncSetAttribute(warm_fb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kFbSmem), "smem attribute")))
        return rc;
    const long long steps_per_epoch = (n_pairs + batch - 1) / batch;
    const long long total = steps_per_epoch * epochs;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    long long step = 0;
    for (int ep = 0; ep < epochs; ++ep) {
        const unsigned long long pa = coprime_near((unsigned long long)n_pairs, hash3(seed, 31, ep) | 1ull);
        const unsigned long long pb = hash3(seed, 37, ep) % (unsigned long long)n_pairs;
        if ((rc = warm_cuda(cudaMemset(w->d_loss, 0, sizeof(double)), "memset"))) return rc;
        for (long long s = 0; s < steps_per_epoch; ++s, ++step) {
            const long long off = s * batch;
            const int b = (int)std::min<long long>(batch, n_pairs - off);
            if ((rc = warm_fb(w, pairs_dev, n_pairs, off, b, pa, pb, 1.0f / (float)b))) return rc;
            // cosine decay of the step size
            const float frac = (float)step / (float)std::max<long long>(1, total - 1);
            const float lr_t = lr * 0.5f * (1.0f + std::cos(3.14159265f * frac));
            const float c1 = 1.0f - std::pow(b1, (float)(step + 1)), c2 = 1.0f - std::pow(b2, (float)(step + 1));
            warm_adamw_kernel<<<(kNParams + 255) / 256, 256>>>(w->d_prm, w->d_g, w->d_m, w->d_v, kNParams, lr_t, b1,
                                                               b2, eps, weight_decay, c1, c2);
        }
        double loss = 0.0;
        if ((rc = warm_cuda(cudaMemcpy(&loss, w->d_loss, sizeof(double), cudaMemcpyDeviceToHost), "loss"))) return rc;
        // each step's loss is sum(err^2)/2 over its batch: the epoch mean per pair
        if (loss_per_epoch) loss_per_epoch[ep] = (float)(loss / (double)n_pairs);
    }
    if ((rc = warm_cuda(cudaMemcpy(w->prm, w->d_prm, sizeof w->prm, cudaMemcpyDeviceToHost), "D2H"))) return rc;
    if ((rc = warm_publish(w))) return rc;
    w->trained = true;
    return warm_cuda(cudaGetLastError(), "training");
}

extern "C" int troute_warm_grad(troute_warm* w, const float* pairs_host, int n, float* grad_out, double* loss_out)
{
    if (!w || !pairs_host || n < 1 || !grad_out) return set_error(TROUTE_EINVAL, "bad arguments");
    int rc = warm_alloc(w);
    if (rc) return rc;
    float* d_pairs = nullptr;
    if ((rc = warm_cuda(cudaMalloc(&d_pairs, (size_t)n * kPairW * sizeof(float)), "cudaMalloc"))) return rc;
    rc = warm_cuda(cudaMemcpy(d_pairs, pairs_host, (size_t)n * kPairW * sizeof(float), cudaMemcpyHostToDevice), "H2D");
    if (!rc) rc = warm_cuda(cudaMemcpy(w->d_prm, w->prm, sizeof w->prm, cudaMemcpyHostToDevice), "H2D");
    if (!rc) rc = warm_cuda(cudaMemset(w->d_loss, 0, sizeof(double)), "memset");
    if (!rc)
        rc = warm_cuda(cudaFuncSetAttribute(warm_fb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFbSmem),
                       "smem attribute");
    if (!rc) rc = warm_fb(w, d_pairs, n, 0, n, 1, 0, 1.0f / (float)n);
    if (!rc) rc = warm_cuda(cudaMemcpy(grad_out, w->d_g, kNParams * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
    double loss = 0.0;
    if (!rc) rc = warm_cuda(cudaMemcpy(&loss, w->d_loss, sizeof(double), cudaMemcpyDeviceToHost), "D2H");
    cudaFree(d_pairs);
    if (loss_out) *loss_out = loss / n;
    return rc;
}

extern "C" int troute_warm_predict(troute_warm* w, const float* raw_host, int n, double* depth_out)
{
    if (!w || !raw_host || n < 1 || !depth_out) return set_error(TROUTE_EINVAL, "bad arguments");
    if (!w->trained) return set_error(TROUTE_ESTATE, "model has no weights (train or set them first)");
    float* d_raw = nullptr;
    double* d_out = nullptr;
    int* d_err = nullptr;
    int rc = warm_cuda(cudaMalloc(&d_raw, (size_t)n * kWIn * sizeof(float)), "cudaMalloc");
    if (!rc) rc = warm_cuda(cudaMalloc(&d_out, (size_t)n * sizeof(double)), "cudaMalloc");
    if (!rc) rc = warm_cuda(cudaMalloc(&d_err, sizeof(int)), "cudaMalloc");
    if (!rc) rc = warm_cuda(cudaMemset(d_err, 0, sizeof(int)), "memset");
    if (!rc) rc = warm_cuda(cudaMemcpy(d_raw, raw_host, (size_t)n * kWIn * sizeof(float), cudaMemcpyHostToDevice), "H2D");
    if (!rc) rc = launch_warm_gemm_raw(w, d_raw, n, d_out, d_err, nullptr);
    int err = 0;
    if (!rc) rc = warm_cuda(cudaMemcpy(depth_out, d_out, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
    if (!rc) rc = warm_cuda(cudaMemcpy(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost), "D2H");
    cudaFree(d_raw);
    cudaFree(d_out);
    cudaFree(d_err);
    if (!rc && err) rc = set_error(err, "warm GEMM: a tensor-core completion wait ran out");
    return rc;
}
