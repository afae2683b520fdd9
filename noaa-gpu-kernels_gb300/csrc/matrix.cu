// Matrix-form linearised Muskingum-Cunge: the reference's fastest
// approximate mode (water-prediction/t-route/wavefront/linear_mc_matrix.cu,
// with the fused one-pass step of linear_mc_matrix_graph.cu).
//
// A reach-level network (one routing unit per reach) with fixed coefficients
// C1..C3, C4/ql at X = 0.25 (compute_mc_coeffs_cpu, linear_mc_matrix.cu:
// 56-86) is linear time-invariant:
//
//   Q_new = C1 N Q_new + C2 N Q_old + C3 Q_old + C4 qlat
//         = P_Q Q_old + P_q qlat,   P_Q = A^-1 (C2 N + C3),  P_q = A^-1 C4,
//
// with A = I - C1 N and N the upstream adjacency. A^-1 is the sum over
// upstream paths of products of C1; the matrices are built once, row by row
// in reach order with entries below a tolerance dropped
// (build_propagation_matrices, :129-216), and every step is then one pass
// over two sparse matrices: no level order, no dependency between reaches
// within a step.
//
// Build (host, once): rows are assembled into the CSR arrays in reach order
// (reaches are numbered upstream first, so an upstream row is always final
// when it is read); row r = C1[r] x (the rows of its upstream reaches, merged
// in upstream-list order), entries with |v| < tol dropped, C2[r] added at each
// upstream reach and C3[r] at r (P_q: C4/ql[r] at r), dropped again -- the
// reference's float operations in its order, so the matrices are bit for bit
// the reference's given the same coefficients.
//
// Step (device): y[r] = sum_k P_Q[r,k] x[k] + sum_k P_q[r,k] ql[k]. The step
// is HBM-bound (8 bytes per stored entry, each entry a (column, value) pair
// read by one streaming load; the ~4 MB vectors stay in L2). The sum keeps the
// reference kernel's arithmetic exactly (kernel_spmv_fused,
// linear_mc_matrix_graph.cu:174-206: lane l of 32 accumulates entries l,
// l + 32, ... of each matrix by fused multiply-add, adds the two partials,
// then the shuffle-down tree 16, 8, 4, 2, 1). Row lengths are heavily skewed
// (on a 1.1 M-reach network the median row holds 1 entry, 14 % of rows hold
// more than 32 and those hold 80 % of the entries), so rows take one of two
// paths:
//  - short rows (at most 32 entries in each matrix) by 4 lanes: lane p holds
//    the reference's lanes p, p + 4, ..., p + 28, performs the tree's first
//    three levels (offsets 16, 8, 4) in registers in the same pairing and the
//    last two by shuffles in its 4-lane group; a warp covers 8 rows;
//  - long rows by the whole warp, lane l being the reference's lane l, each
//    lane issuing the loads of several of its entries before it gathers and
//    adds them, so a row of hundreds of entries costs a few memory round
//    trips instead of one per entry.
// Blocks of 64 threads: a block's slot frees as soon as its two warps finish,
// so warps held up by long rows do not keep idle warps resident. (Measured
// on a 1.1 M-reach network, 144 steps: 8 lanes per short row in blocks of
// 256 22.5 ms, 4 lanes in blocks of 128 16.4 ms, of 64 15.9 ms; 2 lanes
// 23.6 ms; 8 entries per lane and batch on long rows instead of 4 slower.)
//
// A run of n_ts steps is recorded once as a CUDA graph of n_ts launches
// (alternating two discharge buffers) and replayed while the caller's
// buffers and step count stay the same.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <stdexcept>
#include <vector>

#include "troute_internal.h"

namespace tr {
namespace {

constexpr unsigned kFullMask = 0xffffffffu;
#ifndef TROUTE_MAT_THREADS
#define TROUTE_MAT_THREADS 64
#endif
#ifndef TROUTE_MAT_LONG_BATCH
#define TROUTE_MAT_LONG_BATCH 4
#endif
#ifndef TROUTE_MAT_LANES
#define TROUTE_MAT_LANES 4
#endif
constexpr int kMatThreads = TROUTE_MAT_THREADS;
constexpr int kLanesPerRow = TROUTE_MAT_LANES;   // lanes of a short row
constexpr int kRefPerLane = 32 / kLanesPerRow;   // the reference's lanes each of them holds
static_assert(kLanesPerRow >= 2 && kLanesPerRow <= 16 && 32 % kLanesPerRow == 0, "lanes per short row");
constexpr int kRowsPerBlock = kMatThreads / kLanesPerRow;

// Coefficients of one reach at X = 0.25 (linear_mc_matrix.cu:56-86), FP32 in
// the reference's operation order; powf / sqrtf are CUDA's.
__device__ __forceinline__ float4 mat_coeffs(const troute_chparams_f32& p, float dt)
{
    const float z = (p.cs == 0.0f) ? 1.0f : 1.0f / p.cs;
    float bfd;
    if (p.bw > p.tw) bfd = p.bw / 0.00001f;
    else if (p.bw == p.tw) bfd = p.bw / (2.0f * z);
    else bfd = (p.tw - p.bw) / (2.0f * z);
    const float h = fmaxf(0.5f * bfd, 0.1f);
    const float A = (p.bw + h * z) * h;
    const float WP = p.bw + 2.0f * h * sqrtf(1.0f + z * z);
    const float R = (WP > 0.0f) ? A / WP : 0.0f;
    const float r23 = powf(R, 2.0f / 3.0f);
    const float r53 = powf(R, 5.0f / 3.0f);
    const float Ck = fmaxf(1e-6f, (sqrtf(p.s0) / p.n_ch) *
                                      ((5.0f / 3.0f) * r23 -
                                       (2.0f / 3.0f) * r53 * (2.0f * sqrtf(1.0f + z * z) / (p.bw + 2.0f * h * z))));
    const float Km = fmaxf(dt, p.dx / Ck);
    const float X = 0.25f;
    float D = Km * (1.0f - X) + dt / 2.0f;
    if (D == 0.0f) D = 1.0f;
    return make_float4((Km * X + dt / 2.0f) / D, (dt / 2.0f - Km * X) / D, (Km * (1.0f - X) - dt / 2.0f) / D, dt / D);
}

__global__ void mat_coeff_kernel(const troute_chparams_f32* __restrict__ p, int n, float dt, float4* __restrict__ c)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) c[i] = mat_coeffs(p[i], dt);
}

struct MatDev {
    int R;
    const int* qp;     // P_Q row pointers [R + 1]
    const int2* qe;    // P_Q entries: (column, value bits)
    const int* lp;     // P_q row pointers [R + 1]
    const int2* le;    // P_q entries
};

// A row whose two matrices hold at most this many entries each is summed by
// a group of kLanesPerRow lanes (one entry per reference lane at most);
// longer rows by the whole warp.
constexpr int kShortRow = 32;
// Entries a lane loads per matrix before it gathers and adds, on long rows.
constexpr int kLongBatch = TROUTE_MAT_LONG_BATCH;

// Entries are read once per step: streaming loads, evicted first, so the
// gathered discharge and inflow vectors keep their place in L2.
__device__ __forceinline__ int2 ld_entry(const int2* __restrict__ e, int k) { return __ldcs(e + k); }

// Sum of one long row by the whole warp: lane l is the reference's lane l
// (entries l, l + 32, ... of each matrix, fused multiply-add from 0, the two
// partials added, then the shuffle-down tree 16, 8, 4, 2, 1); each lane loads
// kLongBatch entries of each matrix, then gathers them, then adds them in
// order. Returns the row's value in lane 0.
__device__ __forceinline__ float long_row(const MatDev& m, const float* __restrict__ x, const float* __restrict__ ql,
                                          int lane, int qb, int nq, int lb, int nl)
{
    float sq = 0.0f, sl = 0.0f;
    const int n = max(nq, nl);
    for (int k = lane; k < n; k += kLongBatch * 32) {
        int2 eq[kLongBatch], el[kLongBatch];
#pragma unroll
        for (int j = 0; j < kLongBatch; ++j) {
            const int kk = k + 32 * j;
            eq[j] = kk < nq ? ld_entry(m.qe, qb + kk) : make_int2(0, 0);
            el[j] = kk < nl ? ld_entry(m.le, lb + kk) : make_int2(0, 0);
        }
        float xq[kLongBatch], xl[kLongBatch];
#pragma unroll
        for (int j = 0; j < kLongBatch; ++j) {
            const int kk = k + 32 * j;
            xq[j] = kk < nq ? __ldg(x + eq[j].x) : 0.0f;
            xl[j] = kk < nl ? __ldg(ql + el[j].x) : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < kLongBatch; ++j) {
            const int kk = k + 32 * j;
            if (kk < nq) sq = __fmaf_rn(__int_as_float(eq[j].y), xq[j], sq);
            if (kk < nl) sl = __fmaf_rn(__int_as_float(el[j].y), xl[j], sl);
        }
    }
    float u = __fadd_rn(sq, sl);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) u = __fadd_rn(u, __shfl_down_sync(kFullMask, u, off));
    return u;
}

__global__ void __launch_bounds__(kMatThreads) mat_step_kernel(MatDev m, const float* __restrict__ x,
                                                               const float* __restrict__ ql, float* __restrict__ y)
{
    const int lane = threadIdx.x & 31;
    const int p = lane & (kLanesPerRow - 1);
    const int row = blockIdx.x * kRowsPerBlock + threadIdx.x / kLanesPerRow;
    int qb = 0, nq = 0, lb = 0, nl = 0;
    if (row < m.R) {
        qb = __ldg(m.qp + row);
        nq = __ldg(m.qp + row + 1) - qb;
        lb = __ldg(m.lp + row);
        nl = __ldg(m.lp + row + 1) - lb;
    }
    const bool is_long = nq > kShortRow || nl > kShortRow;
    float u = 0.0f;
    if (!is_long) {
        // the entry of each of the reference's lanes p, p + kLanesPerRow, ...
        // (a short row has no other): every entry load is issued before any
        // gather, and every gather before any sum
        int2 eq[kRefPerLane], el[kRefPerLane];
#pragma unroll
        for (int j = 0; j < kRefPerLane; ++j) {
            const int k = p + kLanesPerRow * j;
            eq[j] = k < nq ? ld_entry(m.qe, qb + k) : make_int2(0, 0);
            el[j] = k < nl ? ld_entry(m.le, lb + k) : make_int2(0, 0);
        }
        float xq[kRefPerLane], xl[kRefPerLane];
#pragma unroll
        for (int j = 0; j < kRefPerLane; ++j) {
            const int k = p + kLanesPerRow * j;
            xq[j] = k < nq ? __ldg(x + eq[j].x) : 0.0f;
            xl[j] = k < nl ? __ldg(ql + el[j].x) : 0.0f;
        }
        float s[kRefPerLane];
#pragma unroll
        for (int j = 0; j < kRefPerLane; ++j) {
            const int k = p + kLanesPerRow * j;
            // fma(v, x, 0) where the lane holds an entry, 0 where it holds none
            const float sq = k < nq ? __fmaf_rn(__int_as_float(eq[j].y), xq[j], 0.0f) : 0.0f;
            const float sl = k < nl ? __fmaf_rn(__int_as_float(el[j].y), xl[j], 0.0f) : 0.0f;
            s[j] = __fadd_rn(sq, sl);
        }
        // the reference's shuffle-down levels 16 .. kLanesPerRow in registers:
        // at offset o its lane v adds lane v + o; slot j holds its lane
        // p + kLanesPerRow j, so offset o adds slot j + o / kLanesPerRow onto j
#pragma unroll
        for (int h = kRefPerLane / 2; h >= 1; h >>= 1)
#pragma unroll
            for (int j = 0; j < h; ++j) s[j] = __fadd_rn(s[j], s[j + h]);
        u = s[0];
    }
    // the remaining levels inside the row's lane group (every lane takes part)
#pragma unroll
    for (int off = kLanesPerRow / 2; off >= 1; off >>= 1)
        u = __fadd_rn(u, __shfl_down_sync(kFullMask, u, off, kLanesPerRow));
    if (p == 0 && row < m.R && !is_long) y[row] = u;
    // the warp's long rows, one after another, each by all 32 lanes
    unsigned longs = __ballot_sync(kFullMask, is_long && p == 0);
    while (longs) {
        const int src = __ffs(longs) - 1;
        longs &= longs - 1;
        const int r = __shfl_sync(kFullMask, row, src);
        const float v = long_row(m, x, ql, lane, __shfl_sync(kFullMask, qb, src), __shfl_sync(kFullMask, nq, src),
                                 __shfl_sync(kFullMask, lb, src), __shfl_sync(kFullMask, nl, src));
        if (lane == 0) y[r] = v;
    }
}

template <typename T>
struct MArr {
    T* p = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        if (count <= n && p) return TROUTE_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        const cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e != cudaSuccess) return set_error(TROUTE_ENOMEM, "cudaMalloc: %s", cudaGetErrorString(e));
        n = count;
        return TROUTE_OK;
    }
    ~MArr()
    {
        if (p) cudaFree(p);
    }
};

int mat_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return TROUTE_OK;
    return set_error(e == cudaErrorMemoryAllocation ? TROUTE_ENOMEM : TROUTE_ECUDA, "%s: %s", what,
                     cudaGetErrorString(e));
}

// One matrix in CSR while it is built on the host.
struct HostCsr {
    std::vector<int> ptr, col;
    std::vector<float> val;
};

// Scratch rows of the build: sorted columns with values.
struct Row {
    std::vector<int> col;
    std::vector<float> val;
    void clear()
    {
        col.clear();
        val.clear();
    }
};

// out = acc (+) (row r of m) * scale: columns merged in order; a column in both
// takes acc + m * scale (the product rounded first).
void merge_scaled(const Row& acc, const HostCsr& m, int r, float scale, Row& out)
{
    out.clear();
    int i = 0;
    const int na = (int)acc.col.size();
    int j = m.ptr[r];
    const int je = m.ptr[r + 1];
    while (i < na && j < je) {
        if (acc.col[i] < m.col[j]) {
            out.col.push_back(acc.col[i]);
            out.val.push_back(acc.val[i++]);
        } else if (acc.col[i] > m.col[j]) {
            out.col.push_back(m.col[j]);
            out.val.push_back(m.val[j++] * scale);
        } else {
            const float prod = m.val[j++] * scale;
            out.col.push_back(acc.col[i]);
            out.val.push_back(acc.val[i++] + prod);
        }
    }
    for (; i < na; ++i) {
        out.col.push_back(acc.col[i]);
        out.val.push_back(acc.val[i]);
    }
    for (; j < je; ++j) {
        out.col.push_back(m.col[j]);
        out.val.push_back(m.val[j] * scale);
    }
}

void add_at(Row& row, int c, float v)
{
    const auto it = std::lower_bound(row.col.begin(), row.col.end(), c);
    const size_t k = (size_t)(it - row.col.begin());
    if (it != row.col.end() && *it == c) {
        row.val[k] += v;
        return;
    }
    row.col.insert(it, c);
    row.val.insert(row.val.begin() + (long)k, v);
}

void drop_small(Row& row, float tol)
{
    size_t k = 0;
    for (size_t i = 0; i < row.col.size(); ++i)
        if (!(std::fabs(row.val[i]) < tol)) {
            row.col[k] = row.col[i];
            row.val[k++] = row.val[i];
        }
    row.col.resize(k);
    row.val.resize(k);
}

void append_row(HostCsr& m, const Row& row)
{
    m.col.insert(m.col.end(), row.col.begin(), row.col.end());
    m.val.insert(m.val.end(), row.val.begin(), row.val.end());
    if (m.col.size() > 0x7FFFFFFFu) throw std::length_error("nnz");
    m.ptr.push_back((int)m.col.size());
}

// Builds P_Q and P_q (build_propagation_matrices, linear_mc_matrix.cu:129-216).
int build_matrices(int R, const int* up_ptr, const int* up_idx, const float* c1, const float* c2, const float* c3,
                   const float* c4oq, float tol, HostCsr& PQ, HostCsr& Pq)
{
    PQ = HostCsr();
    Pq = HostCsr();
    PQ.ptr.reserve((size_t)R + 1);
    Pq.ptr.reserve((size_t)R + 1);
    PQ.ptr.push_back(0);
    Pq.ptr.push_back(0);
    Row a, b, la, lb;
    for (int r = 0; r < R; ++r) {
        a.clear();
        la.clear();
        for (int k = up_ptr[r]; k < up_ptr[r + 1]; ++k) {
            const int u = up_idx[k];
            merge_scaled(a, PQ, u, c1[r], b);
            std::swap(a, b);
            merge_scaled(la, Pq, u, c1[r], lb);
            std::swap(la, lb);
        }
        drop_small(a, tol);
        drop_small(la, tol);
        for (int k = up_ptr[r]; k < up_ptr[r + 1]; ++k) add_at(a, up_idx[k], c2[r]);
        add_at(a, r, c3[r]);
        add_at(la, r, c4oq[r]);
        drop_small(a, tol);
        drop_small(la, tol);
        try {
            append_row(PQ, a);
            append_row(Pq, la);
        } catch (const std::exception&) {
            return set_error(TROUTE_ENOMEM, "matrix build: more than 2^31 entries");
        }
    }
    return TROUTE_OK;
}

}  // namespace
}  // namespace tr

using namespace tr;

struct troute_matrix {
    int R = 0;
    long long nnz_Q = 0, nnz_q = 0;
    MArr<int> qp, lp;
    MArr<int2> qe, le;
    MArr<float> tmp;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    const float* g_qlat = nullptr;
    float* g_q = nullptr;
    int g_nts = 0;
    MatDev dev() const { return MatDev{R, qp.p, qe.p, lp.p, le.p}; }
    ~troute_matrix()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (stream) cudaStreamDestroy(stream);
    }
};

extern "C" int troute_matrix_coeffs(const troute_chparams_f32* params, int n_reaches, double dt, float* c1, float* c2,
                                    float* c3, float* c4oq)
{
    if (n_reaches < 0 || !(dt > 0.0)) return set_error(TROUTE_EINVAL, "bad arguments");
    if (n_reaches == 0) return TROUTE_OK;
    if (!params || !c1 || !c2 || !c3 || !c4oq) return set_error(TROUTE_EINVAL, "null array");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");
    MArr<troute_chparams_f32> p;
    MArr<float4> c;
    int rc;
    if ((rc = p.alloc(n_reaches)) || (rc = c.alloc(n_reaches))) return rc;
    if ((rc = mat_cuda(cudaMemcpy(p.p, params, (size_t)n_reaches * sizeof *params, cudaMemcpyHostToDevice), "H2D")))
        return rc;
    mat_coeff_kernel<<<std::min(4096, (n_reaches + 255) / 256), 256>>>(p.p, n_reaches, (float)dt, c.p);
    if ((rc = mat_cuda(cudaGetLastError(), "coefficient launch"))) return rc;
    std::vector<float4> h((size_t)n_reaches);
    if ((rc = mat_cuda(cudaMemcpy(h.data(), c.p, (size_t)n_reaches * sizeof(float4), cudaMemcpyDeviceToHost), "D2H")))
        return rc;
    for (int i = 0; i < n_reaches; ++i) {
        c1[i] = h[i].x;
        c2[i] = h[i].y;
        c3[i] = h[i].z;
        c4oq[i] = h[i].w;
    }
    return TROUTE_OK;
}

extern "C" int troute_matrix_create(troute_matrix** out, int n_reaches, const int* up_ptr, const int* up_idx,
                                    const float* c1, const float* c2, const float* c3, const float* c4oq, float tol)
{
    if (!out) return set_error(TROUTE_EINVAL, "null handle pointer");
    *out = nullptr;
    if (n_reaches < 0 || !(tol >= 0.0f)) return set_error(TROUTE_EINVAL, "bad arguments");
    if (n_reaches > 0 && (!up_ptr || !c1 || !c2 || !c3 || !c4oq)) return set_error(TROUTE_EINVAL, "null array");
    if (n_reaches > 0 && (up_ptr[0] != 0 || (up_ptr[n_reaches] > 0 && !up_idx)))
        return set_error(TROUTE_ETOPO, "bad upstream CSR");
    for (int r = 0; r < n_reaches; ++r) {
        if (up_ptr[r + 1] < up_ptr[r]) return set_error(TROUTE_ETOPO, "reach %d: decreasing upstream pointer", r);
        for (int k = up_ptr[r]; k < up_ptr[r + 1]; ++k)
            if (up_idx[k] < 0 || up_idx[k] >= r)
                return set_error(TROUTE_ETOPO,
                                 "reach %d: upstream reach %d is not numbered before it (the matrix form needs reaches "
                                 "numbered upstream first)", r, up_idx[k]);
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");
    HostCsr PQ, Pq;
    int rc;
    try {
        rc = build_matrices(n_reaches, up_ptr, up_idx, c1, c2, c3, c4oq, tol, PQ, Pq);
    } catch (const std::bad_alloc&) {
        rc = set_error(TROUTE_ENOMEM, "matrix build: host memory");
    }
    if (rc) return rc;
    auto* M = new troute_matrix();
    M->R = n_reaches;
    M->nnz_Q = (long long)PQ.col.size();
    M->nnz_q = (long long)Pq.col.size();
    const size_t R1 = (size_t)n_reaches + 1;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        return bytes ? mat_cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "matrix upload") : TROUTE_OK;
    };
    // entries as (column, value bits) pairs: one 8-byte load per entry
    auto pairs = [](const HostCsr& m) {
        std::vector<int2> e(m.col.size());
        for (size_t k = 0; k < e.size(); ++k) {
            int v;
            std::memcpy(&v, &m.val[k], sizeof v);
            e[k] = make_int2(m.col[k], v);
        }
        return e;
    };
    try {
        const std::vector<int2> eQ = pairs(PQ), eq = pairs(Pq);
        rc = mat_cuda(cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking), "stream");
        if (!rc && !(rc = M->qp.alloc(R1)) && !(rc = M->qe.alloc(eQ.size())) && !(rc = M->lp.alloc(R1)) &&
            !(rc = M->le.alloc(eq.size())) && !(rc = M->tmp.alloc((size_t)std::max(1, n_reaches))) &&
            !(rc = up(M->qp.p, PQ.ptr.data(), R1 * sizeof(int))) &&
            !(rc = up(M->qe.p, eQ.data(), eQ.size() * sizeof(int2))) &&
            !(rc = up(M->lp.p, Pq.ptr.data(), R1 * sizeof(int))))
            rc = up(M->le.p, eq.data(), eq.size() * sizeof(int2));
    } catch (const std::bad_alloc&) {
        rc = set_error(TROUTE_ENOMEM, "matrix upload: host memory");
    }
    if (rc) {
        delete M;
        return rc;
    }
    *out = M;
    return TROUTE_OK;
}

extern "C" int troute_matrix_destroy(troute_matrix* M)
{
    delete M;
    return TROUTE_OK;
}

extern "C" int troute_matrix_info(const troute_matrix* M, int* n_reaches, long long* nnz_Q, long long* nnz_q)
{
    if (!M) return set_error(TROUTE_EINVAL, "null handle");
    if (n_reaches) *n_reaches = M->R;
    if (nnz_Q) *nnz_Q = M->nnz_Q;
    if (nnz_q) *nnz_q = M->nnz_q;
    return TROUTE_OK;
}

extern "C" int troute_matrix_get(const troute_matrix* M, int which, int* ptr, int* col, float* val)
{
    if (!M || (which != 0 && which != 1)) return set_error(TROUTE_EINVAL, "bad arguments");
    const size_t nnz = (size_t)(which ? M->nnz_q : M->nnz_Q);
    const int* dp = which ? M->lp.p : M->qp.p;
    const int2* de = which ? M->le.p : M->qe.p;
    int rc;
    if (ptr && (rc = mat_cuda(cudaMemcpy(ptr, dp, ((size_t)M->R + 1) * sizeof(int), cudaMemcpyDeviceToHost), "D2H")))
        return rc;
    if ((col || val) && nnz) {
        std::vector<int2> e;
        try {
            e.resize(nnz);
        } catch (const std::bad_alloc&) {
            return set_error(TROUTE_ENOMEM, "matrix download: host memory");
        }
        if ((rc = mat_cuda(cudaMemcpy(e.data(), de, nnz * sizeof(int2), cudaMemcpyDeviceToHost), "D2H"))) return rc;
        for (size_t k = 0; k < nnz; ++k) {
            if (col) col[k] = e[k].x;
            if (val) std::memcpy(&val[k], &e[k].y, sizeof(float));
        }
    }
    return TROUTE_OK;
}

// The n_ts launches of a run on `st`: step t reads a and writes b, the two
// alternating between the caller's discharge and the handle's buffer; after an
// odd number of steps the result is copied back into the caller's buffer.
static int enqueue_steps(troute_matrix* M, const float* qlat, int n_ts, float* q, cudaStream_t st)
{
    const int grid = (M->R + kRowsPerBlock - 1) / kRowsPerBlock;
    const MatDev d = M->dev();
    for (int t = 0; t < n_ts; ++t) {
        const float* x = (t & 1) ? M->tmp.p : q;
        float* y = (t & 1) ? q : M->tmp.p;
        mat_step_kernel<<<grid, kMatThreads, 0, st>>>(d, x, qlat + (size_t)t * (size_t)M->R, y);
    }
    int rc = mat_cuda(cudaGetLastError(), "matrix step launch");
    if (!rc && (n_ts & 1))
        rc = mat_cuda(cudaMemcpyAsync(q, M->tmp.p, (size_t)M->R * sizeof(float), cudaMemcpyDeviceToDevice, st),
                      "matrix result copy");
    return rc;
}

extern "C" int troute_matrix_run_device(troute_matrix* M, const float* qlat_ts_device, int n_ts, float* q_device,
                                        void* stream)
{
    if (!M) return set_error(TROUTE_EINVAL, "null handle");
    if (n_ts < 0) return set_error(TROUTE_EINVAL, "n_ts < 0");
    if (n_ts == 0 || M->R == 0) return TROUTE_OK;
    if (!qlat_ts_device || !q_device) return set_error(TROUTE_EINVAL, "null device array");
    const cudaStream_t st = stream ? (cudaStream_t)stream : M->stream;
    int rc;
    if (!M->graph || M->g_qlat != qlat_ts_device || M->g_q != q_device || M->g_nts != n_ts) {
        if (M->graph) {
            cudaGraphExecDestroy(M->graph);
            M->graph = nullptr;
        }
        // record the run once on the handle's stream; replays go to the caller's
        if ((rc = mat_cuda(cudaStreamBeginCapture(M->stream, cudaStreamCaptureModeThreadLocal), "begin capture")))
            return rc;
        rc = enqueue_steps(M, qlat_ts_device, n_ts, q_device, M->stream);
        cudaGraph_t g = nullptr;
        const int rc2 = mat_cuda(cudaStreamEndCapture(M->stream, &g), "end capture");
        if (rc || rc2) {
            if (g) cudaGraphDestroy(g);
            return rc ? rc : rc2;
        }
        rc = mat_cuda(cudaGraphInstantiate(&M->graph, g, 0), "graph instantiate");
        cudaGraphDestroy(g);
        if (rc) {
            M->graph = nullptr;
            return rc;
        }
        M->g_qlat = qlat_ts_device;
        M->g_q = q_device;
        M->g_nts = n_ts;
    }
    return mat_cuda(cudaGraphLaunch(M->graph, st), "matrix graph launch");
}

extern "C" int troute_matrix_route(int n_reaches, const int* up_ptr, const int* up_idx, const float* c1,
                                   const float* c2, const float* c3, const float* c4oq, float tol,
                                   const float* qlat_ts, const float* q0, int n_ts, float* q_out)
{
    if (n_ts < 0) return set_error(TROUTE_EINVAL, "n_ts < 0");
    if (n_reaches > 0 && (!q0 || !q_out || (n_ts > 0 && !qlat_ts))) return set_error(TROUTE_EINVAL, "null array");
    troute_matrix* M = nullptr;
    int rc = troute_matrix_create(&M, n_reaches, up_ptr, up_idx, c1, c2, c3, c4oq, tol);
    if (rc) return rc;
    const size_t R = (size_t)n_reaches;
    MArr<float> q, ql;
    if ((rc = q.alloc(R)) || (rc = ql.alloc((size_t)n_ts * R)) ||
        (rc = mat_cuda(cudaMemcpy(q.p, q0, R * sizeof(float), cudaMemcpyHostToDevice), "H2D")) ||
        (rc = mat_cuda(cudaMemcpy(ql.p, qlat_ts, (size_t)n_ts * R * sizeof(float), cudaMemcpyHostToDevice), "H2D")) ||
        (rc = troute_matrix_run_device(M, ql.p, n_ts, q.p, nullptr)) ||
        (rc = mat_cuda(cudaStreamSynchronize(M->stream), "matrix run")) ||
        (rc = mat_cuda(cudaMemcpy(q_out, q.p, R * sizeof(float), cudaMemcpyDeviceToHost), "D2H"))) {
        troute_matrix_destroy(M);
        return rc;
    }
    troute_matrix_destroy(M);
    return TROUTE_OK;
}
