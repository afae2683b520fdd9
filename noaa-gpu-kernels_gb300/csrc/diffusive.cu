// Diffusive-wave tridiagonal step of t-route (the reference's
// water-prediction/owp_extended_kernels.cu:24-153, after t-route's
// diffusive.f90): per reach, a Crank-Nicolson tridiagonal system along the
// reach's computational nodes, solved by forward elimination and back
// substitution (Thomas), FP32.
//
// Arrays are [n_reaches][max_nodes] (max_nodes = 500 in the reference). The
// reference runs one thread per reach reading its own row (32 rows, i.e. 32
// cache lines, per warp access) with the elimination coefficients in local
// memory. Here a warp still owns 32 reaches and runs each reach's recurrence
// in one lane, in the reference's order of operations (bit-identical), but:
//  - the rows are staged through shared memory 32 nodes at a time with
//    coalesced 128-byte row loads, transposed so each lane reads its reach;
//  - the elimination coefficients go to a node-major scratch [node][reach],
//    written and read back coalesced;
//  - the result is transposed back through shared memory and stored as rows.
// Celerity is an input of the reference's routine but only feeds a Courant
// number that nothing uses; it is not read.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "troute_internal.h"

namespace tr {
namespace {

constexpr int kDW = 32;         // reaches per warp, nodes per tile
constexpr int kDWarps = 4;      // warps per block
constexpr int kTileLd = kDW + 3;  // nodes i0-1 .. i0+32 (+1 pad: odd stride, conflict-free)

struct DiffTiles {
    float dx[kDWarps][kDW][kTileLd];
    float diff[kDWarps][kDW][kTileLd];
    float qp[kDWarps][kDW][kTileLd];
};

// Loads nodes [n0, n0 + cnt) (cnt <= 64) of rows r0..r0+31 of dx and the
// diffusivity and nodes [n0, n0 + cnt + 1) of the previous discharge into
// their tiles, tile[row][j] = node n0 + j (coalesced along the row; nodes
// outside [0, max_nodes) or rows past n_reaches are left untouched). Eight
// rows of all three arrays at a time: their loads are all issued before any is
// stored, so a tile costs four memory round trips for the three arrays.
__device__ __forceinline__ void load_tiles(DiffTiles& T, int w, const float* __restrict__ dx,
                                           const float* __restrict__ diffusivity, const float* __restrict__ qp_prev,
                                           int r0, int n_reaches, int max_nodes, int n0, int cnt, int lane)
{
    const int na = n0 + lane, nb = n0 + lane + kDW;
    const bool in_a = na >= 0 && na < max_nodes, in_b = nb >= 0 && nb < max_nodes;
    const bool ok_a = lane < cnt && in_a, ok_b = lane + kDW < cnt && in_b;          // dx, diffusivity
    const bool okq_a = lane < cnt + 1 && in_a, okq_b = lane + kDW < cnt + 1 && in_b;  // discharge
    for (int row0 = 0; row0 < kDW; row0 += 8) {
        float xa[8], xb[8], da[8], db[8], qa[8], qb[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int r = r0 + row0 + q;
            const bool in = r < n_reaches;
            const size_t o = (size_t)r * (size_t)max_nodes;
            xa[q] = (in && ok_a) ? __ldg(dx + o + na) : 0.0f;
            xb[q] = (in && ok_b) ? __ldg(dx + o + nb) : 0.0f;
            da[q] = (in && ok_a) ? __ldg(diffusivity + o + na) : 0.0f;
            db[q] = (in && ok_b) ? __ldg(diffusivity + o + nb) : 0.0f;
            qa[q] = (in && okq_a) ? __ldg(qp_prev + o + na) : 0.0f;
            qb[q] = (in && okq_b) ? __ldg(qp_prev + o + nb) : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            if (r0 + row0 + q < n_reaches) {
                const int t = row0 + q;
                if (ok_a) T.dx[w][t][lane] = xa[q], T.diff[w][t][lane] = da[q];
                if (ok_b) T.dx[w][t][lane + kDW] = xb[q], T.diff[w][t][lane + kDW] = db[q];
                if (okq_a) T.qp[w][t][lane] = qa[q];
                if (okq_b) T.qp[w][t][lane + kDW] = qb[q];
            }
        }
    }
}

__global__ void __launch_bounds__(kDW * kDWarps) diffusive_kernel(const troute_diff_reach* __restrict__ rp,
                                                                   const float* __restrict__ dx,
                                                                   const float* __restrict__ diffusivity,
                                                                   const float* __restrict__ qp_prev,
                                                                   float* __restrict__ qp_out,
                                                                   float* __restrict__ se, float* __restrict__ sf,
                                                                   int n_reaches, int max_nodes)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DiffTiles& T = *reinterpret_cast<DiffTiles*>(smem_raw);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int r0 = (blockIdx.x * kDWarps + w) * kDW;
    if (r0 >= n_reaches) return;
    const int r = r0 + lane;
    const bool live = r < n_reaches;
    int nc = 0;
    float theta = 0.f, dtini = 0.f;
    if (live) {
        const troute_diff_reach p = rp[r];
        nc = p.ncomp;
        theta = p.theta;
        dtini = p.dtini;
    }
    int nc_max = nc;
    for (int off = 16; off > 0; off >>= 1) nc_max = max(nc_max, __shfl_xor_sync(0xffffffffu, nc_max, off));
    // node-major scratch of this warp's reaches: se/sf[node * n_reaches + r]
    float e_prev = 1.0f, f_prev = 0.0f;  // eei[0], ffi[0]
    if (live) {
        se[r] = 1.0f;
        sf[r] = 0.0f;
    }
    // ---- forward elimination, 32 nodes per tile ----
    for (int i0 = 0; i0 < nc_max; i0 += kDW) {
        __syncwarp();
        // tile column k holds node i0 - 1 + k
        load_tiles(T, w, dx, diffusivity, qp_prev, r0, n_reaches, max_nodes, i0 - 1, kDW + 1, lane);
        __syncwarp();
        if (live) {
            for (int k = 1; k <= kDW; ++k) {
                const int i = i0 - 1 + k;
                if (i < 1) continue;
                if (i >= nc) break;
                float dxi = T.dx[w][lane][k - 1];
                if (dxi < 1.0f) dxi = 1.0f;
                const float alpha = 1.0f;
                float diff_i = T.diff[w][lane][k];
                if (diff_i < 0.01f) diff_i = 0.01f;
                const float ppi = -theta * diff_i * dtini / (dxi * dxi) * 2.0f / (alpha * (alpha + 1.0f)) * alpha;
                const float qqi = 1.0f - ppi * (alpha + 1.0f) / alpha;
                const float rri = ppi / alpha;
                const float qi = T.qp[w][lane][k];
                const float qnext = (i < nc - 1) ? T.qp[w][lane][k + 1] : qi;
                const float ssi = qi + dtini * diff_i * (1.0f - theta) * (T.qp[w][lane][k - 1] - 2.0f * qi + qnext) /
                                           (dxi * dxi);
                float denom = ppi * e_prev + qqi;
                if (fabsf(denom) < 1e-20f) denom = 1e-20f;
                const float e = -rri / denom;
                const float f = (ssi - ppi * f_prev) / denom;
                se[(size_t)i * n_reaches + r] = e;
                sf[(size_t)i * n_reaches + r] = f;
                e_prev = e;
                f_prev = f;
            }
        }
    }
    // ---- back substitution, top tile first; results staged as rows ----
    float next = 0.0f;  // qp_out[i + 1]
    const int top = ((nc_max - 1) / kDW) * kDW;
    for (int i0 = top; i0 >= 0; i0 -= kDW) {
        __syncwarp();
        // the last node of a reach takes the ghost-node value qp_prev[nc - 1]
        if (live && nc - 1 >= i0 && nc - 1 < i0 + kDW) {
            const float ghost = __ldg(qp_prev + (size_t)r * max_nodes + nc - 1);
            next = se[(size_t)(nc - 1) * n_reaches + r] * ghost + sf[(size_t)(nc - 1) * n_reaches + r];
            T.qp[w][lane][nc - 1 - i0] = next;
        }
        if (live) {
            // the tile's elimination coefficients first, eight nodes' loads in
            // flight at a time, into the lane's rows of the dx / diffusivity
            // tiles (free once the forward sweep is done); then the
            // recurrence reads them from shared memory
            for (int k0 = 0; k0 < kDW; k0 += 8) {
                float ev[8], fv[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int i = i0 + k0 + q;
                    ev[q] = i < nc - 1 ? se[(size_t)i * n_reaches + r] : 0.0f;
                    fv[q] = i < nc - 1 ? sf[(size_t)i * n_reaches + r] : 0.0f;
                }
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    T.dx[w][lane][k0 + q] = ev[q];
                    T.diff[w][lane][k0 + q] = fv[q];
                }
            }
            for (int k = kDW - 1; k >= 0; --k) {
                const int i = i0 + k;
                if (i >= nc - 1) continue;
                next = T.dx[w][lane][k] * next + T.diff[w][lane][k];
                T.qp[w][lane][k] = next;
            }
        }
        __syncwarp();
        // rows back to [reach][node], coalesced along each row
        for (int row = 0; row < kDW; ++row) {
            const int rr = r0 + row;
            if (rr >= n_reaches) break;
            const int ncr = __shfl_sync(0xffffffffu, nc, row);
            const int node = i0 + lane;
            if (node < ncr) qp_out[(size_t)rr * max_nodes + node] = T.qp[w][row][lane];
        }
    }
}

int diff_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return TROUTE_OK;
    return set_error(e == cudaErrorMemoryAllocation ? TROUTE_ENOMEM : TROUTE_ECUDA, "%s: %s", what,
                     cudaGetErrorString(e));
}

}  // namespace
}  // namespace tr

using namespace tr;

extern "C" int troute_diffusive_tridiag_device(const troute_diff_reach* rp, const float* dx, const float* diffusivity,
                                               const float* celerity, const float* qp_prev, float* qp_out,
                                               int n_reaches, int max_nodes, float* scratch, void* stream)
{
    (void)celerity;
    if (n_reaches < 0 || max_nodes < 1) return set_error(TROUTE_EINVAL, "bad sizes");
    if (n_reaches == 0) return TROUTE_OK;
    if (!rp || !dx || !diffusivity || !qp_prev || !qp_out || !scratch) return set_error(TROUTE_EINVAL, "null array");
    const int per_block = kDW * kDWarps;
    const int grid = (n_reaches + per_block - 1) / per_block;
    const size_t smem = sizeof(DiffTiles);
    int rc = diff_cuda(cudaFuncSetAttribute(diffusive_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "smem attribute");
    if (rc) return rc;
    float* se = scratch;
    float* sf = scratch + (size_t)n_reaches * max_nodes;
    diffusive_kernel<<<grid, per_block, smem, (cudaStream_t)stream>>>(rp, dx, diffusivity, qp_prev, qp_out, se, sf,
                                                                     n_reaches, max_nodes);
    return diff_cuda(cudaGetLastError(), "diffusive launch");
}

extern "C" int troute_diffusive_tridiag(const troute_diff_reach* rp, const float* dx, const float* diffusivity,
                                        const float* celerity, const float* qp_prev, float* qp_out, int n_reaches,
                                        int max_nodes)
{
    if (n_reaches < 0 || max_nodes < 1) return set_error(TROUTE_EINVAL, "bad sizes");
    if (n_reaches == 0) return TROUTE_OK;
    if (!rp || !dx || !diffusivity || !qp_prev || !qp_out) return set_error(TROUTE_EINVAL, "null array");
    for (int j = 0; j < n_reaches; ++j)
        if (rp[j].ncomp < 1 || rp[j].ncomp > max_nodes)
            return set_error(TROUTE_EINVAL, "reach %d: ncomp %d outside [1, %d]", j, rp[j].ncomp, max_nodes);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(TROUTE_ENODEV, "no CUDA device");
    const size_t n = (size_t)n_reaches * max_nodes;
    troute_diff_reach* d_rp = nullptr;
    float* buf = nullptr;  // dx, diffusivity, qp_prev, qp_out, 2 scratch planes
    int rc = diff_cuda(cudaMalloc(&d_rp, (size_t)n_reaches * sizeof *d_rp), "cudaMalloc");
    if (!rc) rc = diff_cuda(cudaMalloc(&buf, 6 * n * sizeof(float)), "cudaMalloc");
    if (!rc) rc = diff_cuda(cudaMemcpy(d_rp, rp, (size_t)n_reaches * sizeof *rp, cudaMemcpyHostToDevice), "H2D");
    if (!rc) rc = diff_cuda(cudaMemcpy(buf, dx, n * sizeof(float), cudaMemcpyHostToDevice), "H2D");
    if (!rc) rc = diff_cuda(cudaMemcpy(buf + n, diffusivity, n * sizeof(float), cudaMemcpyHostToDevice), "H2D");
    if (!rc) rc = diff_cuda(cudaMemcpy(buf + 2 * n, qp_prev, n * sizeof(float), cudaMemcpyHostToDevice), "H2D");
    // nodes past a reach's ncomp are not written: start from the caller's contents
    if (!rc) rc = diff_cuda(cudaMemcpy(buf + 3 * n, qp_out, n * sizeof(float), cudaMemcpyHostToDevice), "H2D");
    if (!rc)
        rc = troute_diffusive_tridiag_device(d_rp, buf, buf + n, nullptr, buf + 2 * n, buf + 3 * n, n_reaches,
                                             max_nodes, buf + 4 * n, nullptr);
    if (!rc) rc = diff_cuda(cudaMemcpy(qp_out, buf + 3 * n, n * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
    cudaFree(d_rp);
    cudaFree(buf);
    return rc;
}
