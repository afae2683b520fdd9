/*
 * Matrix-form linearised MC, restated in C.
 *
 * TEST INFRASTRUCTURE ONLY (part of libtroute_oracle.so), the checker of the
 * library's matrix form. The reference's matrix form
 * (water-prediction/t-route/wavefront/linear_mc_matrix.cu) routes a
 * reach-level network, one routing unit per reach, with fixed coefficients:
 *
 *   Q_new = P_Q Q_old + P_q qlat,  P_Q = A^-1 (C2 N + C3 I),  P_q = A^-1 C4,
 *   A = I - C1 N   (N[r, u] = 1 for u directly upstream of r),
 *
 * with A^-1 expanded as a series over the upstream paths and entries below a
 * tolerance dropped. Three parts, each following the reference:
 *
 *  - oracle_matrix_coeffs: C1, C2, C3, C4/ql per reach at X = 0.25
 *    (compute_mc_coeffs_cpu, linear_mc_matrix.cu:56-86), float, the C
 *    library's powf / sqrtf as the reference's host code uses;
 *  - oracle_matrix_build: the truncated matrices row by row in reach order
 *    (build_propagation_matrices, :129-216): row r = C1[r] x the rows of its
 *    upstream reaches (merged in upstream-list order, value = row + upstream
 *    x C1 in float), entries below tol dropped, then C2[r] added at each
 *    upstream reach, C3[r] at r itself (C4/ql[r] in P_q), dropped again;
 *  - oracle_matrix_step: one step y = P_Q x + P_q ql with the arithmetic of
 *    the reference's fused warp-per-row kernel (kernel_spmv_fused,
 *    linear_mc_matrix_graph.cu:174-206): lane l of 32 accumulates the row's
 *    entries l, l + 32, ... of each matrix by fused multiply-add (nvcc
 *    contracts `sum += v * x` by default), adds its two partials, and the 32
 *    lane sums are combined by the shuffle-down tree 16, 8, 4, 2, 1.
 *
 * Pinned: tests/test_matrix.py checks the coefficients and the matrices
 * against the reference's own functions compiled from its source
 * (oracle/ref_matrix_shim.cu) and the committed golden fixture.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "troute_oracle.h"

void oracle_matrix_coeffs(const oracle_chparams_f32* params, int n, float dt, float* c1, float* c2, float* c3,
                          float* c4oq)
{
    for (int i = 0; i < n; ++i) {
        const oracle_chparams_f32 p = params[i];
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
        c1[i] = (Km * X + dt / 2.0f) / D;
        c2[i] = (dt / 2.0f - Km * X) / D;
        c3[i] = (Km * (1.0f - X) - dt / 2.0f) / D;
        c4oq[i] = dt / D;
    }
}

/* a sparse row: columns ascending */
typedef struct {
    int n, cap;
    int* col;
    float* val;
} om_row;

static int om_reserve(om_row* r, int cap)
{
    if (cap <= r->cap) return 0;
    int c = r->cap ? r->cap : 4;
    while (c < cap) c *= 2;
    int* nc = (int*)realloc(r->col, sizeof(int) * (size_t)c);
    if (!nc) return 1;
    r->col = nc;
    float* nv = (float*)realloc(r->val, sizeof(float) * (size_t)c);
    if (!nv) return 1;
    r->val = nv;
    r->cap = c;
    return 0;
}

/* dst <- dst (+) src * scale, by column; where both hold a column the value is
 * dst + src * scale (two float roundings) */
static int om_merge_scaled(om_row* dst, const om_row* src, float scale, om_row* tmp)
{
    tmp->n = 0;
    if (om_reserve(tmp, dst->n + src->n)) return 1;
    int i = 0, j = 0;
    while (i < dst->n && j < src->n) {
        if (dst->col[i] < src->col[j]) {
            tmp->col[tmp->n] = dst->col[i];
            tmp->val[tmp->n++] = dst->val[i++];
        } else if (dst->col[i] > src->col[j]) {
            tmp->col[tmp->n] = src->col[j];
            tmp->val[tmp->n++] = src->val[j++] * scale;
        } else {
            const float prod = src->val[j] * scale;
            tmp->col[tmp->n] = dst->col[i];
            tmp->val[tmp->n++] = dst->val[i] + prod;
            ++i;
            ++j;
        }
    }
    for (; i < dst->n; ++i) {
        tmp->col[tmp->n] = dst->col[i];
        tmp->val[tmp->n++] = dst->val[i];
    }
    for (; j < src->n; ++j) {
        tmp->col[tmp->n] = src->col[j];
        tmp->val[tmp->n++] = src->val[j] * scale;
    }
    om_row t = *dst;
    *dst = *tmp;
    *tmp = t;
    return 0;
}

/* adds v at column c (inserted in order, or summed with an existing entry) */
static int om_add(om_row* r, int c, float v)
{
    int lo = 0, hi = r->n;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (r->col[mid] < c) lo = mid + 1; else hi = mid;
    }
    if (lo < r->n && r->col[lo] == c) {
        r->val[lo] += v;
        return 0;
    }
    if (om_reserve(r, r->n + 1)) return 1;
    memmove(r->col + lo + 1, r->col + lo, sizeof(int) * (size_t)(r->n - lo));
    memmove(r->val + lo + 1, r->val + lo, sizeof(float) * (size_t)(r->n - lo));
    r->col[lo] = c;
    r->val[lo] = v;
    r->n++;
    return 0;
}

static void om_prune(om_row* r, float tol)
{
    int k = 0;
    for (int i = 0; i < r->n; ++i)
        if (!(fabsf(r->val[i]) < tol)) {
            r->col[k] = r->col[i];
            r->val[k++] = r->val[i];
        }
    r->n = k;
}

static int om_to_csr(om_row* rows, int R, oracle_csr* m)
{
    m->n = R;
    m->ptr = (int*)malloc(sizeof(int) * (size_t)(R + 1));
    if (!m->ptr) return 1;
    m->ptr[0] = 0;
    for (int r = 0; r < R; ++r) m->ptr[r + 1] = m->ptr[r] + rows[r].n;
    const size_t nnz = (size_t)m->ptr[R];
    m->col = (int*)malloc(sizeof(int) * (nnz ? nnz : 1));
    m->val = (float*)malloc(sizeof(float) * (nnz ? nnz : 1));
    if (!m->col || !m->val) return 1;
    for (int r = 0; r < R; ++r) {
        memcpy(m->col + m->ptr[r], rows[r].col, sizeof(int) * (size_t)rows[r].n);
        memcpy(m->val + m->ptr[r], rows[r].val, sizeof(float) * (size_t)rows[r].n);
    }
    return 0;
}

void oracle_csr_free(oracle_csr* m)
{
    if (!m) return;
    free(m->ptr);
    free(m->col);
    free(m->val);
    m->ptr = m->col = NULL;
    m->val = NULL;
    m->n = 0;
}

int oracle_matrix_build(int R, const int* up_ptr, const int* up_idx, const float* c1, const float* c2,
                        const float* c3, const float* c4oq, float tol, oracle_csr* PQ, oracle_csr* Pq)
{
    memset(PQ, 0, sizeof *PQ);
    memset(Pq, 0, sizeof *Pq);
    if (R < 0) return 3;
    for (int r = 0; r < R; ++r)
        for (int k = up_ptr[r]; k < up_ptr[r + 1]; ++k)
            if (up_idx[k] < 0 || up_idx[k] >= r) return 3; /* reaches must be numbered upstream first */
    om_row* rq = (om_row*)calloc((size_t)(R ? R : 1), sizeof(om_row));
    om_row* rl = (om_row*)calloc((size_t)(R ? R : 1), sizeof(om_row));
    om_row tmp = {0, 0, NULL, NULL};
    int rc = (!rq || !rl) ? 2 : 0;
    for (int r = 0; r < R && !rc; ++r) {
        const int ub = up_ptr[r], ue = up_ptr[r + 1];
        for (int k = ub; k < ue && !rc; ++k) {
            const int u = up_idx[k];
            rc = om_merge_scaled(&rq[r], &rq[u], c1[r], &tmp) || om_merge_scaled(&rl[r], &rl[u], c1[r], &tmp);
        }
        if (rc) break;
        om_prune(&rq[r], tol);
        om_prune(&rl[r], tol);
        for (int k = ub; k < ue && !rc; ++k) rc = om_add(&rq[r], up_idx[k], c2[r]);
        if (!rc) rc = om_add(&rq[r], r, c3[r]);
        if (!rc) rc = om_add(&rl[r], r, c4oq[r]);
        om_prune(&rq[r], tol);
        om_prune(&rl[r], tol);
    }
    if (!rc) rc = om_to_csr(rq, R, PQ) || om_to_csr(rl, R, Pq);
    for (int r = 0; r < R && rq && rl; ++r) {
        free(rq[r].col), free(rq[r].val), free(rl[r].col), free(rl[r].val);
    }
    free(rq), free(rl), free(tmp.col), free(tmp.val);
    if (rc) {
        oracle_csr_free(PQ);
        oracle_csr_free(Pq);
        return rc == 3 ? 3 : 2;
    }
    return 0;
}

void oracle_matrix_step(const oracle_csr* PQ, const oracle_csr* Pq, const float* x, const float* ql, float* y)
{
    for (int r = 0; r < PQ->n; ++r) {
        float s[32];
        for (int l = 0; l < 32; ++l) {
            float sq = 0.f, sl = 0.f;
            for (int k = PQ->ptr[r] + l; k < PQ->ptr[r + 1]; k += 32) sq = fmaf(PQ->val[k], x[PQ->col[k]], sq);
            for (int k = Pq->ptr[r] + l; k < Pq->ptr[r + 1]; k += 32) sl = fmaf(Pq->val[k], ql[Pq->col[k]], sl);
            s[l] = sq + sl;
        }
        for (int off = 16; off > 0; off >>= 1)
            for (int l = 0; l < off; ++l) s[l] = s[l] + s[l + off];
        y[r] = s[0];
    }
}

int oracle_matrix_route(const oracle_csr* PQ, const oracle_csr* Pq, const float* qlat_ts, const float* q0,
                        float* q_final, int n_ts)
{
    const int R = PQ->n;
    float* a = (float*)malloc(sizeof(float) * (size_t)(R ? R : 1));
    float* b = (float*)malloc(sizeof(float) * (size_t)(R ? R : 1));
    if (!a || !b) {
        free(a), free(b);
        return 2;
    }
    memcpy(a, q0, sizeof(float) * (size_t)R);
    for (int t = 0; t < n_ts; ++t) {
        oracle_matrix_step(PQ, Pq, a, qlat_ts + (size_t)t * (size_t)R, b);
        float* tt = a;
        a = b;
        b = tt;
    }
    memcpy(q_final, a, sizeof(float) * (size_t)R);
    free(a), free(b);
    return 0;
}
