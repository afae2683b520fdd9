/*
 * CPU oracle for the t-route Muskingum-Cunge secant routing path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the restated reference algorithm
 * that the CUDA path is compared against; it is called only by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline / reference legs. The product (libtroute_gb300.so
 * and the troute_gb300 Python package) never links, loads or calls it.
 *
 * Pinned against the reference itself: tests/test_oracle.py loads the
 * reference's own cpu_mc (water-prediction/t-route/troute_mc_final.cu:167-252)
 * and cpu_wavefront_fp64 (water-prediction/t-route/wavefront/wavefront_mc.cu:
 * 495-564), compiled from the reference's sources by oracle/Makefile, and
 * checks this restatement bit-for-bit at the reference tolerance;
 * tests/golden/ holds fixtures produced by those compiled reference routines.
 */
#ifndef TROUTE_ORACLE_H
#define TROUTE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-segment channel parameters, same member order and size as the
 * reference's ChParams (troute_mc_final.cu:26-28). */
typedef struct oracle_chparams {
    double dx, bw, tw, twcc, n_ch, ncc, cs, s0;
} oracle_chparams;

/* Secant tolerances. The reference hardcodes rtol = atol = 0.01, maxiter = 100,
 * 5 attempts (troute_mc_final.cu:69-74). */
typedef struct oracle_tol {
    double rtol;
    double atol;
    int maxiter;
    int attempts;
} oracle_tol;

/* Power function used for R^(2/3), R^(5/3): 0 = the C library's pow() (the
 * reference's, default), 1 = correctly rounded values (platform independent).
 * Process-wide; not thread-safe to change while routing. */
void oracle_set_pow_mode(int mode);
void oracle_pow23_53(double x, double* p23, double* p53);
/* The same over an array, mode 0 (C library) or 1 (correctly rounded), on
 * n_threads POSIX threads; returns 0 (2: out of memory). */
int oracle_pow23_53_n(const double* x, long long n, double* p23, double* p53, int mode, int n_threads);

/* One segment solve (troute_mc_final.cu:42-139 / :181-248). Returns qdc and
 * writes depth, velocity and the number of secant iterations run. */
double oracle_mc_solve(double dt, double qup, double quc, double qdp, double ql,
                       const oracle_chparams* p, double depthp,
                       const oracle_tol* tol,
                       double* depthc, double* velc, int* iters);

/* Reach-parallel single step, the reference's cpu_mc (troute_mc_final.cu:167-252)
 * with tolerances as a parameter. iters_total may be NULL. */
void oracle_cpu_mc(const oracle_chparams* p, const double* ql,
                   const int* rs, const int* rl,
                   const double* qu, const double* qd, const double* dp,
                   double* qo, double* vo, double* dpo,
                   double uq, double dt, int nr,
                   const oracle_tol* tol, long long* iters_total);

/* Level-scheduled multi-step tree routing in FP64, the semantics of the
 * reference's cpu_wavefront_fp64 (wavefront_mc.cu:495-564) with FP64
 * parameters and lateral inflow.
 *   qlat_ts   [n_ts][n_segments]
 *   q_hist    optional [n_ts][n_segments] per-step discharge (may be NULL)
 *   q_out/d_out/v_out  final-step discharge/depth/velocity per segment
 *   reach_last_out     final-step discharge of each reach's last segment
 * n_threads <= 1 runs single-threaded; otherwise the reaches of each level are
 * split over n_threads POSIX threads with a barrier between levels (results are
 * identical: reaches within a level are independent). */
int oracle_route_tree(const int* reach_seg_start, const int* reach_seg_len,
                      const int* reach_up_ptr, const int* reach_up_idx,
                      const int* level_ptr, const int* level_reach,
                      int n_reaches, int n_levels, int n_segments,
                      const oracle_chparams* params, const double* qlat_ts,
                      const double* qdp0, const double* dp0, const double* reach_last0,
                      int n_ts, double dt, const oracle_tol* tol,
                      double* q_out, double* d_out, double* v_out,
                      double* reach_last_out, double* q_hist,
                      long long* iters_total, int n_threads);

/* Same, also writing the secant iterations of every solve to it_hist
 * [n_ts][n_segments] (may be NULL). */
int oracle_route_tree_it(const int* reach_seg_start, const int* reach_seg_len,
                         const int* reach_up_ptr, const int* reach_up_idx,
                         const int* level_ptr, const int* level_reach,
                         int n_reaches, int n_levels, int n_segments,
                         const oracle_chparams* params, const double* qlat_ts,
                         const double* qdp0, const double* dp0, const double* reach_last0,
                         int n_ts, double dt, const oracle_tol* tol,
                         double* q_out, double* d_out, double* v_out,
                         double* reach_last_out, double* q_hist, int* it_hist,
                         long long* iters_total, int n_threads);

/* The solve with a learned starting depth. start > 0: the first phase
 * brackets [start (1 - delta), start (1 + delta)] and gets at most warm_k
 * passes; it is accepted when the stop test passes with depth >= 0.01,
 * otherwise the plain solve runs from depthp (a fallback; all passes count in
 * *iters). start <= 0: the plain solve. *warm_state: 0 plain, 1 accepted,
 * 2 fallback. */
double oracle_mc_solve_warm(double dt, double qup, double quc, double qdp, double ql,
                            const oracle_chparams* p, double depthp, const oracle_tol* tol,
                            double start, double delta, int warm_k,
                            double* depthc, double* velc, int* iters, int* warm_state);

/* Options and per-solve outputs of oracle_route_tree_ex. */
typedef struct oracle_tree_opts {
    const double* warm_start; /* [n_ts][n_segments] starting depth per solve (<= 0: plain), or NULL */
    double warm_delta;        /* relative half-width of the warm bracket */
    int warm_k;               /* passes of the warm phase */
    int n_threads;
    double* q_hist;           /* [n_ts][n_segments] discharge, or NULL */
    double* d_hist;           /* [n_ts][n_segments] depth, or NULL */
    int* it_hist;             /* [n_ts][n_segments] secant passes, or NULL */
    long long iters_total;    /* out */
    long long warm_used;      /* out: solves started from warm_start */
    long long warm_fallback;  /* out: of those, solves that fell back */
} oracle_tree_opts;

int oracle_route_tree_ex(const int* reach_seg_start, const int* reach_seg_len,
                         const int* reach_up_ptr, const int* reach_up_idx,
                         const int* level_ptr, const int* level_reach,
                         int n_reaches, int n_levels, int n_segments,
                         const oracle_chparams* params, const double* qlat_ts,
                         const double* qdp0, const double* dp0, const double* reach_last0,
                         int n_ts, double dt, const oracle_tol* tol,
                         double* q_out, double* d_out, double* v_out,
                         double* reach_last_out, oracle_tree_opts* opts);

/* Float parameter record of params.bin (wavefront_mc.cu:41-44). */
typedef struct oracle_chparams_f32 {
    float dx, bw, tw, twcc, n_ch, ncc, cs, s0;
} oracle_chparams_f32;

/* Linearised MC (linear_mc.cu): coefficients (compute_mc_coeffs, :57-100) and
 * the float routing of cpu_linear_mc (:177-232); every reach needs at least
 * one segment. */
void oracle_linear_coeffs(const oracle_chparams_f32* params, int n, float dt, float* c1, float* c2, float* c3,
                          float* c4oq);
int oracle_linear_route(const float* c1, const float* c2, const float* c3, const float* c4oq,
                        const int* reach_seg_start, const int* reach_seg_len, const int* reach_up_ptr,
                        const int* reach_up_idx, const int* level_ptr, const int* level_reach, int n_reaches,
                        int n_levels, int n_segments, const float* qlat_ts, const float* q0, float* q_final,
                        int n_ts);

/* Diffusive-wave tridiagonal step (owp_extended_kernels.cu:24-91), float,
 * arrays [n_reaches][max_nodes]. Returns 1 for an ncomp outside [1, max_nodes]. */
typedef struct oracle_diff_reach {
    int ncomp;
    float theta;
    float dtini;
} oracle_diff_reach;
int oracle_diffusive_tridiag(const oracle_diff_reach* rp, const float* dx, const float* diffusivity,
                             const float* qp_prev, float* qp_out, int n_reaches, int max_nodes);

/* Matrix-form linearised MC (oracle_matrix.c; linear_mc_matrix.cu): a CSR
 * matrix whose arrays the oracle allocates (oracle_csr_free releases them). */
typedef struct oracle_csr {
    int n;
    int* ptr;   /* [n + 1] */
    int* col;   /* [nnz] */
    float* val; /* [nnz] */
} oracle_csr;
void oracle_matrix_coeffs(const oracle_chparams_f32* params, int n, float dt, float* c1, float* c2, float* c3,
                          float* c4oq);
/* Returns 0, 2 (out of memory) or 3 (a reach not numbered after its upstream reaches). */
int oracle_matrix_build(int R, const int* up_ptr, const int* up_idx, const float* c1, const float* c2,
                        const float* c3, const float* c4oq, float tol, oracle_csr* PQ, oracle_csr* Pq);
void oracle_csr_free(oracle_csr* m);
void oracle_matrix_step(const oracle_csr* PQ, const oracle_csr* Pq, const float* x, const float* ql, float* y);
int oracle_matrix_route(const oracle_csr* PQ, const oracle_csr* Pq, const float* qlat_ts, const float* q0,
                        float* q_final, int n_ts);

/* Seeded synthetic inputs (oracle_gen.c), byte for byte the product
 * generator's: tree topology (returns 0, or 1 for bad sizes, 2 out of memory),
 * channel parameters, lateral inflow [n_ts][n_segments] for steps t0..,
 * ensemble member factors (either may be NULL). */
int oracle_gen_tree(uint64_t seed, int n_leaves, int n_segments, int max_len, int* seg_start, int* seg_len,
                    int* up_ptr, int* up_idx);
void oracle_gen_params(uint64_t seed, int n_segments, oracle_chparams* p);
int oracle_gen_qlat(uint64_t seed, int n_segments, int t0, int n_ts, double dt, double* qlat, int n_threads);
void oracle_gen_member(uint64_t seed, int member, int n_segments, double* qfac, double* nfac);
/* Level schedule by the reference's rule (gen_network.py:219-231); returns the
 * number of levels (level_ptr has n_reaches + 1 entries of room). */
int oracle_levels(int n_reaches, const int* up_ptr, const int* up_idx, int* level_ptr, int* level_reach);

#ifdef __cplusplus
}
#endif
#endif
