/*
 * troute_gb300 — GB300 (sm_103a) Muskingum-Cunge secant routing, C ABI.
 *
 * Drop-in boundary for the t-route MC routing path of
 * water-prediction/t-route/troute_mc_final.cu (reach-parallel, cpu_mc) and
 * water-prediction/t-route/wavefront/wavefront_mc.cu (level-scheduled tree,
 * cpu_wavefront_fp64). Every entry point takes plain pointers and sizes, returns
 * a status code (TROUTE_OK == 0) and records a message for troute_last_error().
 * Pointers are host pointers unless the name ends in _device.
 *
 * Threading: one troute_handle per host thread; a handle is not re-entrant.
 * All device-side waits are bounded; a wait that runs out returns
 * TROUTE_ETIMEOUT and leaves the CUDA context usable.
 */
#ifndef TROUTE_GB300_H
#define TROUTE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum troute_status {
    TROUTE_OK = 0,
    TROUTE_EINVAL = 1,   /* bad argument */
    TROUTE_ETOPO = 2,    /* malformed topology (bad CSR, cycle, reach with two outlets) */
    TROUTE_ECUDA = 3,    /* CUDA runtime error */
    TROUTE_ENOMEM = 4,   /* host or device allocation failed */
    TROUTE_ETIMEOUT = 5, /* a bounded device-side wait ran out */
    TROUTE_ENODEV = 6,   /* no CUDA device */
    TROUTE_EIO = 7,      /* file I/O */
    TROUTE_ESTATE = 8    /* handle unusable (earlier timeout) or checkpoint mismatch */
};

/* Per-segment channel parameters. Same members, order and size (8 doubles) as
 * the reference's ChParams, troute_mc_final.cu:26-28, so an array of the
 * reference's struct can be passed as is. */
typedef struct troute_chparams {
    double dx, bw, tw, twcc, n_ch, ncc, cs, s0;
} troute_chparams;

/* Float parameters as read from params.bin, wavefront_mc.cu:41-44. */
typedef struct troute_chparams_f32 {
    float dx, bw, tw, twcc, n_ch, ncc, cs, s0;
} troute_chparams_f32;

/* Secant and launch configuration. troute_cfg_default() gives the reference's
 * constants (rtol = atol = 0.01, maxiter 100, 5 attempts,
 * troute_mc_final.cu:69-74). */
typedef struct troute_cfg {
    double rtol;            /* relative depth change that ends the secant loop */
    double atol;            /* absolute depth change that ends the secant loop */
    int maxiter;            /* iteration cap of the first attempt (+25 per retry) */
    int attempts;           /* bracket-widening attempts */
    int threads_per_block;  /* 0: autotuned / default */
    int blocks_per_sm;      /* 0: occupancy-derived */
    long long wait_cycles;  /* bound on each device-side wait without progress, SM clocks; 0: ~4 s */
    int warm_start;         /* 1: learned warm start (needs troute_set_warm_start; mapping 3) */
    int warm_k;             /* secant passes a warm-started solve gets before the plain solve */
    int record_history;     /* 1: keep per-step discharge of every segment (troute_get_history) */
    int mapping;            /* reach-to-warp mapping: 0 auto (3), 1 one level-block per
                               warp, 2 per-lane refill in level-block order,
                               3 per-lane refill from the ready queue */
    int schedule_flags;     /* mapping 3, bit 0: a lane continues with an item it made ready */
    int max_chunk_steps;    /* steps routed per launch (0: as many as a third of free memory allows) */
    int record_pairs;       /* 1: every solve of a run keeps its training pair (troute_get_pairs) */
    int record_start;       /* 1: every solve of a run keeps its learned starting depth
                               (troute_get_start_history; 0 where the plain start was used) */
    int reserved[2];
} troute_cfg;

/* Counters of one run (summed over all segment solves). */
typedef struct troute_stats {
    unsigned long long solves;        /* segment solves, including early exits */
    unsigned long long iterations;    /* secant iterations */
    unsigned long long retries;       /* solves that needed a widened bracket */
    unsigned long long early_exits;   /* invalid-parameter or zero-flow solves */
    unsigned long long warm_used;     /* solves that started from the learned depth */
    unsigned long long warm_fallback; /* warm-started solves that fell back to the plain secant */
    unsigned long long iter_hist[16]; /* iterations per solve, last bin = 15+ */
    unsigned long long warp_passes;   /* loop passes of the per-lane kernels' warps (mappings 2, 3) */
    unsigned long long lane_busy;     /* lane-passes spent evaluating a depth */
    unsigned long long lane_wait;     /* lane-passes waiting for inputs */
    unsigned long long lane_idle;     /* lane-passes with no work */
    unsigned long long solve_passes;  /* warp passes that evaluated at least one depth
                                         (lane_busy / solve_passes: lanes per FP64 instruction) */
    double kernel_ms;                 /* device time of the routing kernel(s) */
    int timeout;                      /* 1 if a bounded wait ran out */
    int reserved[3];
} troute_stats;

/* River network in the reference's topo.bin terms (wavefront_mc.cu:577-587,
 * gen_network.py:12-25). Reaches are listed so that segments of reach r are
 * reach_seg_start[r] .. +reach_seg_len[r]-1, upstream end first; the upstream
 * CSR lists for each reach the reaches draining into its head. level_ptr and
 * level_reach are optional (NULL): the library derives its own schedule. */
typedef struct troute_topo {
    int n_reaches;
    int n_segments;
    const int* reach_seg_start; /* [n_reaches] */
    const int* reach_seg_len;   /* [n_reaches] */
    const int* reach_up_ptr;    /* [n_reaches + 1] */
    const int* reach_up_idx;    /* [reach_up_ptr[n_reaches]] */
} troute_topo;

typedef struct troute_handle troute_handle;

/* ---- status ------------------------------------------------------------ */
const char* troute_last_error(void);
void troute_cfg_default(troute_cfg* cfg);
int troute_device_info(int* sm_count, int* cc_major, int* cc_minor, size_t* free_bytes);

/* ---- reach-parallel, one step (replaces cpu_mc, troute_mc_final.cu:167-171,
 *      and kernel_mc_gpu, :142-148) ------------------------------------- */
/* Same argument list and meaning as cpu_mc: independent reaches, the first
 * segment's current inflow seeded by uq, reference tolerances. Host arrays. */
int troute_mc_reach_parallel(const troute_chparams* p, const double* ql,
                             const int* rs, const int* rl,
                             const double* qu, const double* qd, const double* dp,
                             double* qo, double* vo, double* dpo,
                             double uq, double dt, int nr);
/* Same with a configuration and counters (cfg/stats may be NULL). */
int troute_mc_reach_parallel_cfg(const troute_chparams* p, const double* ql,
                                 const int* rs, const int* rl,
                                 const double* qu, const double* qd, const double* dp,
                                 double* qo, double* vo, double* dpo,
                                 double uq, double dt, int nr,
                                 const troute_cfg* cfg, troute_stats* stats);
/* Device-pointer form of kernel_mc_gpu (all arrays on the device, n_segments
 * = total segments); asynchronous on `stream` (a cudaStream_t, 0 = default).
 * A reach whose segment range lies outside [0, n_segments) is skipped (its
 * outputs are left unwritten). A CUDA error already pending on the calling
 * thread is reported and left pending; nothing is launched. */
int troute_mc_reach_parallel_device(const troute_chparams* p, const double* ql,
                                    const int* rs, const int* rl,
                                    const double* qu, const double* qd, const double* dp,
                                    double* qo, double* vo, double* dpo,
                                    double uq, double dt, int nr, int n_segments,
                                    const troute_cfg* cfg, void* stream);

/* Same computation as troute_mc_reach_parallel_device for callers that cannot
 * allocate device memory where they route (a host model driver or framework
 * that owns every device buffer through its own pool, or a hot path where an
 * allocation would synchronise the device): its only scratch, the per-block
 * solve counters, is an array compiled into the library (about 1.7 MB per
 * GPU, held until the process exits). No counterpart in the reference. At most
 * 2,097,152 reaches per call (larger calls return TROUTE_EINVAL). The first
 * call on a device looks up the array's address with that device current.
 * Calls that overlap
 * on the GPU share the array and race. With stats non-NULL the call waits for
 * `stream` and returns the counters; only then is a reach with a segment range
 * outside [0, n_segments) reported (TROUTE_EINVAL; its outputs are left
 * unwritten). A CUDA error already pending on the calling thread is reported
 * and left pending; nothing is launched. */
int troute_mc_reach_parallel_device_noalloc(const troute_chparams* p, const double* ql,
                                            const int* rs, const int* rl,
                                            const double* qu, const double* qd, const double* dp,
                                            double* qo, double* vo, double* dpo,
                                            double uq, double dt, int nr, int n_segments,
                                            const troute_cfg* cfg, void* stream,
                                            troute_stats* stats);

/* ---- level-scheduled tree routing, multi-step (replaces
 *      cpu_wavefront_fp64, wavefront_mc.cu:495-507) ----------------------- */
/* Exact argument list of cpu_wavefront_fp64 (float inputs, double outputs,
 * reference tolerances); level_ptr/level_reach are validated against the
 * topology but the schedule is the library's own. */
int troute_wavefront_fp64(const troute_chparams_f32* params,
                          const int* reach_seg_start, const int* reach_seg_len,
                          const int* reach_up_ptr, const int* reach_up_idx,
                          const int* level_ptr, const int* level_reach,
                          int n_reaches, int n_levels, int n_segments,
                          const float* qlat_ts, const float* qdp0_seg,
                          const float* dp0_seg, const float* reach_last0,
                          double* qdc_seg_out_d, double* reach_last_out_d,
                          int n_timesteps, double dt);
/* FP64 one-shot tree routing: qlat_ts is [n_ts][n_segments]; outputs are the
 * final-step discharge, depth, velocity per segment and discharge of each
 * reach's last segment (any output may be NULL). */
int troute_route_tree(const troute_topo* topo, const troute_chparams* params,
                      const double* qlat_ts, const double* qdp0, const double* dp0,
                      const double* reach_last0, int n_ts, double dt,
                      const troute_cfg* cfg,
                      double* q_out, double* d_out, double* v_out,
                      double* reach_last_out, troute_stats* stats);
/* The same call under the name the tree form's drop-in boundary was
 * specified with (cpu_wavefront_fp64's semantics, WF/wavefront_mc.cu:495-507,
 * in FP64 with a configuration and statistics). */
int troute_mc_route_tree(const troute_topo* topo, const troute_chparams* params,
                         const double* qlat_ts, const double* qdp0, const double* dp0,
                         const double* reach_last0, int n_ts, double dt,
                         const troute_cfg* cfg,
                         double* q_out, double* d_out, double* v_out,
                         double* reach_last_out, troute_stats* stats);

/* ---- persistent network handle ---------------------------------------- */
/* Builds the device schedule and uploads parameters (AoS, user order). */
int troute_create(troute_handle** h, const troute_topo* topo,
                  const troute_chparams* params, double dt, const troute_cfg* cfg);
/* Batched form: n_nets independent networks (basins or ensemble members)
 * routed together in one persistent launch. params[i] are each network's
 * parameters. Lateral inflow for the batch is one [n_ts][qlat_cols] matrix:
 * segment s of network i reads column qlat_col[i][s] (NULL: the next
 * sum-of-segments column), scaled by qlat_scale[i][s] (NULL: 1). */
int troute_create_batch(troute_handle** h, int n_nets, const troute_topo* topos,
                        const troute_chparams* const* params,
                        const int* const* qlat_col, const double* const* qlat_scale,
                        int qlat_cols, double dt, const troute_cfg* cfg);
/* Ensemble form: n_members copies of one network in one launch; member m
 * routes the network with Manning's n (channel and floodplain) times
 * n_scale[m][s] and lateral inflow column s times qlat_scale[m][s] (either
 * scale may be NULL = 1). Lateral inflow is one base [n_ts][n_segments]
 * matrix shared by all members; state is member-major. */
int troute_create_ensemble(troute_handle** h, const troute_topo* topo,
                           const troute_chparams* params, int n_members,
                           const double* n_scale, const double* qlat_scale,
                           double dt, const troute_cfg* cfg);
int troute_destroy(troute_handle* h);
int troute_set_cfg(troute_handle* h, const troute_cfg* cfg);
/* Network sizes (any pointer may be NULL). */
int troute_info(const troute_handle* h, int* n_reaches, int* n_segments, int* n_levels,
                int* qlat_cols, long long* steps_done);
/* State in user order over the whole batch (segments then reaches of network
 * 0, then network 1, ...). NULL reach_last: derived from the last segments. */
int troute_set_state(troute_handle* h, const double* qdp, const double* dp,
                     const double* reach_last);
int troute_get_state(troute_handle* h, double* q, double* d, double* v,
                     double* reach_last);
/* Routes n_ts steps; qlat_ts is a host [n_ts][qlat_cols] matrix copied to the
 * device inside the call. */
int troute_run(troute_handle* h, const double* qlat_ts, int n_ts, troute_stats* stats);
/* Same with lateral inflow already on the device ([n_ts][qlat_cols]);
 * asynchronous on `stream`; call troute_sync for counters and status. */
int troute_run_device(troute_handle* h, const double* qlat_ts_device, int n_ts, void* stream);
int troute_sync(troute_handle* h, troute_stats* stats);
/* Captures `n_ts` steps reading `qlat_ts_device` into a CUDA graph, then
 * replays it on each troute_graph_launch (state carries over). */
int troute_graph_capture(troute_handle* h, const double* qlat_ts_device, int n_ts);
int troute_graph_launch(troute_handle* h, void* stream);
/* ---- autotuner --------------------------------------------------------- */
/* Times the handle's candidate launch configurations on a trial run of n_ts
 * steps of qlat_ts_device (each trial from the same saved device state, the
 * minimum of `repeats` runs) and keeps the fastest in the handle's cfg. The
 * candidates: the ready-queue kernel (mapping 3) at every resident-block count
 * from 1 to its occupancy, with and without item continuation; with
 * TROUTE_TUNE_ALL_MAPPINGS also the per-lane refill kernel (mapping 2) at
 * every block count and the one-block-per-warp kernel (mapping 1) at 32, 64
 * and 128 threads per block (not with cfg.warm_start, which needs mapping 3).
 * The schedule does not change results (bit-identical across shapes). The
 * routing state is restored afterwards; a captured graph is released
 * (capture again). */
#define TROUTE_TUNE_ALL_MAPPINGS 1
#define TROUTE_TUNE_MAX_TRIALS 32
typedef struct troute_tune_result {
    int mapping, blocks_per_sm, threads_per_block, schedule_flags;  /* chosen */
    double best_ms;                  /* kernel time of the chosen configuration's trial */
    double default_ms;               /* the default configuration's trial (mapping 3, full occupancy) */
    int n_trials;
    int trial_cfg[TROUTE_TUNE_MAX_TRIALS][4];  /* mapping, blocks per SM, threads, flags */
    double trial_ms[TROUTE_TUNE_MAX_TRIALS];   /* -1: the trial failed */
} troute_tune_result;
int troute_autotune(troute_handle* h, const double* qlat_ts_device, int n_ts, int repeats, int flags,
                    troute_tune_result* result);

/* Per-step discharge history [n_ts][n_segments] of the last run (needs
 * cfg.record_history). */
int troute_get_history(troute_handle* h, double* q_hist, int n_ts);
/* Checkpoint of the routing state (q, depth, velocity, reach outflows, step
 * count). nbytes: in = capacity, out = size; buf NULL queries the size. */
int troute_checkpoint(troute_handle* h, void* buf, size_t* nbytes);
int troute_restore(troute_handle* h, const void* buf, size_t nbytes);

/* ---- learned warm start ------------------------------------------------ */
/* No counterpart in the reference: its solve always starts from the previous
 * depth (troute_mc_final.cu:193). An 8 -> 64 -> 64 -> 1 SiLU MLP predicts a
 * segment's converged depth from log-standardised (qup, quc, qdp, ql, dx, s0,
 * n, bw); trained on the device by the library's own forward / backward /
 * AdamW kernels (FP32), evaluated inside the routing kernel with BF16 tensor
 * cores (FP32 accumulate). A solve with a prediction p brackets
 * [p (1 - delta), p (1 + delta)] for at most cfg.warm_k secant passes, then
 * falls back to the plain solve from the previous depth. */
typedef struct troute_warm troute_warm;
/* Flat model state for get/set: W1 [64][8], b1 [64], W2 [64][64], b2 [64],
 * w3 [64], b3, then the standardisation mu[8], sd[8], mu_y, sd_y. */
#define TROUTE_WARM_NPARAMS 4801
#define TROUTE_WARM_NSTATE (TROUTE_WARM_NPARAMS + 18)
/* Training pair layout (floats): qup quc qdp ql dx s0 n bw depth. */
#define TROUTE_PAIR_FLOATS 9

int troute_warm_create(troute_warm** model, uint64_t seed);
int troute_warm_destroy(troute_warm* model);
int troute_warm_get(const troute_warm* model, float* state, int n);
int troute_warm_set(troute_warm* model, const float* state, int n);
/* Trains on n_pairs device-resident pairs: standardisation from the pairs,
 * then `epochs` passes of shuffled mini-batches (batch a multiple of 64),
 * AdamW (beta 0.9 / 0.999, decoupled weight decay) with a cosine-decayed step
 * size from lr. loss_per_epoch (optional, [epochs]): mean of (err^2)/2 in
 * standardised log-depth units. Synchronous. */
int troute_warm_fit(troute_warm* model, const float* pairs_device, long long n_pairs, int epochs, int batch,
                    float lr, float weight_decay, uint64_t seed, float* loss_per_epoch);
/* Gradient of the loss over n host pairs at the current weights and
 * standardisation (the training kernel's forward and backward pass):
 * grad_out [TROUTE_WARM_NPARAMS], loss_out = mean (err^2)/2. */
int troute_warm_grad(troute_warm* model, const float* pairs_host, int n, float* grad_out, double* loss_out);
/* Predicted depths for n host input rows [n][8], through the GEMM that
 * warm-started runs use: the MLP as BF16 tcgen05 matrix multiplies (M = 128
 * rows per tile, FP32 accumulators in tensor memory); before each
 * warm-started routing launch this GEMM fills the starting depth of every
 * (segment, step) of the launch from the state at the launch's start. */
int troute_warm_predict(troute_warm* model, const float* inputs_host, int n, double* depth_out);

/* Attaches a trained model to a handle (NULL detaches); runs with
 * cfg.warm_start = 1 use it. The model must outlive the handle's runs; a
 * captured graph keeps the model's standardisation and delta of capture time. */
int troute_set_warm_start(troute_handle* h, const troute_warm* model, double delta);
/* Copies the training pairs of the last run (cfg.record_pairs) into a device
 * buffer of `capacity` pairs, ordered by step then segment; *n_pairs = pairs
 * available (solves that exit early have none). */
int troute_get_pairs(troute_handle* h, float* pairs_device, long long capacity, long long* n_pairs);
/* Learned starting depth of every solve of the last run (cfg.record_start),
 * host [n_ts][n_segments]; 0 where the plain start was used. */
int troute_get_start_history(troute_handle* h, double* start_hist, int n_ts);

/* Launches a one-warp kernel whose wait on a flag nothing sets is bounded by
 * wait_cycles; returns TROUTE_ETIMEOUT once the wait gives up and the context
 * stays usable. Exercises the device failure path without faulting. */
int troute_debug_timeout_probe(long long wait_cycles);

/* Measures the current device's FP64 issue rate: independent DMUL chains on
 * every SM (32 warps per SM), launches of >= 20 ms, best of several; returns
 * FP64 warp instructions per second (and the launch time). The routing
 * kernels are bound by this pipe; the benchmark sets their FP64 instruction
 * rate against it. No counterpart in the reference. */
int troute_measure_fp64_rate(double* warp_instr_per_s, double* ms);

/* Evaluates, on the device, the solver's pow(x, 2/3) and pow(x, 5/3) for n
 * host values: out = [ours_23[n], ours_53[n], cuda_pow_23[n], cuda_pow_53[n]]
 * (the last two from CUDA's pow(), for accuracy checks). */
int troute_debug_pow(const double* x, int n, double* out);

/* Evaluates, on the device, the solver's shared-reciprocal quotient a / b
 * (one correctly rounded reciprocal, two FMA corrections) for n host pairs,
 * for comparison with IEEE division. */
int troute_debug_div(const double* a, const double* b, int n, double* out);

/* Evaluates, on the device, the solver's convergence comparison
 * (a / b > c, IEEE quotient, b > 0, c > 0) the way the secant pass does it
 * (an FMA residual against the rounding midpoint above c, IEEE division only
 * in ambiguous cases): out[i] = 1 or 0, for comparison with the host. */
int troute_debug_quot_gt(const double* a, const double* b, double c, int n, int* out);

/* ---- schedule and topology helpers ----------------------------------- */
/* Longest chain of segment solves in the dependency graph of an n_ts-step
 * run (a reach's item of step t follows its item of step t - 1 and the items
 * of step t of its upstream reaches; an item is seg_len solves in order): the
 * critical path that bounds a run's time from below, whatever the
 * parallelism. No counterpart in the reference. */
int troute_critical_path(const troute_topo* topo, int n_ts, long long* solves);
/* Topological levels as the reference builds them (level 0 = headwater,
 * level = 1 + max upstream level; gen_network.py:219-231). level_ptr needs
 * n_reaches + 1 entries of room. */
int troute_levels(int n_reaches, const int* reach_up_ptr, const int* reach_up_idx,
                  int* reach_level, int* level_ptr, int* level_reach, int* n_levels);
/* Checks a topology; returns TROUTE_OK or TROUTE_ETOPO with a message. */
int troute_validate(const troute_topo* topo);

/* ---- matrix-form linearised MC (approximate mode) ----------------------- */
/* The reference's matrix form (water-prediction/t-route/wavefront/
 * linear_mc_matrix.cu, fused step of linear_mc_matrix_graph.cu:174-206): a
 * reach-level network (one routing unit per reach) with fixed coefficients
 * at X = 0.25 is routed as Q_new = P_Q Q_old + P_q qlat with the truncated
 * propagation matrices P_Q = (I - C1 N)^-1 (C2 N + C3), P_q = (I - C1 N)^-1 C4
 * (N: upstream adjacency), FP32. Reaches must be numbered upstream first. */
typedef struct troute_matrix troute_matrix;
/* C1, C2, C3, C4/ql per reach at X = 0.25 (compute_mc_coeffs_cpu,
 * linear_mc_matrix.cu:56-86), evaluated on the device. */
int troute_matrix_coeffs(const troute_chparams_f32* params, int n_reaches, double dt, float* c1, float* c2,
                         float* c3, float* c4oq);
/* Builds P_Q and P_q once on the host (build_propagation_matrices,
 * linear_mc_matrix.cu:129-216; entries with |value| < tol dropped, the
 * reference uses 1e-7) and uploads them. TROUTE_ETOPO when a reach is not
 * numbered after its upstream reaches. */
int troute_matrix_create(troute_matrix** h, int n_reaches, const int* reach_up_ptr, const int* reach_up_idx,
                         const float* c1, const float* c2, const float* c3, const float* c4oq, float tol);
int troute_matrix_destroy(troute_matrix* h);
/* Sizes: reaches and stored entries of P_Q and P_q (any pointer may be NULL). */
int troute_matrix_info(const troute_matrix* h, int* n_reaches, long long* nnz_Q, long long* nnz_q);
/* Host copies of P_Q (which = 0) or P_q (1) in CSR: ptr [n_reaches + 1],
 * col and val [nnz] (any pointer may be NULL). */
int troute_matrix_get(const troute_matrix* h, int which, int* ptr, int* col, float* val);
/* Routes n_ts steps on the device: qlat_ts [n_ts][n_reaches], q [n_reaches]
 * in/out; asynchronous on `stream` (NULL: the handle's own). The run is
 * recorded as a CUDA graph on first use and replayed while the buffers and
 * n_ts stay the same. */
int troute_matrix_run_device(troute_matrix* h, const float* qlat_ts_device, int n_ts, float* q_device, void* stream);
/* One-shot host form: build, route n_ts steps from q0, return the discharge. */
int troute_matrix_route(int n_reaches, const int* reach_up_ptr, const int* reach_up_idx, const float* c1,
                        const float* c2, const float* c3, const float* c4oq, float tol, const float* qlat_ts,
                        const float* q0, int n_ts, float* q_out);

/* ---- linearised MC (approximate mode) --------------------------------- */
/* The reference's linear form (water-prediction/t-route/wavefront/
 * linear_mc.cu): fixed per-segment coefficients C1, C2, C3, C4/ql from the
 * channel at half bankfull depth (linear_mc.cu:57-100), then per step
 * Q_new = C1 Q_up_new + C2 Q_up_old + C3 Q_old + (C4/ql) qlat in topological
 * order (cpu_linear_mc, :177-232), FP32. No secant iteration; its error is
 * measured against the secant path. Every reach needs at least one segment. */
typedef struct troute_linear troute_linear;
/* Coefficients for n segments, computed on the device (FP32, CUDA powf/sqrtf
 * as the reference's kernel_precompute_coeffs). Host arrays. */
int troute_linear_coeffs(const troute_chparams_f32* params, int n_segments, double dt, float* c1, float* c2,
                         float* c3, float* c4oq);
int troute_linear_create(troute_linear** h, const troute_topo* topo, const float* c1, const float* c2,
                         const float* c3, const float* c4oq);
int troute_linear_destroy(troute_linear* h);
/* n_ts steps of device lateral inflow [n_ts][n_segments] (float); q_dev
 * [n_segments] holds the discharge before the run and after it. Synchronous;
 * wait_cycles bounds each device wait without progress (0: ~4 s). */
int troute_linear_run_device(troute_linear* h, const float* qlat_ts_device, int n_ts, float* q_device,
                             long long wait_cycles, void* stream);
/* One-shot host form of cpu_linear_mc's arguments: coefficients, lateral
 * inflow [n_ts][n_segments], initial discharge -> final discharge. */
int troute_linear_route(const troute_topo* topo, const float* c1, const float* c2, const float* c3,
                        const float* c4oq, const float* qlat_ts, const float* q0, int n_ts, float* q_out);

/* ---- diffusive-wave tridiagonal step ----------------------------------- */
/* The reference's t-route diffusive-wave solver (water-prediction/
 * owp_extended_kernels.cu:24-153, cpu_diffusive_tridiag / kernel_diffusive_
 * tridiag): per reach a Crank-Nicolson tridiagonal system over its ncomp
 * computational nodes, forward elimination and back substitution, FP32.
 * Arrays are [n_reaches][max_nodes] (the reference's MAX_NODES is 500); nodes
 * at or past a reach's ncomp are neither read nor written. Bit-identical to
 * the reference's CPU routine. celerity is accepted for the argument list
 * and not read (the reference computes an unused Courant number from it). */
typedef struct troute_diff_reach {
    int ncomp;     /* computational nodes, 1..max_nodes */
    float theta;   /* Crank-Nicolson weight */
    float dtini;   /* time step, s */
} troute_diff_reach;
int troute_diffusive_tridiag(const troute_diff_reach* reaches, const float* dx, const float* diffusivity,
                             const float* celerity, const float* qp_prev, float* qp_out, int n_reaches,
                             int max_nodes);
/* Device arrays; scratch holds 2 * n_reaches * max_nodes floats; asynchronous
 * on `stream`. */
int troute_diffusive_tridiag_device(const troute_diff_reach* reaches, const float* dx, const float* diffusivity,
                                    const float* celerity, const float* qp_prev, float* qp_out, int n_reaches,
                                    int max_nodes, float* scratch, void* stream);

/* ---- on-disk network format ------------------------------------------- */
/* The reference's topo.bin / params.bin / forcings.bin directory format
 * (water-prediction/t-route/wavefront/gen_network.py:292-337, read by
 * wavefront_mc.cu:597-632 load_topo and :655-672). All arrays are owned by
 * the struct; troute_read_network allocates, troute_free_network releases.
 * params are float32 as the reference writes them; qlat is [n_ts][n_segments];
 * qup0 is the per-reach outflow of the step before the first (reach_last0). */
typedef struct troute_netfile {
    int n_reaches, n_segments, n_levels, max_upstream, n_ts;
    int *reach_seg_start, *reach_seg_len, *reach_level, *reach_n_up;
    int *reach_up_ptr, *reach_up_idx;   /* [n_reaches + 1], [nnz] */
    int *level_ptr, *level_reach;       /* [n_levels + 1], [n_reaches] */
    troute_chparams_f32* params;        /* [n_segments] */
    float *qlat, *qup0, *qdp0, *dp0;
} troute_netfile;
/* Reads and checks the three files (short, long or inconsistent files give
 * TROUTE_EIO / TROUTE_ETOPO; the reference's reader exits or reads short). */
int troute_read_network(const char* dir, troute_netfile** net);
void troute_free_network(troute_netfile* net);
/* Writes the three files (byte-compatible with the reference's writer).
 * With qlat, qup0, qdp0 and dp0 all NULL (and n_ts 0) only topo.bin and
 * params.bin are written, as the reference's GeoPackage parser does. */
int troute_write_network(const char* dir, const troute_netfile* net);

/* ---- lateral-inflow pre-processor -------------------------------------- */
/* Pivots a directory of nex-<id>_output.csv files ("step, time, value" rows)
 * into qlat[n_ts][n_reaches] (reach i takes the file whose id is
 * reach_ids[i]; cells without a file stay 0), in parallel over files
 * (n_threads <= 0: all hardware threads). The parsing rules of the reference's
 * water-prediction/t-route/wavefront/data_parsers/parse_qlat_fast_cpp.cpp.
 * matched / missing (optional): files used / files whose id is unknown. */
int troute_qlat_from_csv(const char* csv_dir, const int64_t* reach_ids, int n_reaches, int n_ts, int n_threads,
                         float* qlat, long long* matched, long long* missing);
/* Writes forcings.bin: int32 n_ts, float32 qlat[n_ts][n_segments],
 * qup0[n_reaches], qdp0[n_segments], dp0[n_segments]. */
int troute_write_forcings(const char* path, int n_ts, int n_reaches, int n_segments, const float* qlat,
                          const float* qup0, const float* qdp0, const float* dp0);

/* ---- synthetic inputs (seeded, platform-independent) ------------------ */
/* Uniform random binary river tree (Remy's algorithm) with n_leaves
 * headwaters -> 2*n_leaves-1 reaches, n_segments segments of 1..max_len per
 * reach. Arrays: [2n-1], [2n-1], [2n], [2n-2]. */
int troute_gen_tree(uint64_t seed, int n_leaves, int n_segments, int max_len,
                    int* reach_seg_start, int* reach_seg_len,
                    int* reach_up_ptr, int* reach_up_idx);
/* Channel parameters: dx~U(500,5000), s0~LogU(1e-5,1e-2), n~U(.03,.08),
 * ncc=2n, bw~U(2,50), tw=3bw, twcc=5tw, cs~U(.5,2). */
int troute_gen_params(uint64_t seed, int n_segments, troute_chparams* params);
/* Lateral inflow [n_ts][n_segments] for steps t0..t0+n_ts-1:
 * Gamma(2, 0.05) m3/s x (1 + 0.5 sin(2 pi t dt / 86400 + phase_s)). */
int troute_gen_qlat(uint64_t seed, int n_segments, int t0, int n_ts, double dt,
                    double* qlat);
/* Ensemble member perturbations: qfac ~ LogN(0, 0.3), nfac ~ U(0.8, 1.2). */
int troute_gen_member(uint64_t seed, int member, int n_segments, double* qfac,
                      double* nfac);

#ifdef __cplusplus
}
#endif
#endif
