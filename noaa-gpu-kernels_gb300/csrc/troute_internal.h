// Internal declarations shared by the host (C++) and device (CUDA) halves of
// libtroute_gb300.so. Nothing here is part of the public C ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cmath>

#include <vector_types.h>

#include "../../include/troute_gb300.h"

#if defined(__CUDACC__)
#define TR_HD __host__ __device__
#else
#define TR_HD
#endif

// Records a message for troute_last_error() and returns `code`.
int set_error(int code, const char* fmt, ...);

namespace tr {

uint64_t hash3(uint64_t seed, uint64_t stream, uint64_t ctr);
double u01(uint64_t h);
double det_log(double x);
double det_exp(double x);
double det_sin(double x);

constexpr int kLanes = 32;      // reaches per level-block (one warp)
constexpr int kRing = 4;        // depth of the per-reach outflow ring (steps)
constexpr double kMinDepth = 0.01;  // troute_mc_final.cu:58

// Secant tolerances handed to the device.
struct Tol {
    double rtol, atol;
    int maxiter, attempts;
};

// Per-segment values the solver reads, derived once from ChParams on the host
// with the same IEEE operations the reference performs per solve
// (troute_mc_final.cu:181-183), stored as six double2 planes.
//   p[0] = {dx, bw}        p[1] = {twcc, n_ch}      p[2] = {ncc, s0}
//   p[3] = {z, bfd}        p[4] = {sqrt(s0), 2 sqrt(1+z^2)}
//   p[5] = {sqrt(s0)/n_ch, 2 z}
// The doubled values are exact (scaling by 2), and the reference's products
// 2.0 * z * h and 2.0 * below * sqrt(1+z^2) round to the same double as
// (2z) * h and below * (2 sqrt(1+z^2)): doubling commutes with rounding.
constexpr int kParamPlanes = 6;

struct SegP {
    double dx, bw, twcc, n_ch, ncc, s0, z, bfd, sq_s0, sq2, ck_fac, z2;
};

// Everything static a segment solve reads, in one aligned 128-byte record (one
// L2 line, two DRAM bursts): the six parameter planes' values, the lateral
// inflow scale (1 when the handle has none: x * 1 is exactly x) and column.
// The per-lane kernels take (reach, step) items in any order, so a solve's
// reads are scattered; one record instead of eight separate arrays turns
// eight sector fetches per solve into one line.
struct __align__(128) SegRec {
    double2 p[kParamPlanes];
    double qscale;
    int qcol;
    int reach;   // internal reach of the slot (-1: a slot no segment uses)
    int pos;     // position of the segment in its reach
    int pad[3];
};
static_assert(sizeof(SegRec) == 128, "one 128-byte line per segment");

// Derived values from the reference's parameter record, :181-183.
TR_HD inline SegP derive_seg(const troute_chparams& c)
{
    SegP p;
    p.dx = c.dx; p.bw = c.bw; p.twcc = c.twcc; p.n_ch = c.n_ch; p.ncc = c.ncc; p.s0 = c.s0;
    p.z = (c.cs == 0.0) ? 1.0 : 1.0 / c.cs;
    p.bfd = (c.bw > c.tw) ? c.bw / 0.00001 : (c.bw == c.tw) ? c.bw / (2.0 * p.z) : (c.tw - c.bw) / (2.0 * p.z);
    p.sq_s0 = sqrt(c.s0);
    p.sq2 = 2.0 * sqrt(1.0 + p.z * p.z);
    p.ck_fac = p.sq_s0 / c.n_ch;
    p.z2 = 2.0 * p.z;
    return p;
}

// Device counters of one run.
struct DevStats {
    unsigned long long solves, iterations, retries, early_exits, warm_used, warm_fallback;
    unsigned long long hist[16];
    unsigned long long warp_passes, lane_busy, lane_wait, lane_idle, solve_passes;
    int error;       // 0 ok, TROUTE_ETIMEOUT, TROUTE_EINVAL (bad index seen)
    int err_reach;   // internal reach of the first failure
    int err_step;    // step of the first failure
    int err_where;   // 1 own, 2 upstream, 3 downstream back-pressure, 4 bounds
};

// Static network description on the device (internal order).
struct NetDev {
    int n_blocks;            // level-blocks of kLanes reaches
    int n_levels;            // ALAP levels
    int n_reach_int;         // n_blocks * kLanes
    long long n_seg_int;     // padded tile storage
    const SegRec* seg;       // [n_seg_int] parameters, inflow column and scale
    const int* nseg;         // [n_reach_int], -1 for padding lanes
    const long long* tile_off;  // [n_blocks] first segment slot of a block
    const int* block_level;  // [n_blocks]
    const int* lb_ptr;       // [n_levels + 1] blocks of each level
    const int* up_ptr;       // [n_reach_int + 1]
    const int* up_idx;       // internal reach ids
    const int* down;         // [n_reach_int] internal id or -1
    // mutable state
    double* q;               // [n_seg_int] discharge of the last completed step
    double* d;               // depth
    double* v;               // velocity
    double* ring;            // [kRing][n_reach_int] outflow of each reach per step
    int* done;               // [n_reach_int] cumulative completed steps
};

// One routing run (n_ts steps).
struct RunDev {
    const int* step_base;    // device: cumulative steps before this run
    int n_ts;
    double dt;
    double dt_half;          // dt / 2.0
    const double* qlat;      // [n_ts][qlat_ld]
    long long qlat_ld;
    const unsigned long long* wave_ptr;  // [n_ts + n_levels] ticket prefix per wave
    int n_waves;
    unsigned long long n_tickets;
    unsigned long long* ticket;  // device counter
    DevStats* stats;
    long long wait_cycles;
    Tol tol;
    double* q_hist;          // optional [n_ts][n_seg_int]
    float* pairs;            // optional [n_ts][n_seg_int][9] training pairs (qup quc qdp ql dx s0 n bw depth)
    double* start_hist;      // optional [n_ts][n_seg_int] learned starting depth of each solve (0: plain)
    int warm;                // 1: solves start from the learned depth (dataflow kernel only)
    const float* start_pred; // [n_ts][n_seg_int] learned starting depth of every solve (warm runs)
    int warm_k;              // passes of the warm phase before the plain fallback
    double warm_delta;       // relative half-width of the warm bracket
    double warm_hi, warm_lo; // 1 + warm_delta, 1 - warm_delta
};

// Ready-queue state of one run of the dataflow kernel (mapping 3).
struct DataflowDev {
    int* cnt;                       // [n_ts][n_reach_int] completed dependencies
    int2* rq;                       // [n_items] ready (reach, step) items
    unsigned long long* rq_head;    // claimed slots
    unsigned long long* rq_tail;    // written slots
    unsigned long long* n_done;     // completed items
    double* rh;                     // [n_ts + 1][n_reach_int] reach outflow per step
    const int2* heads;              // (headwater reach, 0) items, ready at the start
    int n_heads;
    int continue_items;             // 1: a lane continues with an item it made ready
    unsigned long long n_items;     // real reaches x n_ts
};

// Launch helpers implemented in kernels.cu (all asynchronous on `stream`).
int launch_reach_parallel(const troute_chparams* p, const double* ql, const int* rs,
                          const int* rl, const double* qu, const double* qd, const double* dp,
                          double* qo, double* vo, double* dpo, double uq, double dt, int nr,
                          int n_segments, const Tol& tol, DevStats* stats, int threads,
                          void* stream);
int launch_route(const NetDev& net, const RunDev& run, int grid, int threads, void* stream);
int route_occupancy(int threads, int* blocks_per_sm);
int launch_route_pool(const NetDev& net, const RunDev& run, int grid, int threads, void* stream);
int route_pool_occupancy(int* blocks_per_sm);
int launch_route_dataflow(const NetDev& net, const RunDev& run, const DataflowDev& df, int grid, void* stream);
// Learned starting depths of a routing launch of T steps (warm_gemm.cu): the
// MLP as one tcgen05 GEMM over every (segment slot, step), features from the
// state at the launch's start; plane [T][n_seg_int]. A stalled wait sets
// *error to TROUTE_ETIMEOUT.
int launch_warm_plane(const troute_warm* w, const NetDev& net, const RunDev& run, int T, float* plane, int* error,
                      void* stream);
// The same GEMM for raw inputs [n][8] (device arrays).
int launch_warm_gemm_raw(const troute_warm* w, const float* raw, long long n, double* depth, int* error,
                         void* stream);
// Learned warm start (warm.cu): whether a model has weights on the device, and
// the compaction of the dense per-solve pair records [n_rows][9] (rows with a
// positive depth) into `out`, in row order; synchronous on `stream`.
bool warm_ready(const troute_warm* w);
int compact_pairs(const float* dense, long long n_rows, float* out, long long capacity, long long* n_valid,
                  void* stream);
int route_dataflow_occupancy(int* blocks_per_sm, bool warm);
int route_dataflow_threads();
int launch_bump_steps(int* step_base, int n_ts, void* stream);
int launch_fill_int(int* p, long long n, const int* value_dev, int value_host, void* stream);
int launch_scatter(const double* src, const long long* map, long long n, double* dst,
                   void* stream);
int launch_gather(const double* src, const long long* map, long long n, double* dst,
                  void* stream);
int launch_timeout_probe(DevStats* stats, long long wait_cycles, void* stream);
int launch_fp64_rate(int blocks, int iters, double* sink, void* stream, double* warp_instr);
int launch_debug_pow(const double* x, int n, double* out, void* stream);
int launch_debug_div(const double* a, const double* b, int n, double* out, void* stream);
int launch_debug_quot_gt(const double* a, const double* b, double c, int n, int* out, void* stream);
int launch_velocity(const NetDev& net, void* stream);

}  // namespace tr
