#!/usr/bin/env python
"""Benchmark of the GB300 MC secant routing path.

Metric: segment-steps per second (segments x routed time steps / s) of FP64
Muskingum-Cunge secant tree routing at secant tolerance rtol = 1e-8
(atol = 1e-10), batched + learned warm start against plain MC.

Default workload c4w (the combined form): a 64-member ensemble over the
2.7M-segment, ~1.1M-reach random binary river tree (~2,400 levels) -- lateral
inflow x LogN(0, 0.3) and Manning's n x U(0.8, 1.2) per member -- routed in one
persistent launch with the learned warm start, FP64 state. The MLP is trained
in the same run, untimed, on (input, converged depth) pairs of an 18-step
plain run of the single network (~49M pairs). One bench "step" = 32 routed
time steps of all 64 members (5.5G segment-steps) in one persistent launch
(longer launches amortise the dependency graph's fill and drain), replayed
from a captured CUDA graph, the state carrying over; 3 timed after 3
warm-up. Beside it, in the same run, the plain single-basin routing of the
same network (144 steps per graph launch) is timed: `plain_single_basin`,
and `speedup_vs_plain` = value / that.

Other workloads: c1 (plain single basin, 144 steps per bench step), c0, c2
(256 uneven basins), c3 (warm start on a fresh-seed c1 network, trained on
pairs of the seed-1001 network), c4 (the ensemble without warm start),
tree:<segments>. Seeded synthetic parameters and lateral inflow (no dataset
is available offline).

`e2e` is the same metric through the public C ABI with host buffers:
troute_run (copies the step's lateral inflow from pinned host memory) plus
troute_get_state (copies the routed discharge, depth, velocity and reach
outflow back).

--impl reference times the reference's CPU algorithm (the oracle port of
cpu_wavefront_fp64, all host threads, one routed time step of the network --
of ensemble member 0 for c4/c4w -- per bench step).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "noaa-gpu-kernels_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "segment-steps/s at 1e-8 depth tol: batched+warm-start vs plain MC, 1 GB300"
UNIT = "seg-steps/s"
TIGHT = dict(rtol=1e-8, atol=1e-10, maxiter=100, attempts=5)
BYTES_PER_SEG_STEP = 112  # params 64 + qlat 8 + q 8 + depth 8 read; q, depth, velocity 24 written


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c4w")
    ap.add_argument("--n-ts", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (profiling runs)")
    ap.add_argument("--no-parity", action="store_true", help="skip the operating-point oracle check")
    ap.add_argument("--no-batched-plain", action="store_true", help="skip the batched plain-start leg")
    ap.add_argument("--warm", action="store_true",
                    help="learned warm start on a single-network workload (trained on its own plain-run pairs)")
    return ap.parse_args()


# --------------------------------------------------------------------------- distributed plumbing
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if torch.cuda.is_available():
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        dev = "cuda" if torch.cuda.is_available() else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        dev = "cuda" if torch.cuda.is_available() else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines = []

    def start(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.gpu_id:
            cmd += ["-i", self.gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------- helpers
def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_file(key: str, name: str):
    """A `key: value` figure from a committed ncu summary under profiles/."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        for ln in open(p):
            if ln.strip().startswith(key + ":"):
                return float(ln.split(":")[1]), name
    except OSError:
        pass
    return None, name


def profiled(key: str, warm: bool):
    """A figure of the routing kernel from the committed ncu summary: the
    warm-started kernel's (an ensemble capture) or the plain kernel's."""
    return profiled_file(key, "route_dataflow_warm_ens256.md" if warm else "route_kernel_c1.md")


def critical_path_bound(T, w, n_ts: int, it_per_solve: float, sm_mhz, kernel_ms: float) -> dict:
    """The dependency graph's critical path of one bench step set against the
    FP64 pipe: the longest chain of segment solves (troute_critical_path), each
    solve at least (iterations + 1) passes, each pass at least its FP64 warp
    instructions x 64 cycles (one FP64 warp instruction per 64 cycles per
    SMSP, however few lanes are busy)."""
    if "batch" in w:
        chain = max(T.critical_path(n["topo"], n_ts) for n in w["batch"])
    else:
        chain = T.critical_path(w["topo"], n_ts)
    out = {"segment_solves": chain, "passes_per_solve": it_per_solve + 1.0}
    instr, src = profiled_file("fp64_instr_per_solving_pass", "route_dataflow_instmix_tree200k.md")
    if instr is None:
        return out
    pass_us = instr * 64.0 / float(sm_mhz or 2070.0)
    bound_ms = chain * (it_per_solve + 1.0) * pass_us / 1e3
    out.update({"fp64_instr_per_pass": instr, "instr_source": f"profiles/{src}", "pass_us_min": pass_us,
                "lower_bound_ms": bound_ms, "kernel_ms": kernel_ms, "kernel_over_bound": kernel_ms / bound_ms})
    return out


def workload(name: str, n_ts: int | None, members: tuple | None = None):
    """Single networks ('c1', 'c0', 'tree:<segments>', 'c3' = fresh-seed c1
    with warm start) or the batched forms: 'c2' (256 basins with
    LogU(500, 200,000) segments, 288 steps), 'c4' / 'c4w' (64 ensemble
    members of the c1 network, without / with warm start; 32 steps per bench
    step). `members` = (first, end): the share of the ensemble members (or of
    the c2 basins, by index) one rank routes."""
    from troute_gb300 import synth

    if name == "c2":
        T = 288 if n_ts is None else n_ts
        sizes = synth.basin_sizes(1002, 256)
        nets = synth.basins(seed=1002, n_trees=256, which=members)
        qlat = synth.make_qlat(1002, int(sizes.sum()), T)
        if members is not None:
            # the same inflow columns as in the unsharded batch
            offs = np.concatenate([[0], np.cumsum(sizes)])
            qlat = np.ascontiguousarray(np.concatenate([qlat[:, offs[i]:offs[i + 1]] for i in members], axis=1))
        S = sum(n["topo"]["n_segments"] for n in nets)
        w = {"name": name, "batch": nets, "n_ts": T, "dt": synth.DT, "qlat": qlat}
        w["q0"] = np.full(S, synth.Q0)
        w["d0"] = np.full(S, synth.D0)
        w["rl0"] = np.concatenate([np.full(len(n["topo"]["reach_seg_start"]), synth.Q0) for n in nets])
        w["S"], w["R"] = S, len(w["rl0"])
        return w
    if name in ("c4", "c4w") or name.startswith("ens:"):
        # ens:<members>:<segments>[:w] -- a smaller ensemble of a tree:<segments>
        # network (profiling cases), ':w' with the warm start
        if name.startswith("ens:"):
            parts = name.split(":")
            M, base_net = int(parts[1]), f"tree:{int(parts[2])}"
        else:
            M, base_net = 64, "c1"
        T = 32 if n_ts is None else n_ts
        w = synth.network(base_net, n_ts=T)
        w["base"] = base_net
        S = w["topo"]["n_segments"]
        m0, m1 = (0, M) if members is None else members
        qf = np.empty((m1 - m0, S))
        nf = np.empty((m1 - m0, S))
        for k, m in enumerate(range(m0, m1)):
            qf[k], nf[k] = synth.make_member(1004, m, S)
        w.update(name=name, members=m1 - m0, member_range=(m0, m1), members_total=M, qfac=qf, nfac=nf,
                 warm=(name == "c4w" or name.endswith(":w")))
        w["S"], w["R"] = (m1 - m0) * S, (m1 - m0) * len(w["topo"]["reach_seg_start"])
        w["q0_1"], w["d0_1"], w["rl0_1"] = w["q0"], w["d0"], w["rl0"]
        w["q0"], w["d0"], w["rl0"] = (np.tile(w["q0"], m1 - m0), np.tile(w["d0"], m1 - m0),
                                      np.tile(w["rl0"], m1 - m0))
        return w
    w = synth.network(name, n_ts=n_ts)
    if name == "c3":
        w["warm"] = True
    w["S"], w["R"] = w["topo"]["n_segments"], len(w["topo"]["reach_seg_start"])
    return w


def seeds_of(w: dict, model: bool = False) -> dict:
    """The generator seeds of a workload, recorded in the JSON line's config:
    the network's (or c2's basin set's), the ensemble members' perturbations,
    and the warm-start model's initialisation and shuffling."""
    if w.get("name") == "c2":
        out = {"basins": 1002}
    else:
        out = {"network": w.get("seed")}
    if "members" in w:
        out["members"] = 1004
    if model:
        out["model"] = 1001
    return out


def shard(name: str, dist) -> tuple | None:
    """The rank's share of a batched workload (members or basins), or None
    (single networks run as replicas)."""
    from troute_gb300 import parallel, synth

    if dist.world <= 1:
        return None
    if name in ("c4", "c4w") or name.startswith("ens:"):
        M = int(name.split(":")[1]) if name.startswith("ens:") else 64
        return parallel.member_range(M, dist.world, dist.rank)
    if name == "c2":
        return tuple(parallel.partition([int(x) for x in synth.basin_sizes(1002, 256)], dist.world)[dist.rank])
    return None


def make_network(T, w, cfg):
    if "batch" in w:
        nets = w["batch"]
        return T.Network([n["topo"] for n in nets], [n["params"] for n in nets], cfg=cfg)
    if "members" in w:
        return T.Network.ensemble(w["topo"], w["params"], w["members"], n_scale=w["nfac"], qlat_scale=w["qfac"],
                                  cfg=cfg)
    return T.Network(w["topo"], w["params"], cfg=cfg)


def describe(w) -> str:
    ws = ", learned warm start" if w.get("warm") else ", plain secant start"
    if "batch" in w:
        return f"batched: {len(w['batch'])} independent basins in one launch" + ws
    if "members" in w:
        return f"batched: {w['members']}-member ensemble in one launch" + ws
    return "single basin" + ws


WARM_DELTA = 0.05   # relative half-width of the bracket around the learned depth
WARM_K = 16         # secant passes before the plain fallback
PAIR_STEPS = 18     # plain steps whose solves give the training pairs (~49M for c1)


def nvtx_push(name: str) -> None:
    try:
        import torch

        torch.cuda.nvtx.range_push(name)
    except Exception:
        pass


def nvtx_pop() -> None:
    try:
        import torch

        torch.cuda.nvtx.range_pop()
    except Exception:
        pass


def train_and_plain(T, torch, dev, stream, plain_steps: int, plain_warmup: int, base: str = "c1") -> tuple:
    """Untimed set-up of the warm-started workloads, on the base network (the
    seed-1001 c1 network for c3/c4w, else the workload's own network): the
    training pairs of an 18-step plain run, the MLP trained on them, then the
    plain single-basin routing timed (144 steps per graph launch, the same
    method as the c1 workload)."""
    from troute_gb300 import synth

    w = synth.network(base, n_ts=144)
    S = w["topo"]["n_segments"]
    ql = torch.from_numpy(np.ascontiguousarray(w["qlat"])).to(dev)
    net = T.Network(w["topo"], w["params"], cfg=T.make_cfg(**TIGHT, record_pairs=1))
    net.set_state(w["q0"], w["d0"], w["rl0"])
    t0 = time.perf_counter()
    net.run_device(ql.data_ptr(), PAIR_STEPS, stream.cuda_stream)
    net.sync()
    n = net.pairs()
    pairs = torch.empty((n, 9), dtype=torch.float32, device=dev)
    net.pairs(pairs.data_ptr(), n)
    torch.cuda.synchronize(dev)
    t_pairs = time.perf_counter() - t0
    model = T.WarmModel(1001)
    t0 = time.perf_counter()
    loss = model.fit(pairs.data_ptr(), n, epochs=3, batch=8192, lr=2e-3, seed=1001)
    t_fit = time.perf_counter() - t0
    del pairs
    # plain single-basin routing, graph-replayed 144-step runs, in the launch
    # shape the autotuner picks for it (all mappings; 16-step trials)
    net.set_cfg(T.make_cfg(**TIGHT))
    tune = net.autotune(ql.data_ptr(), 16, repeats=1, all_mappings=True)
    net.graph_capture(ql.data_ptr(), 144)
    for _ in range(plain_warmup):
        net.graph_launch(stream.cuda_stream)
    torch.cuda.synchronize(dev)
    net.sync()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(plain_steps):
        net.graph_launch(stream.cuda_stream)
    b.record(stream)
    torch.cuda.synchronize(dev)
    st = net.sync()
    ms = a.elapsed_time(b)
    net.close()
    del ql
    torch.cuda.empty_cache()
    plain = {"value": S * 144 * plain_steps / (ms / 1e3), "unit": UNIT,
             "workload": f"{base}: the {S}-segment network alone, plain secant start, 144 steps per graph "
                         f"launch, {plain_steps} timed launches after {plain_warmup}",
             "iterations_per_solve": st["iterations"] / max(1, st["solves"]), "ms_per_run": ms / plain_steps,
             "launch_shape": {k: tune[k] for k in ("mapping", "blocks_per_sm", "threads_per_block", "schedule_flags")}}
    info = {"pairs": int(n), "pair_steps": PAIR_STEPS, "pairs_s": round(t_pairs, 2), "epochs": 3, "batch": 8192,
            "fit_s": round(t_fit, 2), "loss_per_epoch": [round(float(x), 5) for x in loss],
            "delta": WARM_DELTA, "k": WARM_K, "trained_on": f"{base} (seed {w['seed']}), plain run from the initial state"}
    return model, info, plain


def topology_bytes_per_seg_step(w) -> float:
    """Reach-topology bytes a step reads per segment, beside the algorithmic
    112 B: per reach its segment range, upstream CSR row and downstream index
    (16 B), per upstream link 4 B."""
    if "batch" in w:
        topos = [n["topo"] for n in w["batch"]]
    else:
        topos = [w["topo"]] * int(w.get("members", 1))
    R = sum(len(t["reach_seg_start"]) for t in topos)
    links = sum(len(t["reach_up_idx"]) for t in topos)
    S = sum(int(t["n_segments"]) for t in topos)
    return (16.0 * R + 4.0 * links) / max(1, S)


def host_cpu() -> dict:
    """The host the CPU legs ran on: hardware threads and the CPU model."""
    model = ""
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                key = ln.split(":", 1)[0].strip().lower()
                if key in ("model name", "cpu model", "hardware"):
                    model = ln.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if not model:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            model = next((ln.split(":", 1)[1].strip() for ln in out.splitlines() if ln.startswith("Model name")), "")
        except (OSError, subprocess.SubprocessError):
            model = ""
    return {"nproc": os.cpu_count() or 1, "cpu_model": model or platform.machine()}


def cpu_baseline(w, win=None) -> dict:
    """The oracle port of cpu_wavefront_fp64 (the C library's pow(), the
    reference's arithmetic), one core, one routed step of network 0 of the
    workload (ensemble member 0, basin 0 or the network) from the start state
    of the GPU arm's timed window (the initial state without `win`)."""
    from oracle import troute_oracle as O

    O.build(ref=False)
    tol = (TIGHT["rtol"], TIGHT["atol"], TIGHT["maxiter"], TIGHT["attempts"])
    ss, rs, cs = member_slice(w, 0)
    topo, params, qs, label = network_k(w, 0)
    Sn = topo["n_segments"]
    ql = w["qlat"][:1, cs] * (qs[None, :] if qs is not None else 1.0)
    if win is None:
        q, d, rl, where = w["q0"][ss], w["d0"][ss], w["rl0"][rs], "its initial state"
    else:
        q, d, rl, where = win[0][ss], win[1][ss], win[3][rs], "the start state of the timed window"
    t0 = time.perf_counter()
    O.route_tree(topo, params, ql, q, d, rl, tol=tol, threads=1)
    dt = time.perf_counter() - t0
    return {"value": Sn / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"1 routed step of {label} {Sn}-segment network from {where}, rtol 1e-8, single thread "
                      f"({dt:.1f} s)", "host": host_cpu()}


# --------------------------------------------------------------------------- reference arm
def reference_inputs(name: str, n_ts: int | None):
    """(network, label, routed steps per bench step) of the reference arm, built
    with the oracle's own restatement of the seeded generator: this process
    never loads the product library. The ensembles route member 0."""
    from oracle import troute_oracle as O

    if name in ("c4", "c4w"):
        T = 32 if n_ts is None else n_ts
        w = O.ensemble_member(O.network("c1", n_ts=T), 0)
        return w, f"member 0 of the 64-member ensemble over the {w['topo']['n_segments']}-segment c1 network", T
    if name.startswith("ens:"):
        parts = name.split(":")
        T = 32 if n_ts is None else n_ts
        w = O.ensemble_member(O.network(f"tree:{int(parts[2])}", n_ts=T), 0)
        return w, f"member 0 of the {int(parts[1])}-member ensemble over the tree:{int(parts[2])} network", T
    if name in ("c0", "c1", "c3") or name.startswith("tree:"):
        w = O.network(name, n_ts=n_ts)
        return w, f"the {w['topo']['n_segments']}-segment {name} network", w["n_ts"]
    return None, "", 0


def run_reference(args, dist: Dist):
    """The reference's CPU algorithm (the oracle port of cpu_wavefront_fp64 in
    FP64, level-parallel over all host threads; the reference's own routine is
    single-threaded and is not built on the aarch64 host) on the routed-step
    window the GPU arm times: the network is first advanced untimed through
    the GPU arm's warm-up bench steps, then each timed bench step routes the
    same routed steps as a GPU bench step (lateral inflow rows t mod n_ts, as
    the GPU arm's graph replays them)."""
    if dist.rank != 0:
        return
    from oracle import troute_oracle as O

    O.build(ref=False)
    w, label, per_step = reference_inputs(args.workload, args.n_ts)
    if w is None:
        print(json.dumps({"impl": "reference", "unavailable": "the CPU arm routes single networks and ensemble "
                                                            "members; run it with --workload c1 for c2"}))
        return
    topo, params, qlat = w["topo"], w["params"], w["qlat"]
    q, d, rl = w["q0"], w["d0"], w["rl0"]
    S, R = topo["n_segments"], len(topo["reach_seg_start"])
    nth = os.cpu_count() or 1
    tol = (TIGHT["rtol"], TIGHT["atol"], TIGHT["maxiter"], TIGHT["attempts"])
    lp, lr = O.levels_c(topo["reach_up_ptr"], topo["reach_up_idx"], R)
    n_ts = qlat.shape[0]
    per_step = min(per_step, n_ts)

    def route(rows):
        nonlocal q, d, rl
        o = O.route_tree(topo, params, rows, q, d, rl, tol=tol, threads=nth, level_ptr=lp, level_reach=lr)
        q, d, rl = o["q"], o["d"], o["reach_last"]
        return o["iterations"]

    t0 = time.perf_counter()
    for _ in range(args.warmup):   # the GPU arm's warm-up bench steps, untimed
        route(qlat[:per_step])
    advance_s = time.perf_counter() - t0
    times, iters = [], 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        iters += route(qlat[:per_step])
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = S * per_step * len(times) / tot
    first = args.warmup * per_step
    window = f"routed steps {first}-{first + args.steps * per_step - 1}"
    sample = (f"{label}: {window} ({args.steps} bench steps of {per_step} routed steps, after {first} untimed "
              f"routed steps from the initial state in {advance_s:.0f} s), rtol 1e-8, {nth} threads "
              f"(level-parallel oracle port of cpu_wavefront_fp64; the reference routine is single-threaded)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator, the oracle's restatement)",
            "config": {"workload": f"{args.workload}: FP64 MC secant tree routing of {label}, {R} reaches, "
                                   f"{len(lp) - 1} levels, plain secant start (the reference's), {window}",
                       "segments": S, "reaches": R, "levels": len(lp) - 1, "routed_steps_per_step": per_step,
                       "first_timed_routed_step": first, "threads": nth},
            "solver": {"iterations_per_solve": iters / max(1, S * per_step * len(times))},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port", "sample": sample,
                             "host": host_cpu()},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- our arm
def member_slice(w, k: int = 0):
    """(segment slice, reach slice, inflow columns) of network k of the handle
    (an ensemble member or a basin of the batch) in the handle's user order."""
    if "members" in w:
        S1, R1 = w["topo"]["n_segments"], len(w["topo"]["reach_seg_start"])
        return slice(k * S1, (k + 1) * S1), slice(k * R1, (k + 1) * R1), slice(0, S1)
    if "batch" in w:
        s0 = sum(n["topo"]["n_segments"] for n in w["batch"][:k])
        r0 = sum(len(n["topo"]["reach_seg_start"]) for n in w["batch"][:k])
        n = w["batch"][k]
        S1, R1 = n["topo"]["n_segments"], len(n["topo"]["reach_seg_start"])
        return slice(s0, s0 + S1), slice(r0, r0 + R1), slice(s0, s0 + S1)
    return slice(0, w["S"]), slice(0, w["R"]), slice(0, w["S"])


def network_k(w, k: int = 0):
    """(topo, params, inflow scale or None, label) of network k of the handle."""
    if "members" in w:
        p = w["params"].copy()
        p["n_ch"] *= w["nfac"][k]
        p["ncc"] *= w["nfac"][k]
        m = w["member_range"][0] + k
        return w["topo"], p, w["qfac"][k], f"ensemble member {m} of the"
    if "batch" in w:
        n = w["batch"][k]
        return n["topo"], n["params"], None, f"basin {n['index']} of the batch: the"
    return w["topo"], w["params"], None, "the"


def operating_point_parity(T, w, model, win, after, n_steps: int, qlat_rows) -> dict:
    """Discharge of network 0 of the handle (ensemble member 0, basin 0 or the
    network) after the first `n_steps` routed steps of the timed window,
    routed alone from the window-start state with the start depths recorded,
    against (a) the same network inside the batched launch (`after`: the
    handle's state after those steps, or None) and (b) the oracle replaying
    those solves: correctly rounded powers (bit-identical expected) and the C
    library's pow() (the reference's arithmetic; ulp-sensitive at rtol 1e-8)."""
    from oracle import troute_oracle as O

    ss, rs, cs = member_slice(w, 0)
    topo, params, qs, label = network_k(w, 0)
    Sn = topo["n_segments"]
    cfg = T.make_cfg(**TIGHT, warm_start=1 if model else 0, warm_k=WARM_K, record_start=1 if model else 0)
    if qs is not None:
        net = T.Network.ensemble(topo, w["params"], 1, n_scale=w["nfac"][0], qlat_scale=qs, cfg=cfg)
    else:
        net = T.Network(topo, params, cfg=cfg)
    if model:
        net.set_warm_start(model, WARM_DELTA)
    net.set_state(win[0][ss], win[1][ss], win[3][rs])
    rows = np.ascontiguousarray(qlat_rows[:n_steps, cs])
    net.run(rows)
    q = net.get_state()[0]
    start = net.start_history(n_steps) if model else None
    net.close()
    ql = rows * qs[None, :] if qs is not None else rows
    tol = (TIGHT["rtol"], TIGHT["atol"], TIGHT["maxiter"], TIGHT["attempts"])
    nth = os.cpu_count() or 1
    lp, lr = O.levels_c(topo["reach_up_ptr"], topo["reach_up_idx"], len(topo["reach_seg_start"]))
    out = {"network": f"{label} {Sn}-segment network", "routed_steps": n_steps,
           "window": "the first routed steps of the timed window, from the window-start state",
           "warm_start_replayed": bool(model)}
    for mode, key in ((1, "max_rel_err"), (0, "max_rel_err_libm_pow")):
        with O.pow_mode(mode):
            o = O.route_tree(topo, params, ql, win[0][ss], win[1][ss], win[3][rs], tol=tol, threads=nth,
                             level_ptr=lp, level_reach=lr, warm_start=start, warm_delta=WARM_DELTA if model else 0.0,
                             warm_k=WARM_K if model else 0)
        den = np.maximum(np.abs(o["q"]), 1e-300)
        out[key] = float(np.max(np.where(q == o["q"], 0.0, np.abs(q - o["q"]) / den)))
        if mode == 1:
            out["bit_identical"] = bool(np.array_equal(q, o["q"]))
    out["oracle_pow"] = {"max_rel_err": "correctly rounded R^(2/3), R^(5/3) (the device's)",
                         "max_rel_err_libm_pow": "the C library's pow() (the reference's)"}
    if after is not None:
        out["alone_vs_batched_bit_identical"] = bool(np.array_equal(q, after[ss]))
    return out


def run_ours(args, dist: Dist):
    import torch

    import troute_gb300 as T

    dev = torch.device("cuda", dist.local if dist.world > 1 else 0)
    torch.cuda.set_device(dev)
    share = shard(args.workload, dist)
    w = workload(args.workload, args.n_ts, members=share)
    S, R = w["S"], w["R"]
    n_ts = w["qlat"].shape[0]
    cols = w["qlat"].shape[1]
    stream = torch.cuda.Stream(dev)   # a real stream: 0 would mean "the handle's own stream"
    fp64_rate = T.measure_fp64_rate()  # the FP64 pipe's measured issue rate (roofline peak), untimed
    model = warm_info = plain = None
    if args.warm and "topo" in w and "members" not in w:
        w["warm"] = True
    if w.get("warm"):
        base = w.get("base", "c1") if w["name"] in ("c3", "c4w") or "members" in w else w["name"]
        model, warm_info, plain = train_and_plain(T, torch, dev, stream, plain_steps=2, plain_warmup=1, base=base)
    cfg = T.make_cfg(**TIGHT, warm_start=1 if model else 0, warm_k=WARM_K)
    net = make_network(T, w, cfg)
    if model:
        net.set_warm_start(model, WARM_DELTA)
    net.set_state(w["q0"], w["d0"], w["rl0"])
    qlat_host = torch.empty((n_ts, cols), dtype=torch.float64, pin_memory=True)
    qlat_host.numpy()[:] = w["qlat"]
    qlat_dev = qlat_host.to(dev, non_blocking=False)
    levels = net.n_levels
    tune = None
    shape = {}
    if ("batch" in w or "members" in w) and not args.no_tune:
        # the batched forms pick their launch shape with the autotuner (a trial of
        # a quarter bench step per candidate, from the same state; untimed)
        t0 = time.perf_counter()
        trial = max(1, n_ts // 4)
        tune = net.autotune(qlat_dev.data_ptr(), trial, repeats=1, all_mappings=not model)
        tune["tune_s"] = round(time.perf_counter() - t0, 2)
        tune["trial_steps"] = trial
        shape = dict(mapping=tune["mapping"], blocks_per_sm=tune["blocks_per_sm"],
                     schedule_flags=tune["schedule_flags"],
                     threads_per_block=tune["threads_per_block"] if tune["mapping"] == 1 else 0)
    net.graph_capture(qlat_dev.data_ptr(), n_ts)
    for _ in range(args.warmup):
        net.graph_launch(stream.cuda_stream)
    torch.cuda.synchronize(dev)
    net.sync()
    # state at the start of the timed window (host copies): the e2e leg, the
    # batched plain leg, the parity check and the CPU sample start from it
    win = net.get_state()

    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    sampler = ClockSampler(uuid)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    dist.barrier()
    torch.cuda.synchronize(dev)
    sampler.start()
    time.sleep(0.3)
    e_start = torch.cuda.Event(enable_timing=True)
    e_stop = torch.cuda.Event(enable_timing=True)
    # the NVTX range "timed" lets a profiler capture exactly the timed launches
    # (ncu --nvtx --nvtx-include "timed/")
    nvtx_push("timed")
    e_start.record(stream)
    for k in range(args.steps):
        evs[k][0].record(stream)
        net.graph_launch(stream.cuda_stream)
        evs[k][1].record(stream)
    e_stop.record(stream)
    torch.cuda.synchronize(dev)
    nvtx_pop()
    dist.barrier()
    clocks = sampler.stop()
    stats = net.sync()
    ms_total = dist.max(e_start.elapsed_time(e_stop))
    ms_step = ms_total / args.steps
    kernel_ms = statistics.mean(a.elapsed_time(b) for a, b in evs)
    seg_steps = S * n_ts
    total_seg_steps = dist.sum(seg_steps) if share is not None else seg_steps * dist.world
    value = total_seg_steps * args.steps / (ms_total / 1e3)

    # roofline: the FP64 pipe (the bound) from this run's own solving warp passes,
    # against the measured FP64 issue rate; the HBM fraction beside it
    instr, instr_src = profiled_file("fp64_instr_per_solving_pass", "route_dataflow_instmix_tree200k.md")
    fp64_warp_instr = stats["solve_passes"] * (instr or 0.0)
    achieved = fp64_warp_instr * 32 / (kernel_ms / 1e3) / 1e12
    peak = fp64_rate["warp_instr_per_s"] * 32 / 1e12
    hbm_peak, peak_kind = measured_peak_hbm()
    alg_bytes = BYTES_PER_SEG_STEP * seg_steps
    hbm_achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    tr, tr_src = profiled("dram_bytes_per_seg_step", bool(model))
    roofline = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": (tr * seg_steps if tr is not None else None),
                "definition": "FP64 pipe: solving warp passes of the last timed launch (run statistics) x FP64 warp "
                              "instructions per solving pass x 32 lanes / launch time; peak = the FP64 issue rate "
                              "measured in this run (troute_measure_fp64_rate, independent DMUL chains on every SM) "
                              "x 32 lanes; the solver has no FMA contraction, so an FP64 lane operation is a flop",
                "fp64_instr_per_solving_pass": instr, "instr_source": f"profiles/{instr_src} (ncu instruction mix)",
                "fp64_peak_warp_instr_per_s": fp64_rate["warp_instr_per_s"],
                "traffic_source": f"scaled: DRAM bytes per segment-step of the ncu capture in profiles/{tr_src} x "
                                  f"the segment-steps of one launch (this launch is too large to capture)",
                "hbm": {"achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_achieved / hbm_peak,
                        "alg_bytes_per_seg_step": BYTES_PER_SEG_STEP,
                        "topology_bytes_per_seg_step": topology_bytes_per_seg_step(w),
                        "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                        else "fallback"}}

    # batched plain leg: the same batch and launch shape without the warm start,
    # from the window-start state (splits the headline into batching and learning)
    batched_plain = None
    if model and ("members" in w or "batch" in w) and not args.no_batched_plain:
        net.set_state(win[0], win[1], win[3])
        net.set_cfg(T.make_cfg(**TIGHT, **shape))
        net.graph_capture(qlat_dev.data_ptr(), n_ts)
        k_plain = min(args.steps, 2)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        a.record(stream)
        for _ in range(k_plain):
            net.graph_launch(stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize(dev)
        stp = net.sync()
        bp_ms = dist.max(a.elapsed_time(b))
        batched_plain = {"value": total_seg_steps * k_plain / (bp_ms / 1e3), "unit": UNIT,
                         "workload": f"the same batch and launch shape, plain secant start, the first {k_plain} bench "
                                     f"steps of the timed window from its start state",
                         "iterations_per_solve": stp["iterations"] / max(1, stp["solves"]),
                         "ms_per_step": bp_ms / k_plain}
    net.close()

    e2e = None
    after = None
    if not args.no_e2e:
        # public C-ABI path with host buffers: H2D of the step's lateral inflow
        # from pinned memory inside troute_run, D2H of the routed state into
        # pinned buffers; the same routed steps as the timed window's first bench
        # steps (from the window-start state)
        qh = qlat_host.numpy()
        net2 = make_network(T, w, cfg)
        if model:
            net2.set_warm_start(model, WARM_DELTA)
        if shape:
            net2.set_cfg(T.make_cfg(**TIGHT, warm_start=1 if model else 0, warm_k=WARM_K, **shape))
        # two sets of pinned state buffers, used in turn: the first bench step's
        # discharge stays readable for the parity check without a copy in the loop
        outs = []
        for _ in range(2):
            o = [torch.empty(S, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
            outs.append(o + [torch.empty(R, dtype=torch.float64, pin_memory=True).numpy()])
        e2e_steps = min(args.steps, 2) if ("members" in w or "batch" in w) else args.steps
        net2.set_state(win[0], win[1], win[3])
        torch.cuda.synchronize(dev)
        dist.barrier()
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            net2.run(qh)
            net2.get_state(out=outs[k % 2])
        t1 = time.perf_counter()
        after = outs[0][0]
        dist.barrier()
        e2e_s = dist.max(t1 - t0)
        e2e = {"value": total_seg_steps * e2e_steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(qh.nbytes), "d2h_bytes_per_step": int((3 * S + R) * 8),
               "steps": e2e_steps, "window": "the first bench steps of the timed window, from its start state"}
        net2.close()

    parity = cpu = None
    if dist.rank == 0 and not args.no_parity:
        n_par = min(n_ts, 32)
        parity = operating_point_parity(T, w, model, win, after if n_par == n_ts else None, n_par, w["qlat"])
    if dist.rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, win)
    it = stats["iterations"]
    crit = critical_path_bound(T, w, n_ts, it / max(1, stats["solves"]), clocks.get("sm_mhz"), kernel_ms)
    if share is not None:
        par = (f"{dist.world} ranks, batch sharded without exchange: rank 0 routes "
               + (f"members {share[0]}-{share[1] - 1}" if "members" in w else f"{len(share)} basins"))
        scaling = "strong"
    else:
        par = "replicas" if dist.world > 1 else "single GPU"
        scaling = "weak"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": scaling,
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": f"{args.workload}: FP64 MC secant tree routing ({describe(w)}), "
                                   f"{S} segments, {R} reaches, {levels} levels, {n_ts} steps of "
                                   f"{w['dt']:.0f} s per bench step, rtol 1e-8 atol 1e-10; timed window: routed "
                                   f"steps {args.warmup * n_ts}-{(args.warmup + args.steps) * n_ts - 1}",
                       "segments": S, "reaches": R, "levels": levels, "timesteps_per_step": n_ts,
                       "first_timed_routed_step": args.warmup * n_ts,
                       "l2": f"inputs larger than L2 (129 MB): lateral inflow {w['qlat'].nbytes / 1e9:.2f} GB and "
                             f"segment parameters {S * 96 / 1e9:.2f} GB read per bench step",
                       "parallelism": par, "seeds": seeds_of(w, bool(model))},
            "roofline": roofline, "critical_path": crit, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": (5 if model else 4) * args.steps, "parity": parity,
            "max_rel_err": None if parity is None else parity["max_rel_err"],
            "solver": {"iterations_per_solve": it / max(1, stats["solves"]), "retries": stats["retries"],
                       "early_exits": stats["early_exits"], "warm_used": stats["warm_used"],
                       "warm_fallback_rate": stats["warm_fallback"] / max(1, stats["warm_used"]),
                       "busy_lanes_per_warp_pass": stats["lane_busy"] / max(1, stats["warp_passes"]),
                       "busy_lanes_per_solving_pass": stats["lane_busy"] / max(1, stats["solve_passes"]),
                       "solving_passes_share": stats["solve_passes"] / max(1, stats["warp_passes"]),
                       "solving_warp_passes": stats["solve_passes"]}}
    if tune:
        line["autotune"] = tune
    if model:
        line["warm_model"] = warm_info
        line["plain_single_basin"] = plain
        line["speedup_vs_plain"] = value / plain["value"]
        if batched_plain:
            line["batched_plain"] = batched_plain
            line["speedup_split"] = {"batching": batched_plain["value"] / plain["value"],
                                     "learned_warm_start": value / batched_plain["value"]}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def _event_timed(torch, stream, fn, warmup: int, steps: int):
    """Runs fn() warmup times, then times `steps` calls with CUDA events on
    `stream` (synchronised on both sides); returns ms per call."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def _line(metric, value, unit, args, dist, ms, dtype, workload, extra):
    out = {"metric": metric, "value": value, "unit": unit, "n_gpus": dist.world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded generator)", "config": {"workload": workload}}
    out.update(extra)
    if dist.rank == 0:
        print(json.dumps(out), flush=True)


def run_linear(args, dist: Dist):
    """lin:<network>: the linearised-MC approximate mode (FP32, one persistent
    launch per run) on a single network; one bench step = one run of n_ts steps
    from the carried-over discharge, timed with CUDA events. Reported on its
    own metric line."""
    import torch

    import troute_gb300 as T

    dev = torch.device("cuda", dist.local if dist.world > 1 else 0)
    torch.cuda.set_device(dev)
    w = workload(args.workload.split(":", 1)[1], args.n_ts)
    S, n_ts = w["S"], w["qlat"].shape[0]
    p32 = np.asarray(w["params"].view("<f8").reshape(-1, 8), np.float32)
    coeffs = T.linear_coeffs(p32, w["dt"])
    ql = torch.from_numpy(w["qlat"].astype(np.float32)).to(dev)
    q = torch.from_numpy(w["q0"].astype(np.float32)).to(dev)
    stream = torch.cuda.Stream(dev)   # a real stream (0 would mean the handle's own)
    torch.cuda.synchronize(dev)
    net = T.LinearNetwork(w["topo"], coeffs)
    dist.barrier()
    ms = dist.max(_event_timed(torch, stream, lambda: net.run_device(ql.data_ptr(), n_ts, q.data_ptr(),
                                                                     stream=stream.cuda_stream),
                               args.warmup, args.steps))
    net.close()
    value = S * n_ts * dist.world / (ms / 1e3)
    _line("segment-steps/s, linearised MC (approximate mode, FP32)", value, UNIT, args, dist, ms, "f32",
          f"{args.workload}: {S} segments, {n_ts} steps per bench step (one persistent dataflow launch), "
          f"CUDA-event timed", {"config": {"workload": f"{args.workload}: {S} segments, {n_ts} steps per bench step",
                                          "segments": S, "timesteps_per_step": n_ts}})


def matrix_inputs(name: str, n_ts: int | None):
    """The matrix form's reach-level network from a synthetic tree: reach r
    takes parameter record r and inflow column r (as the reference's main()
    reads its network files), initial discharge 0.1 m3/s."""
    from troute_gb300 import synth

    w = synth.network(name, n_ts=n_ts)
    t = w["topo"]
    R = len(t["reach_seg_start"])
    p32 = np.ascontiguousarray(np.asarray(w["params"].view("<f8").reshape(-1, 8)[:R], np.float32))
    ql = np.ascontiguousarray(w["qlat"][:, :R], np.float32)
    return t["reach_up_ptr"], t["reach_up_idx"], p32, ql, np.full(R, 0.1, np.float32), w["dt"]


def run_matrix(args, dist: Dist):
    """mat:<network>: the matrix-form linear MC (FP32): one bench step = one
    n_ts-step run (a graph of n_ts fused step launches) over the reach-level
    form of the network, timed with CUDA events. HBM roofline: every step
    streams both matrices (8 B per stored entry), their row pointers, the
    step's lateral inflow and writes the discharge."""
    import torch

    import troute_gb300 as T
    from oracle import troute_oracle as O

    dev = torch.device("cuda", dist.local if dist.world > 1 else 0)
    torch.cuda.set_device(dev)
    name = args.workload.split(":", 1)[1]
    up_ptr, up_idx, p32, ql_h, q0, dt = matrix_inputs(name, args.n_ts)
    R, n_ts = len(q0), ql_h.shape[0]
    coeffs = T.matrix_coeffs(p32, dt)
    t0 = time.perf_counter()
    net = T.MatrixNetwork(up_ptr, up_idx, coeffs)
    build_s = time.perf_counter() - t0
    ql = torch.from_numpy(ql_h).to(dev)
    q = torch.from_numpy(q0.copy()).to(dev)
    stream = torch.cuda.Stream(dev)   # a real stream (0 would mean the handle's own)
    torch.cuda.synchronize(dev)
    dist.barrier()
    ms = dist.max(_event_timed(torch, stream, lambda: net.run_device(ql.data_ptr(), n_ts, q.data_ptr(),
                                                                     stream.cuda_stream), args.warmup, args.steps))
    value = R * n_ts * dist.world / (ms / 1e3)
    bytes_step = 8 * (net.nnz_Q + net.nnz_q) + 8 * (R + 1) + 12 * R
    hbm_peak, kind = measured_peak_hbm()
    achieved = bytes_step * n_ts / (ms / 1e3) / 1e9
    # DRAM bytes of one step launch from the ncu capture of mat:c1 (the same
    # workload, small enough to capture whole)
    tr, tr_src = profiled_file("dram_bytes_per_step", "mat_step_c1.md") if name == "c1" else (None, None)
    # parity: 8 steps from the initial discharge against the oracle (the
    # reference kernel's arithmetic on the same matrices), bit for bit
    k = min(8, n_ts)
    qa = torch.from_numpy(q0.copy()).to(dev)
    net.run_device(ql.data_ptr(), k, qa.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    m = net.matrices()
    want = O.matrix_route(m[0], m[1], ql_h[:k], q0)
    got = qa.cpu().numpy()
    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        t0 = time.perf_counter()
        O.matrix_route(m[0], m[1], ql_h[:2], q0)
        el = time.perf_counter() - t0
        cpu = {"value": R * 2 / el, "unit": "reach-steps/s", "cores": 1, "kind": "port",
               "sample": f"2 steps of the {R}-reach network from the initial discharge, single thread (the oracle's "
                         f"restatement of the reference's step on the same matrices; the reference's step runs only "
                         f"on the GPU)", "host": host_cpu()}
    net.close()
    _line("reach-steps/s, matrix-form linear MC (approximate mode, FP32)", value, "reach-steps/s", args, dist, ms,
          "f32", f"{args.workload}", {
              "config": {"workload": f"{args.workload}: reach-level form of the {name} network ({R} reaches, one "
                                     f"routing unit per reach), truncated propagation matrices at tol 1e-7 "
                                     f"(P_Q {net.nnz_Q} entries, P_q {net.nnz_q}), {n_ts} steps per bench step",
                         "reaches": R, "nnz_PQ": net.nnz_Q, "nnz_Pq": net.nnz_q, "timesteps_per_step": n_ts,
                         "build_s": round(build_s, 2),
                         "l2": f"matrices {8 * (net.nnz_Q + net.nnz_q) / 1e6:.0f} MB streamed per step"},
              "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                           "frac": achieved / hbm_peak, "traffic": tr,
                           "traffic_source": (f"profiles/{tr_src}: dram__bytes_read.sum + dram__bytes_write.sum of "
                                              f"one step launch" if tr is not None else None),
                           "alg_bytes_per_step": bytes_step,
                           "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if kind == "measured" else "fallback"},
              "parity": {"steps": k, "bit_identical_to_oracle": bool(np.array_equal(got, want))},
              "cpu_baseline": cpu, "gpu_launches": n_ts * args.steps})


def run_diffusive(args, dist: Dist):
    """diff:<reaches>: the diffusive-wave tridiagonal step on reaches with the
    reference's benchmark distributions (20-99 nodes of at most 500, theta
    0.6, dt 60 s, dx U(100, 600) m, diffusivity U(10, 110), discharge
    U(1, 51)); one bench step = one launch over all reaches, CUDA-event timed.
    HBM roofline: per computational node dx, diffusivity and the previous
    discharge are read and the new discharge written (16 B)."""
    import torch

    import troute_gb300 as T
    from oracle import troute_oracle as O

    dev = torch.device("cuda", dist.local if dist.world > 1 else 0)
    torch.cuda.set_device(dev)
    n = int(args.workload.split(":", 1)[1])
    M = 500
    rng = np.random.default_rng(2027)
    rp = np.zeros(n, T.api.DIFF_REACH_DTYPE)
    rp["ncomp"] = rng.integers(20, 100, n)
    rp["theta"] = 0.6
    rp["dtini"] = 60.0
    dx = rng.uniform(100.0, 600.0, (n, M)).astype(np.float32)
    df = rng.uniform(10.0, 110.0, (n, M)).astype(np.float32)
    qp = rng.uniform(1.0, 51.0, (n, M)).astype(np.float32)
    nodes = int(rp["ncomp"].sum())
    g = {k: torch.from_numpy(v).to(dev) for k, v in (("dx", dx), ("df", df), ("qp", qp))}
    g["rp"] = torch.from_numpy(rp.view(np.uint8)).to(dev)
    out = torch.zeros((n, M), dtype=torch.float32, device=dev)
    scratch = torch.empty(2 * n * M, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)   # a real stream (0 would mean the handle's own)
    torch.cuda.synchronize(dev)
    L = T.lib()

    def step():
        rc = L.troute_diffusive_tridiag_device(g["rp"].data_ptr(), g["dx"].data_ptr(), g["df"].data_ptr(), None,
                                               g["qp"].data_ptr(), out.data_ptr(), n, M, scratch.data_ptr(),
                                               stream.cuda_stream)
        if rc:
            raise RuntimeError(L.troute_last_error())

    dist.barrier()
    ms = dist.max(_event_timed(torch, stream, step, args.warmup, args.steps))
    value = nodes * dist.world / (ms / 1e3)
    hbm_peak, kind = measured_peak_hbm()
    achieved = 16.0 * nodes / (ms / 1e3) / 1e9
    sample = min(n, 2000)
    want = O.diffusive_tridiag(rp[:sample], dx[:sample], df[:sample], qp[:sample])
    got = out.cpu().numpy()[:sample]
    mask = np.arange(M)[None, :] < rp["ncomp"][:sample, None]
    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        t0 = time.perf_counter()
        O.diffusive_tridiag(rp[:sample], dx[:sample], df[:sample], qp[:sample])
        el = time.perf_counter() - t0
        cpu = {"value": int(rp["ncomp"][:sample].sum()) / el, "unit": "node-steps/s", "cores": 1, "kind": "port",
               "sample": f"the first {sample} reaches, single thread (the oracle's restatement of "
                         f"cpu_diffusive_tridiag, bit-identical to it)", "host": host_cpu()}
    _line("node-steps/s, diffusive-wave tridiagonal step (FP32)", value, "node-steps/s", args, dist, ms, "f32",
          args.workload, {
              "config": {"workload": f"{args.workload}: {n} reaches x {M} node slots, {nodes} computational nodes "
                                     f"(20-99 per reach), one launch per bench step", "reaches": n, "nodes": nodes,
                         "l2": f"inputs {3 * n * M * 4 / 1e9:.2f} GB (larger than L2)"},
              "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                           "frac": achieved / hbm_peak, "traffic": None, "alg_bytes_per_node": 16,
                           "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if kind == "measured" else "fallback"},
              "parity": {"reaches_checked": sample, "bit_identical_to_oracle": bool(np.array_equal(got[mask],
                                                                                                  want[mask]))},
              "cpu_baseline": cpu, "gpu_launches": args.steps})


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        elif args.workload.startswith("lin:"):
            run_linear(args, dist)
        elif args.workload.startswith("mat:"):
            run_matrix(args, dist)
        elif args.workload.startswith("diff:"):
            run_diffusive(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
