"""bench.py's JSON contract where it runs without a GPU: the reference arm
(`--impl reference`, the oracle port of cpu_wavefront_fp64 on the host
threads) prints one line with the metric, the baseline description and a
zero-copy e2e block, never loads the product library, and times the routed
steps the GPU arm times (after the same warm-up)."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# runs bench.py in this interpreter, then reports which shared objects of the
# repository the process mapped
_WRAP = """
import runpy, sys
sys.argv = ["bench.py"] + sys.argv[1:]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("MAPPED", sorted({ln.split()[-1].rsplit("/", 1)[-1] for ln in maps.splitlines() if ln.endswith(".so")
                        and "libtroute" in ln}))
"""


def test_reference_arm_line():
    out = subprocess.run([sys.executable, "-c", _WRAP, "--impl", "reference", "--workload", "c0", "--n-ts", "8",
                          "--steps", "2", "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = out.stdout.strip().splitlines()
    mapped = lines[-1]
    assert mapped.startswith("MAPPED") and "libtroute_gb300" not in mapped and "libtroute_oracle" in mapped, mapped
    line = json.loads(lines[-2])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 1 and line["higher_is_better"] is True
    assert line["unit"] == "seg-steps/s" and line["dtype"] == "f64"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert cb["host"]["nproc"] >= cb["cores"] and cb["host"]["cpu_model"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # the GPU arm's window: 1 warm-up bench step of 8 routed steps, then 2 timed ones
    cfg = line["config"]
    assert cfg["routed_steps_per_step"] == 8 and cfg["first_timed_routed_step"] == 8
    assert "routed steps 8-23" in cfg["workload"] and cfg["threads"] == cb["cores"]


def _bench_module():
    import importlib.util

    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_line_helpers_of_the_gpu_arm():
    """The parts of the GPU arm's line that run on the host: topology bytes,
    the critical-path bound, the host description, the committed profile
    figures it reads."""
    import troute_gb300 as T

    b = _bench_module()
    for name in ("c0", "ens:3:2000:w"):
        w = b.workload(name, 4)
        tb = b.topology_bytes_per_seg_step(w)
        assert 2.0 < tb < 40.0
        cp = b.critical_path_bound(T, w, 4, 6.5, 2070.0, 100.0)
        assert cp["segment_solves"] == T.critical_path(w["topo"], 4)
        assert cp["passes_per_solve"] == 7.5 and cp["fp64_instr_per_pass"] > 0
        assert abs(cp["lower_bound_ms"] - cp["segment_solves"] * 7.5 * cp["pass_us_min"] / 1e3) < 1e-9
    for warm in (False, True):
        for key in ("dram_bytes_per_seg_step", "fp64_pipe_active_pct"):
            v, src = b.profiled(key, warm)
            assert v is not None and v > 0, (key, src)
    assert b.profiled_file("fp64_instr_per_solving_pass", "route_dataflow_instmix_tree200k.md")[0] > 0
    assert b.host_cpu()["nproc"] >= 1
    # network 0 of an ensemble share: member m0's factors, its slices of the state
    w = b.workload("ens:4:2000:w", 4, members=(2, 4))
    S1, R1 = w["topo"]["n_segments"], len(w["topo"]["reach_seg_start"])
    assert w["members"] == 2 and w["S"] == 2 * S1
    ss, rs, cs = b.member_slice(w, 1)
    assert (ss.start, ss.stop, rs.start, rs.stop, cs.stop) == (S1, 2 * S1, R1, 2 * R1, S1)
    topo, p, qs, label = b.network_k(w, 0)
    from troute_gb300 import synth

    qf, nf = synth.make_member(1004, 2, S1)
    assert "member 2" in label and np.array_equal(qs, qf) and np.array_equal(p["n_ch"], w["params"]["n_ch"] * nf)


def test_shares_of_the_batched_workloads():
    b = _bench_module()

    class D:
        world, rank = 3, 1

    assert b.shard("c4w", D) == (22, 43)
    share = b.shard("c2", D)
    parts = [b.shard("c2", type("D", (), {"world": 3, "rank": r})) for r in range(3)]
    assert share == parts[1] and sorted(i for p in parts for i in p) == list(range(256))
    assert b.shard("c1", D) is None


def test_profiles_carry_the_figures_the_bench_reads():
    """The roofline figures bench.py takes from the committed ncu summaries:
    each file exists, holds its `key: value` line once, and the value is in a
    plausible range (FP64 warp instructions per solving pass, DRAM bytes per
    segment-step of the single-network and ensemble captures, DRAM bytes of
    one matrix step)."""
    sys.path.insert(0, ROOT)
    import bench

    want = {
        ("fp64_instr_per_solving_pass", "route_dataflow_instmix_tree200k.md"): (150.0, 400.0),
        ("dram_bytes_per_seg_step", "route_kernel_c1.md"): (112.0, 2000.0),
        ("dram_bytes_per_seg_step", "route_dataflow_warm_ens256.md"): (112.0, 2000.0),
        ("fp64_pipe_active_pct", "route_dataflow_warm_ens256.md"): (1.0, 100.0),
        ("dram_bytes_per_step", "mat_step_c1.md"): (3.0e8, 4.0e8),
    }
    for (key, name), (lo, hi) in want.items():
        text = open(os.path.join(ROOT, "profiles", name)).read()
        assert sum(ln.strip().startswith(key + ":") for ln in text.splitlines()) == 1, (key, name)
        value, src = bench.profiled_file(key, name)
        assert src == name and value is not None and lo <= value <= hi, (key, name, value)


def test_seeds_are_recorded_for_every_workload_form():
    """The JSON line's config names the generator seeds: the network's (c1 is
    seed 1010, 3,016 levels), the ensemble members' perturbations and the
    warm-start model's."""
    sys.path.insert(0, ROOT)
    import bench

    assert bench.seeds_of(bench.workload("c0", 2)) == {"network": 1000}
    assert bench.seeds_of(bench.workload("c1", 1)) == {"network": 1010}
    assert bench.seeds_of(bench.workload("c3", 1), model=True) == {"network": 2006, "model": 1001}
    assert bench.seeds_of(bench.workload("ens:2:2000:w", 2), model=True) == {"network": 7, "members": 1004,
                                                                             "model": 1001}
    assert bench.seeds_of({"name": "c2"}) == {"basins": 1002}
