"""bench.py's JSON contract where it runs without a GPU: the reference arm
(`--impl reference`, the oracle port of cpu_wavefront_fp64 on the host
threads) prints one line with the metric, the baseline description and a
zero-copy e2e block."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "c0",
                          "--steps", "2", "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
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
    assert b.host_cpu()["nproc"] >= 1
