"""Linearised MC (the reference's approximate mode, water-prediction/t-route/
wavefront/linear_mc.cu) against the reference's own routines and the oracle.

CPU: the oracle's coefficient function and float routing against the
reference's compute_mc_coeffs and cpu_linear_mc compiled from its source (bit
for bit), and against the golden fixture those produced. GPU: the dataflow
kernel against the fixture and the oracle (bit for bit, given the same
coefficients), the device coefficients against the oracle's (CUDA's powf and
the C library's differ in the last bits), chunked runs, and the secant path
as the yardstick of the linear form's error.
"""
import os

import numpy as np
import pytest

import troute_gb300 as T
from golden_inputs import GOLDEN
from oracle import troute_oracle as O
from troute_gb300 import synth

REFNET = os.path.join(GOLDEN, "refnet")


def refnet():
    n = T.read_network(REFNET)
    topo = {k: n[k] for k in ("reach_seg_start", "reach_seg_len", "reach_up_ptr", "reach_up_idx")}
    topo["n_segments"] = n["n_segments"]
    return n, topo


def synthetic(seed=3, segs=20000, n_ts=24):
    c = synth.network(f"tree:{segs}", seed=seed, n_ts=n_ts)
    p32 = np.asarray(c["params"].view("<f8").reshape(-1, 8), np.float32)
    q0 = np.random.default_rng(seed).uniform(0.0, 15.0, c["topo"]["n_segments"]).astype(np.float32)
    return c, p32, c["qlat"].astype(np.float32), q0


def test_oracle_matches_golden_fixture():
    n, topo = refnet()
    g = np.load(os.path.join(GOLDEN, "refnet_out.npz"))
    c = O.linear_coeffs(n["params"], 300.0)
    for k, v in zip(("lin_c1", "lin_c2", "lin_c3", "lin_c4oq"), c):
        np.testing.assert_array_equal(v, g[k])
    q = O.linear_route(c, topo, n["qlat"], n["qdp0"], level_ptr=n["level_ptr"], level_reach=n["level_reach"])
    np.testing.assert_array_equal(q, g["lin_q"])


@pytest.mark.skipif(not O.ref_available(), reason="needs the reference checkout (compiled reference)")
def test_oracle_matches_compiled_reference():
    c, p32, ql, q0 = synthetic()
    co = O.linear_coeffs(p32)
    cr = O.linear_coeffs(p32, use_ref=True)
    for a, b in zip(co, cr):
        np.testing.assert_array_equal(a, b)
    qo = O.linear_route(co, c["topo"], ql, q0)
    qr = O.linear_route(co, c["topo"], ql, q0, use_ref=True)
    np.testing.assert_array_equal(qo, qr)


@pytest.mark.skipif(not O.ref_available(), reason="needs the reference checkout (compiled reference)")
@pytest.mark.parametrize("kind,R", [("chain", 500), ("star", 300), ("single", 1)])
def test_oracle_matches_compiled_reference_on_special_shapes(kind, R):
    """A 500-reach chain (one reach per level), a star whose outlet takes 299
    upstream reaches, a single reach; zero coefficients' segments (invalid
    parameters) mixed in."""
    rng = np.random.default_rng(R + 1)
    if kind == "chain":
        up_ptr, up_idx = [0] + list(range(R)), list(range(R - 1))
    elif kind == "star":
        up_ptr, up_idx = [0] * R + [R - 1], list(range(R - 1))
    else:
        up_ptr, up_idx = [0, 0], []
    seg_len = rng.integers(1, 7, R).astype(np.int32)
    topo = {"n_segments": int(seg_len.sum()), "reach_seg_start": np.concatenate([[0], np.cumsum(seg_len)[:-1]]).astype(np.int32),
            "reach_seg_len": seg_len, "reach_up_ptr": np.array(up_ptr, np.int32), "reach_up_idx": np.array(up_idx, np.int32)}
    S = topo["n_segments"]
    _, p32, _, _ = synthetic(seed=17, segs=3000, n_ts=1)
    p32 = np.ascontiguousarray(p32[rng.integers(0, len(p32), S)])
    p32[rng.random(S) < 0.03, 4] = 0.0   # n_ch = 0
    co = O.linear_coeffs(p32)
    for a, b in zip(co, O.linear_coeffs(p32, use_ref=True)):
        np.testing.assert_array_equal(a, b)
    ql = rng.uniform(0.0, 2.0, (8, S)).astype(np.float32)
    q0 = rng.uniform(0.0, 15.0, S).astype(np.float32)
    np.testing.assert_array_equal(O.linear_route(co, topo, ql, q0), O.linear_route(co, topo, ql, q0, use_ref=True))


@pytest.mark.gpu
def test_gpu_matches_golden_and_oracle_bit_for_bit():
    n, topo = refnet()
    g = np.load(os.path.join(GOLDEN, "refnet_out.npz"))
    coeffs = [g[k] for k in ("lin_c1", "lin_c2", "lin_c3", "lin_c4oq")]
    q = T.linear_route(topo, coeffs, n["qlat"], n["qdp0"])
    np.testing.assert_array_equal(q, g["lin_q"])
    c, p32, ql, q0 = synthetic()
    co = O.linear_coeffs(p32)
    np.testing.assert_array_equal(T.linear_route(c["topo"], co, ql, q0), O.linear_route(co, c["topo"], ql, q0))


@pytest.mark.gpu
def test_device_coefficients_within_float_rounding():
    c, p32, _, _ = synthetic()
    gd = T.linear_coeffs(p32)
    ho = O.linear_coeffs(p32)
    # C1..C4/ql are at most ~1 in magnitude; C2 and C3 cancel (dt/2 - Km X)
    # when Km is near dt, so the bound is absolute at that scale
    for a, b in zip(gd, ho):
        assert np.all(np.abs(a - b) <= 4e-6 * np.maximum(np.abs(b), 1.0))


@pytest.mark.gpu
def test_chunked_device_runs_equal_one_run():
    torch = pytest.importorskip("torch")
    c, p32, ql, q0 = synthetic(seed=5, n_ts=20)
    co = O.linear_coeffs(p32)
    qlat = torch.from_numpy(ql).cuda()
    with T.LinearNetwork(c["topo"], co) as net:
        a = torch.from_numpy(q0.copy()).cuda()
        net.run_device(qlat.data_ptr(), 20, a.data_ptr())
        b = torch.from_numpy(q0.copy()).cuda()
        net.run_device(qlat.data_ptr(), 7, b.data_ptr())
        net.run_device(qlat[7:].contiguous().data_ptr(), 13, b.data_ptr())
    np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
    np.testing.assert_array_equal(a.cpu().numpy(), O.linear_route(co, c["topo"], ql, q0))


@pytest.mark.gpu
def test_linear_form_measured_against_the_secant_path():
    """The secant routing is the yardstick: the linear form's discharge after a
    day of steps, relative to the secant path's on the same inputs, is
    reported and sanity-checked (finite, same total order of magnitude)."""
    c, p32, ql, q0 = synthetic(seed=9, segs=5000, n_ts=48)
    co = T.linear_coeffs(p32)
    ql_lin = ql
    q_lin = T.linear_route(c["topo"], co, ql_lin, q0)
    topo = c["topo"]
    r = T.route_tree(topo, p32.astype(np.float64), ql.astype(np.float64), q0.astype(np.float64),
                     np.full(topo["n_segments"], 0.5), None)
    q_sec = r["q"]
    assert np.isfinite(q_lin).all()
    rel = np.abs(q_lin - q_sec) / np.maximum(np.abs(q_sec), 1e-6)
    total = q_lin.sum() / q_sec.sum()
    print(f"\nlinear vs secant after 48 steps: median rel {np.median(rel):.3f}, p90 {np.quantile(rel, 0.9):.3f}, "
          f"total ratio {total:.3f}")
    assert 0.2 < total < 5.0
