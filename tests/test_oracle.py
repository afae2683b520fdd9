"""The CPU oracle against the reference: golden fixtures made by the
reference's own compiled routines, and (where the reference checkout exists)
the compiled reference itself on fresh inputs."""
import os

import numpy as np
import pytest

from golden_inputs import GOLDEN, make_golden
from oracle import troute_oracle as O


def test_cpu_mc_matches_golden():
    p, ql, rs, rl, qu, qd, dp = make_golden.cpu_mc_inputs()
    g = np.load(os.path.join(GOLDEN, "cpu_mc_c0.npz"))
    assert make_golden.sha(p, ql, rs, rl, qu, qd, dp) == str(g["input_sha"])
    qo, vo, dpo, _ = O.cpu_mc(p, ql, rs, rl, qu, qd, dp, uq=10.0, dt=300.0)
    np.testing.assert_array_equal(qo, g["qo"])
    np.testing.assert_array_equal(vo, g["vo"])
    np.testing.assert_array_equal(dpo, g["dpo"])
    # edge cases really were exercised: invalid parameters give zeros
    for s in (5, 17, 23):
        assert qo[s] == 0.0 and vo[s] == 0.0 and dpo[s] == 0.0


@pytest.mark.parametrize("T", [1, 24, 288])
def test_wavefront_matches_golden(T):
    topo, p32, ql32, q0, d0, r0 = make_golden.wavefront_inputs()
    g = np.load(os.path.join(GOLDEN, "wavefront_c0.npz"))
    assert make_golden.sha(topo["reach_seg_start"], topo["reach_seg_len"], topo["reach_up_ptr"],
                           topo["reach_up_idx"], p32, ql32, q0, d0, r0) == str(g["input_sha"])
    o = O.route_tree(topo, p32.astype(np.float64), ql32[:T].astype(np.float64), q0.astype(np.float64),
                     d0.astype(np.float64), r0.astype(np.float64))
    np.testing.assert_array_equal(o["q"], g[f"q_{T}"])
    np.testing.assert_array_equal(o["reach_last"], g[f"reach_last_{T}"])


def _reference_gen(seed, nr):
    """Inputs shaped like the reference's own gen() (troute_mc_final.cu:254-274)."""
    rng = np.random.default_rng(seed)
    rl = rng.integers(1, 21, nr).astype(np.int32)
    rs = np.concatenate([[0], np.cumsum(rl)[:-1]]).astype(np.int32)
    S = int(rl.sum())
    p = np.zeros((S, 8))
    p[:, 0] = 500.0 + rng.integers(0, 5000, S)
    p[:, 1] = 5.0 + rng.integers(0, 50, S)
    p[:, 2] = p[:, 1] + rng.integers(0, 20, S)
    p[:, 3] = p[:, 2] + rng.integers(0, 100, S)
    p[:, 4] = 0.02 + 0.06 * rng.random(S)
    p[:, 5] = p[:, 4] * 1.5
    p[:, 6] = 0.5 + 2.0 * rng.random(S)
    p[:, 7] = 0.0001 + 0.005 * rng.random(S)
    ql = 0.5 * rng.random(S)
    bq = 5.0 + 50.0 * rng.random(S)
    return p, ql, rs, rl, bq * 0.95, bq, 0.5 + 3.0 * rng.random(S)


@pytest.mark.skipif(not O.ref_available(), reason="reference checkout not present")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_cpu_mc_matches_compiled_reference(seed):
    p, ql, rs, rl, qu, qd, dp = _reference_gen(seed, 400)
    a = O.cpu_mc(p, ql, rs, rl, qu, qd, dp, uq=10.0, dt=300.0)
    b = O.ref_cpu_mc(p, ql, rs, rl, qu, qd, dp, uq=10.0, dt=300.0)
    for x, y in zip(a[:3], b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.skipif(not O.ref_available(), reason="reference checkout not present")
def test_wavefront_matches_compiled_reference_other_seed():
    from troute_gb300 import synth

    c = synth.network("tree:3000", seed=99, n_ts=12)
    p32 = np.asarray(c["params"].view("<f8").reshape(-1, 8), np.float32)
    ql32 = c["qlat"].astype(np.float32)
    q0 = np.random.default_rng(5).uniform(0.0, 15.0, c["topo"]["n_segments"]).astype(np.float32)
    d0 = np.random.default_rng(6).uniform(0.3, 3.0, c["topo"]["n_segments"]).astype(np.float32)
    r0 = np.random.default_rng(7).uniform(0.0, 10.0, len(c["topo"]["reach_seg_start"])).astype(np.float32)
    qr, rlr = O.ref_wavefront_fp64(c["topo"], p32, ql32, q0, d0, r0)
    o = O.route_tree(c["topo"], p32.astype(np.float64), ql32.astype(np.float64), q0.astype(np.float64),
                     d0.astype(np.float64), r0.astype(np.float64))
    np.testing.assert_array_equal(o["q"], qr)
    np.testing.assert_array_equal(o["reach_last"], rlr)


def _special_topo(kind, R, rng):
    """Reach topologies the random trees rarely produce: a chain (reach r
    drains r - 1), a star (every other reach drains into the last), a single
    reach; 1-6 segments per reach."""
    if kind == "chain":
        up_ptr, up_idx = [0] + list(range(R)), list(range(R - 1))
    elif kind == "star":
        up_ptr, up_idx = [0] * R + [R - 1], list(range(R - 1))
    else:
        R, up_ptr, up_idx = 1, [0, 0], []
    seg_len = rng.integers(1, 7, R).astype(np.int32)
    seg_start = np.concatenate([[0], np.cumsum(seg_len)[:-1]]).astype(np.int32)
    return {"n_segments": int(seg_len.sum()), "reach_seg_start": seg_start, "reach_seg_len": seg_len,
            "reach_up_ptr": np.array(up_ptr, np.int32), "reach_up_idx": np.array(up_idx or [0], np.int32)[:len(up_idx)]}


@pytest.mark.skipif(not O.ref_available(), reason="reference checkout not present")
@pytest.mark.parametrize("kind,R", [("chain", 400), ("star", 300), ("single", 1)])
def test_wavefront_matches_compiled_reference_on_special_shapes(kind, R):
    """A 400-reach chain (a critical path as long as the network), a star
    whose outlet sums 299 upstream outflows, a single reach; with dry
    segments (zero inflow and state) and segments of invalid parameters
    (the reference's early exits) mixed in."""
    from troute_gb300 import synth

    rng = np.random.default_rng(R)
    t = _special_topo(kind, R, rng)
    S = t["n_segments"]
    base = synth.network("tree:3000", seed=98, n_ts=2)
    p32 = np.asarray(base["params"].view("<f8").reshape(-1, 8), np.float32)
    p32 = np.ascontiguousarray(p32[rng.integers(0, len(p32), S)])
    p32[rng.random(S) < 0.03, 4] = 0.0           # n_ch = 0: invalid parameters, an early exit
    T = 10
    ql32 = rng.uniform(0.0, 3.0, (T, S)).astype(np.float32)
    q0 = rng.uniform(0.0, 15.0, S).astype(np.float32)
    d0 = rng.uniform(0.3, 3.0, S).astype(np.float32)
    dry = rng.random(S) < 0.05                     # no flow at all: the other early exit
    ql32[:, dry] = 0.0
    q0[dry] = 0.0
    r0 = rng.uniform(0.0, 10.0, len(t["reach_seg_len"])).astype(np.float32)
    qr, rlr = O.ref_wavefront_fp64(t, p32, ql32, q0, d0, r0)
    o = O.route_tree(t, p32.astype(np.float64), ql32.astype(np.float64), q0.astype(np.float64),
                     d0.astype(np.float64), r0.astype(np.float64))
    np.testing.assert_array_equal(o["q"], qr)
    np.testing.assert_array_equal(o["reach_last"], rlr)


def test_threaded_oracle_identical():
    from troute_gb300 import synth

    c = synth.network("c0", n_ts=48)
    a = O.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"], threads=1)
    b = O.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"], threads=3)
    for k in ("q", "d", "v", "reach_last"):
        np.testing.assert_array_equal(a[k], b[k])
    assert a["iterations"] == b["iterations"]


def test_tolerance_parameter():
    """At the reference tolerance the parameterised loop is the reference's;
    a tighter tolerance runs more iterations, and one step from a common state
    at 1e-8 and at 1e-10 agrees to well below 1e-6."""
    from troute_gb300 import synth

    c = synth.network("c0", n_ts=24)
    args = (c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    a = O.route_tree(*args, tol=(0.01, 0.01, 100, 5))
    b = O.route_tree(*args, tol=(1e-8, 1e-10, 100, 5))
    assert b["iterations"] > a["iterations"]
    # single segment solves (no chaining): the iteration's limit is reached
    p = c["params"]
    rel = []
    for s in range(0, 1000, 7):
        a8 = O.mc_solve(300.0, 0.3, 0.35, 0.1, c["qlat"][0, s], p[s:s + 1], 0.1, tol=(1e-8, 1e-10, 100, 5))
        a10 = O.mc_solve(300.0, 0.3, 0.35, 0.1, c["qlat"][0, s], p[s:s + 1], 0.1, tol=(1e-10, 1e-12, 100, 5))
        assert a10[3] >= a8[3]
        if a10[3] <= 100:   # a tighter run that exhausts maxiter restarts from a wider bracket
            rel.append(abs(a8[0] - a10[0]) / abs(a10[0]))
    assert len(rel) > 100 and max(rel) < 1e-6


def test_tight_tolerance_trajectories_are_ulp_sensitive():
    """Property of the reference algorithm that sets how multi-step parity is
    tested: its two secant residuals use different X clamps (troute_mc_final.cu
    :86 vs :105), so the iteration converges linearly to a point that depends
    on the starting bracket, i.e. on the previous depth. At rtol = 1e-8 a 1-ulp
    change of one step's lateral inflow grows to >1e-4 over the run; at the
    reference tolerance it stays below 1e-10."""
    from troute_gb300 import synth

    c = synth.network("c0", n_ts=96)
    ql2 = c["qlat"].copy()
    ql2[0] = np.nextafter(ql2[0], np.inf)
    for tol, lo, hi in (((1e-8, 1e-10, 100, 5), 1e-4, 1.0), ((0.01, 0.01, 100, 5), 0.0, 1e-10)):
        a = O.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"], tol=tol)
        b = O.route_tree(c["topo"], c["params"], ql2, c["q0"], c["d0"], c["rl0"], tol=tol)
        rel = (np.abs(a["q"] - b["q"]) / np.maximum(np.abs(a["q"]), 1e-300)).max()
        assert lo <= rel < hi, (tol, rel)


def test_planted_mistake_is_caught():
    """A deliberately wrong oracle run (lateral inflow scaled by 1 + 1e-9)
    must fail the 1e-10 discharge parity bar used by the GPU tests."""
    from troute_gb300 import synth

    c = synth.network("c0", n_ts=24)
    a = O.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"], tol=(1e-8, 1e-10, 100, 5))
    b = O.route_tree(c["topo"], c["params"], c["qlat"] * (1 + 1e-9), c["q0"], c["d0"], c["rl0"],
                     tol=(1e-8, 1e-10, 100, 5))
    rel = np.abs(a["q"] - b["q"]) / np.maximum(np.abs(a["q"]), 1e-300)
    assert rel.max() > 1e-10


def test_correctly_rounded_powers_against_libm_and_mpmath():
    """Pow mode 1 gives the correctly rounded R^fl(2/3), R^fl(5/3); the C
    library's pow() agrees except for rare 1-ulp misroundings."""
    rng = np.random.default_rng(3)
    xs = np.exp(rng.uniform(np.log(1e-4), np.log(1e3), 20000))
    a = np.array([O.pow23_53(x, 0) for x in xs])
    b = np.array([O.pow23_53(x, 1) for x in xs])
    ulp = np.abs(a.view(np.int64) - b.view(np.int64))
    assert ulp.max() <= 1 and (ulp > 0).mean() < 0.005
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    e2, e5 = mpmath.mpf(2.0 / 3.0), mpmath.mpf(5.0 / 3.0)
    for x, (p23, p53) in zip(xs[:2000], b[:2000]):
        assert p23 == float(mpmath.mpf(x) ** e2) and p53 == float(mpmath.mpf(x) ** e5)


def test_pow_mode_changes_nothing_at_reference_tolerance():
    """The correctly rounded powers change whole 288-step runs at the
    reference tolerance by far less than the 1e-10 parity bar."""
    from troute_gb300 import synth

    c = synth.network("c0")
    args = (c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    a = O.route_tree(*args, history=True)
    with O.pow_mode(1):
        b = O.route_tree(*args, history=True)
    rel = np.abs(a["q_hist"] - b["q_hist"]) / np.maximum(np.abs(a["q_hist"]), 1e-300)
    assert rel.max() < 1e-10


def test_warm_started_oracle_semantics():
    """The oracle's warm-started solve (the restatement the GPU's warm runs
    are replayed against): no learned depth (0) is the plain solve exactly.
    Starting from the plain run's own converged depths, a 5 % bracket takes
    fewer secant iterations than the plain start, but a 0.2 % bracket takes
    more: the reference's two residuals use different X clamps, so a bracket
    too narrow for their offset sends the secant away (and into fallbacks)."""
    from troute_gb300 import synth

    c = synth.network("tree:3000", seed=21, n_ts=6)
    args = (c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    tight = (1e-8, 1e-10, 100, 5)
    plain = O.route_tree(*args, tol=tight, depth_history=True)
    S = c["topo"]["n_segments"]
    zero = O.route_tree(*args, tol=tight, warm_start=np.zeros((6, S)), warm_delta=0.05, warm_k=16)
    np.testing.assert_array_equal(zero["q"], plain["q"])
    assert zero["iterations"] == plain["iterations"] and zero["warm_used"] == 0
    wide = O.route_tree(*args, tol=tight, warm_start=plain["d_hist"], warm_delta=0.05, warm_k=16)
    narrow = O.route_tree(*args, tol=tight, warm_start=plain["d_hist"], warm_delta=0.002, warm_k=16)
    for w in (wide, narrow):
        assert w["warm_used"] == S * 6 and 0 < w["warm_fallback"] < w["warm_used"]
    assert wide["iterations"] < 0.9 * plain["iterations"] < narrow["iterations"]
    assert narrow["warm_fallback"] > wide["warm_fallback"]
