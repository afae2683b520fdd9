"""GPU parity: the CUDA path through the C ABI against the oracle and the
reference-made golden fixtures.

The solver's powers R^fl(2/3), R^fl(5/3) are correctly rounded on the device
and the rest of its arithmetic is compiled without FMA contraction, so:
  - against the oracle with correctly rounded powers (oracle pow mode 1) the
    GPU is bit-identical: whole multi-step trajectories, every tolerance;
  - against the reference's own routines and the oracle with the C library's
    pow() (which misrounds ~0.1% of these powers by 1 ulp), discharge agrees
    to 1e-10 relative over whole runs at the reference tolerance
    (rtol = atol = 0.01). At rtol = 1e-8 the reference algorithm itself is
    ulp-sensitive over many steps (test_oracle.py::
    test_tight_tolerance_trajectories_are_ulp_sensitive), so there the libm
    comparison is statistical.
"""
import os

import numpy as np
import pytest

import troute_gb300 as T
from golden_inputs import GOLDEN, make_golden
from oracle import troute_oracle as O
from troute_gb300 import synth

pytestmark = pytest.mark.gpu

REL = 1e-10
TIGHT = (1e-8, 1e-10, 100, 5)


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    den = np.maximum(np.abs(b), 1e-300)
    e = np.where((a == b), 0.0, np.abs(a - b) / den)
    return float(e.max()) if e.size else 0.0


def cfg_of(tol, **kw):
    return T.make_cfg(rtol=tol[0], atol=tol[1], maxiter=tol[2], attempts=tol[3], **kw)


# ---------------------------------------------------------------- reach-parallel
def test_reach_parallel_matches_reference_golden():
    p, ql, rs, rl, qu, qd, dp = make_golden.cpu_mc_inputs()
    g = np.load(os.path.join(GOLDEN, "cpu_mc_c0.npz"))
    qo, vo, dpo, st = T.mc_reach_parallel(p, ql, rs, rl, qu, qd, dp, uq=10.0, dt=300.0, return_stats=True)
    assert rel_err(qo, g["qo"]) < REL
    assert rel_err(dpo, g["dpo"]) < REL
    assert rel_err(vo, g["vo"]) < REL
    assert st["solves"] == len(qo) and st["early_exits"] >= 3


def test_reach_parallel_bit_identical_to_oracle():
    p, ql, rs, rl, qu, qd, dp = make_golden.cpu_mc_inputs()
    for tol in (O.REF_TOL, TIGHT):
        with O.pow_mode(1):
            a = O.cpu_mc(p, ql, rs, rl, qu, qd, dp, tol=tol)
        qo, vo, dpo, st = T.mc_reach_parallel(p, ql, rs, rl, qu, qd, dp, cfg=cfg_of(tol), return_stats=True)
        np.testing.assert_array_equal(qo, a[0])
        np.testing.assert_array_equal(vo, a[1])
        np.testing.assert_array_equal(dpo, a[2])
        assert st["iterations"] == a[3]


def test_device_powers_are_correctly_rounded():
    rng = np.random.default_rng(11)
    x = np.concatenate([np.exp(rng.uniform(np.log(1e-6), np.log(1e4), 200000)),
                        [0.0, 1.0, 8.0, 27.0, 0.125, 1e-310, 1e300, 5e-324]])
    o23, o53, c23, c53 = T.debug_pow(x)
    r23 = np.array([O.pow23_53(v, mode=1)[0] for v in x])
    r53 = np.array([O.pow23_53(v, mode=1)[1] for v in x])
    np.testing.assert_array_equal(o23, r23)
    np.testing.assert_array_equal(o53, r53)
    # against CUDA's pow() (documented max error 2 ulp): within 2 ulp everywhere
    ulp = lambda a, b: np.abs(a.view(np.int64) - b.view(np.int64))
    assert ulp(o23, c23).max() <= 2 and ulp(o53, c53).max() <= 2


def test_device_powers_equal_the_oracle_over_200m_arguments():
    """Over 200 M arguments spanning the hydraulic radii the solver meets
    (log-uniform over [1e-4, 1e3]), the device's powers equal the oracle's
    correctly rounded ones bit for bit: the device's rounding test sends every
    argument whose single-precision offset term could tip the rounding to the
    accurate path. (Before that test existed, ~1 argument in 2^21 rounded the
    other way, enough for whole 144-step runs at rtol 1e-8 to drift apart.)"""
    rng = np.random.default_rng(12)
    bad = 0
    for chunk in range(20):
        x = np.exp(rng.uniform(np.log(1e-4), np.log(1e3), 10_000_000))
        o23, o53 = T.debug_pow(x)[:2]
        r23, r53 = O.pow23_53_n(x, mode=1)
        bad += int(np.count_nonzero(o23 != r23) + np.count_nonzero(o53 != r53))
    assert bad == 0


# ---------------------------------------------------------------- tree, reference tolerance
@pytest.mark.parametrize("T_", [1, 24, 288])
def test_wavefront_fp64_dropin_matches_reference_golden(T_):
    topo, p32, ql32, q0, d0, r0 = make_golden.wavefront_inputs()
    g = np.load(os.path.join(GOLDEN, "wavefront_c0.npz"))
    lp, lr = O.levels(topo["reach_up_ptr"], topo["reach_up_idx"], len(topo["reach_seg_start"]))
    q, rl = T.wavefront_fp64(p32, topo["reach_seg_start"], topo["reach_seg_len"], topo["reach_up_ptr"],
                             topo["reach_up_idx"], lp, lr, ql32[:T_], q0, d0, r0, T_, 300.0)
    assert rel_err(q, g[f"q_{T_}"]) < REL
    assert rel_err(rl, g[f"reach_last_{T_}"]) < REL


def test_tree_full_history_matches_oracle_reference_tol():
    c = synth.network("c0")
    args = (c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    o = O.route_tree(*args, history=True)
    g = T.route_tree(*args, history=True)
    for t in range(c["n_ts"]):
        assert rel_err(g["q_hist"][t], o["q_hist"][t]) < REL, t
    assert rel_err(g["d"], o["d"]) < REL and rel_err(g["v"], o["v"]) < REL
    assert rel_err(g["reach_last"], o["reach_last"]) < REL
    assert g["stats"]["iterations"] == o["iterations"]


# ---------------------------------------------------------------- tree, bit-identical
@pytest.mark.parametrize("tol", [O.REF_TOL, TIGHT], ids=["ref_tol", "rtol_1e-8"])
def test_tree_full_history_bit_identical_to_oracle(tol):
    c = synth.network("c0")
    args = (c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    with O.pow_mode(1):
        o = O.route_tree(*args, tol=tol, history=True)
    g = T.route_tree(*args, cfg=cfg_of(tol), history=True)
    np.testing.assert_array_equal(g["q_hist"], o["q_hist"])
    for k in ("q", "d", "v", "reach_last"):
        np.testing.assert_array_equal(g[k], o[k])
    assert g["stats"]["iterations"] == o["iterations"]


def test_tree_tight_tolerance_trajectory_statistics():
    """Whole 288-step run at 1e-8: iteration counts agree within 1% and the
    network outflow agrees closely (the trajectories are ulp-sensitive)."""
    c = synth.network("c0")
    args = (c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    o = O.route_tree(*args, tol=TIGHT)
    g = T.route_tree(*args, cfg=cfg_of(TIGHT))
    assert abs(g["stats"]["iterations"] - o["iterations"]) <= 0.01 * o["iterations"]
    assert abs(g["q"].sum() - o["q"].sum()) <= 1e-3 * o["q"].sum()


# ---------------------------------------------------------------- structure and edge cases
def _topo(seg_len, ups):
    seg_len = np.asarray(seg_len, np.int32)
    return {"n_segments": int(seg_len.sum()),
            "reach_seg_start": (np.cumsum(seg_len) - seg_len).astype(np.int32),
            "reach_seg_len": seg_len,
            "reach_up_ptr": np.concatenate([[0], np.cumsum([len(u) for u in ups])]).astype(np.int32),
            "reach_up_idx": np.array([x for u in ups for x in u], np.int32)}


@pytest.mark.parametrize("case", ["y", "zero_len", "single", "isolated", "wide", "invalid", "dry"])
def test_edge_cases_match_oracle(case):
    rng = np.random.default_rng(3)
    if case == "y":
        topo = _topo([3, 2, 4], [[], [], [0, 1]])
    elif case == "zero_len":
        topo = _topo([2, 0, 3, 1], [[], [], [0, 1], [2]])
    elif case == "single":
        topo = _topo([1], [[]])
    elif case == "isolated":
        topo = _topo([1] * 70, [[]] * 70)
    elif case == "wide":   # one reach with 40 upstream reaches (max fan-in case)
        topo = _topo([1] * 40 + [5], [[]] * 40 + [list(range(40))])
    else:
        topo = _topo([3, 3, 2], [[], [], [0, 1]])
    S = topo["n_segments"]
    params = synth.make_params(77, S)
    qlat = synth.make_qlat(77, S, 12)
    q0 = np.full(S, 0.1)
    d0 = np.full(S, 0.1)
    rl0 = np.full(len(topo["reach_seg_start"]), 0.1)
    if case == "invalid":
        params["n_ch"][1] = 0.0
        params["bw"][4] = -1.0
    if case == "dry":
        qlat[:] = 0.0
        q0[:] = 0.0
        rl0[:] = 0.0
    o = O.route_tree(topo, params, qlat, q0, d0, rl0, history=True)
    g = T.route_tree(topo, params, qlat, q0, d0, rl0, history=True)
    assert rel_err(g["q_hist"], o["q_hist"]) < REL
    assert rel_err(g["d"], o["d"]) < REL and rel_err(g["reach_last"], o["reach_last"]) < REL
    if case == "dry":
        assert not g["q"].any()


def test_zero_steps_and_empty_network():
    c = synth.network("c0", n_ts=1)
    g = T.route_tree(c["topo"], c["params"], c["qlat"][:0], c["q0"], c["d0"], c["rl0"])
    np.testing.assert_array_equal(g["q"], c["q0"])
    with T.Network(_topo([], []), np.zeros((0, 8))) as net:
        assert net.n_reaches == 0
        net.run(np.zeros((3, 0)))


def test_batch_equals_separate_runs():
    nets = [synth.network(f"tree:{S}", seed=s, n_ts=20) for S, s in ((1500, 1), (400, 2), (3000, 3))]
    cols = sum(n["topo"]["n_segments"] for n in nets)
    qlat = np.concatenate([n["qlat"] for n in nets], axis=1)
    with T.Network([n["topo"] for n in nets], [n["params"] for n in nets]) as b:
        assert b.qlat_cols == cols
        b.set_state(np.concatenate([n["q0"] for n in nets]), np.concatenate([n["d0"] for n in nets]),
                    np.concatenate([n["rl0"] for n in nets]))
        b.run(qlat)
        qb, db, vb, rb = b.get_state()
    off = 0
    for n in nets:
        S = n["topo"]["n_segments"]
        s = T.route_tree(n["topo"], n["params"], n["qlat"], n["q0"], n["d0"], n["rl0"])
        np.testing.assert_array_equal(qb[off:off + S], s["q"])
        np.testing.assert_array_equal(db[off:off + S], s["d"])
        off += S


def test_ensemble_column_map_and_scale():
    c = synth.network("tree:2000", seed=4, n_ts=10)
    S = c["topo"]["n_segments"]
    qf, nf = synth.make_member(5, 1, S)
    p1 = c["params"].copy()
    p1["n_ch"] *= nf
    p1["ncc"] *= nf
    with T.Network([c["topo"], c["topo"]], [c["params"], p1], qlat_col=[np.arange(S), np.arange(S)],
                   qlat_scale=[None, qf], qlat_cols=S) as b:
        b.set_state(np.tile(c["q0"], 2), np.tile(c["d0"], 2), np.tile(c["rl0"], 2))
        b.run(c["qlat"])
        qb = b.get_state()[0]
    o0 = O.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    o1 = O.route_tree(c["topo"], p1, c["qlat"] * qf[None, :], c["q0"], c["d0"], c["rl0"])
    assert rel_err(qb[:S], o0["q"]) < REL and rel_err(qb[S:], o1["q"]) < REL


def test_checkpoint_resume_is_bit_identical():
    c = synth.network("c0", n_ts=40)
    with T.Network(c["topo"], c["params"]) as a:
        a.set_state(c["q0"], c["d0"], c["rl0"])
        a.run(c["qlat"][:15])
        blob = a.checkpoint()
        a.run(c["qlat"][15:])
        full = a.get_state()
    with T.Network(c["topo"], c["params"]) as b:
        b.restore(blob)
        assert b.steps_done == 15
        b.run(c["qlat"][15:])
        resumed = b.get_state()
    for x, y in zip(full, resumed):
        np.testing.assert_array_equal(x, y)


def test_launch_shape_does_not_change_results():
    """The schedule (grid size, block shape, reach-to-warp mapping, which lane
    takes which reach, whether a lane continues with an item it made ready)
    is not part of the arithmetic: identical bits for all."""
    c = synth.network("tree:20000", seed=8, n_ts=16)
    args = (c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    ref = None
    for mapping, shapes in ((3, ((0, 0, 0), (128, 1, 0), (128, 2, 1), (0, 0, 1))),
                            (2, ((0, 0, 0), (128, 1, 0))), (1, ((128, 0, 0), (64, 1, 0), (32, 2, 0)))):
        outs = [T.route_tree(*args, cfg=T.make_cfg(mapping=mapping, threads_per_block=tpb, blocks_per_sm=bps,
                                                   schedule_flags=fl))["q"]
                for tpb, bps, fl in shapes]
        if ref is None:
            ref = outs[0]
        for x in outs:
            np.testing.assert_array_equal(x, ref)


def test_bounded_wait_times_out_cleanly():
    assert T.timeout_probe(200_000) == 5   # TROUTE_ETIMEOUT
    c = synth.network("c0", n_ts=3)        # context still usable
    g = T.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    o = O.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    assert rel_err(g["q"], o["q"]) < REL


def test_tiny_wait_budget_reports_timeout_or_completes():
    """With a wait budget of a few cycles the run either finishes (no wait was
    needed) or returns TROUTE_ETIMEOUT; it never hangs, and the handle
    refuses further runs until its state is reset."""
    c = synth.network("tree:50000", seed=9, n_ts=8)
    with T.Network(c["topo"], c["params"], cfg=T.make_cfg(wait_cycles=1)) as net:
        net.set_state(c["q0"], c["d0"], c["rl0"])
        try:
            net.run(c["qlat"])
        except T.TrouteError as e:
            assert e.code == 5
            with pytest.raises(T.TrouteError) as e2:
                net.run(c["qlat"])
            assert e2.value.code == 8
            net.set_state(c["q0"], c["d0"], c["rl0"])
            net.set_cfg(T.make_cfg())
            net.run(c["qlat"])


def test_ensemble_members_bit_identical_to_single_runs():
    c = synth.network("c0", n_ts=30)
    S = c["topo"]["n_segments"]
    M = 3
    nf = np.stack([synth.make_member(21, m, S)[1] for m in range(M)])
    qf = np.stack([synth.make_member(21, m, S)[0] for m in range(M)])
    cfg = cfg_of(TIGHT)
    with T.Network.ensemble(c["topo"], c["params"], M, n_scale=nf, qlat_scale=qf, cfg=cfg) as net:
        assert net.n_segments == M * S and net.qlat_cols == S
        net.set_state(np.tile(c["q0"], M), np.tile(c["d0"], M), np.tile(c["rl0"], M))
        net.run(c["qlat"])
        q, d, v, rl = net.get_state()
    R = len(c["topo"]["reach_seg_start"])
    for m in range(M):
        p = c["params"].copy()
        p["n_ch"] *= nf[m]
        p["ncc"] *= nf[m]
        with O.pow_mode(1):
            o = O.route_tree(c["topo"], p, c["qlat"] * qf[m][None, :], c["q0"], c["d0"], c["rl0"], tol=TIGHT)
        np.testing.assert_array_equal(q[m * S:(m + 1) * S], o["q"])
        np.testing.assert_array_equal(d[m * S:(m + 1) * S], o["d"])
        np.testing.assert_array_equal(v[m * S:(m + 1) * S], o["v"])
        np.testing.assert_array_equal(rl[m * R:(m + 1) * R], o["reach_last"])


@pytest.mark.parametrize("mapping", [3, 2, 1])
def test_chunked_run_equals_single_launch(mapping):
    c = synth.network("tree:5000", seed=12, n_ts=40)
    args = (c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    a = T.route_tree(*args, cfg=T.make_cfg(mapping=mapping), history=True)
    b = T.route_tree(*args, cfg=T.make_cfg(mapping=mapping, max_chunk_steps=7), history=True)
    for k in ("q", "d", "v", "reach_last", "q_hist"):
        np.testing.assert_array_equal(a[k], b[k])
    assert a["stats"]["iterations"] == b["stats"]["iterations"]


def test_graph_replay_equals_runs():
    torch = pytest.importorskip("torch")
    c = synth.network("tree:5000", seed=13, n_ts=10)
    ql = torch.from_numpy(np.ascontiguousarray(c["qlat"])).cuda()
    with T.Network(c["topo"], c["params"], cfg=T.make_cfg(max_chunk_steps=4)) as g:
        g.set_state(c["q0"], c["d0"], c["rl0"])
        g.graph_capture(ql.data_ptr(), 10)
        g.graph_launch()
        g.graph_launch()
        g.sync()
        assert g.steps_done == 20
        qg = g.get_state()
    with T.Network(c["topo"], c["params"]) as r:
        r.set_state(c["q0"], c["d0"], c["rl0"])
        r.run(c["qlat"])
        r.run(c["qlat"])
        qr = r.get_state()
    for x, y in zip(qg, qr):
        np.testing.assert_array_equal(x, y)


def test_autotuner_keeps_state_and_results():
    """The tuner times every candidate shape from the same saved state, keeps
    the fastest, leaves the routing state as it was, and the tuned handle
    routes bit-identically to an untuned one."""
    torch = pytest.importorskip("torch")
    c = synth.network("tree:20000", seed=21, n_ts=8)
    ql = torch.from_numpy(np.ascontiguousarray(c["qlat"])).cuda()
    cfg = cfg_of(TIGHT)
    with T.Network(c["topo"], c["params"], cfg=cfg) as a:
        a.set_state(c["q0"], c["d0"], c["rl0"])
        a.run(c["qlat"][:3])
        before = a.get_state()
        res = a.autotune(ql.data_ptr(), 8, repeats=1, all_mappings=True)
        after = a.get_state()
        for x, y in zip(before, after):
            np.testing.assert_array_equal(x, y)
        assert a.steps_done == 3
        assert len(res["trials"]) >= 6
        assert all(t["ms"] > 0 for t in res["trials"])
        assert {t["mapping"] for t in res["trials"]} == {1, 2, 3}
        assert res["best_ms"] == min(t["ms"] for t in res["trials"])
        a.run(c["qlat"])
        qa = a.get_state()
    with T.Network(c["topo"], c["params"], cfg=cfg) as b:
        b.set_state(c["q0"], c["d0"], c["rl0"])
        b.run(c["qlat"][:3])
        b.run(c["qlat"])
        qb = b.get_state()
    for x, y in zip(qa, qb):
        np.testing.assert_array_equal(x, y)


def test_convergence_comparison_matches_ieee_quotient():
    """The secant pass's stop test compares |h_1 - h| / h with rtol through an
    FMA residual instead of dividing; it must give the IEEE quotient's answer
    for every operand: quotients within a few ulps of rtol and of the rounding
    midpoint above it, random operands over the whole range, subnormal,
    infinite, zero and NaN operands, several rtol values."""
    rng = np.random.default_rng(31)
    for c in (1e-8, 0.01, 1e-6, 0.3, 2.0 ** -30, np.nextafter(1e-8, 1.0)):
        n = 400_000
        b = np.exp(rng.uniform(np.log(1e-4), np.log(1e4), n))
        a0 = b * c
        steps = rng.integers(-6, 7, n)
        a = a0.copy()
        for j in range(1, 7):
            a = np.where(steps >= j, np.nextafter(a, np.inf), a)
            a = np.where(steps <= -j, np.nextafter(a, -np.inf), a)
        # random magnitudes over the whole range
        a2 = np.ldexp(rng.uniform(1, 2, n), rng.integers(-1074, 1024, n))
        b2 = np.ldexp(rng.uniform(1, 2, n), rng.integers(-1074, 1024, n))
        special = np.array([0.0, np.inf, np.nan, 5e-324, 1e-310, 1e308, 1.0, c])
        a3 = np.repeat(special, 4)
        b3 = np.tile(np.array([5e-324, 1e-310, 1.0, 1e308]), special.size)
        A = np.concatenate([a, a2, a3])
        B = np.concatenate([b, b2, b3])
        with np.errstate(all="ignore"):
            ref = (A / B) > c
        got = T.debug_quot_gt(A, B, c)
        bad = got != ref
        assert not bad.any(), (c, A[bad][:5], B[bad][:5])
        assert 0.2 < ref[:n].mean() < 0.8  # the first set straddles c


def test_shared_reciprocal_division_is_ieee():
    """The solver's quotients that share one reciprocal (Markstein's
    correction) equal IEEE division bit for bit: random operands over the
    whole exponent range (the far ranges take the IEEE path), significands of
    all ones and powers of two, the solver's own operand ranges, zeros,
    infinities and NaNs."""
    rng = np.random.default_rng(23)
    n = 2_000_000
    a = np.ldexp(rng.uniform(1, 2, n), rng.integers(-1070, 1024, n)) * rng.choice([-1, 1], n)
    b = np.ldexp(rng.uniform(1, 2, n), rng.integers(-1070, 1024, n)) * rng.choice([-1, 1], n)
    # the coefficient divisions of the solver: numerators up to ~1e6, denominators 150..1e9
    a2 = rng.uniform(-1e6, 1e6, n)
    b2 = np.exp(rng.uniform(np.log(150.0), np.log(1e9), n))
    allones = np.ldexp(2.0 - np.ldexp(1.0, -52), rng.integers(-60, 60, 200000))
    pow2 = np.ldexp(1.0, rng.integers(-60, 60, 200000))
    a3 = np.concatenate([allones, pow2, rng.uniform(1, 2, 200000), allones])
    b3 = np.concatenate([rng.uniform(1, 2, 200000), allones, allones, pow2])
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, 5e-324, 1e308])
    a4 = np.repeat(special, special.size)
    b4 = np.tile(special, special.size)
    A = np.concatenate([a, a2, a3, a4])
    B = np.concatenate([b, b2, b3, b4])
    with np.errstate(all="ignore"):
        ref = A / B
    got = T.debug_div(A, B)
    same = (got.view(np.int64) == ref.view(np.int64)) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), (A[~same][:5], B[~same][:5], got[~same][:5], ref[~same][:5])
