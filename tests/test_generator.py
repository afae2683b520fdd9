"""Seeded synthetic inputs: determinism, sizes, ranges and tree shape."""
import hashlib

import numpy as np

import troute_gb300 as T
from troute_gb300 import synth


def h(*a):
    m = hashlib.sha256()
    for x in a:
        m.update(np.ascontiguousarray(x).tobytes())
    return m.hexdigest()


def test_deterministic():
    a = synth.network("c0", n_ts=8)
    b = synth.network("c0", n_ts=8)
    assert h(a["params"], a["qlat"], a["topo"]["reach_up_idx"]) == h(b["params"], b["qlat"], b["topo"]["reach_up_idx"])
    c = synth.network("c0", seed=5, n_ts=8)
    assert h(a["params"]) != h(c["params"])


def test_c0_shape():
    c = synth.network("c0")
    t = c["topo"]
    assert t["n_segments"] == 1000 and len(t["reach_seg_start"]) == 199
    assert t["reach_seg_len"].min() >= 1 and t["reach_seg_len"].max() <= 10
    assert c["qlat"].shape == (288, 1000)
    T.validate(t["reach_seg_start"], t["reach_seg_len"], t["reach_up_ptr"], t["reach_up_idx"], t["n_segments"])
    ups = np.diff(t["reach_up_ptr"])
    assert set(np.unique(ups)) <= {0, 2} and (ups == 0).sum() == 100   # binary merge tree, 100 headwaters


def test_parameter_ranges():
    p = synth.make_params(3, 20000)
    assert 500 <= p["dx"].min() and p["dx"].max() <= 5000
    assert 1e-5 <= p["s0"].min() and p["s0"].max() <= 1e-2
    ls = np.log10(p["s0"])   # log-uniform
    assert abs(ls.mean() + 3.5) < 0.05
    assert np.allclose(p["ncc"], 2 * p["n_ch"]) and np.allclose(p["tw"], 3 * p["bw"]) and np.allclose(p["twcc"], 5 * p["tw"])
    assert 0.5 <= p["cs"].min() and p["cs"].max() <= 2.0


def test_lateral_inflow_distribution():
    q = synth.make_qlat(4, 5000, 288)
    assert q.min() > 0
    # Gamma(2, 0.05) mean 0.1 times a diurnal factor of mean 1
    assert abs(q.mean() - 0.1) < 0.003
    day = q.mean(axis=1)
    assert day.max() / day.min() < 1.2   # per-segment phases average the sine out


def test_deep_tree_levels():
    t = synth.make_tree(1001, 20000, 49000)
    lv, lp, lr = T.levels(t["reach_up_ptr"], t["reach_up_idx"])
    # uniform random binary tree: height ~ 2 sqrt(pi n)
    assert 200 < len(lp) - 1 < 2000


def test_member_factors():
    qf, nf = synth.make_member(9, 3, 20000)
    assert abs(np.log(qf).std() - 0.3) < 0.01 and abs(np.log(qf).mean()) < 0.01
    assert 0.8 <= nf.min() and nf.max() <= 1.2


def test_oracle_generator_is_byte_identical():
    """The CPU legs build their inputs with the oracle's restatement of the
    generator (they must not load the product library): every array equals
    the product's, byte for byte, including a multi-threaded inflow matrix."""
    from oracle import troute_oracle as O

    for seed, leaves, segs in ((1000, 100, 1000), (7, 4081, 20000), (1010, 20000, 49000)):
        a, b = synth.make_tree(seed, leaves, segs), O.gen_tree(seed, leaves, segs)
        for k in ("reach_seg_start", "reach_seg_len", "reach_up_ptr", "reach_up_idx"):
            assert a[k].tobytes() == b[k].tobytes(), (seed, k)
        assert synth.make_params(seed, segs).tobytes() == O.gen_params(seed, segs).tobytes()
    for t0 in (0, 96):
        assert synth.make_qlat(11, 30000, 40, t0=t0).tobytes() == O.gen_qlat(11, 30000, 40, t0=t0, threads=4).tobytes()
    for m in (0, 63):
        qa, na = synth.make_member(1004, m, 30000)
        qb, nb = O.gen_member(1004, m, 30000)
        assert qa.tobytes() == qb.tobytes() and na.tobytes() == nb.tobytes()
    for name in ("c0", "tree:20000"):
        a, b = synth.network(name, n_ts=4), O.network(name, n_ts=4)
        assert a["seed"] == b["seed"] and a["params"].tobytes() == b["params"].tobytes()
        assert a["qlat"].tobytes() == b["qlat"].tobytes()
    # the named seeds agree (c1 and c3 themselves are checked on their topology)
    assert (O.C1_SEED, O.C3_SEED) == (synth.C1_SEED, synth.C3_SEED)


def test_oracle_levels_in_c_match_the_reference_rule():
    from oracle import troute_oracle as O

    t = synth.make_tree(5, 3000, 7400)
    R = len(t["reach_seg_start"])
    lp, lr = O.levels(t["reach_up_ptr"], t["reach_up_idx"], R)
    lp2, lr2 = O.levels_c(t["reach_up_ptr"], t["reach_up_idx"], R)
    np.testing.assert_array_equal(lp, lp2)
    np.testing.assert_array_equal(lr, lr2)
    lv, lp3, lr3 = T.levels(t["reach_up_ptr"], t["reach_up_idx"])
    np.testing.assert_array_equal(lp, lp3)
    np.testing.assert_array_equal(lr, lr3)


def test_c1_has_about_3000_levels():
    from oracle import troute_oracle as O

    t = synth.make_tree(synth.C1_SEED, 550_000, 2_700_000)
    lv, lp, lr = T.levels(t["reach_up_ptr"], t["reach_up_idx"])
    assert len(lp) - 1 == 3016 and len(t["reach_seg_start"]) == 1_099_999
    b = O.gen_tree(O.C1_SEED, 550_000, 2_700_000)
    assert b["reach_up_idx"].tobytes() == t["reach_up_idx"].tobytes()
    assert b["reach_seg_len"].tobytes() == t["reach_seg_len"].tobytes()
