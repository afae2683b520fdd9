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
