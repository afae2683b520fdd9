"""Topology checks and the reference level schedule (host logic, no GPU)."""
import numpy as np
import pytest

import troute_gb300 as T
from oracle import troute_oracle as O
from troute_gb300 import synth


def topo(seg_len, ups):
    seg_len = np.asarray(seg_len, np.int32)
    seg_start = np.concatenate([[0], np.cumsum(seg_len)[:-1]]).astype(np.int32)
    up_ptr = np.concatenate([[0], np.cumsum([len(u) for u in ups])]).astype(np.int32)
    up_idx = np.array([x for u in ups for x in u], np.int32)
    return seg_start, seg_len, up_ptr, up_idx, int(seg_len.sum())


def test_valid_y_network():
    T.validate(*topo([2, 3, 1], [[], [], [0, 1]]))


def test_zero_length_reach_and_empty_network_are_valid():
    T.validate(*topo([2, 0, 1], [[], [], [0, 1]]))
    T.validate(np.zeros(0), np.zeros(0), np.zeros(1), np.zeros(0), 0)


@pytest.mark.parametrize("bad", [
    ([1, 1], [[1], [0]]),            # cycle
    ([1, 1, 1], [[], [0], [0]]),     # reach 0 drains into two reaches
    ([1, 1], [[], [5]]),             # upstream index out of range
    ([1, 1], [[], [1]]),             # self loop
])
def test_invalid_topologies_rejected(bad):
    with pytest.raises(T.TrouteError) as e:
        T.validate(*topo(*bad))
    assert e.value.code == 2


def test_overlapping_segments_rejected():
    s, l, p, i, S = topo([2, 2], [[], [0]])
    s[1] = 1
    with pytest.raises(T.TrouteError):
        T.validate(s, l, p, i, S)


def test_levels_match_reference_construction():
    t = synth.make_tree(11, 500, 2500)
    lv, lp, lr = T.levels(t["reach_up_ptr"], t["reach_up_idx"])
    lp2, lr2 = O.levels(t["reach_up_ptr"], t["reach_up_idx"], len(t["reach_seg_start"]))
    np.testing.assert_array_equal(lp, lp2)
    np.testing.assert_array_equal(lr, lr2)


def _critical_path_brute(topo, n_ts):
    """Longest path in the explicit (reach, step) graph, by memoised recursion
    from every item backwards."""
    import functools

    R = len(topo["reach_seg_start"])
    ups = [list(topo["reach_up_idx"][topo["reach_up_ptr"][r]:topo["reach_up_ptr"][r + 1]]) for r in range(R)]

    @functools.lru_cache(maxsize=None)
    def ending_at(r, t):
        best = 0
        if t > 0:
            best = ending_at(r, t - 1)
        for u in ups[r]:
            best = max(best, ending_at(int(u), t))
        return best + int(topo["reach_seg_len"][r])

    return max((ending_at(r, t) for r in range(R) for t in range(n_ts)), default=0)


def test_critical_path_matches_the_explicit_graph():
    from troute_gb300 import synth

    for seed, S, n_ts in ((1, 300, 1), (2, 500, 5), (3, 800, 12)):
        topo = synth.network(f"tree:{S}", seed=seed, n_ts=1, with_qlat=False)["topo"]
        assert T.critical_path(topo, n_ts) == _critical_path_brute(topo, n_ts)
    c0 = synth.network("c0", n_ts=1, with_qlat=False)["topo"]
    # one step: the most segments on a headwater-to-outlet path; more steps add at least one reach per step
    one = T.critical_path(c0, 1)
    assert one == _critical_path_brute(c0, 1)
    assert T.critical_path(c0, 4) > one and T.critical_path(c0, 0) == 0


def test_critical_path_rejects_bad_topologies():
    bad = {"n_segments": 3, "reach_seg_start": np.array([0, 1, 2], np.int32), "reach_seg_len": np.ones(3, np.int32),
           "reach_up_ptr": np.array([0, 1, 2, 3], np.int32), "reach_up_idx": np.array([2, 0, 1], np.int32)}
    with pytest.raises(T.TrouteError) as e:
        T.critical_path(bad, 4)       # a cycle
    assert e.value.code == 2
    ok = dict(bad, reach_up_ptr=np.array([0, 0, 1, 2], np.int32), reach_up_idx=np.array([0, 1], np.int32))
    assert T.critical_path(ok, 1) == 3 and T.critical_path(ok, 5) == 7   # a 3-reach chain: 3 + 1 per extra step
