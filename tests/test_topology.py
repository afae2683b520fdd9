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
