"""Matrix-form linearised MC (the reference's water-prediction/t-route/
wavefront/linear_mc_matrix.cu, fused step of linear_mc_matrix_graph.cu)
against the reference's own functions, the golden fixture and the oracle.

CPU: the oracle's coefficients and truncated propagation matrices against the
reference's compute_mc_coeffs_cpu and build_propagation_matrices compiled
from its source (bit for bit) and against the fixture those produced on the
reference's own network; the oracle's step, as a check independent of its
restatement of the reference kernel's summation, against the reference's own
cpu_linear_mc on one-segment-per-reach networks given the same coefficients
(the two forms differ only by the dropped entries and float rounding).
GPU: the library's matrices (host build) and routed discharge (fused step
kernel, odd and even step counts, graph replays) bit for bit against the
fixture and the oracle; device coefficients within float rounding of the C
library's; the matrix form measured against the secant path.
"""
import os

import numpy as np
import pytest

import troute_gb300 as T
from golden_inputs import GOLDEN
from oracle import troute_oracle as O
from troute_gb300 import synth


def fixture():
    return np.load(os.path.join(GOLDEN, "matrix_ref.npz"))


def fixture_setup():
    n = T.read_network(os.path.join(GOLDEN, "refnet"))
    return n["reach_up_ptr"], n["reach_up_idx"], n["params"]


def reach_level(segs=20000, seed=3, n_ts=8):
    """A reach-level network (one routing unit per reach) from the synthetic
    tree: reach r gets parameter record r and inflow column r, as the
    reference's main() reads its files."""
    c = synth.network(f"tree:{segs}", seed=seed, n_ts=n_ts)
    t = c["topo"]
    R = len(t["reach_seg_start"])
    p32 = np.asarray(c["params"].view("<f8").reshape(-1, 8)[:R], np.float32)
    ql = np.ascontiguousarray(c["qlat"][:, :R], np.float32)
    q0 = np.random.default_rng(seed).uniform(0.05, 20.0, R).astype(np.float32)
    return t["reach_up_ptr"], t["reach_up_idx"], p32, ql, q0


def assert_same_matrices(a, b):
    for m, n in zip(a, b):
        for x, y in zip(m, n):
            np.testing.assert_array_equal(x, y)


def test_oracle_matches_golden_fixture():
    g = fixture()
    up_ptr, up_idx, params = fixture_setup()
    R = len(up_ptr) - 1
    c = O.matrix_coeffs(params[:R], 300.0)
    for k, v in zip(("c1", "c2", "c3", "c4oq"), c):
        np.testing.assert_array_equal(v, g[k])
    m = O.matrix_build(up_ptr, up_idx, c, 1e-7)
    assert_same_matrices(m, ((g["PQ_ptr"], g["PQ_col"], g["PQ_val"]), (g["Pq_ptr"], g["Pq_col"], g["Pq_val"])))
    np.testing.assert_array_equal(O.matrix_route(m[0], m[1], g["qlat"], g["q0"]), g["q_final"])


@pytest.mark.skipif(not O.ref_available(), reason="needs the reference checkout (compiled reference)")
@pytest.mark.parametrize("segs,seed,tol", [(20000, 3, 1e-7), (60000, 4, 1e-7), (20000, 5, 1e-4), (3000, 6, 0.0)])
def test_oracle_matches_compiled_reference(segs, seed, tol):
    up_ptr, up_idx, p32, _, _ = reach_level(segs, seed)
    co = O.matrix_coeffs(p32)
    cr = O.matrix_coeffs(p32, use_ref=True)
    for a, b in zip(co, cr):
        np.testing.assert_array_equal(a, b)
    assert_same_matrices(O.matrix_build(up_ptr, up_idx, co, tol), O.matrix_build(up_ptr, up_idx, co, tol, use_ref=True))


def _shape(kind, R):
    """Upstream CSR of special networks: a chain (reach r drains r - 1), a star
    (every other reach drains into the last one), a binary comb."""
    if kind == "chain":
        return np.array([0] + list(range(R)), np.int32), np.arange(R - 1, dtype=np.int32)
    if kind == "star":
        return np.array([0] * R + [R - 1], np.int32), np.arange(R - 1, dtype=np.int32)
    if kind == "comb":   # reach r (odd) drains a headwater r - 1 and the previous spine reach r - 2
        ups, ptr = [], [0]
        for r in range(R):
            if r % 2 == 1:
                ups += [r - 1] + ([r - 2] if r >= 3 else [])
            ptr.append(len(ups))
        return np.array(ptr, np.int32), np.array(ups, np.int32)
    raise ValueError(kind)


@pytest.mark.skipif(not O.ref_available(), reason="needs the reference checkout (compiled reference)")
@pytest.mark.parametrize("kind,R,tol", [("chain", 3000, 1e-7), ("chain", 200, 0.0), ("star", 2000, 1e-7),
                                        ("comb", 4001, 1e-7), ("chain", 1, 1e-7)])
def test_oracle_matches_compiled_reference_on_special_shapes(kind, R, tol):
    """Long rows (a chain accumulates its whole truncated ancestry; with tol 0
    nothing is dropped), one very wide row (a star), a single reach: the
    oracle's build and routing against the reference's build_propagation_matrices."""
    up_ptr, up_idx = _shape(kind, R)
    _, _, p32, _, _ = reach_level(max(4 * R, 2000), 21)   # a tree of more than R reaches: their records
    assert len(p32) >= R
    p32 = np.ascontiguousarray(p32[:R])
    c = O.matrix_coeffs(p32)
    m = O.matrix_build(up_ptr, up_idx, c, tol)
    assert_same_matrices(m, O.matrix_build(up_ptr, up_idx, c, tol, use_ref=True))
    lens = np.diff(m[0][0])
    if kind == "star":
        assert lens[-1] == R     # C2 at every upstream reach and C3 at itself: the step's whole-warp path
    if kind == "chain" and tol == 0.0:
        assert (lens == np.arange(1, R + 1)).all()   # nothing dropped: row r holds reaches 0..r
    rng = np.random.default_rng(R)
    ql = rng.uniform(0.0, 2.0, (6, R)).astype(np.float32)
    q0 = rng.uniform(0.05, 20.0, R).astype(np.float32)
    q = O.matrix_route(m[0], m[1], ql, q0)
    assert np.isfinite(q).all()


def test_oracle_rejects_reaches_not_numbered_upstream_first():
    up_ptr = np.array([0, 1, 1], np.int32)
    up_idx = np.array([1], np.int32)     # reach 0's upstream reach is reach 1
    c = [np.ones(2, np.float32) * 0.3] * 4
    with pytest.raises(ValueError):
        O.matrix_build(up_ptr, up_idx, c)


def _f32_products(v, x):
    """fma(v, x, +0) in float32: the product of two floats is exact in
    double, rounded once; adding +0 turns a -0 product into +0 as the fused
    operation does."""
    return (np.float32(v) * np.float32(x)).astype(np.float32) + np.float32(0.0)


def _reference_short_row(pq, pl):
    """The reference kernel's sum of one row with at most 32 entries per
    matrix: lane l holds its entry l of each matrix (0 where it has none),
    adds the two, then the shuffle-down tree 16, 8, 4, 2, 1."""
    s = (np.pad(pq, (0, 32 - len(pq))) + np.pad(pl, (0, 32 - len(pl)))).astype(np.float32)
    for off in (16, 8, 4, 2, 1):
        s[:off] = s[:off] + s[off:2 * off]
    return s[0]


def _lane_group_short_row(pq, pl, G):
    """The library's form with G lanes per row: lane p holds the reference's
    lanes p, p + G, ...; the tree levels 16 .. G in its registers (offset o
    adds slot j + o / G onto j), then shuffles G/2 .. 1 across the group."""
    s = (np.pad(pq, (0, 32 - len(pq))) + np.pad(pl, (0, 32 - len(pl)))).astype(np.float32)
    J = 32 // G
    u = np.empty(G, np.float32)
    for p in range(G):
        slot = s[p::G].copy()          # slot j = reference lane p + G j
        h = J // 2
        while h >= 1:
            slot[:h] = slot[:h] + slot[h:2 * h]
            h //= 2
        u[p] = slot[0]
    off = G // 2
    while off >= 1:
        u[:off] = u[:off] + u[off:2 * off]
        off //= 2
    return u[0]


def test_lane_groups_sum_short_rows_in_the_reference_order():
    """The step kernel's short-row mapping (4 lanes per row, the tree's first
    levels in registers) equals the reference kernel's 32-lane tree bit for
    bit, for every group width the kernel can be built with."""
    rng = np.random.default_rng(12)
    for _ in range(3000):
        nq, nl = rng.integers(0, 33, 2)
        scale = 10.0 ** rng.uniform(-6, 6)
        pq = _f32_products(rng.standard_normal(nq) * scale, rng.standard_normal(nq))
        pl = _f32_products(rng.standard_normal(nl), rng.standard_normal(nl) * scale)
        want = _reference_short_row(pq, pl)
        for G in (2, 4, 8, 16):
            assert _lane_group_short_row(pq, pl, G).tobytes() == want.tobytes(), (nq, nl, G)


def one_segment_topo(up_ptr, R):
    return {"n_segments": R, "reach_seg_start": np.arange(R, dtype=np.int32),
            "reach_seg_len": np.ones(R, np.int32), "reach_up_ptr": up_ptr, "reach_up_idx": None}


def test_matrix_step_agrees_with_the_sequential_linear_form():
    """With every reach one segment, the reference's cpu_linear_mc (here the
    oracle's bit-identical restatement of it) routes exactly the linear system
    the matrices expand; given the matrix form's coefficients the two differ
    by the dropped entries (1e-7) and float rounding only."""
    up_ptr, up_idx, p32, ql, q0 = reach_level(20000, 7, n_ts=24)
    R = len(up_ptr) - 1
    c = O.matrix_coeffs(p32)
    m = O.matrix_build(up_ptr, up_idx, c, 1e-7)
    q_mat = O.matrix_route(m[0], m[1], ql, q0)
    topo = one_segment_topo(up_ptr, R)
    topo["reach_up_idx"] = up_idx
    q_lin = O.linear_route(c, topo, ql, q0)
    rel = np.abs(q_mat - q_lin) / np.maximum(np.abs(q_lin), 1e-3)
    print(f"\nmatrix vs sequential linear form, 24 steps: max rel {rel.max():.2e}, median {np.median(rel):.2e}")
    assert rel.max() < 1e-4 and np.median(rel) < 1e-6


@pytest.mark.gpu
def test_gpu_matches_fixture_bit_for_bit():
    g = fixture()
    up_ptr, up_idx, _ = fixture_setup()
    coeffs = [g[k] for k in ("c1", "c2", "c3", "c4oq")]
    with T.MatrixNetwork(up_ptr, up_idx, coeffs) as net:
        assert_same_matrices(net.matrices(),
                             ((g["PQ_ptr"], g["PQ_col"], g["PQ_val"]), (g["Pq_ptr"], g["Pq_col"], g["Pq_val"])))
    np.testing.assert_array_equal(T.matrix_route(up_ptr, up_idx, coeffs, g["qlat"], g["q0"]), g["q_final"])


@pytest.mark.gpu
@pytest.mark.parametrize("segs,seed,n_ts", [(20000, 3, 7), (200000, 11, 24)])
def test_gpu_matches_oracle_bit_for_bit(segs, seed, n_ts):
    up_ptr, up_idx, p32, ql, q0 = reach_level(segs, seed, n_ts)
    c = O.matrix_coeffs(p32)
    m = O.matrix_build(up_ptr, up_idx, c, 1e-7)
    with T.MatrixNetwork(up_ptr, up_idx, c) as net:
        assert_same_matrices(net.matrices(), m)
    np.testing.assert_array_equal(T.matrix_route(up_ptr, up_idx, c, ql, q0), O.matrix_route(m[0], m[1], ql, q0))


@pytest.mark.gpu
def test_graph_replays_and_split_runs_equal_one_run():
    torch = pytest.importorskip("torch")
    up_ptr, up_idx, p32, ql, q0 = reach_level(20000, 5, 20)
    c = O.matrix_coeffs(p32)
    qlat = torch.from_numpy(ql).cuda()
    with T.MatrixNetwork(up_ptr, up_idx, c) as net:
        a = torch.from_numpy(q0.copy()).cuda()
        net.run_device(qlat.data_ptr(), 20, a.data_ptr())
        b = torch.from_numpy(q0.copy()).cuda()
        tail = qlat[7:].contiguous()
        net.run_device(qlat.data_ptr(), 7, b.data_ptr())
        net.run_device(tail.data_ptr(), 13, b.data_ptr())
        c2 = torch.from_numpy(q0.copy()).cuda()
        for _ in range(2):   # the second call replays the recorded graph
            net.run_device(qlat.data_ptr(), 10, c2.data_ptr())
        torch.cuda.synchronize()
    m = O.matrix_build(up_ptr, up_idx, c, 1e-7)
    want = O.matrix_route(m[0], m[1], ql, q0)
    np.testing.assert_array_equal(a.cpu().numpy(), want)
    np.testing.assert_array_equal(b.cpu().numpy(), want)
    ql2 = np.concatenate([ql[:10], ql[:10]])
    np.testing.assert_array_equal(c2.cpu().numpy(), O.matrix_route(m[0], m[1], ql2, q0))


@pytest.mark.gpu
def test_device_coefficients_within_float_rounding():
    _, _, p32, _, _ = reach_level()
    gd = T.matrix_coeffs(p32)
    for a, b in zip(gd, O.matrix_coeffs(p32)):
        assert np.all(np.abs(a - b) <= 4e-6 * np.maximum(np.abs(b), 1.0))


@pytest.mark.gpu
def test_rejects_reaches_not_numbered_upstream_first():
    c = [np.ones(2, np.float32) * 0.3] * 4
    with pytest.raises(T.TrouteError):
        T.MatrixNetwork(np.array([0, 1, 1], np.int32), np.array([1], np.int32), c)


@pytest.mark.gpu
def test_matrix_form_measured_against_the_secant_path():
    """The secant routing is the yardstick of the approximate form: on a one-segment-per-
    reach network the matrix form's discharge after a day of steps is set
    against the FP64 secant path's on the same inputs (reported, and sanity-
    checked: finite, same total order of magnitude)."""
    up_ptr, up_idx, p32, ql, q0 = reach_level(5000, 9, n_ts=48)
    R = len(up_ptr) - 1
    q_mat = T.matrix_route(up_ptr, up_idx, T.matrix_coeffs(p32), ql, q0)
    topo = one_segment_topo(up_ptr, R)
    topo["reach_up_idx"] = up_idx
    r = T.route_tree(topo, p32.astype(np.float64), ql.astype(np.float64), q0.astype(np.float64),
                     np.full(R, 0.5), None)
    q_sec = r["q"]
    assert np.isfinite(q_mat).all()
    rel = np.abs(q_mat - q_sec) / np.maximum(np.abs(q_sec), 1e-6)
    total = q_mat.sum() / q_sec.sum()
    print(f"\nmatrix form vs secant after 48 steps: median rel {np.median(rel):.3f}, p90 {np.quantile(rel, 0.9):.3f}, "
          f"total ratio {total:.3f}")
    assert 0.2 < total < 5.0
