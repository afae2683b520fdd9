"""ctypes access to the CPU oracle and, where it was built, to the compiled
reference routines.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, which compare the CUDA path with it. The product package
never imports it.

  oracle_cpu_mc / oracle_route_tree   our C restatement (troute_oracle.c),
      built into oracle/_build/libtroute_oracle.so by `make -C oracle oracle`;
  ref_cpu_mc / ref_cpu_wavefront_fp64  the reference's own cpu_mc
      (water-prediction/t-route/troute_mc_final.cu:167-252) and
      cpu_wavefront_fp64 (water-prediction/t-route/wavefront/wavefront_mc.cu:
      495-564), compiled unmodified into oracle/_ref/libtroute_ref.so by
      `make -C oracle ref` where the reference checkout exists.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libtroute_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libtroute_ref.so")
# the reference checkout: $TROUTE_REF_ROOT, else a checkout named `reference`
# beside this repository
REF_ROOT = os.environ.get("TROUTE_REF_ROOT") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))

CHP = np.dtype([(n, "<f8") for n in ("dx", "bw", "tw", "twcc", "n_ch", "ncc", "cs", "s0")])
CHP32 = np.dtype([(n, "<f4") for n in ("dx", "bw", "tw", "twcc", "n_ch", "ncc", "cs", "s0")])


class Tol(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("maxiter", C.c_int), ("attempts", C.c_int)]


REF_TOL = (0.01, 0.01, 100, 5)


def build(ref: bool = True) -> None:
    """Builds the oracle (always) and the reference library (when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if ref and os.path.exists(os.path.join(REF_ROOT, "water-prediction", "t-route", "troute_mc_final.cu")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={REF_ROOT}"], check=True)


_ORC = None
_REF = None
_P = C.c_void_p


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def oracle():
    global _ORC
    if _ORC is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        L = C.CDLL(ORACLE_SO)
        L.oracle_cpu_mc.argtypes = [_P] * 10 + [C.c_double, C.c_double, C.c_int, _P, _P]
        L.oracle_cpu_mc.restype = None
        L.oracle_route_tree.argtypes = [_P] * 6 + [C.c_int] * 3 + [_P] * 5 + [C.c_int, C.c_double, _P] + [_P] * 6 + [C.c_int]
        L.oracle_route_tree.restype = C.c_int
        L.oracle_mc_solve.argtypes = [C.c_double] * 5 + [_P, C.c_double, _P, _P, _P, _P]
        L.oracle_mc_solve.restype = C.c_double
        L.oracle_route_tree_ex.argtypes = [_P] * 6 + [C.c_int] * 3 + [_P] * 5 + [C.c_int, C.c_double, _P] + [_P] * 5
        L.oracle_route_tree_ex.restype = C.c_int
        L.oracle_mc_solve_warm.argtypes = ([C.c_double] * 5 + [_P, C.c_double, _P, C.c_double, C.c_double, C.c_int]
                                           + [_P] * 4)
        L.oracle_mc_solve_warm.restype = C.c_double
        L.oracle_linear_coeffs.argtypes = [_P, C.c_int, C.c_float] + [_P] * 4
        L.oracle_linear_coeffs.restype = None
        L.oracle_linear_route.argtypes = [_P] * 10 + [C.c_int] * 3 + [_P] * 3 + [C.c_int]
        L.oracle_linear_route.restype = C.c_int
        L.oracle_diffusive_tridiag.argtypes = [_P] * 5 + [C.c_int, C.c_int]
        L.oracle_diffusive_tridiag.restype = C.c_int
        L.oracle_set_pow_mode.argtypes = [C.c_int]
        L.oracle_set_pow_mode.restype = None
        L.oracle_pow23_53.argtypes = [C.c_double, _P, _P]
        L.oracle_pow23_53.restype = None
        L.oracle_pow23_53_n.argtypes = [_P, C.c_longlong, _P, _P, C.c_int, C.c_int]
        L.oracle_pow23_53_n.restype = C.c_int
        L.oracle_gen_tree.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int] + [_P] * 4
        L.oracle_gen_tree.restype = C.c_int
        L.oracle_gen_params.argtypes = [C.c_uint64, C.c_int, _P]
        L.oracle_gen_params.restype = None
        L.oracle_gen_qlat.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_double, _P, C.c_int]
        L.oracle_gen_qlat.restype = C.c_int
        L.oracle_gen_member.argtypes = [C.c_uint64, C.c_int, C.c_int, _P, _P]
        L.oracle_gen_member.restype = None
        L.oracle_levels.argtypes = [C.c_int, _P, _P, _P, _P]
        L.oracle_levels.restype = C.c_int
        L.oracle_matrix_coeffs.argtypes = [_P, C.c_int, C.c_float] + [_P] * 4
        L.oracle_matrix_coeffs.restype = None
        L.oracle_matrix_build.argtypes = [C.c_int, _P, _P, _P, _P, _P, _P, C.c_float, _P, _P]
        L.oracle_matrix_build.restype = C.c_int
        L.oracle_csr_free.argtypes = [_P]
        L.oracle_csr_free.restype = None
        L.oracle_matrix_route.argtypes = [_P, _P, _P, _P, _P, C.c_int]
        L.oracle_matrix_route.restype = C.c_int
        _ORC = L
    return _ORC


class pow_mode:
    """Context manager: route the oracle's R^(2/3), R^(5/3) through the C
    library's pow() (0, the reference's) or the correctly rounded form (1)."""

    def __init__(self, mode: int):
        self.mode = mode

    def __enter__(self):
        oracle().oracle_set_pow_mode(self.mode)
        return self

    def __exit__(self, *a):
        oracle().oracle_set_pow_mode(0)


def pow23_53(x: float, mode: int = 0):
    a, b = C.c_double(), C.c_double()
    with pow_mode(mode):
        oracle().oracle_pow23_53(float(x), C.byref(a), C.byref(b))
    return a.value, b.value


def pow23_53_n(x, mode: int = 1, threads: int = 0):
    """pow23_53 over an array (all host threads by default) -> (p23, p53)."""
    x = np.ascontiguousarray(x, np.float64)
    a, b = np.empty_like(x), np.empty_like(x)
    if oracle().oracle_pow23_53_n(_ptr(x), x.size, _ptr(a), _ptr(b), int(mode), int(threads or os.cpu_count() or 1)):
        raise MemoryError("oracle_pow23_53_n")
    return a, b


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _REF
    if _REF is None:
        L = C.CDLL(REF_SO)
        L.ref_cpu_mc.argtypes = [_P] * 10 + [C.c_double, C.c_double, C.c_int]
        L.ref_cpu_mc.restype = None
        L.ref_cpu_wavefront_fp64.argtypes = [_P] * 7 + [C.c_int] * 3 + [_P] * 6 + [C.c_int, C.c_double]
        L.ref_cpu_wavefront_fp64.restype = None
        L.ref_linear_coeffs.argtypes = [_P, C.c_int, C.c_float] + [_P] * 4
        L.ref_linear_coeffs.restype = None
        L.ref_cpu_linear_mc.argtypes = [_P] * 10 + [C.c_int] * 3 + [_P] * 3 + [C.c_int]
        L.ref_cpu_linear_mc.restype = None
        L.ref_cpu_diffusive_tridiag.argtypes = [_P] * 6 + [C.c_int]
        L.ref_cpu_diffusive_tridiag.restype = None
        L.ref_diffusive_max_nodes.restype = C.c_int
        L.ref_matrix_coeffs.argtypes = [_P, C.c_int, C.c_float] + [_P] * 4
        L.ref_matrix_coeffs.restype = None
        L.ref_matrix_build.argtypes = [C.c_int, _P, _P, _P, _P, _P, _P, C.c_float, _P, _P]
        L.ref_matrix_build.restype = None
        L.ref_matrix_fetch.argtypes = [C.c_int, _P, _P, _P]
        L.ref_matrix_fetch.restype = None
        _REF = L
    return _REF


def _tol(t):
    return Tol(*t) if not isinstance(t, Tol) else t


def _params(p):
    p = np.ascontiguousarray(p)
    if p.dtype.names is not None:
        return np.ascontiguousarray(p.astype(CHP))
    return np.ascontiguousarray(np.asarray(p, np.float64).reshape(-1, 8)).view(CHP).reshape(-1)


def cpu_mc(p, ql, rs, rl, qu, qd, dp, uq=10.0, dt=300.0, tol=REF_TOL):
    """Oracle restatement of cpu_mc -> (qo, vo, dpo, iterations)."""
    p = _params(p)
    n = p.shape[0]
    ql, qu, qd, dp = (np.ascontiguousarray(x, np.float64) for x in (ql, qu, qd, dp))
    rs, rl = np.ascontiguousarray(rs, np.int32), np.ascontiguousarray(rl, np.int32)
    qo, vo, dpo = np.zeros(n), np.zeros(n), np.zeros(n)
    it = C.c_longlong()
    t = _tol(tol)
    oracle().oracle_cpu_mc(_ptr(p), _ptr(ql), _ptr(rs), _ptr(rl), _ptr(qu), _ptr(qd), _ptr(dp), _ptr(qo), _ptr(vo),
                           _ptr(dpo), float(uq), float(dt), int(rs.size), C.byref(t), C.byref(it))
    return qo, vo, dpo, it.value


def mc_solve(dt, qup, quc, qdp, ql, p_record, depthp, tol=REF_TOL):
    """One segment solve -> (q, depth, velocity, iterations)."""
    p = _params(np.asarray(p_record).reshape(1, -1) if np.asarray(p_record).dtype.names is None else p_record)
    d, v, it = C.c_double(), C.c_double(), C.c_int()
    t = _tol(tol)
    q = oracle().oracle_mc_solve(dt, qup, quc, qdp, ql, _ptr(p), depthp, C.byref(t), C.byref(d), C.byref(v),
                                 C.byref(it))
    return q, d.value, v.value, it.value


class TreeOpts(C.Structure):
    _fields_ = [("warm_start", C.c_void_p), ("warm_delta", C.c_double), ("warm_k", C.c_int), ("n_threads", C.c_int),
                ("q_hist", C.c_void_p), ("d_hist", C.c_void_p), ("it_hist", C.c_void_p),
                ("iters_total", C.c_longlong), ("warm_used", C.c_longlong), ("warm_fallback", C.c_longlong)]


def route_tree(topo, params, qlat_ts, qdp0, dp0, reach_last0, dt=300.0, tol=REF_TOL, history=False, threads=1,
               level_ptr=None, level_reach=None, warm_start=None, warm_delta=0.0, warm_k=0, depth_history=False,
               iter_history=False):
    """Oracle tree routing (cpu_wavefront_fp64 semantics, FP64 inputs).

    warm_start: optional [n_ts][n_segments] starting depth of every solve
    (<= 0: plain start), with the warm bracket half-width warm_delta and
    warm_k passes before the plain fallback (oracle_mc_solve_warm)."""
    seg_start = np.ascontiguousarray(topo["reach_seg_start"], np.int32)
    seg_len = np.ascontiguousarray(topo["reach_seg_len"], np.int32)
    up_ptr = np.ascontiguousarray(topo["reach_up_ptr"], np.int32)
    up_idx = np.ascontiguousarray(topo["reach_up_idx"] if len(topo["reach_up_idx"]) else [0], np.int32)
    R, S = seg_start.size, int(topo["n_segments"])
    if level_ptr is None:
        level_ptr, level_reach = levels(up_ptr, up_idx, R)
    level_ptr = np.ascontiguousarray(level_ptr, np.int32)
    level_reach = np.ascontiguousarray(level_reach, np.int32)
    p = _params(params)
    ql = np.ascontiguousarray(qlat_ts, np.float64)
    T = ql.shape[0]
    q0, d0, r0 = (np.ascontiguousarray(x, np.float64) for x in (qdp0, dp0, reach_last0))
    q, d, v, rl = np.zeros(S), np.zeros(S), np.zeros(S), np.zeros(R)
    hist = np.zeros((T, S)) if history else None
    dhist = np.zeros((T, S)) if depth_history else None
    ihist = np.zeros((T, S), np.int32) if iter_history else None
    ws = None
    if warm_start is not None:
        ws = np.ascontiguousarray(warm_start, np.float64)
        if ws.shape != (T, S):
            raise ValueError(f"warm_start must be [{T}][{S}]")
    o = TreeOpts(_ptr(ws), float(warm_delta), int(warm_k), int(threads), _ptr(hist), _ptr(dhist), _ptr(ihist), 0, 0, 0)
    t = _tol(tol)
    rc = oracle().oracle_route_tree_ex(_ptr(seg_start), _ptr(seg_len), _ptr(up_ptr), _ptr(up_idx), _ptr(level_ptr),
                                       _ptr(level_reach), R, level_ptr.size - 1, S, _ptr(p), _ptr(ql), _ptr(q0),
                                       _ptr(d0), _ptr(r0), T, float(dt), C.byref(t), _ptr(q), _ptr(d), _ptr(v),
                                       _ptr(rl), C.byref(o))
    if rc != 0:
        raise RuntimeError(f"oracle_route_tree failed: {rc}")
    out = {"q": q, "d": d, "v": v, "reach_last": rl, "iterations": o.iters_total,
           "warm_used": o.warm_used, "warm_fallback": o.warm_fallback}
    if history:
        out["q_hist"] = hist
    if depth_history:
        out["d_hist"] = dhist
    if iter_history:
        out["it_hist"] = ihist
    return out


def mc_solve_warm(dt, qup, quc, qdp, ql, p_record, depthp, start, delta, k, tol=REF_TOL):
    """One warm-started segment solve -> (q, depth, velocity, iterations, warm_state)."""
    p = _params(np.asarray(p_record).reshape(1, -1) if np.asarray(p_record).dtype.names is None else p_record)
    d, v, it, st = C.c_double(), C.c_double(), C.c_int(), C.c_int()
    t = _tol(tol)
    q = oracle().oracle_mc_solve_warm(dt, qup, quc, qdp, ql, _ptr(p), depthp, C.byref(t), float(start), float(delta),
                                      int(k), C.byref(d), C.byref(v), C.byref(it), C.byref(st))
    return q, d.value, v.value, it.value, st.value


def levels(up_ptr, up_idx, R):
    """Reference level construction (gen_network.py:219-231), numpy only."""
    up_ptr = np.asarray(up_ptr)
    up_idx = np.asarray(up_idx)
    down = np.full(R, -1)
    for r in range(R):
        for k in range(up_ptr[r], up_ptr[r + 1]):
            down[up_idx[k]] = r
    indeg = np.diff(up_ptr).copy()
    order = [r for r in range(R) if indeg[r] == 0]
    i = 0
    while i < len(order):
        d = down[order[i]]
        if d >= 0:
            indeg[d] -= 1
            if indeg[d] == 0:
                order.append(d)
        i += 1
    level = np.zeros(R, np.int32)
    for r in order:
        ups = up_idx[up_ptr[r]:up_ptr[r + 1]]
        if len(ups):
            level[r] = 1 + level[ups].max()
    L = int(level.max()) + 1 if R else 0
    level_reach = np.argsort(level, kind="stable").astype(np.int32)
    counts = np.bincount(level, minlength=L).astype(np.int32)
    level_ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    return level_ptr, level_reach


def ref_cpu_mc(p, ql, rs, rl, qu, qd, dp, uq=10.0, dt=300.0):
    """The reference's own cpu_mc (compiled from its source)."""
    p = _params(p)
    n = p.shape[0]
    ql, qu, qd, dp = (np.ascontiguousarray(x, np.float64) for x in (ql, qu, qd, dp))
    rs, rl = np.ascontiguousarray(rs, np.int32), np.ascontiguousarray(rl, np.int32)
    qo, vo, dpo = np.zeros(n), np.zeros(n), np.zeros(n)
    ref().ref_cpu_mc(_ptr(p), _ptr(ql), _ptr(rs), _ptr(rl), _ptr(qu), _ptr(qd), _ptr(dp), _ptr(qo), _ptr(vo),
                     _ptr(dpo), float(uq), float(dt), int(rs.size))
    return qo, vo, dpo


def ref_wavefront_fp64(topo, params_f32, qlat_f32, qdp0_f32, dp0_f32, reach_last0_f32, dt=300.0,
                       level_ptr=None, level_reach=None):
    """The reference's own cpu_wavefront_fp64 -> (q_final, reach_last_final)."""
    seg_start = np.ascontiguousarray(topo["reach_seg_start"], np.int32)
    seg_len = np.ascontiguousarray(topo["reach_seg_len"], np.int32)
    up_ptr = np.ascontiguousarray(topo["reach_up_ptr"], np.int32)
    up_idx = np.ascontiguousarray(topo["reach_up_idx"] if len(topo["reach_up_idx"]) else [0], np.int32)
    R, S = seg_start.size, int(topo["n_segments"])
    if level_ptr is None:
        level_ptr, level_reach = levels(up_ptr, up_idx, R)
    level_ptr = np.ascontiguousarray(level_ptr, np.int32)
    level_reach = np.ascontiguousarray(level_reach, np.int32)
    p = np.ascontiguousarray(params_f32)
    if p.dtype != CHP32:
        p = np.ascontiguousarray(np.asarray(p, np.float32).reshape(-1, 8)).view(CHP32).reshape(-1)
    ql = np.ascontiguousarray(qlat_f32, np.float32)
    q0, d0, r0 = (np.ascontiguousarray(x, np.float32) for x in (qdp0_f32, dp0_f32, reach_last0_f32))
    q, rl = np.zeros(S), np.zeros(R)
    ref().ref_cpu_wavefront_fp64(_ptr(p), _ptr(seg_start), _ptr(seg_len), _ptr(up_ptr), _ptr(up_idx),
                                 _ptr(level_ptr), _ptr(level_reach), R, level_ptr.size - 1, S, _ptr(ql), _ptr(q0),
                                 _ptr(d0), _ptr(r0), _ptr(q), _ptr(rl), int(ql.shape[0]), float(dt))
    return q, rl


def _params_f32(p):
    p = np.ascontiguousarray(p)
    if p.dtype != CHP32:
        p = np.ascontiguousarray(np.asarray(p, np.float32).reshape(-1, 8)).view(CHP32).reshape(-1)
    return p


def linear_coeffs(params_f32, dt=300.0, use_ref=False):
    """Linearised-MC coefficients (C1, C2, C3, C4/ql) per segment: the oracle's
    restatement of compute_mc_coeffs, or (use_ref) the reference's own."""
    p = _params_f32(params_f32)
    n = p.shape[0]
    c = [np.zeros(n, np.float32) for _ in range(4)]
    f = ref().ref_linear_coeffs if use_ref else oracle().oracle_linear_coeffs
    f(_ptr(p), n, float(dt), *(_ptr(x) for x in c))
    return c


def _linear_args(coeffs, topo, level_ptr, level_reach):
    seg_start = np.ascontiguousarray(topo["reach_seg_start"], np.int32)
    seg_len = np.ascontiguousarray(topo["reach_seg_len"], np.int32)
    up_ptr = np.ascontiguousarray(topo["reach_up_ptr"], np.int32)
    up_idx = np.ascontiguousarray(topo["reach_up_idx"] if len(topo["reach_up_idx"]) else [0], np.int32)
    R = seg_start.size
    if level_ptr is None:
        level_ptr, level_reach = levels(up_ptr, up_idx, R)
    lp = np.ascontiguousarray(level_ptr, np.int32)
    lr = np.ascontiguousarray(level_reach, np.int32)
    cs = [np.ascontiguousarray(c, np.float32) for c in coeffs]
    return cs, [seg_start, seg_len, up_ptr, up_idx, lp, lr], R, lp.size - 1


def linear_route(coeffs, topo, qlat_ts, q0, level_ptr=None, level_reach=None, use_ref=False):
    """Float routing of cpu_linear_mc: the oracle's restatement or (use_ref)
    the reference's own; returns the final discharge."""
    cs, ints, R, L = _linear_args(coeffs, topo, level_ptr, level_reach)
    S = int(topo["n_segments"])
    ql = np.ascontiguousarray(qlat_ts, np.float32)
    q0 = np.ascontiguousarray(q0, np.float32)
    out = np.zeros(S, np.float32)
    args = [_ptr(x) for x in cs] + [_ptr(x) for x in ints] + [R, L, S, _ptr(ql), _ptr(q0), _ptr(out), ql.shape[0]]
    if use_ref:
        ref().ref_cpu_linear_mc(*args)
    else:
        rc = oracle().oracle_linear_route(*args)
        if rc:
            raise RuntimeError(f"oracle_linear_route failed: {rc}")
    return out


DIFF_REACH = np.dtype([("ncomp", "<i4"), ("theta", "<f4"), ("dtini", "<f4")])


def diffusive_tridiag(reaches, dx, diffusivity, qp_prev, qp_out=None, use_ref=False, celerity=None):
    """Diffusive-wave tridiagonal step over [n_reaches][max_nodes] arrays: the
    oracle's restatement, or (use_ref) the reference's cpu_diffusive_tridiag
    (whose arrays are [n][MAX_NODES = 500])."""
    rp = np.ascontiguousarray(reaches, DIFF_REACH)
    dx, df, qp = (np.ascontiguousarray(a, np.float32) for a in (dx, diffusivity, qp_prev))
    n, m = qp.shape
    out = np.zeros_like(qp) if qp_out is None else np.ascontiguousarray(qp_out, np.float32).copy()
    if use_ref:
        assert m == ref().ref_diffusive_max_nodes()
        cel = np.zeros_like(qp) if celerity is None else np.ascontiguousarray(celerity, np.float32)
        ref().ref_cpu_diffusive_tridiag(_ptr(rp), _ptr(dx), _ptr(df), _ptr(cel), _ptr(qp), _ptr(out), n)
    else:
        rc = oracle().oracle_diffusive_tridiag(_ptr(rp), _ptr(dx), _ptr(df), _ptr(qp), _ptr(out), n, m)
        if rc:
            raise RuntimeError(f"oracle_diffusive_tridiag failed: {rc}")
    return out


# --------------------------------------------------------------------------- seeded inputs
# The benchmark's synthetic workloads, built by the oracle's own restatement of
# the product's seeded generator (oracle_gen.c), so that the CPU legs never load
# the product library. tests/test_generator.py checks every array against the
# product generator byte for byte.
DT, Q0, D0 = 300.0, 0.1, 0.1
SEG_PER_REACH = 2.7e6 / 1.1e6
C1_SEED, C3_SEED, C0_SEED, TREE_SEED, MEMBER_SEED = 1010, 2006, 1000, 7, 1004


def gen_tree(seed: int, n_leaves: int, n_segments: int, max_len: int = 10) -> dict:
    R = 2 * n_leaves - 1
    seg_start, seg_len = np.zeros(R, np.int32), np.zeros(R, np.int32)
    up_ptr, up_idx = np.zeros(R + 1, np.int32), np.zeros(max(R - 1, 1), np.int32)
    rc = oracle().oracle_gen_tree(seed, n_leaves, n_segments, max_len, _ptr(seg_start), _ptr(seg_len), _ptr(up_ptr),
                                  _ptr(up_idx))
    if rc:
        raise ValueError(f"oracle_gen_tree: {rc}")
    return {"n_segments": int(n_segments), "reach_seg_start": seg_start, "reach_seg_len": seg_len,
            "reach_up_ptr": up_ptr, "reach_up_idx": up_idx[: R - 1]}


def gen_params(seed: int, n_segments: int) -> np.ndarray:
    p = np.zeros(n_segments, CHP)
    oracle().oracle_gen_params(seed, n_segments, _ptr(p))
    return p


def gen_qlat(seed: int, n_segments: int, n_ts: int, t0: int = 0, dt: float = DT, threads: int = 0) -> np.ndarray:
    q = np.zeros((n_ts, n_segments))
    rc = oracle().oracle_gen_qlat(seed, n_segments, t0, n_ts, dt, _ptr(q), int(threads or os.cpu_count() or 1))
    if rc:
        raise MemoryError("oracle_gen_qlat")
    return q


def gen_member(seed: int, member: int, n_segments: int):
    qf, nf = np.zeros(n_segments), np.zeros(n_segments)
    oracle().oracle_gen_member(seed, member, n_segments, _ptr(qf), _ptr(nf))
    return qf, nf


def levels_c(up_ptr, up_idx, R: int):
    """levels() computed in C (the same schedule, for networks of millions of reaches)."""
    up_ptr = np.ascontiguousarray(up_ptr, np.int32)
    up_idx = np.ascontiguousarray(up_idx if len(up_idx) else [0], np.int32)
    lp, lr = np.zeros(R + 1, np.int32), np.zeros(max(R, 1), np.int32)
    L = oracle().oracle_levels(R, _ptr(up_ptr), _ptr(up_idx), _ptr(lp), _ptr(lr))
    if L < 0:
        raise MemoryError("oracle_levels")
    return lp[: L + 1], lr[:R]


def tree_size(n_segments: int) -> int:
    """Headwaters of a tree with ~2.45 segments per reach."""
    n_leaves = max(1, int(round(n_segments / SEG_PER_REACH / 2.0)))
    return min(n_leaves, (n_segments + 1) // 2)


def network(name: str, seed: int | None = None, n_ts: int | None = None, t0: int = 0) -> dict:
    """The single-network workloads: 'c0' (1,000 segments, 288 steps), 'c1'
    (2.7M segments, ~3,000 levels, 144 steps), 'c3' (c1's sizes on a fresh
    seed) and 'tree:<segments>' (24 steps); lateral inflow of steps t0.."""
    if name == "c0":
        seed = C0_SEED if seed is None else seed
        topo, T = gen_tree(seed, 100, 1000, 10), 288
    elif name in ("c1", "c3"):
        seed = (C1_SEED if name == "c1" else C3_SEED) if seed is None else seed
        topo, T = gen_tree(seed, 550_000, 2_700_000, 10), 144
    elif name.startswith("tree:"):
        S = int(name.split(":")[1])
        seed = TREE_SEED if seed is None else seed
        topo, T = gen_tree(seed, tree_size(S), S, 10), 24
    else:
        raise ValueError(name)
    T = T if n_ts is None else n_ts
    S = topo["n_segments"]
    R = len(topo["reach_seg_start"])
    return {"name": name, "seed": seed, "topo": topo, "params": gen_params(seed, S), "n_ts": T, "dt": DT,
            "qlat": gen_qlat(seed, S, T, t0), "q0": np.full(S, Q0), "d0": np.full(S, D0), "rl0": np.full(R, Q0)}


def ensemble_member(w: dict, member: int, seed: int = MEMBER_SEED) -> dict:
    """Member `member` of an ensemble over network w: Manning's n (channel and
    floodplain) times U(0.8, 1.2) and lateral inflow times LogN(0, 0.3), per
    segment, the products formed in FP64 as the library forms them."""
    S = w["topo"]["n_segments"]
    qf, nf = gen_member(seed, member, S)
    p = w["params"].copy()
    p["n_ch"] *= nf
    p["ncc"] *= nf
    out = dict(w)
    out.update(params=p, qlat=w["qlat"] * qf[None, :], qfac=qf, nfac=nf, member=member)
    return out


# --------------------------------------------------------------------------- matrix form
class CSR(C.Structure):
    _fields_ = [("n", C.c_int), ("ptr", C.POINTER(C.c_int)), ("col", C.POINTER(C.c_int)),
                ("val", C.POINTER(C.c_float))]


def matrix_coeffs(params_f32, dt=300.0, use_ref=False):
    """Matrix-form coefficients (C1, C2, C3, C4/ql) at X = 0.25 per reach: the
    oracle's restatement of compute_mc_coeffs_cpu or (use_ref) the reference's own."""
    p = _params_f32(params_f32)
    n = p.shape[0]
    c = [np.zeros(n, np.float32) for _ in range(4)]
    f = ref().ref_matrix_coeffs if use_ref else oracle().oracle_matrix_coeffs
    f(_ptr(p), n, float(dt), *(_ptr(x) for x in c))
    return c


def _csr_arrays(m: CSR):
    n = m.n
    ptr = np.ctypeslib.as_array(m.ptr, shape=(n + 1,)).copy()
    nnz = int(ptr[-1])
    col = np.ctypeslib.as_array(m.col, shape=(max(nnz, 1),))[:nnz].copy()
    val = np.ctypeslib.as_array(m.val, shape=(max(nnz, 1),))[:nnz].copy()
    return ptr, col, val


def matrix_build(up_ptr, up_idx, coeffs, tol=1e-7, use_ref=False):
    """The truncated propagation matrices ((ptr, col, val) of P_Q, of P_q): the
    oracle's restatement of build_propagation_matrices or (use_ref) the
    reference's own."""
    up_ptr = np.ascontiguousarray(up_ptr, np.int32)
    up_idx = np.ascontiguousarray(up_idx if len(up_idx) else [0], np.int32)
    R = up_ptr.size - 1
    cs = [np.ascontiguousarray(c, np.float32) for c in coeffs]
    if use_ref:
        nq, nl = C.c_int(), C.c_int()
        ref().ref_matrix_build(R, _ptr(up_ptr), _ptr(up_idx), *(_ptr(c) for c in cs), float(tol), C.byref(nq),
                               C.byref(nl))
        out = []
        for which, nnz in ((0, nq.value), (1, nl.value)):
            ptr, col, val = np.zeros(R + 1, np.int32), np.zeros(max(nnz, 1), np.int32), np.zeros(max(nnz, 1), np.float32)
            ref().ref_matrix_fetch(which, _ptr(ptr), _ptr(col), _ptr(val))
            out.append((ptr, col[:nnz], val[:nnz]))
        return tuple(out)
    PQ, Pq = CSR(), CSR()
    rc = oracle().oracle_matrix_build(R, _ptr(up_ptr), _ptr(up_idx), *(_ptr(c) for c in cs), float(tol), C.byref(PQ),
                                      C.byref(Pq))
    if rc:
        raise ValueError(f"oracle_matrix_build: {rc}")
    try:
        return _csr_arrays(PQ), _csr_arrays(Pq)
    finally:
        oracle().oracle_csr_free(C.byref(PQ))
        oracle().oracle_csr_free(C.byref(Pq))


def matrix_route(PQ, Pq, qlat_ts, q0):
    """The matrix form routed n_ts steps (the reference's fused kernel's
    arithmetic, oracle_matrix_step); returns the final discharge."""
    keep = []

    def csr(m):
        ptr, col, val = (np.ascontiguousarray(m[0], np.int32), np.ascontiguousarray(m[1] if len(m[1]) else [0], np.int32),
                         np.ascontiguousarray(m[2] if len(m[2]) else [0], np.float32))
        keep.extend((ptr, col, val))
        return CSR(ptr.size - 1, ptr.ctypes.data_as(C.POINTER(C.c_int)), col.ctypes.data_as(C.POINTER(C.c_int)),
                   val.ctypes.data_as(C.POINTER(C.c_float)))

    a, b = csr(PQ), csr(Pq)
    ql = np.ascontiguousarray(qlat_ts, np.float32)
    q0 = np.ascontiguousarray(q0, np.float32)
    out = np.zeros(a.n, np.float32)
    rc = oracle().oracle_matrix_route(C.byref(a), C.byref(b), _ptr(ql), _ptr(q0), _ptr(out), int(ql.shape[0]))
    if rc:
        raise MemoryError("oracle_matrix_route")
    return out
