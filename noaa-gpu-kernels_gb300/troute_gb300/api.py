"""Python mirror of the t-route MC routing interface over libtroute_gb300.so.

Function names and argument meaning follow the reference's entry points:
  mc_reach_parallel  <- cpu_mc / kernel_mc_gpu
                        (water-prediction/t-route/troute_mc_final.cu:142-171)
  wavefront_fp64     <- cpu_wavefront_fp64
                        (water-prediction/t-route/wavefront/wavefront_mc.cu:495-507)
  route_tree / Network  FP64 multi-step tree routing with persistent state.
Every call goes through the C ABI declared in include/troute_gb300.h; a
non-zero status raises TrouteError with the library's message. The CUDA
library must have been built (troute_gb300.build.build()); there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

# ---------------------------------------------------------------------------
# library loading
# ---------------------------------------------------------------------------
_LIB = None


class TrouteError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"troute error {code}: {msg}")
        self.code = code


OK, EINVAL, ETOPO, ECUDA, ENOMEM, ETIMEOUT, ENODEV, EIO, ESTATE = range(9)


class ChParams(C.Structure):
    """Same layout as the reference's ChParams (troute_mc_final.cu:26-28)."""

    _fields_ = [(n, C.c_double) for n in ("dx", "bw", "tw", "twcc", "n_ch", "ncc", "cs", "s0")]


CHPARAMS_DTYPE = np.dtype([(n, "<f8") for n in ("dx", "bw", "tw", "twcc", "n_ch", "ncc", "cs", "s0")])
CHPARAMS_F32_DTYPE = np.dtype([(n, "<f4") for n in ("dx", "bw", "tw", "twcc", "n_ch", "ncc", "cs", "s0")])


class Cfg(C.Structure):
    _fields_ = [
        ("rtol", C.c_double),
        ("atol", C.c_double),
        ("maxiter", C.c_int),
        ("attempts", C.c_int),
        ("threads_per_block", C.c_int),
        ("blocks_per_sm", C.c_int),
        ("wait_cycles", C.c_longlong),
        ("warm_start", C.c_int),
        ("warm_k", C.c_int),
        ("record_history", C.c_int),
        ("mapping", C.c_int),
        ("schedule_flags", C.c_int),
        ("max_chunk_steps", C.c_int),
        ("record_pairs", C.c_int),
        ("record_start", C.c_int),
        ("reserved", C.c_int * 2),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("solves", C.c_ulonglong),
        ("iterations", C.c_ulonglong),
        ("retries", C.c_ulonglong),
        ("early_exits", C.c_ulonglong),
        ("warm_used", C.c_ulonglong),
        ("warm_fallback", C.c_ulonglong),
        ("iter_hist", C.c_ulonglong * 16),
        ("warp_passes", C.c_ulonglong),
        ("lane_busy", C.c_ulonglong),
        ("lane_wait", C.c_ulonglong),
        ("lane_idle", C.c_ulonglong),
        ("solve_passes", C.c_ulonglong),
        ("kernel_ms", C.c_double),
        ("timeout", C.c_int),
        ("reserved", C.c_int * 3),
    ]

    def as_dict(self) -> dict:
        return {
            "solves": int(self.solves),
            "iterations": int(self.iterations),
            "retries": int(self.retries),
            "early_exits": int(self.early_exits),
            "warm_used": int(self.warm_used),
            "warm_fallback": int(self.warm_fallback),
            "iter_hist": [int(x) for x in self.iter_hist],
            "warp_passes": int(self.warp_passes),
            "lane_busy": int(self.lane_busy),
            "lane_wait": int(self.lane_wait),
            "lane_idle": int(self.lane_idle),
            "solve_passes": int(self.solve_passes),
            "kernel_ms": float(self.kernel_ms),
            "timeout": int(self.timeout),
        }


class Topo(C.Structure):
    _fields_ = [
        ("n_reaches", C.c_int),
        ("n_segments", C.c_int),
        ("reach_seg_start", C.POINTER(C.c_int)),
        ("reach_seg_len", C.POINTER(C.c_int)),
        ("reach_up_ptr", C.POINTER(C.c_int)),
        ("reach_up_idx", C.POINTER(C.c_int)),
    ]


_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_U64 = C.c_uint64

# name -> argtypes (restype is int unless noted)
_SIGS = {
    "troute_last_error": ([], C.c_char_p),
    "troute_cfg_default": ([_P], None),
    "troute_device_info": ([_P, _P, _P, _P], _I),
    "troute_mc_reach_parallel": ([_P] * 10 + [_D, _D, _I], _I),
    "troute_mc_reach_parallel_cfg": ([_P] * 10 + [_D, _D, _I, _P, _P], _I),
    "troute_mc_reach_parallel_device": ([_P] * 10 + [_D, _D, _I, _I, _P, _P], _I),
    "troute_mc_reach_parallel_device_noalloc": ([_P] * 10 + [_D, _D, _I, _I, _P, _P, _P], _I),
    "troute_wavefront_fp64": ([_P] * 7 + [_I, _I, _I] + [_P] * 6 + [_I, _D], _I),
    "troute_route_tree": ([_P] * 6 + [_I, _D, _P] + [_P] * 5, _I),
    "troute_mc_route_tree": ([_P] * 6 + [_I, _D, _P] + [_P] * 5, _I),
    "troute_create": ([_P, _P, _P, _D, _P], _I),
    "troute_create_batch": ([_P, _I, _P, _P, _P, _P, _I, _D, _P], _I),
    "troute_create_ensemble": ([_P, _P, _P, _I, _P, _P, _D, _P], _I),
    "troute_destroy": ([_P], _I),
    "troute_set_cfg": ([_P, _P], _I),
    "troute_info": ([_P, _P, _P, _P, _P, _P], _I),
    "troute_set_state": ([_P, _P, _P, _P], _I),
    "troute_get_state": ([_P, _P, _P, _P, _P], _I),
    "troute_run": ([_P, _P, _I, _P], _I),
    "troute_run_device": ([_P, _P, _I, _P], _I),
    "troute_sync": ([_P, _P], _I),
    "troute_graph_capture": ([_P, _P, _I], _I),
    "troute_graph_launch": ([_P, _P], _I),
    "troute_get_history": ([_P, _P, _I], _I),
    "troute_checkpoint": ([_P, _P, _P], _I),
    "troute_restore": ([_P, _P, C.c_size_t], _I),
    "troute_warm_create": ([_P, _U64], _I),
    "troute_warm_destroy": ([_P], _I),
    "troute_warm_get": ([_P, _P, _I], _I),
    "troute_warm_set": ([_P, _P, _I], _I),
    "troute_warm_fit": ([_P, _P, C.c_longlong, _I, _I, C.c_float, C.c_float, _U64, _P], _I),
    "troute_warm_grad": ([_P, _P, _I, _P, _P], _I),
    "troute_warm_predict": ([_P, _P, _I, _P], _I),
    "troute_set_warm_start": ([_P, _P, _D], _I),
    "troute_get_pairs": ([_P, _P, C.c_longlong, _P], _I),
    "troute_get_start_history": ([_P, _P, _I], _I),
    "troute_autotune": ([_P, _P, _I, _I, _I, _P], _I),
    "troute_diffusive_tridiag": ([_P] * 6 + [_I, _I], _I),
    "troute_diffusive_tridiag_device": ([_P] * 6 + [_I, _I, _P, _P], _I),
    "troute_linear_coeffs": ([_P, _I, _D, _P, _P, _P, _P], _I),
    "troute_linear_create": ([_P, _P, _P, _P, _P, _P], _I),
    "troute_linear_destroy": ([_P], _I),
    "troute_linear_run_device": ([_P, _P, _I, _P, C.c_longlong, _P], _I),
    "troute_linear_route": ([_P, _P, _P, _P, _P, _P, _P, _I, _P], _I),
    "troute_matrix_coeffs": ([_P, _I, _D, _P, _P, _P, _P], _I),
    "troute_matrix_create": ([_P, _I, _P, _P, _P, _P, _P, _P, C.c_float], _I),
    "troute_matrix_destroy": ([_P], _I),
    "troute_matrix_info": ([_P, _P, _P, _P], _I),
    "troute_matrix_get": ([_P, _I, _P, _P, _P], _I),
    "troute_matrix_run_device": ([_P, _P, _I, _P, _P], _I),
    "troute_matrix_route": ([_I, _P, _P, _P, _P, _P, _P, C.c_float, _P, _P, _I, _P], _I),
    "troute_qlat_from_csv": ([C.c_char_p, _P, _I, _I, _I, _P, _P, _P], _I),
    "troute_write_forcings": ([C.c_char_p, _I, _I, _I, _P, _P, _P, _P], _I),
    "troute_read_network": ([C.c_char_p, _P], _I),
    "troute_free_network": ([_P], None),
    "troute_write_network": ([C.c_char_p, _P], _I),
    "troute_debug_timeout_probe": ([C.c_longlong], _I),
    "troute_debug_pow": ([_P, _I, _P], _I),
    "troute_measure_fp64_rate": ([_P, _P], _I),
    "troute_debug_div": ([_P, _P, _I, _P], _I),
    "troute_debug_quot_gt": ([_P, _P, C.c_double, _I, _P], _I),
    "troute_levels": ([_I, _P, _P, _P, _P, _P, _P], _I),
    "troute_critical_path": ([_P, _I, _P], _I),
    "troute_validate": ([_P], _I),
    "troute_gen_tree": ([_U64, _I, _I, _I, _P, _P, _P, _P], _I),
    "troute_gen_params": ([_U64, _I, _P], _I),
    "troute_gen_qlat": ([_U64, _I, _I, _I, _D, _P], _I),
    "troute_gen_member": ([_U64, _I, _I, _P, _P], _I),
}


def library_path() -> str:
    return _build.LIB


def lib():
    """Loads libtroute_gb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        path = _build.LIB
        if not os.path.exists(path):
            raise ImportError(f"{path} is missing: build it with troute_gb300.build.build()")
        L = C.CDLL(path)
        for name, (argt, rest) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = argt
            fn.restype = rest
        _LIB = L
    return _LIB


def exported_symbols() -> list:
    return list(_SIGS)


def _check(rc: int):
    if rc != OK:
        raise TrouteError(rc, lib().troute_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _params(p):
    p = np.ascontiguousarray(p)
    if p.dtype == CHPARAMS_DTYPE:
        return p
    if p.dtype.names is not None:
        return np.ascontiguousarray(p.astype(CHPARAMS_DTYPE))
    p = np.ascontiguousarray(p, dtype=np.float64)
    if p.ndim != 2 or p.shape[1] != 8:
        raise ValueError("params must be a ChParams record array or an (n, 8) float array")
    return p.view(CHPARAMS_DTYPE).reshape(-1)


def make_cfg(rtol=0.01, atol=0.01, maxiter=100, attempts=5, **kw) -> Cfg:
    c = Cfg()
    lib().troute_cfg_default(C.byref(c))
    c.rtol, c.atol, c.maxiter, c.attempts = rtol, atol, maxiter, attempts
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def timeout_probe(wait_cycles: int = 2_000_000) -> int:
    """Runs the bounded-wait probe kernel; returns the status code (ETIMEOUT expected)."""
    return lib().troute_debug_timeout_probe(int(wait_cycles))


def measure_fp64_rate() -> dict:
    """The device's FP64 issue rate (independent DMUL chains on every SM):
    FP64 warp instructions per second and the probe launch's time."""
    r, ms = C.c_double(), C.c_double()
    _check(lib().troute_measure_fp64_rate(C.byref(r), C.byref(ms)))
    return {"warp_instr_per_s": r.value, "ms": ms.value}


def debug_pow(x):
    """Device evaluation of the solver's powers and CUDA's pow():
    (ours_23, ours_53, cuda_23, cuda_53)."""
    x = _f64(x)
    out = np.zeros(4 * x.size)
    _check(lib().troute_debug_pow(_ptr(x), int(x.size), _ptr(out)))
    return tuple(out.reshape(4, -1))


def debug_div(a, b):
    """The solver's shared-reciprocal quotient a / b evaluated on the device."""
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    out = np.zeros_like(a)
    _check(lib().troute_debug_div(_ptr(a), _ptr(b), a.size, _ptr(out)))
    return out


def debug_quot_gt(a, b, c):
    """The solver's convergence comparison a / b > c evaluated on the device
    (boolean array)."""
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    out = np.zeros(a.size, np.int32)
    _check(lib().troute_debug_quot_gt(_ptr(a), _ptr(b), float(c), a.size, _ptr(out)))
    return out.astype(bool)


def device_info() -> dict:
    sm, ma, mi, fr = _I(), _I(), _I(), C.c_size_t()
    _check(lib().troute_device_info(C.byref(sm), C.byref(ma), C.byref(mi), C.byref(fr)))
    return {"sm_count": sm.value, "cc": (ma.value, mi.value), "free_bytes": fr.value}


# ---------------------------------------------------------------------------
# reach-parallel (cpu_mc)
# ---------------------------------------------------------------------------
def mc_reach_parallel(p, ql, rs, rl, qu, qd, dp, uq: float = 10.0, dt: float = 300.0, cfg: Cfg | None = None,
                      return_stats: bool = False):
    """cpu_mc on the GPU: returns (qo, vo, dpo) (+ stats dict)."""
    p = _params(p)
    n = p.shape[0]
    ql, qu, qd, dp = (_f64(x, n) for x in (ql, qu, qd, dp))
    rs, rl = _i32(rs), _i32(rl)
    qo, vo, dpo = np.zeros(n), np.zeros(n), np.zeros(n)
    st = Stats()
    _check(lib().troute_mc_reach_parallel_cfg(
        _ptr(p), _ptr(ql), _ptr(rs), _ptr(rl), _ptr(qu), _ptr(qd), _ptr(dp), _ptr(qo), _ptr(vo), _ptr(dpo),
        float(uq), float(dt), int(rs.size), C.byref(cfg) if cfg is not None else None, C.byref(st)))
    return (qo, vo, dpo, st.as_dict()) if return_stats else (qo, vo, dpo)


# ---------------------------------------------------------------------------
# topology helpers
# ---------------------------------------------------------------------------
def _topo_struct(seg_start, seg_len, up_ptr, up_idx, n_segments):
    arrs = [_i32(seg_start), _i32(seg_len), _i32(up_ptr), _i32(up_idx if len(up_idx) else np.zeros(1, np.int32))]
    t = Topo()
    t.n_reaches = int(arrs[0].size)
    t.n_segments = int(n_segments)
    t.reach_seg_start, t.reach_seg_len, t.reach_up_ptr, t.reach_up_idx = (
        a.ctypes.data_as(C.POINTER(C.c_int)) for a in arrs)
    return t, arrs


def levels(up_ptr, up_idx):
    """Reference-style levels (gen_network.py:219-231): (reach_level, level_ptr, level_reach)."""
    up_ptr, up_idx = _i32(up_ptr), _i32(up_idx if len(up_idx) else np.zeros(1, np.int32))
    R = up_ptr.size - 1
    lv = np.zeros(max(R, 1), np.int32)
    lp = np.zeros(R + 1, np.int32)
    lr = np.zeros(max(R, 1), np.int32)
    nl = _I()
    _check(lib().troute_levels(R, _ptr(up_ptr), _ptr(up_idx), _ptr(lv), _ptr(lp), _ptr(lr), C.byref(nl)))
    return lv[:R], lp[: nl.value + 1], lr[:R]


def validate(seg_start, seg_len, up_ptr, up_idx, n_segments):
    t, _keep = _topo_struct(seg_start, seg_len, up_ptr, up_idx, n_segments)
    _check(lib().troute_validate(C.byref(t)))


def critical_path(topo: dict, n_ts: int) -> int:
    """Longest chain of segment solves in the (reach, step) dependency graph
    of an n_ts-step run (troute_critical_path)."""
    t, _keep = _topo_struct(topo["reach_seg_start"], topo["reach_seg_len"], topo["reach_up_ptr"],
                            topo["reach_up_idx"], topo["n_segments"])
    out = C.c_longlong()
    _check(lib().troute_critical_path(C.byref(t), int(n_ts), C.byref(out)))
    return int(out.value)


# ---------------------------------------------------------------------------
# tree routing
# ---------------------------------------------------------------------------
def wavefront_fp64(params_f32, seg_start, seg_len, up_ptr, up_idx, level_ptr, level_reach, qlat_ts_f32,
                   qdp0_f32, dp0_f32, reach_last0_f32, n_timesteps: int, dt: float = 300.0):
    """cpu_wavefront_fp64 drop-in: float inputs, (q_final, reach_last_final) doubles."""
    p = np.ascontiguousarray(params_f32)
    if p.dtype != CHPARAMS_F32_DTYPE:
        p = np.ascontiguousarray(np.asarray(p, np.float32).reshape(-1, 8)).view(CHPARAMS_F32_DTYPE).reshape(-1)
    S, R = p.shape[0], len(seg_start)
    ints = [_i32(x) for x in (seg_start, seg_len, up_ptr, up_idx if len(up_idx) else [0], level_ptr, level_reach)]
    fl = [np.ascontiguousarray(x, np.float32) for x in (qlat_ts_f32, qdp0_f32, dp0_f32, reach_last0_f32)]
    q, rl = np.zeros(S), np.zeros(R)
    _check(lib().troute_wavefront_fp64(_ptr(p), *(_ptr(a) for a in ints), R, len(level_ptr) - 1, S,
                                       *(_ptr(a) for a in fl), _ptr(q), _ptr(rl), int(n_timesteps), float(dt)))
    return q, rl


class Network:
    """A routed network (or a batch of networks) with device-resident state."""

    def __init__(self, topos, params, dt: float = 300.0, cfg: Cfg | None = None, qlat_col=None, qlat_scale=None,
                 qlat_cols: int = 0, _handle=None):
        if _handle is not None:
            self._h = _handle
            self._keep = []
            self._info()
            return
        if isinstance(topos, dict):
            topos, params = [topos], [params]
            qlat_col = None if qlat_col is None else [qlat_col]
            qlat_scale = None if qlat_scale is None else [qlat_scale]
        n = len(topos)
        self._keep = []
        tarr = (Topo * n)()
        parr = (C.c_void_p * n)()
        carr = (C.c_void_p * n)()
        sarr = (C.c_void_p * n)()
        self.n_segments_each = []
        self.n_reaches_each = []
        for i, t in enumerate(topos):
            ts, keep = _topo_struct(t["reach_seg_start"], t["reach_seg_len"], t["reach_up_ptr"], t["reach_up_idx"],
                                    t["n_segments"])
            tarr[i] = ts
            pp = _params(params[i])
            self._keep += keep + [pp]
            parr[i] = pp.ctypes.data
            self.n_segments_each.append(int(t["n_segments"]))
            self.n_reaches_each.append(int(len(t["reach_seg_start"])))
            if qlat_col is not None and qlat_col[i] is not None:
                c = _i32(qlat_col[i])
                self._keep.append(c)
                carr[i] = c.ctypes.data
            if qlat_scale is not None and qlat_scale[i] is not None:
                s = _f64(qlat_scale[i])
                self._keep.append(s)
                sarr[i] = s.ctypes.data
        h = C.c_void_p()
        _check(lib().troute_create_batch(C.byref(h), n, tarr, parr, carr if qlat_col is not None else None,
                                         sarr if qlat_scale is not None else None, int(qlat_cols), float(dt),
                                         C.byref(cfg) if cfg is not None else None))
        self._h = h
        self._keep = []  # the library copied everything
        self._info()

    def _info(self):
        R, S, L, Q, T = _I(), _I(), _I(), _I(), C.c_longlong()
        _check(lib().troute_info(self._h, C.byref(R), C.byref(S), C.byref(L), C.byref(Q), C.byref(T)))
        self.n_reaches, self.n_segments, self.n_levels, self.qlat_cols = R.value, S.value, L.value, Q.value

    @classmethod
    def ensemble(cls, topo: dict, params, n_members: int, n_scale=None, qlat_scale=None, dt: float = 300.0,
                 cfg: Cfg | None = None):
        """n_members copies of one network (Manning's n and lateral inflow
        scaled per member and segment); lateral inflow is the base
        [n_ts][n_segments] matrix."""
        ts, keep = _topo_struct(topo["reach_seg_start"], topo["reach_seg_len"], topo["reach_up_ptr"],
                                topo["reach_up_idx"], topo["n_segments"])
        pp = _params(params)
        S = int(topo["n_segments"])
        ns = None if n_scale is None else _f64(n_scale, n_members * S)
        qs = None if qlat_scale is None else _f64(qlat_scale, n_members * S)
        h = C.c_void_p()
        _check(lib().troute_create_ensemble(C.byref(h), C.byref(ts), _ptr(pp), int(n_members), _ptr(ns), _ptr(qs),
                                            float(dt), C.byref(cfg) if cfg is not None else None))
        return cls(None, None, _handle=h)

    def close(self):
        if getattr(self, "_h", None):
            lib().troute_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def steps_done(self) -> int:
        T = C.c_longlong()
        _check(lib().troute_info(self._h, None, None, None, None, C.byref(T)))
        return T.value

    def set_cfg(self, cfg: Cfg):
        _check(lib().troute_set_cfg(self._h, C.byref(cfg)))

    def set_state(self, qdp, dp, reach_last=None):
        q = _f64(qdp, self.n_segments)
        d = _f64(dp, self.n_segments)
        r = None if reach_last is None else _f64(reach_last, self.n_reaches)
        _check(lib().troute_set_state(self._h, _ptr(q), _ptr(d), _ptr(r)))

    def get_state(self, out=None):
        """(discharge, depth, velocity, reach outflow) in user order; `out`: four
        caller arrays (e.g. pinned host memory) to fill instead of new ones."""
        if out is None:
            out = (np.zeros(self.n_segments), np.zeros(self.n_segments), np.zeros(self.n_segments),
                   np.zeros(self.n_reaches))
        q, d, v, r = out
        for a, n in ((q, self.n_segments), (d, self.n_segments), (v, self.n_segments), (r, self.n_reaches)):
            if a.dtype != np.float64 or a.size != n or not a.flags["C_CONTIGUOUS"] or not a.flags["WRITEABLE"]:
                raise ValueError("get_state: out arrays must be contiguous writable float64 of the state's sizes")
        _check(lib().troute_get_state(self._h, _ptr(q), _ptr(d), _ptr(v), _ptr(r)))
        return q, d, v, r

    def run(self, qlat_ts) -> dict:
        ql = np.ascontiguousarray(qlat_ts, dtype=np.float64)
        if ql.ndim != 2 or ql.shape[1] != self.qlat_cols:
            raise ValueError(f"qlat must be [n_ts][{self.qlat_cols}]")
        st = Stats()
        _check(lib().troute_run(self._h, _ptr(ql), int(ql.shape[0]), C.byref(st)))
        return st.as_dict()

    def run_device(self, qlat_dev_ptr: int, n_ts: int, stream: int = 0):
        _check(lib().troute_run_device(self._h, C.c_void_p(qlat_dev_ptr), int(n_ts), C.c_void_p(stream)))

    def sync(self) -> dict:
        st = Stats()
        _check(lib().troute_sync(self._h, C.byref(st)))
        return st.as_dict()

    def graph_capture(self, qlat_dev_ptr: int, n_ts: int):
        _check(lib().troute_graph_capture(self._h, C.c_void_p(qlat_dev_ptr), int(n_ts)))

    def graph_launch(self, stream: int = 0):
        _check(lib().troute_graph_launch(self._h, C.c_void_p(stream)))

    def history(self, n_ts: int):
        out = np.zeros((n_ts, self.n_segments))
        _check(lib().troute_get_history(self._h, _ptr(out), int(n_ts)))
        return out

    def autotune(self, qlat_dev_ptr: int, n_ts: int, repeats: int = 1, all_mappings: bool = True) -> dict:
        """Times the candidate launch configurations on n_ts steps of the device
        lateral inflow at qlat_dev_ptr and keeps the fastest (state unchanged)."""
        r = TuneResult()
        _check(lib().troute_autotune(self._h, C.c_void_p(qlat_dev_ptr), int(n_ts), int(repeats),
                                     TUNE_ALL_MAPPINGS if all_mappings else 0, C.byref(r)))
        return r.as_dict()

    def set_warm_start(self, model: "WarmModel | None", delta: float = 0.05):
        """Attaches a trained model (None detaches); runs use it with cfg.warm_start = 1."""
        self._warm = model
        _check(lib().troute_set_warm_start(self._h, None if model is None else model._h, float(delta)))

    def pairs(self, out_dev_ptr: int = 0, capacity: int = 0) -> int:
        """Training pairs of the last run (cfg.record_pairs): copies up to
        `capacity` into the device buffer at out_dev_ptr; returns how many exist."""
        n = C.c_longlong()
        _check(lib().troute_get_pairs(self._h, C.c_void_p(out_dev_ptr or None), int(capacity), C.byref(n)))
        return n.value

    def start_history(self, n_ts: int):
        """Learned starting depth of every solve of the last run (cfg.record_start), 0 = plain start."""
        out = np.zeros((n_ts, self.n_segments))
        _check(lib().troute_get_start_history(self._h, _ptr(out), int(n_ts)))
        return out

    def checkpoint(self) -> bytes:
        n = C.c_size_t(0)
        _check(lib().troute_checkpoint(self._h, None, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        _check(lib().troute_checkpoint(self._h, buf, C.byref(n)))
        return buf.raw[: n.value]

    def restore(self, blob: bytes):
        buf = C.create_string_buffer(blob, len(blob))
        _check(lib().troute_restore(self._h, buf, len(blob)))


class TuneResult(C.Structure):
    _fields_ = [("mapping", C.c_int), ("blocks_per_sm", C.c_int), ("threads_per_block", C.c_int),
                ("schedule_flags", C.c_int), ("best_ms", C.c_double), ("default_ms", C.c_double),
                ("n_trials", C.c_int), ("trial_cfg", (C.c_int * 4) * 32), ("trial_ms", C.c_double * 32)]

    def as_dict(self) -> dict:
        n = self.n_trials
        return {"mapping": self.mapping, "blocks_per_sm": self.blocks_per_sm,
                "threads_per_block": self.threads_per_block, "schedule_flags": self.schedule_flags,
                "best_ms": self.best_ms, "default_ms": self.default_ms,
                "trials": [{"mapping": self.trial_cfg[i][0], "blocks_per_sm": self.trial_cfg[i][1],
                            "threads": self.trial_cfg[i][2], "flags": self.trial_cfg[i][3], "ms": self.trial_ms[i]}
                           for i in range(n)]}


TUNE_ALL_MAPPINGS = 1


class NetFile(C.Structure):
    _fields_ = [("n_reaches", C.c_int), ("n_segments", C.c_int), ("n_levels", C.c_int), ("max_upstream", C.c_int),
                ("n_ts", C.c_int)] + [(k, C.c_void_p) for k in (
                    "reach_seg_start", "reach_seg_len", "reach_level", "reach_n_up", "reach_up_ptr", "reach_up_idx",
                    "level_ptr", "level_reach", "params", "qlat", "qup0", "qdp0", "dp0")]


_NET_INT = ("reach_seg_start", "reach_seg_len", "reach_level", "reach_n_up", "reach_up_ptr", "reach_up_idx",
            "level_ptr", "level_reach")


def read_network(path: str) -> dict:
    """Reads a topo.bin / params.bin / forcings.bin directory (the reference's
    format) -> dict of numpy arrays (params as float32 ChParams records)."""
    ptr = C.POINTER(NetFile)()
    _check(lib().troute_read_network(os.fsencode(path), C.byref(ptr)))
    try:
        n = ptr.contents
        R, S, L, T = n.n_reaches, n.n_segments, n.n_levels, n.n_ts
        nnz = int(np.ctypeslib.as_array(C.cast(n.reach_up_ptr, C.POINTER(C.c_int)), (R + 1,))[R])
        sizes = {"reach_seg_start": R, "reach_seg_len": R, "reach_level": R, "reach_n_up": R,
                 "reach_up_ptr": R + 1, "reach_up_idx": nnz, "level_ptr": L + 1, "level_reach": R}
        out = {"n_reaches": R, "n_segments": S, "n_levels": L, "max_upstream": n.max_upstream, "n_ts": T}
        for k, m in sizes.items():
            a = getattr(n, k)
            out[k] = np.ctypeslib.as_array(C.cast(a, C.POINTER(C.c_int)), (m,)).copy() if m else np.zeros(0, np.int32)
        pf = np.ctypeslib.as_array(C.cast(n.params, C.POINTER(C.c_float)), (S * 8,)).copy() if S else np.zeros(0, np.float32)
        out["params"] = pf.view(CHPARAMS_F32_DTYPE).reshape(-1)
        f = lambda a, m: (np.ctypeslib.as_array(C.cast(a, C.POINTER(C.c_float)), (m,)).copy() if m
                          else np.zeros(0, np.float32))
        out["qlat"] = f(n.qlat, T * S).reshape(T, S)
        out["qup0"], out["qdp0"], out["dp0"] = f(n.qup0, R), f(n.qdp0, S), f(n.dp0, S)
        return out
    finally:
        lib().troute_free_network(ptr)


def write_network(path: str, net: dict):
    """Writes a dict as returned by read_network as the reference's three files
    (topo.bin and params.bin only when the dict has no "qlat")."""
    keep = {}

    def arr(k, dt):
        a = np.ascontiguousarray(net[k], dt)
        keep[k] = a
        return a.ctypes.data_as(C.c_void_p)

    n = NetFile()
    n.n_reaches, n.n_segments, n.n_levels = int(net["n_reaches"]), int(net["n_segments"]), int(net["n_levels"])
    has_forcings = net.get("qlat") is not None
    n.max_upstream, n.n_ts = int(net["max_upstream"]), int(net["qlat"].shape[0]) if has_forcings else 0
    for k in _NET_INT:
        setattr(n, k, arr(k, np.int32))
    p = np.ascontiguousarray(net["params"])
    if p.dtype != CHPARAMS_F32_DTYPE:
        p = np.ascontiguousarray(np.asarray(p, np.float32).reshape(-1, 8)).view(CHPARAMS_F32_DTYPE).reshape(-1)
    keep["params"] = p
    n.params = p.ctypes.data_as(C.c_void_p)
    if has_forcings:
        for k in ("qlat", "qup0", "qdp0", "dp0"):
            setattr(n, k, arr(k, np.float32))
    os.makedirs(path, exist_ok=True)
    _check(lib().troute_write_network(os.fsencode(path), C.byref(n)))


def _f32_params(p):
    p = np.ascontiguousarray(p)
    if p.dtype != CHPARAMS_F32_DTYPE:
        p = np.ascontiguousarray(np.asarray(p, np.float32).reshape(-1, 8)).view(CHPARAMS_F32_DTYPE).reshape(-1)
    return p


def linear_coeffs(params_f32, dt: float = 300.0):
    """Linearised-MC coefficients (C1, C2, C3, C4/ql), float32, computed on the device."""
    p = _f32_params(params_f32)
    n = p.shape[0]
    c = [np.zeros(n, np.float32) for _ in range(4)]
    _check(lib().troute_linear_coeffs(_ptr(p), n, float(dt), *(_ptr(x) for x in c)))
    return c


def linear_route(topo: dict, coeffs, qlat_ts, q0):
    """cpu_linear_mc drop-in on the GPU: float coefficients, lateral inflow
    [n_ts][n_segments] and initial discharge -> final discharge (float32)."""
    S = int(topo["n_segments"])
    t = _topo_struct(topo["reach_seg_start"], topo["reach_seg_len"], topo["reach_up_ptr"], topo["reach_up_idx"], S)
    cs = [np.ascontiguousarray(c, np.float32) for c in coeffs]
    ql = np.ascontiguousarray(qlat_ts, np.float32)
    q = np.ascontiguousarray(q0, np.float32)
    out = np.zeros(S, np.float32)
    _check(lib().troute_linear_route(C.byref(t[0]), *(_ptr(c) for c in cs), _ptr(ql), _ptr(q), int(ql.shape[0]),
                                     _ptr(out)))
    return out


def matrix_coeffs(params_f32, dt: float = 300.0):
    """Matrix-form coefficients (C1, C2, C3, C4/ql) at X = 0.25 per reach,
    float32, computed on the device."""
    p = _f32_params(params_f32)
    n = p.shape[0]
    c = [np.zeros(n, np.float32) for _ in range(4)]
    _check(lib().troute_matrix_coeffs(_ptr(p), n, float(dt), *(_ptr(x) for x in c)))
    return c


def matrix_route(up_ptr, up_idx, coeffs, qlat_ts, q0, tol: float = 1e-7):
    """The matrix form on the GPU, one shot: reach-level upstream CSR (reaches
    numbered upstream first), coefficients, lateral inflow [n_ts][n_reaches]
    and initial discharge -> final discharge (float32)."""
    up_ptr, up_idx = _i32(up_ptr), _i32(up_idx if len(up_idx) else np.zeros(1, np.int32))
    R = up_ptr.size - 1
    cs = [np.ascontiguousarray(c, np.float32) for c in coeffs]
    ql = np.ascontiguousarray(qlat_ts, np.float32)
    q = np.ascontiguousarray(q0, np.float32)
    out = np.zeros(R, np.float32)
    _check(lib().troute_matrix_route(R, _ptr(up_ptr), _ptr(up_idx), *(_ptr(c) for c in cs), float(tol), _ptr(ql),
                                     _ptr(q), int(ql.shape[0]), _ptr(out)))
    return out


class MatrixNetwork:
    """Persistent device form of the matrix-form linear MC (troute_matrix_*)."""

    def __init__(self, up_ptr, up_idx, coeffs, tol: float = 1e-7):
        up_ptr, up_idx = _i32(up_ptr), _i32(up_idx if len(up_idx) else np.zeros(1, np.int32))
        cs = [np.ascontiguousarray(c, np.float32) for c in coeffs]
        self._h = C.c_void_p()
        _check(lib().troute_matrix_create(C.byref(self._h), up_ptr.size - 1, _ptr(up_ptr), _ptr(up_idx),
                                          *(_ptr(c) for c in cs), float(tol)))
        R, nq, nl = _I(), C.c_longlong(), C.c_longlong()
        _check(lib().troute_matrix_info(self._h, C.byref(R), C.byref(nq), C.byref(nl)))
        self.n_reaches, self.nnz_Q, self.nnz_q = R.value, nq.value, nl.value

    def matrices(self):
        """((ptr, col, val) of P_Q, (ptr, col, val) of P_q), host copies."""
        out = []
        for which, nnz in ((0, self.nnz_Q), (1, self.nnz_q)):
            ptr = np.zeros(self.n_reaches + 1, np.int32)
            col, val = np.zeros(max(nnz, 1), np.int32), np.zeros(max(nnz, 1), np.float32)
            _check(lib().troute_matrix_get(self._h, which, _ptr(ptr), _ptr(col), _ptr(val)))
            out.append((ptr, col[:nnz], val[:nnz]))
        return tuple(out)

    def run_device(self, qlat_dev_ptr: int, n_ts: int, q_dev_ptr: int, stream: int = 0):
        _check(lib().troute_matrix_run_device(self._h, C.c_void_p(qlat_dev_ptr), int(n_ts), C.c_void_p(q_dev_ptr),
                                              C.c_void_p(stream)))

    def close(self):
        if self._h:
            lib().troute_matrix_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


DIFF_REACH_DTYPE = np.dtype([("ncomp", "<i4"), ("theta", "<f4"), ("dtini", "<f4")])


def diffusive_tridiag(reaches, dx, diffusivity, qp_prev, qp_out=None, celerity=None):
    """cpu_diffusive_tridiag drop-in on the GPU: [n_reaches][max_nodes] float
    arrays, reaches with (ncomp, theta, dtini); returns qp_out."""
    rp = np.ascontiguousarray(reaches, DIFF_REACH_DTYPE)
    dx, df, qp = (np.ascontiguousarray(a, np.float32) for a in (dx, diffusivity, qp_prev))
    n, m = qp.shape
    out = np.zeros_like(qp) if qp_out is None else np.ascontiguousarray(qp_out, np.float32).copy()
    cel = None if celerity is None else np.ascontiguousarray(celerity, np.float32)
    _check(lib().troute_diffusive_tridiag(_ptr(rp), _ptr(dx), _ptr(df), _ptr(cel), _ptr(qp), _ptr(out), n, m))
    return out


class LinearNetwork:
    """Persistent device form of the linearised MC (troute_linear_*)."""

    def __init__(self, topo: dict, coeffs):
        S = int(topo["n_segments"])
        self._t = _topo_struct(topo["reach_seg_start"], topo["reach_seg_len"], topo["reach_up_ptr"],
                               topo["reach_up_idx"], S)
        cs = [np.ascontiguousarray(c, np.float32) for c in coeffs]
        self._h = C.c_void_p()
        _check(lib().troute_linear_create(C.byref(self._h), C.byref(self._t[0]), *(_ptr(c) for c in cs)))
        self.n_segments = S

    def run_device(self, qlat_dev_ptr: int, n_ts: int, q_dev_ptr: int, wait_cycles: int = 0, stream: int = 0):
        _check(lib().troute_linear_run_device(self._h, C.c_void_p(qlat_dev_ptr), int(n_ts), C.c_void_p(q_dev_ptr),
                                              int(wait_cycles), C.c_void_p(stream)))

    def close(self):
        if self._h:
            lib().troute_linear_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def qlat_from_csv(csv_dir: str, reach_ids, n_ts: int, n_threads: int = 0):
    """Parallel pivot of nex-<id>_output.csv files -> (qlat [n_ts][n_reaches]
    float32, files matched, files missing)."""
    ids = np.ascontiguousarray(reach_ids, np.int64)
    out = np.zeros((n_ts, ids.size), np.float32)
    m, x = C.c_longlong(), C.c_longlong()
    _check(lib().troute_qlat_from_csv(os.fsencode(csv_dir), _ptr(ids), ids.size, int(n_ts), int(n_threads),
                                      _ptr(out), C.byref(m), C.byref(x)))
    return out, m.value, x.value


def write_forcings(path: str, qlat, qup0, qdp0, dp0):
    """forcings.bin writer (n_reaches from qup0, n_segments from qdp0)."""
    ql = np.ascontiguousarray(qlat, np.float32)
    a, b, c = (np.ascontiguousarray(v, np.float32) for v in (qup0, qdp0, dp0))
    _check(lib().troute_write_forcings(os.fsencode(path), ql.shape[0], a.size, b.size, _ptr(ql), _ptr(a), _ptr(b),
                                       _ptr(c)))


WARM_NPARAMS = 4801
WARM_NSTATE = WARM_NPARAMS + 18
PAIR_FLOATS = 9


class WarmModel:
    """The learned warm start's MLP (8 -> 64 -> 64 -> 1, SiLU), held by the library.

    State vector (get_state / set_state): W1 [64][8], b1 [64], W2 [64][64],
    b2 [64], w3 [64], b3, then mu[8], sd[8], mu_y, sd_y (standardisation of
    the log inputs and log depth)."""

    def __init__(self, seed: int = 0):
        self._h = C.c_void_p()
        _check(lib().troute_warm_create(C.byref(self._h), C.c_uint64(seed)))

    def close(self):
        if self._h:
            lib().troute_warm_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_state(self) -> np.ndarray:
        out = np.zeros(WARM_NSTATE, np.float32)
        _check(lib().troute_warm_get(self._h, _ptr(out), out.size))
        return out

    def set_state(self, state):
        st = np.ascontiguousarray(state, np.float32)
        if st.size != WARM_NSTATE:
            raise ValueError(f"state must hold {WARM_NSTATE} floats")
        _check(lib().troute_warm_set(self._h, _ptr(st), st.size))

    def fit(self, pairs_dev_ptr: int, n_pairs: int, epochs: int = 4, batch: int = 8192, lr: float = 2e-3,
            weight_decay: float = 1e-4, seed: int = 0) -> np.ndarray:
        """Trains on device-resident pairs [n_pairs][9]; returns the loss of each epoch."""
        loss = np.zeros(epochs, np.float32)
        _check(lib().troute_warm_fit(self._h, C.c_void_p(pairs_dev_ptr), int(n_pairs), int(epochs), int(batch),
                                     float(lr), float(weight_decay), C.c_uint64(seed), _ptr(loss)))
        return loss

    def grad(self, pairs) -> tuple:
        """(gradient [WARM_NPARAMS], loss) of mean (err^2)/2 over host pairs [n][9]."""
        pr = np.ascontiguousarray(pairs, np.float32).reshape(-1, PAIR_FLOATS)
        g = np.zeros(WARM_NPARAMS, np.float32)
        loss = C.c_double()
        _check(lib().troute_warm_grad(self._h, _ptr(pr), pr.shape[0], _ptr(g), C.byref(loss)))
        return g, loss.value

    def predict(self, inputs) -> np.ndarray:
        """Predicted depths for host rows [n][8] (qup quc qdp ql dx s0 n bw), through
        the tcgen05 GEMM that fills a warm-started launch's starting depths."""
        x = np.ascontiguousarray(inputs, np.float32).reshape(-1, 8)
        out = np.zeros(x.shape[0])
        _check(lib().troute_warm_predict(self._h, _ptr(x), x.shape[0], _ptr(out)))
        return out



def route_tree(topo: dict, params, qlat_ts, qdp0, dp0, reach_last0=None, dt: float = 300.0, cfg: Cfg | None = None,
               history: bool = False):
    """One-shot FP64 tree routing; returns dict(q, d, v, reach_last, stats[, q_hist])."""
    c = cfg if cfg is not None else make_cfg()
    if history:
        c = Cfg.from_buffer_copy(c)
        c.record_history = 1
    with Network(topo, params, dt=dt, cfg=c) as net:
        net.set_state(qdp0, dp0, reach_last0)
        ql = np.ascontiguousarray(qlat_ts, dtype=np.float64)
        st = net.run(ql)
        q, d, v, r = net.get_state()
        out = {"q": q, "d": d, "v": v, "reach_last": r, "stats": st}
        if history:
            out["q_hist"] = net.history(ql.shape[0])
        return out
