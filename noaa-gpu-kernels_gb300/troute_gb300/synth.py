"""Seeded synthetic workloads of the MC routing benchmark (host-side, via the
library's platform-independent generator).

  c0  random binary merge tree, 1,000 segments in ~200 reaches of 1-10
      segments, 288 steps (CPU-runnable parity case)
  c1  2.7M segments in ~1.1M reaches (uniform random binary tree with 550,000
      headwaters: Horton bifurcation ratio ~4), 144 steps. The depth of such
      a tree varies with the seed (1,666 to 4,287 levels over seeds
      1001-1030); seed 1010 gives 3,016 levels, the specified ~3,000
  c3  c1's sizes on a fresh seed (2006: 2,912 levels), for the warm start
      trained on c1
  c2  256 independent trees with LogU(500, 200,000) segments, 288 steps
  c4  64 ensemble members of the c1 network: lateral inflow x LogN(0, 0.3),
      Manning's n x U(0.8, 1.2), 288 steps
Parameters: dx~U(500,5000) m, s0~LogU(1e-5,1e-2), n~U(.03,.08), ncc=2n,
bw~U(2,50) m, tw=3bw, twcc=5tw, cs~U(.5,2); lateral inflow Gamma(2, 0.05)
m3/s x diurnal sine; initial discharge 0.1 m3/s, initial depth 0.1 m; dt=300 s.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .api import CHPARAMS_DTYPE, _check, _ptr, lib

DT = 300.0
Q0 = 0.1
D0 = 0.1
SEG_PER_REACH = 2.7e6 / 1.1e6
C1_SEED = 1010   # 3,016 levels
C3_SEED = 2006   # 2,912 levels


def make_tree(seed: int, n_leaves: int, n_segments: int, max_len: int = 10) -> dict:
    R = 2 * n_leaves - 1
    seg_start = np.zeros(R, np.int32)
    seg_len = np.zeros(R, np.int32)
    up_ptr = np.zeros(R + 1, np.int32)
    up_idx = np.zeros(max(R - 1, 1), np.int32)
    _check(lib().troute_gen_tree(C.c_uint64(seed), int(n_leaves), int(n_segments), int(max_len), _ptr(seg_start),
                                 _ptr(seg_len), _ptr(up_ptr), _ptr(up_idx)))
    return {"n_segments": int(n_segments), "reach_seg_start": seg_start, "reach_seg_len": seg_len,
            "reach_up_ptr": up_ptr, "reach_up_idx": up_idx[: R - 1]}


def make_params(seed: int, n_segments: int) -> np.ndarray:
    p = np.zeros(n_segments, CHPARAMS_DTYPE)
    _check(lib().troute_gen_params(C.c_uint64(seed), int(n_segments), _ptr(p)))
    return p


def make_qlat(seed: int, n_segments: int, n_ts: int, t0: int = 0, dt: float = DT) -> np.ndarray:
    q = np.zeros((n_ts, n_segments))
    _check(lib().troute_gen_qlat(C.c_uint64(seed), int(n_segments), int(t0), int(n_ts), float(dt), _ptr(q)))
    return q


def make_member(seed: int, member: int, n_segments: int):
    qf, nf = np.zeros(n_segments), np.zeros(n_segments)
    _check(lib().troute_gen_member(C.c_uint64(seed), int(member), int(n_segments), _ptr(qf), _ptr(nf)))
    return qf, nf


def initial_state(topo: dict):
    S = topo["n_segments"]
    q0 = np.full(S, Q0)
    d0 = np.full(S, D0)
    rl0 = np.full(len(topo["reach_seg_start"]), Q0)
    return q0, d0, rl0


def tree_size(n_segments: int) -> int:
    """Headwaters for a tree with ~2.45 segments per reach."""
    n_leaves = max(1, int(round(n_segments / SEG_PER_REACH / 2.0)))
    return min(n_leaves, (n_segments + 1) // 2)


def network(name: str, seed: int | None = None, n_ts: int | None = None, with_qlat: bool = True) -> dict:
    """One of the single-network workloads ('c0', 'c1', 'c3' or 'tree:<segments>')."""
    if name == "c0":
        seed = 1000 if seed is None else seed
        topo = make_tree(seed, 100, 1000, 10)
        T = 288 if n_ts is None else n_ts
    elif name in ("c1", "c3"):
        seed = (C1_SEED if name == "c1" else C3_SEED) if seed is None else seed
        topo = make_tree(seed, 550_000, 2_700_000, 10)
        T = 144 if n_ts is None else n_ts
    elif name.startswith("tree:"):
        # tree:<segments>
        S = int(name.split(":")[1])
        seed = 7 if seed is None else seed
        topo = make_tree(seed, tree_size(S), S, 10)
        T = 24 if n_ts is None else n_ts
    else:
        raise ValueError(name)
    S = topo["n_segments"]
    out = {"name": name, "seed": seed, "topo": topo, "params": make_params(seed, S), "n_ts": T, "dt": DT}
    out["q0"], out["d0"], out["rl0"] = initial_state(topo)
    if with_qlat:
        out["qlat"] = make_qlat(seed, S, T)
    return out


def basin_sizes(seed: int = 1002, n_trees: int = 256, lo: float = 500.0, hi: float = 200_000.0,
                scale: float = 1.0) -> np.ndarray:
    """c2's segment counts: LogU(lo, hi) per tree (times `scale`), at least 3."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n_trees)) * scale
    return np.maximum(3, np.round(sizes)).astype(int)


def basins(seed: int = 1002, n_trees: int = 256, lo: float = 500.0, hi: float = 200_000.0, scale: float = 1.0,
           which=None):
    """c2: independent trees with LogU(lo, hi) segments each (times `scale`);
    `which` selects basins by index (a rank's share), default all."""
    sizes = basin_sizes(seed, n_trees, lo, hi, scale)
    nets = []
    for i in (range(n_trees) if which is None else which):
        S = int(sizes[i])
        s = seed * 1000 + i
        topo = make_tree(s, tree_size(S), S, 10)
        nets.append({"topo": topo, "params": make_params(s, S), "seed": s, "index": int(i)})
    return nets
