"""Hydrofabric ingest: a GeoPackage's `flowpaths` and `flowpath-attributes`
tables -> the river network the routing takes (one segment per waterbody),
written as topo.bin / params.bin plus the waterbody id of every reach.

The rules are those of the reference's
water-prediction/t-route/wavefront/data_parsers/parse_gpkg.py (:43-270), so
the files agree byte for byte:
- ids are the integer after the first '-' ("wb-12" -> 12); rows whose id has
  none are skipped, a repeated waterbody id keeps its first row;
- flow goes from wb-X to wb-M when X's toid is nex-M (or any other prefix)
  and wb-M exists; otherwise wb-X is an outlet;
- reaches are renumbered in the order of a last-in-first-out Kahn
  topological sort of that graph (headwaters in index order on the stack);
  a cycle is an error;
- a reach's level is 1 + the largest level upstream; levels are listed in
  reach order;
- channel parameters start from defaults (dx 1000 m, bw 20 m, tw 25 m,
  twcc 60 m, n 0.06, ncc 0.12, cs 2, s0 0.001) and each attribute row of a
  known waterbody, in table order, overrides the positive values it has,
  with floors (dx >= 100 m, n >= 0.01, ncc >= 0.02, cs >= 0.1,
  s0 >= 1e-5); a top width not above the bottom width becomes 1.2 bw, a
  compound-channel top width not above the top width becomes 3 tw; the
  parameters are float32 and are computed as such.
"""
from __future__ import annotations

import os
import sqlite3

import numpy as np

from .api import CHPARAMS_F32_DTYPE, write_network

_DEFAULTS = (1000.0, 20.0, 25.0, 60.0, 0.06, 0.12, 2.0, 0.001)  # dx bw tw twcc n ncc cs s0


def _id_of(s):
    """The integer after the first '-' of an id string, else None."""
    if s is None or "-" not in s:
        return None
    try:
        return int(s.split("-", 1)[1])
    except ValueError:
        return None


def _positive(v) -> bool:
    return bool(v) and v > 0


def _graph(con):
    """Waterbody ids in first-seen order and, per waterbody, the indices of
    those draining into it."""
    wb, down_id = [], []
    seen = set()
    for id_s, toid_s in con.execute("SELECT id, toid FROM flowpaths"):
        w = _id_of(id_s)
        if w is None or w in seen:
            continue
        seen.add(w)
        wb.append(w)
        t = _id_of(toid_s)
        down_id.append(-1 if t is None else t)
    index = {w: i for i, w in enumerate(wb)}
    ups = [[] for _ in wb]
    for i, t in enumerate(down_id):
        if t >= 0 and t in index:
            ups[index[t]].append(i)
    return np.asarray(wb, np.int64), index, ups


def _topological_order(ups):
    """Last-in-first-out Kahn order of the reaches (upstream before downstream)."""
    n = len(ups)
    pending = np.array([len(u) for u in ups], np.int64)
    downs = [[] for _ in range(n)]
    for v, us in enumerate(ups):
        for u in us:
            downs[u].append(v)
    stack = [i for i in range(n) if pending[i] == 0]
    order = []
    while stack:
        u = stack.pop()
        order.append(u)
        for d in downs[u]:
            pending[d] -= 1
            if pending[d] == 0:
                stack.append(d)
    if len(order) != n:
        raise ValueError(f"the flowpaths contain a cycle ({n - len(order)} waterbodies never become ready)")
    return np.asarray(order, np.int64)


def _apply_attributes(p, row):
    """One attribute row onto a reach's float32 parameters p (dx bw tw twcc n ncc cs s0)."""
    length_m, n_ch, ncc, bw, tw, twcc, cs, s0 = row
    if _positive(length_m):
        p[0] = max(100.0, float(length_m))
    if _positive(bw):
        p[1] = float(bw)
    # widths are compared with, and scaled from, the stored float32 values
    # (a NumPy float32 scalar against a Python float, as the files were made)
    p[2] = tw if (_positive(tw) and tw > p[1]) else p[1] * 1.2
    p[3] = twcc if (_positive(twcc) and twcc > p[2]) else p[2] * 3.0
    if _positive(n_ch):
        p[4] = max(0.01, float(n_ch))
    if _positive(ncc):
        p[5] = max(0.02, float(ncc))
    if _positive(cs):
        p[6] = max(0.1, float(cs))
    if _positive(s0):
        p[7] = max(1e-5, float(s0))


def read_gpkg(path: str) -> dict:
    """The network of a GeoPackage hydrofabric: the arrays of
    troute_gb300.read_network (without forcings) plus `topo_to_wbid`, the
    waterbody id of each reach."""
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    con = sqlite3.connect(f"file:{path}?mode=ro", uri=True)
    try:
        wb, index, ups = _graph(con)
        n = wb.size
        if n == 0:
            raise ValueError(f"{path}: no waterbodies in flowpaths")
        order = _topological_order(ups)
        new_of = np.empty(n, np.int64)
        new_of[order] = np.arange(n)
        new_ups = [None] * n
        for old, us in enumerate(ups):
            new_ups[new_of[old]] = sorted(int(new_of[u]) for u in us)
        level = np.zeros(n, np.int32)
        for r in range(n):
            if new_ups[r]:
                level[r] = 1 + max(level[u] for u in new_ups[r])
        n_up = np.array([len(u) for u in new_ups], np.int32)
        params = np.tile(np.asarray(_DEFAULTS, np.float32), (n, 1))
        for link, *row in con.execute('SELECT link, "Length_m", "n", "nCC", "BtmWdth", "TopWdth", "TopWdthCC", '
                                      '"ChSlp", "So" FROM "flowpath-attributes"'):
            w = _id_of(link)
            if w is None or w not in index:
                continue
            _apply_attributes(params[new_of[index[w]]], row)
    finally:
        con.close()
    n_levels = int(level.max()) + 1
    counts = np.bincount(level, minlength=n_levels)
    topo_to_wbid = np.empty(n, np.int64)
    topo_to_wbid[new_of] = wb
    return {
        "n_reaches": int(n), "n_segments": int(n), "n_levels": n_levels, "max_upstream": int(n_up.max()),
        "reach_seg_start": np.arange(n, dtype=np.int32), "reach_seg_len": np.ones(n, np.int32),
        "reach_level": level, "reach_n_up": n_up,
        "reach_up_ptr": np.concatenate([[0], np.cumsum(n_up)]).astype(np.int32),
        "reach_up_idx": np.fromiter((u for us in new_ups for u in us), np.int32, int(n_up.sum())),
        "level_ptr": np.concatenate([[0], np.cumsum(counts)]).astype(np.int32),
        "level_reach": np.argsort(level, kind="stable").astype(np.int32),
        "params": np.ascontiguousarray(params).view(CHPARAMS_F32_DTYPE).reshape(-1),
        "topo_to_wbid": topo_to_wbid,
    }


def gpkg_to_network(gpkg: str, out_dir: str) -> dict:
    """Writes out_dir/topo.bin, params.bin (the library's network writer) and
    topo_to_wbid.npy for a GeoPackage hydrofabric; returns the network."""
    net = read_gpkg(gpkg)
    write_network(out_dir, net)
    np.save(os.path.join(out_dir, "topo_to_wbid.npy"), net["topo_to_wbid"])
    return net
