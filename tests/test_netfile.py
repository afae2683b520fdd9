"""The reference's on-disk network format (topo.bin, params.bin, forcings.bin).

tests/golden/refnet/ was written by the reference's own generator and writers
(water-prediction/t-route/wavefront/gen_network.py) and refnet_out.npz by the
reference's own cpu_wavefront_fp64 on those files (tests/golden/make_refnet.py).
CPU tests: the library's reader against an independent parse of the documented
layout, byte-identical round trips through its writer, rejection of damaged
files, and the oracle against the reference's outputs. GPU tests: the CUDA
routing of the file-loaded network against the same outputs.
"""
import os
import shutil
import struct

import numpy as np
import pytest

import troute_gb300 as T
from golden_inputs import GOLDEN
from oracle import troute_oracle as O

REFNET = os.path.join(GOLDEN, "refnet")
FILES = ("topo.bin", "params.bin", "forcings.bin")


def parse_by_hand(d):
    """Independent numpy parse of the layout written by gen_network.py:292-337."""
    topo = open(os.path.join(d, "topo.bin"), "rb").read()
    R, S, L, mx = struct.unpack_from("<iiii", topo, 0)
    a = np.frombuffer(topo, "<i4", offset=16)
    o = 0
    out = {"n_reaches": R, "n_segments": S, "n_levels": L, "max_upstream": mx}
    for k, n in (("reach_seg_start", R), ("reach_seg_len", R), ("reach_level", R), ("reach_n_up", R),
                 ("reach_up_ptr", R + 1)):
        out[k] = a[o:o + n]
        o += n
    nnz = int(out["reach_up_ptr"][-1])
    out["reach_up_idx"] = a[o:o + nnz]
    o += nnz
    out["level_ptr"] = a[o:o + L + 1]
    o += L + 1
    out["level_reach"] = a[o:o + R]
    o += R
    assert o == a.size
    out["params"] = np.fromfile(os.path.join(d, "params.bin"), "<f4").reshape(S, 8)
    f = open(os.path.join(d, "forcings.bin"), "rb").read()
    nts = struct.unpack_from("<i", f, 0)[0]
    b = np.frombuffer(f, "<f4", offset=4)
    out["n_ts"] = nts
    out["qlat"] = b[:nts * S].reshape(nts, S)
    out["qup0"] = b[nts * S:nts * S + R]
    out["qdp0"] = b[nts * S + R:nts * S + R + S]
    out["dp0"] = b[nts * S + R + S:]
    assert out["dp0"].size == S
    return out


def test_reader_matches_the_documented_layout():
    n = T.read_network(REFNET)
    h = parse_by_hand(REFNET)
    for k, v in h.items():
        if k == "params":
            np.testing.assert_array_equal(n["params"].view("<f4").reshape(-1, 8), v)
        elif isinstance(v, np.ndarray):
            np.testing.assert_array_equal(n[k], v)
        else:
            assert n[k] == v, k
    assert n["n_reaches"] > 200 and n["n_ts"] == 12


def test_writer_round_trip_is_byte_identical(tmp_path):
    n = T.read_network(REFNET)
    T.write_network(str(tmp_path), n)
    for f in FILES:
        assert open(os.path.join(REFNET, f), "rb").read() == open(tmp_path / f, "rb").read(), f


@pytest.mark.parametrize("damage", ["truncate_topo", "trailing_params", "bad_csr", "bad_level", "missing"])
def test_damaged_files_are_rejected(tmp_path, damage):
    for f in FILES:
        shutil.copy(os.path.join(REFNET, f), tmp_path / f)
    p = tmp_path / "topo.bin"
    raw = bytearray(open(p, "rb").read())
    R = struct.unpack_from("<i", raw, 0)[0]
    if damage == "truncate_topo":
        open(p, "wb").write(raw[:-5])
    elif damage == "trailing_params":
        open(tmp_path / "params.bin", "ab").write(b"\0\0\0\0")
    elif damage == "bad_csr":
        # an upstream index outside [0, n_reaches)
        off = 16 + 4 * (4 * R + R + 1)
        struct.pack_into("<i", raw, off, R + 5)
        open(p, "wb").write(raw)
    elif damage == "bad_level":
        # reach 0 claims a level beyond n_levels
        struct.pack_into("<i", raw, 16 + 4 * 2 * R, 10 ** 6)
        open(p, "wb").write(raw)
    else:
        os.remove(tmp_path / "forcings.bin")
    with pytest.raises(T.TrouteError) as e:
        T.read_network(str(tmp_path))
    assert e.value.code in (2, 7)  # TROUTE_ETOPO, TROUTE_EIO


def _topo(n):
    t = {k: n[k] for k in ("reach_seg_start", "reach_seg_len", "reach_up_ptr", "reach_up_idx")}
    t["n_segments"] = n["n_segments"]
    return t


def test_oracle_matches_reference_outputs_on_the_files():
    n = T.read_network(REFNET)
    g = np.load(os.path.join(GOLDEN, "refnet_out.npz"))
    p64 = n["params"].view("<f4").reshape(-1, 8).astype(np.float64)
    for steps in (1, 12):
        o = O.route_tree(_topo(n), p64, n["qlat"][:steps].astype(np.float64), n["qdp0"].astype(np.float64),
                         n["dp0"].astype(np.float64), n["qup0"].astype(np.float64),
                         level_ptr=n["level_ptr"], level_reach=n["level_reach"])
        np.testing.assert_array_equal(o["q"], g[f"q_{steps}"])
        np.testing.assert_array_equal(o["reach_last"], g[f"reach_last_{steps}"])


@pytest.mark.gpu
def test_gpu_routing_of_the_files_matches_reference_outputs():
    n = T.read_network(REFNET)
    g = np.load(os.path.join(GOLDEN, "refnet_out.npz"))
    for steps in (1, 12):
        q, rl = T.wavefront_fp64(n["params"], n["reach_seg_start"], n["reach_seg_len"], n["reach_up_ptr"],
                                 n["reach_up_idx"], n["level_ptr"], n["level_reach"], n["qlat"][:steps], n["qdp0"],
                                 n["dp0"], n["qup0"], steps)
        den = np.maximum(np.abs(g[f"q_{steps}"]), 1e-300)
        assert (np.abs(q - g[f"q_{steps}"]) / den).max() < 1e-10
        assert (np.abs(rl - g[f"reach_last_{steps}"]) / np.maximum(np.abs(g[f"reach_last_{steps}"]), 1e-300)).max() < 1e-10
    # the persistent handle at the tight tolerance, bit-identical to the oracle
    tight = (1e-8, 1e-10, 100, 5)
    p64 = n["params"].view("<f4").reshape(-1, 8).astype(np.float64)
    args = (_topo(n), p64, n["qlat"].astype(np.float64), n["qdp0"].astype(np.float64),
            n["dp0"].astype(np.float64), n["qup0"].astype(np.float64))
    r = T.route_tree(*args, cfg=T.make_cfg(rtol=tight[0], atol=tight[1], maxiter=tight[2], attempts=tight[3]))
    with O.pow_mode(1):
        o = O.route_tree(*args, tol=tight)
    np.testing.assert_array_equal(r["q"], o["q"])
    np.testing.assert_array_equal(r["reach_last"], o["reach_last"])
