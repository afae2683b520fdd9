"""GeoPackage hydrofabric ingest (the reference's
water-prediction/t-route/wavefront/data_parsers/parse_gpkg.py) against the
reference's own parser: the committed fixture (tests/golden/gpkg/, made by
tests/golden/make_gpkg.py running that parser) byte for byte, fresh
hydrofabrics against the parser run live where the reference checkout is
present, the ingested network read back and routed by the oracle, and the
error cases."""
import filecmp
import importlib.util
import os
import sqlite3

import numpy as np
import pytest

import troute_gb300 as T
from golden_inputs import GOLDEN
from oracle import troute_oracle as O

GPKG_DIR = os.path.join(GOLDEN, "gpkg")
REF_ROOT = O.REF_ROOT  # the reference checkout, where present


def _make_gpkg():
    spec = importlib.util.spec_from_file_location("make_gpkg", os.path.join(GOLDEN, "make_gpkg.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _same_files(a, b):
    for f in ("topo.bin", "params.bin"):
        assert filecmp.cmp(os.path.join(a, f), os.path.join(b, f), shallow=False), f
    np.testing.assert_array_equal(np.load(os.path.join(a, "topo_to_wbid.npy")),
                                  np.load(os.path.join(b, "topo_to_wbid.npy")))


def test_fixture_reproduced_byte_for_byte(tmp_path):
    net = T.gpkg_to_network(os.path.join(GPKG_DIR, "hydrofabric.gpkg"), str(tmp_path))
    _same_files(str(tmp_path), GPKG_DIR)
    assert not os.path.exists(os.path.join(tmp_path, "forcings.bin"))
    assert net["n_reaches"] == 1200 and net["n_segments"] == 1200


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "water-prediction")),
                    reason="needs the reference checkout (the parser is run live)")
@pytest.mark.parametrize("seed", [3, 4])
def test_fresh_hydrofabrics_match_the_reference_parser(tmp_path, seed):
    mg = _make_gpkg()
    gpkg = str(tmp_path / "h.gpkg")
    mg.make_hydrofabric(gpkg, 900, seed)
    ref = str(tmp_path / "ref")
    mg.run_reference(REF_ROOT, gpkg, ref)
    ours = str(tmp_path / "ours")
    T.gpkg_to_network(gpkg, ours)
    _same_files(ours, ref)


def test_ingested_network_reads_back_and_routes(tmp_path):
    net = T.gpkg_to_network(os.path.join(GPKG_DIR, "hydrofabric.gpkg"), str(tmp_path))
    R, S, n_ts = net["n_reaches"], net["n_segments"], 6
    rng = np.random.default_rng(5)
    qlat = rng.gamma(2.0, 0.05, (n_ts, S)).astype(np.float32)
    T.write_forcings(str(tmp_path / "forcings.bin"), qlat, np.full(R, 0.1, np.float32), np.full(S, 0.1, np.float32),
                     np.full(S, 0.1, np.float32))
    back = T.read_network(str(tmp_path))     # the library's reader checks the topology
    for k in ("reach_up_ptr", "reach_up_idx", "level_ptr", "level_reach", "reach_level"):
        np.testing.assert_array_equal(back[k], net[k])
    topo = {k: back[k] for k in ("reach_seg_start", "reach_seg_len", "reach_up_ptr", "reach_up_idx")}
    topo["n_segments"] = S
    p64 = np.zeros(S, T.CHPARAMS_DTYPE)
    for f in p64.dtype.names:
        p64[f] = back["params"][f]
    o = O.route_tree(topo, p64, back["qlat"].astype(np.float64), np.full(S, 0.1), np.full(S, 0.1), np.full(R, 0.1))
    assert np.isfinite(o["q"]).all() and (o["q"] >= 0).all()


def _tiny(path, flow, attrs=()):
    con = sqlite3.connect(path)
    con.execute("CREATE TABLE flowpaths (id TEXT, toid TEXT, hydroseq INTEGER, lengthkm REAL, areasqkm REAL)")
    con.executemany("INSERT INTO flowpaths VALUES (?, ?, 1, 1.0, 1.0)", flow)
    con.execute('CREATE TABLE "flowpath-attributes" (link TEXT, "Length_m" REAL, "n" REAL, "nCC" REAL, '
                '"BtmWdth" REAL, "TopWdth" REAL, "TopWdthCC" REAL, "ChSlp" REAL, "So" REAL)')
    con.executemany('INSERT INTO "flowpath-attributes" VALUES (?, ?, ?, ?, ?, ?, ?, ?, ?)', attrs)
    con.commit()
    con.close()


def test_rules_on_a_small_hydrofabric(tmp_path):
    path = str(tmp_path / "t.gpkg")
    # wb-7 and wb-3 drain into wb-5, wb-5 leaves through a terminal nexus;
    # the repeated wb-3 row and the malformed row are ignored
    _tiny(path, [("wb-7", "nex-5"), ("wb-3", "nex-5"), ("wb-5", "tnx-1"), ("wb-3", "nex-7"), ("x", "nex-3")],
          [("wb-5", 50.0, 0.005, None, 10.0, 8.0, 11.0, 0.01, 0.0),     # floors, tw <= bw, twcc <= tw
           ("wb-3", 2000.0, 0.04, 0.08, 12.0, 30.0, 90.0, 1.5, 0.003)])
    net = T.read_gpkg(path)
    assert net["n_reaches"] == 3 and net["n_levels"] == 2
    wb = list(net["topo_to_wbid"])
    r5 = wb.index(5)
    assert net["reach_level"][r5] == 1 and net["reach_n_up"][r5] == 2
    p = net["params"]
    assert p["dx"][r5] == np.float32(100.0) and p["n_ch"][r5] == np.float32(0.01)
    assert p["tw"][r5] == np.float32(10.0) * np.float32(1.2)
    assert p["twcc"][r5] == p["tw"][r5] * np.float32(3.0)
    assert p["s0"][r5] == np.float32(0.001) and p["ncc"][r5] == np.float32(0.12)   # defaults kept
    r7 = wb.index(7)
    assert p["dx"][r7] == np.float32(1000.0) and p["bw"][r7] == np.float32(20.0)   # no attributes: defaults


def test_errors(tmp_path):
    with pytest.raises(FileNotFoundError):
        T.read_gpkg(str(tmp_path / "missing.gpkg"))
    cyc = str(tmp_path / "cycle.gpkg")
    _tiny(cyc, [("wb-1", "nex-2"), ("wb-2", "nex-1"), ("wb-3", "nex-1")])
    with pytest.raises(ValueError):
        T.read_gpkg(cyc)
    empty = str(tmp_path / "empty.gpkg")
    _tiny(empty, [("lake", "nex-1")])
    with pytest.raises(ValueError):
        T.read_gpkg(empty)
