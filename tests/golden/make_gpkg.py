"""Writes tests/golden/gpkg/: a small synthetic hydrofabric (hydrofabric.gpkg,
an SQLite file with the two tables the reference's GeoPackage parser reads,
`flowpaths` and `flowpath-attributes`) and what the reference's own parser
(water-prediction/t-route/wavefront/data_parsers/parse_gpkg.py, run
unmodified from the reference checkout) makes of it: topo.bin, params.bin and
topo_to_wbid.npy.

The synthetic hydrofabric exercises the parser's rules: waterbody ids that
are sparse and shuffled, flow through nexus ids (nex-M feeds wb-M), terminal
nexuses (tnx-*), NULL and unknown downstream ids, repeated flowpath ids (the
first row counts), malformed ids, attribute rows with NULL, zero, negative or
out-of-range values, top widths below the bottom width, repeated attribute
rows and attribute rows for unknown waterbodies.

This script needs the reference checkout and only runs in the build
container; the files it writes are committed.

Run from the repo root:  python tests/golden/make_gpkg.py <reference root> [seed] [out dir]
"""
import os
import shutil
import sqlite3
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "gpkg")
N_WB, SEED = 1200, 11
# where the reference's parser expects its input, relative to its working directory
REF_GPKG = os.path.join("extract", "big_one_fixed_1", "config", "big_one_fixed_subset.gpkg")
REF_OUT = "net_real_309k"


def make_hydrofabric(path: str, n_wb: int, seed: int):
    rng = np.random.default_rng(seed)
    ids = rng.choice(np.arange(1, 1_000_000), size=n_wb, replace=False)
    # a random forest: each waterbody drains into one placed later in a random
    # order, or leaves the network (about 4 %)
    order = rng.permutation(n_wb)
    pos = np.empty(n_wb, np.int64)
    pos[order] = np.arange(n_wb)
    flow = []
    for i in range(n_wb):
        later = n_wb - 1 - pos[i]
        r = rng.random()
        if later == 0 or r < 0.02:
            toid = f"tnx-{int(rng.integers(1, 10_000))}"
        elif r < 0.03:
            toid = None
        elif r < 0.04:
            toid = f"nex-{int(rng.integers(1_000_000, 2_000_000))}"  # not a waterbody: terminal
        else:
            d = order[pos[i] + 1 + int(rng.integers(0, min(later, 40)))]
            toid = f"nex-{int(ids[d])}"
        flow.append((f"wb-{int(ids[i])}", toid, int(rng.integers(1, 10**7)), float(rng.uniform(0.05, 8.0)),
                     float(rng.uniform(0.1, 50.0))))
    # repeated ids (the first row counts) and malformed ids
    for i in rng.choice(n_wb, 15, replace=False):
        flow.append((f"wb-{int(ids[i])}", f"tnx-{int(rng.integers(1, 10))}", 1, 1.0, 1.0))
    flow += [("wb-", "nex-1", 1, 1.0, 1.0), ("lake-x", "nex-2", 1, 1.0, 1.0), ("cat-", None, 1, 1.0, 1.0)]
    perm = rng.permutation(len(flow) - 18)
    flow = [flow[k] for k in perm] + flow[len(flow) - 18:]

    def maybe(v, p_none=0.03, p_zero=0.03, p_neg=0.02):
        r = rng.random()
        if r < p_none:
            return None
        if r < p_none + p_zero:
            return 0.0
        if r < p_none + p_zero + p_neg:
            return -abs(v)
        return v

    attrs = []
    for i in range(n_wb):
        if rng.random() < 0.07:
            continue  # no attributes: the parser's defaults
        bw = float(rng.uniform(1.0, 60.0))
        tw = bw * float(rng.uniform(0.7, 3.0))      # sometimes below the bottom width
        twcc = tw * float(rng.uniform(0.5, 6.0))    # sometimes below the top width
        attrs.append((f"wb-{int(ids[i])}", maybe(float(rng.uniform(20.0, 6000.0))), maybe(float(rng.uniform(0.005, 0.2))),
                      maybe(float(rng.uniform(0.01, 0.3))), maybe(bw), maybe(tw), maybe(twcc),
                      maybe(float(rng.uniform(0.05, 3.0))), maybe(float(np.exp(rng.uniform(np.log(1e-7), np.log(0.05)))))))
    for i in rng.choice(n_wb, 20, replace=False):  # a second row for the same link
        attrs.append((f"wb-{int(ids[i])}", None, 0.09, None, float(rng.uniform(1, 10)), 0.0, None, 1.5, 0.002))
    attrs += [("wb-999999999", 100.0, 0.05, 0.1, 5.0, 8.0, 30.0, 1.0, 0.01), ("junk", 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0)]
    perm = rng.permutation(len(attrs))
    attrs = [attrs[k] for k in perm]

    if os.path.exists(path):
        os.remove(path)
    con = sqlite3.connect(path)
    con.execute("CREATE TABLE flowpaths (fid INTEGER PRIMARY KEY AUTOINCREMENT, id TEXT, toid TEXT, "
                "hydroseq INTEGER, lengthkm REAL, areasqkm REAL)")
    con.executemany("INSERT INTO flowpaths (id, toid, hydroseq, lengthkm, areasqkm) VALUES (?, ?, ?, ?, ?)", flow)
    con.execute('CREATE TABLE "flowpath-attributes" (fid INTEGER PRIMARY KEY AUTOINCREMENT, link TEXT, '
                '"Length_m" REAL, "n" REAL, "nCC" REAL, "BtmWdth" REAL, "TopWdth" REAL, "TopWdthCC" REAL, '
                '"ChSlp" REAL, "So" REAL)')
    con.executemany('INSERT INTO "flowpath-attributes" (link, "Length_m", "n", "nCC", "BtmWdth", "TopWdth", '
                    '"TopWdthCC", "ChSlp", "So") VALUES (?, ?, ?, ?, ?, ?, ?, ?, ?)', attrs)
    con.commit()
    con.close()


def run_reference(ref_root: str, gpkg: str, out_dir: str):
    """Runs the reference's parser unmodified on `gpkg`; its three outputs go
    to out_dir."""
    script = os.path.join(ref_root, "water-prediction", "t-route", "wavefront", "data_parsers", "parse_gpkg.py")
    with tempfile.TemporaryDirectory() as tmp:
        dst = os.path.join(tmp, REF_GPKG)
        os.makedirs(os.path.dirname(dst))
        shutil.copyfile(gpkg, dst)
        subprocess.run([sys.executable, script], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        os.makedirs(out_dir, exist_ok=True)
        for f in ("topo.bin", "params.bin", "topo_to_wbid.npy"):
            shutil.copyfile(os.path.join(tmp, REF_OUT, f), os.path.join(out_dir, f))


def main(ref_root: str, seed: int = SEED, out: str = OUT):
    os.makedirs(out, exist_ok=True)
    gpkg = os.path.join(out, "hydrofabric.gpkg")
    make_hydrofabric(gpkg, N_WB, seed)
    run_reference(ref_root, gpkg, out)
    print(f"wrote {out}")


if __name__ == "__main__":
    main(sys.argv[1], *(int(a) for a in sys.argv[2:3]), *sys.argv[3:4])
