"""Lateral-inflow pre-processor (the reference's data_parsers/
parse_qlat_fast_cpp.cpp): the library's parallel CSV pivot and forcings.bin
writer against a plain-Python statement of the parsing rules and, where the
reference checkout is present, against the reference tool itself built from
its source (byte-identical forcings.bin)."""
import os
import subprocess

import numpy as np
import pytest

import troute_gb300 as T
from oracle import troute_oracle as O

REF_TOOL = os.path.join(os.path.dirname(O.REF_SO), "parse_qlat_fast")


def make_csv_dir(d, n_reaches=300, n_ts=24, seed=11):
    rng = np.random.default_rng(seed)
    ids = rng.choice(np.arange(1000, 10_000_000), n_reaches, replace=False).astype(np.int64)
    for k, wb in enumerate(ids):
        if k % 17 == 5:
            continue  # a reach without a file
        vals = rng.gamma(2.0, 0.05, n_ts).astype(np.float32)
        lines = [" Time Step, Time, q_lateral"]  # header: read as step 0, then overwritten
        for t in range(n_ts + (2 if k % 11 == 0 else 0)):  # some files run past n_ts
            v = vals[t] if t < n_ts else 99.0
            lines.append(f"{t}, 2017-01-01 {t:02d}:00:00, {v:.8g}")
        if k % 7 == 0:
            lines.append("")  # trailing blank line
            lines.append("1,")  # too short
        eol = "\r\n" if k % 13 == 0 else "\n"
        (d / f"nex-{wb}_output.csv").write_text(eol.join(lines) + eol)
    (d / "nex-999_output.csv").write_text("0, x, 1.0\n")  # id not in the table
    (d / "cat-5_output.csv").write_text("0, x, 1.0\n")    # not a nexus file
    (d / "nex-12_other.csv").write_text("0, x, 1.0\n")    # not an output file
    return ids


def python_pivot(d, ids, n_ts):
    """The parsing rules, restated in plain Python."""
    import ctypes

    libc = ctypes.CDLL(None)
    libc.atof.restype = ctypes.c_double
    index = {int(w): i for i, w in enumerate(ids)}
    q = np.zeros((n_ts, len(ids)), np.float32)
    for name in sorted(os.listdir(d)):
        if not (name.startswith("nex-") and "_output.csv" in name):
            continue
        wb = int(name[4:name.index("_", 4)])
        if wb not in index:
            continue
        for line in open(os.path.join(d, name), "rb").read().split(b"\n"):
            if len(line) < 5 or b"," not in line:
                continue
            ts = libc.atoi(line)
            v = np.float32(libc.atof(line[line.rindex(b",") + 1:]))
            if 0 <= ts < n_ts:
                q[ts, index[wb]] = v
    return q


def test_pivot_matches_python_statement(tmp_path):
    ids = make_csv_dir(tmp_path)
    for threads in (1, 3, 0):
        q, matched, missing = T.qlat_from_csv(str(tmp_path), ids, 24, n_threads=threads)
        np.testing.assert_array_equal(q, python_pivot(tmp_path, ids, 24))
        assert matched == sum(1 for k in range(len(ids)) if k % 17 != 5) and missing == 1


@pytest.mark.skipif(not os.path.exists(REF_TOOL), reason="needs the reference checkout (reference tool)")
def test_forcings_bin_identical_to_reference_tool(tmp_path):
    csv = tmp_path / "csv"
    csv.mkdir()
    ids = make_csv_dir(csv, seed=12)
    np.save(tmp_path / "topo_to_wbid.npy", ids)
    ref_out = tmp_path / "ref_forcings.bin"
    subprocess.run([REF_TOOL, str(csv), str(tmp_path / "topo_to_wbid.npy"), str(ref_out), "24", "4"], check=True,
                   stdout=subprocess.DEVNULL)
    q, _, _ = T.qlat_from_csv(str(csv), ids, 24, n_threads=4)
    n = len(ids)
    ours = tmp_path / "forcings.bin"
    T.write_forcings(str(ours), q, np.zeros(n), np.zeros(n), np.full(n, 0.5))
    assert open(ours, "rb").read() == open(ref_out, "rb").read()
