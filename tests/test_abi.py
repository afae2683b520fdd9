"""The C ABI: every declared entry point is exported, struct layouts agree,
and the host-side logic behaves without a GPU (no compute calls)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, has_gpu

HEADER = os.path.join(ROOT, "include", "troute_gb300.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(troute_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    import troute_gb300 as T

    L = T.lib()
    names = declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(T.exported_symbols())


def test_struct_layouts_match_c():
    import troute_gb300 as T
    from troute_gb300 import api

    prog = r"""
#include <stdio.h>
#include <stddef.h>
#include "troute_gb300.h"
int main(void){
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(troute_chparams), sizeof(troute_chparams_f32),
         sizeof(troute_cfg), sizeof(troute_stats), sizeof(troute_topo),
         offsetof(troute_stats, kernel_ms), offsetof(troute_cfg, wait_cycles));
  return 0; }
"""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "l.c")
        open(src, "w").write(prog)
        exe = os.path.join(d, "l")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        got = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [C.sizeof(api.ChParams), api.CHPARAMS_F32_DTYPE.itemsize, C.sizeof(api.Cfg), C.sizeof(api.Stats),
                   C.sizeof(api.Topo), api.Stats.kernel_ms.offset, api.Cfg.wait_cycles.offset]
    assert got[0] == 64 == T.CHPARAMS_DTYPE.itemsize


def test_cfg_defaults_are_the_reference_constants():
    from troute_gb300 import make_cfg

    c = make_cfg()
    assert (c.rtol, c.atol, c.maxiter, c.attempts) == (0.01, 0.01, 100, 5)


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_device_is_reported_not_faked():
    """Without a GPU the product path fails loudly (no CPU fallback)."""
    import troute_gb300 as T
    from troute_gb300 import synth

    with pytest.raises(T.TrouteError) as e:
        T.device_info()
    assert e.value.code == 6  # TROUTE_ENODEV
    c = synth.network("c0", n_ts=2)
    with pytest.raises(T.TrouteError) as e:
        T.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"])
    assert e.value.code in (6, 3)
    t = c["topo"]
    with pytest.raises(T.TrouteError):
        T.mc_reach_parallel(c["params"], c["qlat"][0], t["reach_seg_start"], t["reach_seg_len"], c["q0"], c["q0"],
                            c["d0"])
    # the tree form under both of its names, called through the C ABI directly
    from troute_gb300 import api

    arrs = [np.ascontiguousarray(t[k], np.int32) for k in ("reach_seg_start", "reach_seg_len", "reach_up_ptr",
                                                             "reach_up_idx")]
    topo, _keep = api._topo_struct(*arrs, t["n_segments"])
    S = t["n_segments"]
    p = np.ascontiguousarray(c["params"])   # structured ChParams records (64 B each)
    ql = np.ascontiguousarray(c["qlat"], np.float64)
    q0, d0 = np.ascontiguousarray(c["q0"], np.float64), np.ascontiguousarray(c["d0"], np.float64)
    q = np.zeros(S)
    for name in ("troute_route_tree", "troute_mc_route_tree"):
        rc = getattr(T.lib(), name)(C.byref(topo), p.ctypes.data_as(C.c_void_p), ql.ctypes.data_as(C.c_void_p),
                                    q0.ctypes.data_as(C.c_void_p), d0.ctypes.data_as(C.c_void_p), None, ql.shape[0],
                                    300.0, None, q.ctypes.data_as(C.c_void_p), None, None, None, None)
        assert rc in (6, 3), (name, rc)


def test_bad_arguments_rejected_before_device():
    import troute_gb300 as T

    p = np.zeros((1, 8))
    with pytest.raises(T.TrouteError) as e:
        T.mc_reach_parallel(p, [0.0], [0], [1], [0.0], [0.0], [0.0], cfg=T.make_cfg(rtol=2.0))
    assert e.value.code == 1
    with pytest.raises(T.TrouteError) as e:
        T.mc_reach_parallel(p, [0.0], [-1], [1], [0.0], [0.0], [0.0])
    assert e.value.code == 1


def test_makefile_builds_the_same_library(tmp_path):
    """noaa-gpu-kernels_gb300/Makefile (the build for C callers without
    Python) produces a library exporting every declared entry point."""
    out = tmp_path / "libtroute_gb300.so"
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "noaa-gpu-kernels_gb300"), f"-j{os.cpu_count() or 2}",
                        f"BUILD={tmp_path / 'obj'}", f"OUT={out}"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    nm = subprocess.run(["nm", "-D", "--defined-only", str(out)], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (troute_[a-z0-9_]+)$", nm, flags=re.M))
    assert set(declared()) <= exported
