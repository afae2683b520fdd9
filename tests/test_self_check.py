"""The self-checking build (TROUTE_CHECK=1).

Built into its own directory and loaded in a child process, so the default
library of this session is untouched. In this build the dataflow kernel's
reach-outflow history is NaN-filled before every run and each (reach, step)
item verifies on the device, before it starts, that every value it reads has
been written and its own output slot has not; a violation is reported as an
error instead of being assumed away. A c0 run at rtol 1e-8 must report no
violation and stay bit-identical to the oracle (correctly rounded powers);
so must a 16-member ensemble of a 20,000-segment tree (many items in flight).
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu

_CHILD = r"""
import sys
import numpy as np
sys.path[:0] = [ROOT, ROOT + "/noaa-gpu-kernels_gb300"]
from troute_gb300 import build as B
B.build(force=True)
import troute_gb300 as T
from oracle import troute_oracle as O
from troute_gb300 import synth
assert T.library_path().startswith(LIBDIR), T.library_path()
TIGHT = (1e-8, 1e-10, 100, 5)
cfg = T.make_cfg(rtol=1e-8, atol=1e-10)
c = synth.network("c0", n_ts=48)
g = T.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"], cfg=cfg)
with O.pow_mode(1):
    o = O.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"], tol=TIGHT)
np.testing.assert_array_equal(g["q"], o["q"])
w = synth.network("tree:20000", n_ts=8)
M, S = 16, w["topo"]["n_segments"]
qf = np.stack([synth.make_member(1004, m, S)[0] for m in range(M)])
with T.Network.ensemble(w["topo"], w["params"], M, qlat_scale=qf, cfg=cfg) as net:
    net.set_state(np.tile(w["q0"], M), np.tile(w["d0"], M), np.tile(w["rl0"], M))
    st = net.run(w["qlat"])
    q = net.get_state()[0]
assert st["solves"] == M * S * 8, st
with O.pow_mode(1):
    o = O.route_tree(w["topo"], w["params"], w["qlat"] * qf[5][None, :], w["q0"], w["d0"], w["rl0"], tol=TIGHT)
np.testing.assert_array_equal(q[5 * S:6 * S], o["q"])
print("SELF-CHECK OK")
"""


def test_self_check_build_reports_no_violation(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    env = dict(os.environ, TROUTE_CHECK="1", TROUTE_BUILD_DIR=str(tmp_path / "_build"),
               TROUTE_LIB_DIR=str(tmp_path / "lib"))
    code = f"ROOT = {ROOT!r}\nLIBDIR = {str(tmp_path / 'lib')!r}\n" + _CHILD
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert "SELF-CHECK OK" in r.stdout
