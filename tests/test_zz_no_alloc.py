"""The no-allocation reach-parallel entry point.

Callers that cannot allocate device memory where they route (a model driver
whose device buffers all come from its own pool, or a hot path where an
allocation would synchronise the device) use
troute_mc_reach_parallel_device_noalloc, whose only scratch is an array
compiled into the library. Through the C ABI, two calls in a row must give the
same results as the allocating device entry point on the same device arrays,
and the same bits as the oracle's cpu_mc (correctly rounded powers).
"""
import ctypes as C

import numpy as np
import pytest

import troute_gb300 as T
from golden_inputs import make_golden
from oracle import troute_oracle as O

pytestmark = pytest.mark.gpu


def test_no_alloc_entry_point_matches_allocating_one_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda", 0)
    p, ql, rs, rl, qu, qd, dp = make_golden.cpu_mc_inputs()
    S, nr = len(ql), len(rs)
    pv = np.ascontiguousarray(p.view("<f8").reshape(-1, 8))
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in dict(p=pv, ql=ql, qu=qu, qd=qd, dp=dp).items()}
    ti = {k: torch.from_numpy(np.ascontiguousarray(v, np.int32)).to(dev) for k, v in dict(rs=rs, rl=rl).items()}
    L = T.lib()

    def outs():
        return [torch.zeros(S, dtype=torch.float64, device=dev) for _ in range(3)]

    def args(o):
        return [C.c_void_p(x.data_ptr()) for x in (t["p"], t["ql"], ti["rs"], ti["rl"], t["qu"], t["qd"], t["dp"],
                                                   *o)] + [10.0, 300.0, nr, S, None, None]

    ref = outs()
    assert L.troute_mc_reach_parallel_device(*args(ref)) == 0
    torch.cuda.synchronize()
    st_ref = T.Stats()
    qo, vo, dpo = (np.zeros(S) for _ in range(3))
    # counters of the same computation through the host entry point
    assert L.troute_mc_reach_parallel_cfg(*(x.ctypes.data_as(C.c_void_p) for x in (pv, ql, np.int32(rs), np.int32(rl),
                                                                                     qu, qd, dp, qo, vo, dpo)),
                                          10.0, 300.0, nr, None, C.byref(st_ref)) == 0
    with O.pow_mode(1):
        oq, ov, od, _ = O.cpu_mc(p, ql, rs, rl, qu, qd, dp, uq=10.0, dt=300.0)
    for _ in range(2):
        o = outs()
        st = T.Stats()
        assert L.troute_mc_reach_parallel_device_noalloc(*args(o), C.byref(st)) == 0, L.troute_last_error()
        for a, b in zip(o, ref):
            x, y = a.cpu().numpy(), b.cpu().numpy()
            rel = np.abs(x - y) / np.maximum(np.abs(y), 1e-300)
            assert rel.max() < 1e-10
        assert st.solves == S and st.iterations == st_ref.iterations
        for a, b in zip(o, (oq, ov, od)):
            np.testing.assert_array_equal(a.cpu().numpy(), b)


def test_no_alloc_rejects_oversized_calls():
    L = T.lib()
    rc = L.troute_mc_reach_parallel_device_noalloc(*([C.c_void_p(1)] * 10), 10.0, 300.0, 2_097_153, 10, None, None,
                                                   None)
    assert rc == 1 and b"no-alloc limit" in L.troute_last_error()
