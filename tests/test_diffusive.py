"""Diffusive-wave tridiagonal step (the reference's t-route diffusive solver,
water-prediction/owp_extended_kernels.cu:24-153): the oracle against the
reference's own cpu_diffusive_tridiag (compiled from its source) and its
golden fixture, bit for bit; the GPU kernel against both, bit for bit."""
import importlib.util
import os

import numpy as np
import pytest

import troute_gb300 as T
from golden_inputs import GOLDEN
from oracle import troute_oracle as O

_spec = importlib.util.spec_from_file_location("make_diffusive", os.path.join(GOLDEN, "make_diffusive.py"))
MD = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(MD)


def fixture():
    rp, dx, diff, cel, qp = MD.diffusive_inputs()
    g = np.load(os.path.join(GOLDEN, "diffusive_ref.npz"))
    assert str(g["inputs_sha256"]) == MD.sha(rp, dx, diff, cel, qp)
    return rp, dx, diff, cel, qp, g["qp_out"]


def test_oracle_matches_golden():
    rp, dx, diff, cel, qp, ref = fixture()
    np.testing.assert_array_equal(O.diffusive_tridiag(rp, dx, diff, qp), ref)


@pytest.mark.skipif(not O.ref_available(), reason="needs the reference checkout (compiled reference)")
def test_oracle_matches_compiled_reference_other_seed():
    rp, dx, diff, cel, qp = MD.diffusive_inputs(n_reaches=300, seed=77)
    np.testing.assert_array_equal(O.diffusive_tridiag(rp, dx, diff, qp),
                                  O.diffusive_tridiag(rp, dx, diff, qp, use_ref=True, celerity=cel))


@pytest.mark.skipif(not O.ref_available(), reason="needs the reference checkout (compiled reference)")
def test_oracle_matches_compiled_reference_at_the_edges():
    """Reaches of 1, 2 and 3 nodes and of the maximum 500, theta 0 and 1,
    diffusivity and dx below the solver's floors, zero discharge: the oracle
    against the reference's cpu_diffusive_tridiag, bit for bit."""
    rp, dx, diff, cel, qp = MD.diffusive_inputs(n_reaches=64, seed=91)
    rng = np.random.default_rng(92)
    rp["ncomp"][:8] = [1, 2, 3, 500, 2, 500, 4, 1]
    rp["theta"][8:16] = 0.0
    rp["theta"][16:24] = 1.0
    diff[24:32] = rng.uniform(0.0, 0.02, diff[24:32].shape)   # below the 0.01 floor for some nodes
    dx[32:40] = rng.uniform(0.0, 2.0, dx[32:40].shape)        # below the 1 m floor for some nodes
    qp[40:48] = 0.0
    np.testing.assert_array_equal(O.diffusive_tridiag(rp, dx, diff, qp),
                                  O.diffusive_tridiag(rp, dx, diff, qp, use_ref=True, celerity=cel))


def test_bad_ncomp_rejected_by_the_library():
    rp, dx, diff, cel, qp = MD.diffusive_inputs(n_reaches=8)
    rp["ncomp"][1] = 0
    with pytest.raises(T.TrouteError):
        T.diffusive_tridiag(rp, dx, diff, qp)


@pytest.mark.gpu
def test_gpu_matches_golden_bit_for_bit():
    rp, dx, diff, cel, qp, ref = fixture()
    np.testing.assert_array_equal(T.diffusive_tridiag(rp, dx, diff, qp, celerity=cel), ref)


@pytest.mark.gpu
@pytest.mark.parametrize("n_reaches,max_nodes,seed", [(1000, 500, 3), (333, 500, 4), (5000, 500, 5), (77, 120, 6)])
def test_gpu_matches_oracle(n_reaches, max_nodes, seed):
    rp, dx, diff, cel, qp = MD.diffusive_inputs(n_reaches=n_reaches, seed=seed)
    rp["ncomp"] = np.minimum(rp["ncomp"], max_nodes)
    dx, diff, qp = (np.ascontiguousarray(a[:, :max_nodes]) for a in (dx, diff, qp))
    start = np.full_like(qp, -7.0)  # nodes past ncomp must stay untouched
    g = T.diffusive_tridiag(rp, dx, diff, qp, qp_out=start)
    o = O.diffusive_tridiag(rp, dx, diff, qp, qp_out=start)
    np.testing.assert_array_equal(g, o)
