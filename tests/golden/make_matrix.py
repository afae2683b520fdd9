"""Writes tests/golden/matrix_ref.npz: the reference's matrix form
(water-prediction/t-route/wavefront/linear_mc_matrix.cu) set up on the
committed reference network tests/golden/refnet/ exactly as the reference's
main() sets it up (:266-310):

  - coefficients from the first n_reaches parameter records (main passes
    params[r] for reach r) by the reference's own compute_mc_coeffs_cpu
    (:56-86), at dt = 300 s;
  - P_Q and P_q by the reference's own build_propagation_matrices (:129-216)
    at its default tolerance 1e-7;
  - lateral inflow as main reads it (the first n_ts x n_reaches values of
    forcings.bin, step t at offset t x n_reaches) and the first n_reaches
    initial discharges.

Both functions are compiled unmodified from the reference's source into
oracle/_ref/libtroute_ref.so (oracle/ref_matrix_shim.cu). The reference's
step runs only on the GPU (cuSPARSE, or kernel_spmv_fused of
linear_mc_matrix_graph.cu:174-206), so the routed discharge stored here
(`q_final`, 12 steps) is the oracle's restatement of that kernel's arithmetic
(oracle_matrix_step), on the reference's matrices.

Run from the repo root (needs the reference checkout):
    python tests/golden/make_matrix.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "noaa-gpu-kernels_gb300")]

from oracle import troute_oracle as O  # noqa: E402
import troute_gb300 as T  # noqa: E402

STEPS, TOL, DT = 12, 1e-7, 300.0


def reference_setup():
    """(up_ptr, up_idx, params [R], qlat [STEPS][R], q0 [R]) as main() reads refnet."""
    n = T.read_network(os.path.join(HERE, "refnet"))
    R = len(n["reach_up_ptr"]) - 1
    flat = np.ascontiguousarray(n["qlat"], np.float32).reshape(-1)
    qlat = flat[: STEPS * R].reshape(STEPS, R)
    return n["reach_up_ptr"], n["reach_up_idx"], n["params"][:R], qlat, np.asarray(n["qdp0"][:R], np.float32)


def main():
    O.build(ref=True)
    assert O.ref_available(), "needs the reference checkout"
    up_ptr, up_idx, p, qlat, q0 = reference_setup()
    c = O.matrix_coeffs(p, DT, use_ref=True)
    (qp, qc, qv), (lp, lc, lv) = O.matrix_build(up_ptr, up_idx, c, TOL, use_ref=True)
    q = O.matrix_route((qp, qc, qv), (lp, lc, lv), qlat, q0)
    np.savez_compressed(os.path.join(HERE, "matrix_ref.npz"), c1=c[0], c2=c[1], c3=c[2], c4oq=c[3], PQ_ptr=qp,
                        PQ_col=qc, PQ_val=qv, Pq_ptr=lp, Pq_col=lc, Pq_val=lv, qlat=qlat, q0=q0, q_final=q)
    print(f"matrix_ref: {len(qp) - 1} reaches, P_Q {len(qc)} entries, P_q {len(lc)} entries, {STEPS} steps")


if __name__ == "__main__":
    main()
