"""Writes tests/golden/diffusive_ref.npz: the reference's own diffusive-wave
tridiagonal step (cpu_diffusive_tridiag, water-prediction/
owp_extended_kernels.cu:35-91, compiled unmodified into
oracle/_ref/libtroute_ref.so by make -C oracle ref) on seeded inputs with the
distributions of the reference's gen_diff_data (:347-362): 20-99 nodes per
reach, theta 0.6, dt 60 s, dx U(100, 600) m, diffusivity U(10, 110),
celerity U(0.5, 2.5), discharge U(1, 51) -- plus a few edge reaches (one
node, two nodes, the full 500 nodes, dx below 1 m, diffusivity below 0.01).

The inputs are regenerated from their seed by diffusive_inputs() (numpy
PCG64); a SHA-256 of them is stored with the outputs.

Run from the repo root:  python tests/golden/make_diffusive.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
MAX_NODES = 500


def diffusive_inputs(n_reaches=96, seed=2026):
    rng = np.random.default_rng(seed)
    rp = np.zeros(n_reaches, np.dtype([("ncomp", "<i4"), ("theta", "<f4"), ("dtini", "<f4")]))
    rp["ncomp"] = rng.integers(20, 100, n_reaches)
    rp["theta"] = 0.6
    rp["dtini"] = 60.0
    shape = (n_reaches, MAX_NODES)
    dx = rng.uniform(100.0, 600.0, shape).astype(np.float32)
    diff = rng.uniform(10.0, 110.0, shape).astype(np.float32)
    cel = rng.uniform(0.5, 2.5, shape).astype(np.float32)
    qp = rng.uniform(1.0, 51.0, shape).astype(np.float32)
    # edge reaches
    rp["ncomp"][0], rp["ncomp"][1], rp["ncomp"][2] = 1, 2, MAX_NODES
    dx[3, :10] = 0.25
    diff[4, :10] = 0.001
    rp["theta"][5] = 1.0
    return rp, dx, diff, cel, qp


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main():
    from oracle import troute_oracle as O

    O.build(ref=True)
    rp, dx, diff, cel, qp = diffusive_inputs()
    out = O.diffusive_tridiag(rp, dx, diff, qp, use_ref=True, celerity=cel)
    np.savez_compressed(os.path.join(HERE, "diffusive_ref.npz"), qp_out=out, inputs_sha256=sha(rp, dx, diff, cel, qp))
    print("diffusive_ref.npz:", out.shape)


if __name__ == "__main__":
    main()
