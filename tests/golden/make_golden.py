"""Writes the golden fixtures of this directory from the reference's OWN CPU
routines, compiled unmodified from the reference checkout into
oracle/_ref/libtroute_ref.so (make -C oracle ref):

  cpu_mc_c0.npz     cpu_mc (water-prediction/t-route/troute_mc_final.cu:167-252)
                    on the c0 network's reaches, one step, uq = 10, dt = 300;
  wavefront_c0.npz  cpu_wavefront_fp64 (water-prediction/t-route/wavefront/
                    wavefront_mc.cu:495-564) on the c0 network with inputs
                    rounded to float32 (the reference routine takes floats),
                    final state after 1, 24 and 288 steps.

Inputs are regenerated from their seeds by troute_gb300.synth (a
platform-independent generator) and numpy's PCG64; a SHA-256 of the inputs is
stored with each fixture so drift in either is caught.

Run from the repo root:  python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "noaa-gpu-kernels_gb300"))

HERE = os.path.dirname(os.path.abspath(__file__))


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def cpu_mc_inputs():
    """c0 reach structure, random single-step state (PCG64 seed 2024),
    including zero-flow and invalid-parameter segments."""
    from troute_gb300 import synth

    c = synth.network("c0", n_ts=1)
    topo = c["topo"]
    S = topo["n_segments"]
    rng = np.random.default_rng(2024)
    p = c["params"].copy()
    qu = rng.uniform(0.0, 50.0, S)
    qd = rng.uniform(0.0, 50.0, S)
    dp = rng.uniform(0.0, 3.0, S)
    ql = rng.gamma(2.0, 0.05, S)
    # edge cases the reference handles explicitly (troute_mc_final.cu:54-63)
    p["n_ch"][5] = 0.0
    p["s0"][17] = -1e-4
    p["bw"][23] = 0.0
    p["cs"][31] = 0.0      # z = 1 branch
    p["tw"][40] = p["bw"][40]  # bw == tw branch
    p["tw"][41] = 0.5 * p["bw"][41]  # bw > tw branch
    p["twcc"][50] = 0.0    # no floodplain
    for s in (60, 61, 62):
        qu[s] = qd[s] = ql[s] = 0.0
    dp[70] = -1.0
    return p, ql, topo["reach_seg_start"], topo["reach_seg_len"], qu, qd, dp


def wavefront_inputs():
    from troute_gb300 import synth

    c = synth.network("c0")
    p32 = np.asarray(c["params"].view("<f8").reshape(-1, 8), np.float32)
    return (c["topo"], p32, c["qlat"].astype(np.float32), c["q0"].astype(np.float32),
            c["d0"].astype(np.float32), c["rl0"].astype(np.float32))


def main():
    from oracle import troute_oracle as O

    O.build(ref=True)
    if not O.ref_available():
        raise SystemExit("reference library not built (reference checkout missing)")
    p, ql, rs, rl, qu, qd, dp = cpu_mc_inputs()
    qo, vo, dpo = O.ref_cpu_mc(p, ql, rs, rl, qu, qd, dp, uq=10.0, dt=300.0)
    np.savez_compressed(os.path.join(HERE, "cpu_mc_c0.npz"), qo=qo, vo=vo, dpo=dpo,
                        input_sha=sha(p, ql, rs, rl, qu, qd, dp))
    topo, p32, ql32, q0, d0, r0 = wavefront_inputs()
    out = {}
    for T in (1, 24, 288):
        q, rlast = O.ref_wavefront_fp64(topo, p32, ql32[:T], q0, d0, r0)
        out[f"q_{T}"] = q
        out[f"reach_last_{T}"] = rlast
    np.savez_compressed(os.path.join(HERE, "wavefront_c0.npz"),
                        input_sha=sha(topo["reach_seg_start"], topo["reach_seg_len"], topo["reach_up_ptr"],
                                      topo["reach_up_idx"], p32, ql32, q0, d0, r0), **out)
    print("golden fixtures written")


if __name__ == "__main__":
    main()
