"""Writes tests/golden/refnet/ (topo.bin, params.bin, forcings.bin) with the
reference's OWN network generator and writers, imported from the reference
checkout (water-prediction/t-route/wavefront/gen_network.py: build_network,
generate_params, generate_forcings, write_network, write_params,
write_forcings), and tests/golden/refnet_out.npz with the reference's own
cpu_wavefront_fp64 (water-prediction/t-route/wavefront/wavefront_mc.cu:495-564,
compiled unmodified into oracle/_ref/libtroute_ref.so by make -C oracle ref)
routing those files: final discharge and reach outflow after 1 and 12 steps;
and the reference's linearised form (linear_mc.cu): its coefficients
(compute_mc_coeffs, host instance) and cpu_linear_mc's final discharge after
the 12 steps.

The network is small (target 300 reaches, 12 steps, seed 7) so the files stay
a few hundred KB. This script needs the reference checkout and only runs in
the build container; the files it writes are committed.

Run from the repo root:  python tests/golden/make_refnet.py <reference root>
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "noaa-gpu-kernels_gb300"))
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "refnet")

REACHES, STEPS, SEED = 300, 12, 7


def main(ref_root: str):
    sys.path.insert(0, os.path.join(ref_root, "water-prediction", "t-route", "wavefront"))
    import gen_network as G  # the reference's generator

    net = G.build_network(G.NetworkSpec(n_reaches=REACHES, seed=SEED, mean_chain=3, mean_segments_per_reach=4))
    params = G.generate_params(net["n_segments"], SEED)
    qlat, qup0, qdp0, dp0 = G.generate_forcings(net["n_reaches"], net["n_segments"], STEPS, SEED)
    os.makedirs(OUT, exist_ok=True)
    G.write_network(OUT, net)
    G.write_params(OUT, params)
    G.write_forcings(OUT, STEPS, qlat, qup0, qdp0, dp0)

    from oracle import troute_oracle as O

    O.build(ref=True)
    import troute_gb300 as T

    n = T.read_network(OUT)
    topo = {k: n[k] for k in ("reach_seg_start", "reach_seg_len", "reach_up_ptr", "reach_up_idx")}
    topo["n_segments"] = n["n_segments"]
    out = {}
    for steps in (1, STEPS):
        q, rl = O.ref_wavefront_fp64(topo, n["params"], n["qlat"][:steps], n["qdp0"], n["dp0"], n["qup0"],
                                     level_ptr=n["level_ptr"], level_reach=n["level_reach"])
        out[f"q_{steps}"], out[f"reach_last_{steps}"] = q, rl
    # the linearised form (linear_mc.cu): the reference's coefficient function
    # (host instance) and its cpu_linear_mc over all steps from qdp0
    c = O.linear_coeffs(n["params"], 300.0, use_ref=True)
    for k, v in zip(("lin_c1", "lin_c2", "lin_c3", "lin_c4oq"), c):
        out[k] = v
    out["lin_q"] = O.linear_route(c, topo, n["qlat"], n["qdp0"], level_ptr=n["level_ptr"],
                                  level_reach=n["level_reach"], use_ref=True)
    np.savez_compressed(os.path.join(HERE, "refnet_out.npz"), **out)
    print(f"refnet: {n['n_reaches']} reaches, {n['n_segments']} segments, {n['n_levels']} levels, "
          f"{n['n_ts']} steps")


if __name__ == "__main__":
    from oracle.troute_oracle import REF_ROOT  # $TROUTE_REF_ROOT, else ../reference beside the repository

    main(sys.argv[1] if len(sys.argv) > 1 else REF_ROOT)
