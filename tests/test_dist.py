"""Multi-rank host logic on CPU (gloo, world size 2): partitioning batched
networks across ranks and gathering their results must reproduce the
single-process routing exactly. The per-rank compute here is the oracle (no
GPU on this machine); the GPU path routes each rank's share the same way."""
import os
import socket

import numpy as np
import pytest

from troute_gb300.parallel import member_range, partition


def test_partition_is_complete_and_balanced():
    rng = np.random.default_rng(0)
    sizes = list(np.exp(rng.uniform(np.log(500), np.log(2e5), 256)).astype(int))
    for w in (1, 2, 3, 8):
        parts = partition(sizes, w)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)
    assert [member_range(64, 3, r) for r in range(3)] == [(0, 22), (22, 43), (43, 64)]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "noaa-gpu-kernels_gb300")):
        sys.path.insert(0, p)
    import torch.distributed as dist

    from oracle import troute_oracle as O
    from troute_gb300 import synth
    from troute_gb300.parallel import partition

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    nets = [synth.network(f"tree:{S}", seed=s, n_ts=6) for S, s in ((800, 1), (300, 2), (1500, 3), (200, 4))]
    mine = partition([n["topo"]["n_segments"] for n in nets], world)[rank]
    res = {}
    for i in mine:
        n = nets[i]
        res[i] = O.route_tree(n["topo"], n["params"], n["qlat"], n["q0"], n["d0"], n["rl0"])["q"]
    gathered = [None] * world
    dist.all_gather_object(gathered, res)
    if rank == 0:
        merged = {k: v for d in gathered for k, v in d.items()}
        np.savez(os.path.join(out_dir, "dist.npz"), **{str(k): v for k, v in merged.items()})
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_batch_routing_matches_single_process(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    from oracle import troute_oracle as O
    from troute_gb300 import synth

    got = np.load(tmp_path / "dist.npz")
    assert sorted(got.files, key=int) == ["0", "1", "2", "3"]
    for i, (S, s) in enumerate(((800, 1), (300, 2), (1500, 3), (200, 4))):
        n = synth.network(f"tree:{S}", seed=s, n_ts=6)
        q = O.route_tree(n["topo"], n["params"], n["qlat"], n["q0"], n["d0"], n["rl0"])["q"]
        np.testing.assert_array_equal(got[str(i)], q)
