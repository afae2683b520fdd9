"""Sharding batched routing across ranks.

- Host logic on CPU (gloo, world size 2): partitioning batched networks across
  ranks and gathering their results reproduces the single-process routing
  exactly. Each rank routes its share with the library where a GPU exists,
  else with the oracle.
- On the GPU: the shares of an ensemble (member ranges) and of a basin batch
  (partitioned basins), routed one after another as separate launches, are
  bit-identical to the unsharded launch -- what bench.py --gpus N relies on
  when it gives every rank its share instead of a replica."""
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
    gpu = False
    try:
        import torch

        gpu = torch.cuda.is_available()
    except Exception:
        pass
    res = {}
    if mine and gpu:
        import troute_gb300 as T

        share = [nets[i] for i in mine]
        with T.Network([n["topo"] for n in share], [n["params"] for n in share]) as b:
            b.set_state(np.concatenate([n["q0"] for n in share]), np.concatenate([n["d0"] for n in share]),
                        np.concatenate([n["rl0"] for n in share]))
            b.run(np.concatenate([n["qlat"] for n in share], axis=1))
            q = b.get_state()[0]
        off = 0
        for i, n in zip(mine, share):
            res[i] = q[off:off + n["topo"]["n_segments"]]
            off += n["topo"]["n_segments"]
    for i in ([] if gpu else mine):
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
        # the reference tolerance: the GPU matches the C-library-pow oracle to 1e-10
        np.testing.assert_allclose(got[str(i)], q, rtol=1e-10, atol=0)


@pytest.mark.gpu
def test_sequential_shards_equal_the_unsharded_launch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import troute_gb300 as T
    from troute_gb300 import synth

    cfg = T.make_cfg(rtol=1e-8, atol=1e-10)
    # ensemble members: ranges of 2 ranks against all 6 members in one launch
    w = synth.network("tree:20000", n_ts=6)
    S, R, M = w["topo"]["n_segments"], len(w["topo"]["reach_seg_start"]), 6
    fac = [synth.make_member(1004, m, S) for m in range(M)]

    def route_members(m0, m1):
        qf = np.stack([fac[m][0] for m in range(m0, m1)])
        nf = np.stack([fac[m][1] for m in range(m0, m1)])
        k = m1 - m0
        with T.Network.ensemble(w["topo"], w["params"], k, n_scale=nf, qlat_scale=qf, cfg=cfg) as net:
            net.set_state(np.tile(w["q0"], k), np.tile(w["d0"], k), np.tile(w["rl0"], k))
            net.run(w["qlat"])
            return net.get_state()

    full = route_members(0, M)
    parts = [route_members(*member_range(M, 2, r)) for r in range(2)]
    for a, n in ((0, S), (1, S), (2, S), (3, R)):
        np.testing.assert_array_equal(np.concatenate([p[a] for p in parts]), full[a])
    # basins: the partition of 5 basins over 2 ranks against one launch of all
    nets = synth.basins(seed=1002, n_trees=5, lo=500.0, hi=20000.0)
    sizes = [n["topo"]["n_segments"] for n in nets]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    qlat = synth.make_qlat(1002, int(offs[-1]), 6)

    def route_basins(which):
        sub = [nets[i] for i in which]
        ql = np.ascontiguousarray(np.concatenate([qlat[:, offs[i]:offs[i + 1]] for i in which], axis=1))
        Ss = sum(sizes[i] for i in which)
        Rs = sum(len(nets[i]["topo"]["reach_seg_start"]) for i in which)
        with T.Network([n["topo"] for n in sub], [n["params"] for n in sub], cfg=cfg) as b:
            b.set_state(np.full(Ss, synth.Q0), np.full(Ss, synth.D0), np.full(Rs, synth.Q0))
            b.run(ql)
            return b.get_state()[0]

    q_all = route_basins(range(5))
    for which in partition(sizes, 2):
        q = route_basins(which)
        off = 0
        for i in which:
            np.testing.assert_array_equal(q[off:off + sizes[i]], q_all[offs[i]:offs[i + 1]])
            off += sizes[i]
