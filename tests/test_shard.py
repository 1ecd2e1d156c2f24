"""Multi-rank sharding of independent slices (CPU, gloo, world size 2): the assignment covers
every unit exactly once, balances the CT-XAFS stack's costs, and the ranks' reconstructions
(oracle OS-EM on each rank's share) gathered together equal one process doing all of them.
The only collective is the timing's maximum over ranks."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_slice_range_covers_all():
    from xct import shard
    for n in (0, 1, 7, 100):
        for world in (1, 2, 3, 8):
            got = []
            for r in range(world):
                a, b = shard.slice_range(n, r, world)
                got.extend(range(a, b))
                assert (b - a) in (n // world, n // world + 1)
            assert got == list(range(n))
    with pytest.raises(ValueError):
        shard.slice_range(4, 2, 2)


def test_balance_ctxafs_costs():
    from xct import phantom, shard
    specs = phantom.ctxafs_item_specs(64, seed=3)
    costs = [shard.item_cost(w, len(a)) for w, a in specs]
    for world in (2, 4, 8):
        parts = shard.balance(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        # LPT is within 4/3 of the optimum; the mean load bounds the optimum from below
        assert max(loads) <= (4.0 / 3.0) * max(np.mean(loads), max(costs)) + 1e-6


def _worker(rank, world, port, out_dir):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    for p in (os.path.join(os.path.dirname(here), "ct-xafs_analysis_gb300"), os.path.join(os.path.dirname(here), "oracle")):
        sys.path.insert(0, p)
    import torch.distributed as dist
    import oracle as O
    from xct import phantom as P, shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    specs = [(24, 20), (32, 30), (16, 12), (40, 36), (24, 24)]
    parts = shard.balance([shard.item_cost(w, a) for w, a in specs], world)
    res = {}
    for i in parts[rank]:
        w, a = specs[i]
        ang = P.uniform_angles(a)
        img = P.ellipse_phantom(w, 4, 10 + i, axes=(2, w / 4))
        y = P.noisy_log_sinogram(O.projection(img, ang, w), 1e5, i)
        res[i] = O.osem_run(np.ones((w, w), np.float32), y, ang, 4, 2, order=O.ORDER_LITERAL)
    gathered = [None] * world
    dist.all_gather_object(gathered, res)
    t = shard.max_over_ranks(float(rank + 1))
    if rank == 0:
        merged = {}
        for g in gathered:
            assert not set(g) & set(merged), "a unit was reconstructed twice"
            merged.update(g)
        np.savez(os.path.join(out_dir, "merged.npz"), **{str(k): v for k, v in merged.items()}, tmax=t)
    dist.destroy_process_group()


def test_two_ranks_match_one_process(oracle_lib, tmp_path):
    import torch.multiprocessing as mp
    from xct import phantom as P
    O = oracle_lib
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    merged = dict(np.load(tmp_path / "merged.npz"))
    assert float(merged.pop("tmax")) == 2.0
    specs = [(24, 20), (32, 30), (16, 12), (40, 36), (24, 24)]
    assert sorted(int(k) for k in merged) == list(range(len(specs)))
    for i, (w, a) in enumerate(specs):
        ang = P.uniform_angles(a)
        img = P.ellipse_phantom(w, 4, 10 + i, axes=(2, w / 4))
        y = P.noisy_log_sinogram(O.projection(img, ang, w), 1e5, i)
        want = O.osem_run(np.ones((w, w), np.float32), y, ang, 4, 2, order=O.ORDER_LITERAL)
        assert np.array_equal(merged[str(i)], want)
