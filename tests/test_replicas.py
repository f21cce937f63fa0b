"""Multi-process host logic of the replica path on CPU (gloo, world size 2): instance
sharding, the ordered gather of per-instance results and the max-over-ranks timing."""
import os
import socket

import numpy as np
import pytest

from nd_gb300.replicas import gather_instances, max_over_ranks, shard


def test_shard_covers_every_instance_once():
    for n in (0, 1, 7, 4096):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            assert [i for p in parts for i in p] == list(range(n))
            assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root / "networkdynamics.jl_gb300"))
    sys.path.insert(0, str(root))
    import torch.distributed as dist

    from nd_gb300.replicas import gather_instances, max_over_ranks, shard
    from oracle import oracle as O
    import nd_gb300 as nd
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # per-instance work: the oracle RHS of small swing networks, instances sharded by rank
    n = 9
    res = []
    for i in shard(n, rank, world):
        g = nd.barabasi_albert(40 + i, 2, seed=i)
        on = O.OracleNetwork.from_graph(g, O.V_SWING, O.E_KURAMOTO)
        rng = np.random.default_rng(i)
        u = rng.normal(size=on.dim)
        p = np.concatenate([np.tile([1.0, 0.1, 0.0], g.nv), rng.uniform(5, 10, g.ne)])
        res.append(np.abs(on.rhs(u, p)).max())
    full = gather_instances(np.array(res).reshape(-1), world)
    slowest = max_over_ranks(float(rank + 1), world)
    if rank == 0:
        np.save(out, np.concatenate([full, [slowest]]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_gather(tmp_path):
    import torch.multiprocessing as mp

    from oracle import oracle as O
    import nd_gb300 as nd
    out = str(tmp_path / "r.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
    got = np.load(out)
    ref = []
    for i in range(9):
        g = nd.barabasi_albert(40 + i, 2, seed=i)
        on = O.OracleNetwork.from_graph(g, O.V_SWING, O.E_KURAMOTO)
        rng = np.random.default_rng(i)
        u = rng.normal(size=on.dim)
        p = np.concatenate([np.tile([1.0, 0.1, 0.0], g.nv), rng.uniform(5, 10, g.ne)])
        ref.append(np.abs(on.rhs(u, p)).max())
    np.testing.assert_array_equal(got[:-1], np.array(ref))
    assert got[-1] == 2.0


def test_single_process_helpers_need_no_process_group():
    assert max_over_ranks(3.5, 1) == 3.5
    np.testing.assert_array_equal(gather_instances([1, 2], 1), [1, 2])
