"""Multi-rank host logic on CPU: gloo, world_size 2, one process per rank."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, sizes, out):
    import torch.distributed as dist
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "fmm-rainbow_gb300"))
    from rfmm import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = replicas.shard_scenes(sizes, world)[rank]
    work = float(sum(sizes[i] for i in mine))
    seconds = 1.0 + rank  # rank 1 is the slowest
    value, total, slowest = replicas.reduce_throughput(work, seconds)
    out[rank] = (mine, value, total, slowest)
    dist.barrier()
    dist.destroy_process_group()


def test_scene_sharding_and_throughput_reduction_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    sizes = [4096, 262144, 70000, 16384, 120000, 9000, 50000]
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), sizes, out), nprocs=world, join=True)
        res = dict(out)
    owned = sorted(i for r in range(world) for i in res[r][0])
    assert owned == list(range(len(sizes)))          # every scene exactly once
    for r in range(world):
        assert res[r][2] == sum(sizes) and res[r][3] == 2.0
        assert res[r][1] == pytest.approx(sum(sizes) / 2.0)
    loads = [sum(sizes[i] for i in res[r][0]) for r in range(world)]
    assert abs(loads[0] - loads[1]) <= max(sizes)


def test_shard_scenes_is_balanced_and_deterministic():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "fmm-rainbow_gb300"))
    from rfmm import replicas
    sizes = list(range(1, 50))
    a = replicas.shard_scenes(sizes, 4)
    assert a == replicas.shard_scenes(sizes, 4)
    loads = [sum(sizes[i] for i in r) for r in a]
    assert max(loads) - min(loads) <= max(sizes)
