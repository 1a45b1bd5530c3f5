"""Several ranks without a GPU: the batch's scenes are split between two
gloo ranks (every scene exactly once, loads balanced), and the job time is
the max over ranks -- the host logic bench.py runs at N > 1."""
import os
import socket

import pytest

from voxel_cone_tracing_gb300 import replicas

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_partitions_and_balances():
    costs = [replicas.scene_cost(w, h, g, c, t) for (w, h, g, c, t) in
             [(1920, 1080, 256, 0, 500_000), (256, 256, 32, 1, 1_000), (1280, 720, 128, 0, 200_000),
              (640, 480, 64, 1, 50_000), (1920, 1080, 64, 1, 900_000), (512, 384, 256, 0, 10_000)] * 5]
    for world in (1, 2, 3, 4, 8):
        parts = replicas.shard(costs, world)
        assert len(parts) == world
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs) + 1e-9  # greedy bound
    assert replicas.shard(costs, 2) == replicas.shard(list(costs), 2)  # deterministic


def _worker(rank, world, port, costs, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = replicas.shard(costs, world)[rank]
    local = sum(costs[i] for i in mine)
    t = replicas.job_time(local, dist)
    q.put((rank, mine, local, t))
    dist.destroy_process_group()


def test_two_gloo_ranks_split_the_batch():
    import torch.multiprocessing as mp
    costs = [float(c) for c in [5, 3, 8, 1, 1, 2, 9, 4, 4, 6, 2, 7]]
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, costs, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    seen = sorted(i for _, mine, _, _ in out for i in mine)
    assert seen == list(range(len(costs)))
    assert set(out[0][1]).isdisjoint(out[1][1])
    slowest = max(local for _, _, local, _ in out)
    assert all(t == slowest for _, _, _, t in out)
