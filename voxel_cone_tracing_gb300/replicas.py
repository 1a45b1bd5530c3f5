"""Several GPUs: the path has no exchange step (a frame's voxel maps, G-buffer
and trace belong to one scene on one GPU), so N GPUs run N replicas of a
frame, or split the independent scenes of a batch between them.  Nothing
here moves scene data between ranks; the only collective is the
max-over-ranks of a time (the job ends when its slowest rank ends).

Works with any torch.distributed backend (gloo on CPU, nccl on GPUs).
"""
from __future__ import annotations


def scene_cost(width: int, height: int, grid: int, cone_set: int, n_tris: int) -> float:
    """Relative cost of one batch scene: trace work ~ pixels x cones, plus
    voxelization ~ triangles and grid volume (weights from the bench frame:
    1080p traces in ~4.2 ms, 500k triangles voxelize in ~0.3 ms at 256^3)."""
    cones = 9 if cone_set == 0 else 6
    trace = width * height * (cones + 2) / (1920 * 1080 * 11) * 4.2
    vox = n_tris / 500_000 * 0.2 + (grid / 256) ** 3 * 0.1
    return trace + vox


def shard(costs, world: int) -> list:
    """Split scenes (given their costs) between `world` ranks: longest job
    first onto the least loaded rank; ties go to the lower rank.  Returns the
    scene indices of every rank, each in ascending order (deterministic on
    every rank)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def my_scenes(items, rank: int, world: int) -> list:
    """The batch items (scene, width, height, grid, cone_set) of this rank."""
    costs = [scene_cost(w, h, g, c, s.n_tris) for s, w, h, g, c in items]
    return [items[i] for i in shard(costs, world)[rank]]


def job_time(local_ms: float, dist=None, device=None) -> float:
    """Max over ranks of a per-rank time (identity without a process group)."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return float(local_ms)
    import torch
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
