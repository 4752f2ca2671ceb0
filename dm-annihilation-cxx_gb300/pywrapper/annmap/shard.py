"""Particle-sharded rendering over several ranks (one GPU each).

Particles are independent and the map is a sum over them, so N ranks can
each render a contiguous 1/N of the particles into a full partial map and
one sum reduction of the FP64 maps gives the whole map.  Each rank's shard
is [n*r/N, n*(r+1)/N).  This is the data path of a node with several GPUs
(NCCL on CUDA tensors); its arithmetic is tested with gloo ranks on the CPU.
"""
from __future__ import annotations


def shard_bounds(n: int, rank: int, world: int) -> tuple:
    return (n * rank) // world, (n * (rank + 1)) // world


def shard(parts: dict, rank: int, world: int) -> dict:
    n = len(next(iter(parts.values())))
    i0, i1 = shard_bounds(n, rank, world)
    return {k: v[i0:i1] for k, v in parts.items()}


def render_sharded(render, parts: dict, nside: int, *, rank: int = None, world: int = None,
                   group=None):
    """Renders this rank's shard with ``render(parts, nside) -> map`` (a
    float64 torch tensor, e.g. a Renderer.render into a CUDA map) and sums
    the partial maps over the process group in place.  Returns the summed
    map (every rank holds it)."""
    import torch.distributed as dist
    if rank is None:
        rank = dist.get_rank(group)
    if world is None:
        world = dist.get_world_size(group)
    m = render(shard(parts, rank, world), nside)
    dist.all_reduce(m, op=dist.ReduceOp.SUM, group=group)
    return m
