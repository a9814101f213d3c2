"""Sharding a frame's sample passes over ranks, one process per GPU.

A frame of N sample passes is N independent images of the same pixels (each
pass draws its own seeds from the tile state machine's frame numbers,
Renderer.cpp:745-783), so ranks render disjoint contiguous pass ranges with
no exchange during rendering, and the frame's accumulation is the sum of the
ranks' accumulations: one sum-all-reduce of the RGBA32F buffer at the end.
The scene is replicated on every rank.

`render` is any callable (first_pass, num_passes) -> accumulation array of
this rank (GpuRenderer.render_passes + accum on a GPU); `reduce_sum` uses
torch.distributed when a process group is initialised (NCCL on GPUs, gloo on
CPUs) and is the identity otherwise.
"""
from __future__ import annotations

import numpy as np


def pass_range(rank: int, world: int, first_pass: int, num_passes: int) -> tuple[int, int]:
    """Contiguous share of passes [first_pass, first_pass + num_passes) for
    `rank` of `world`: the first num_passes % world ranks take one extra."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    if num_passes < 0 or first_pass < 0:
        raise ValueError("negative pass range")
    base, extra = divmod(num_passes, world)
    start = first_pass + rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def reduce_sum(accum: np.ndarray) -> np.ndarray:
    """Sum of every rank's accumulation (float32), returned on every rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return accum
    backend = dist.get_backend()
    t = torch.from_numpy(np.ascontiguousarray(accum, dtype=np.float32))
    if backend == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()


def render_sharded(render, first_pass: int, num_passes: int) -> np.ndarray:
    """Render this rank's share of the passes, then sum over ranks."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        rank, world = dist.get_rank(), dist.get_world_size()
    else:
        rank, world = 0, 1
    start, count = pass_range(rank, world, first_pass, num_passes)
    return reduce_sum(render(start, count))
