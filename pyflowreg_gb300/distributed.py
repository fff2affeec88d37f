"""Frame sharding over ranks (one process per GPU) and the only cross-frame
exchange of pyflowreg's batch loop.

Frames of a batch are independent once ``w_init`` is fixed
(motion_correction/parallelization/sequential.py:97-163), so ranks take
contiguous frame ranges and register them with no communication.  Between
batches pyflowreg sets the next initial field to the mean of the last (up to
20) flows of the batch (motion_correction/compensate_recording.py:801-806);
with frames sharded, the ranks exchange the flows of that tail and each sums
them in frame order, so every rank gets numpy's float32 mean bit for bit.
Everything here runs over any torch.distributed backend (NCCL on GPUs, gloo
on CPU for tests).
"""

from __future__ import annotations

from typing import Callable, Optional, Sequence

import numpy as np


def shard_range(n_frames: int, rank: int, world: int) -> tuple:
    """Contiguous [start, stop) of the frames rank `rank` registers; the first
    n_frames % world ranks take one extra frame."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(n_frames), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def _dist():
    import torch.distributed as dist

    return dist


def numpy_mean0_f32(frames: np.ndarray) -> np.ndarray:
    """np.mean(frames, axis=0) of a float32 stack, as numpy computes it: the
    leading axis is reduced element-wise, one frame after another, in float32,
    then divided by the count in float32."""
    acc = np.array(frames[0], dtype=np.float32, copy=True)
    for i in range(1, frames.shape[0]):
        acc += frames[i]
    return acc / np.float32(frames.shape[0])


def next_w_init(local_flows, start: int, n_total: int, last: int = 20, group=None) -> np.ndarray:
    """Mean of the last `last` flows of the whole batch (all of them when the
    batch has no more than `last` frames), from each rank's contiguous share,
    equal bit for bit to pyflowreg's ``np.mean(w[-20:], axis=0)``
    (motion_correction/compensate_recording.py:801-806).

    local_flows: (t, H, W, 2) flows of global frames [start, start + t).  The
    ranks exchange their frames of the tail (at most `last` flows in all), so
    that every rank sums the same frames in frame order.  Returns (H, W, 2)
    float32 on every rank.
    """
    import torch

    flows = np.asarray(local_flows, dtype=np.float32)
    first = n_total - last if n_total > last else 0
    count = n_total - first
    if count <= 0:
        raise ValueError("empty batch")
    t = flows.shape[0]
    dist = _dist()
    world = dist.get_world_size(group) if (dist.is_available() and dist.is_initialized()) else 1
    if world == 1:
        if start != 0 or t != n_total:
            raise ValueError("a single process must hold the whole batch")
        return numpy_mean0_f32(flows[first:])
    # this rank's frames of the tail in their slots, the others zero
    slots = np.zeros((count,) + flows.shape[1:], np.float32)
    a, b = max(first, start), min(n_total, start + t)
    if a < b:
        slots[a - first:b - first] = flows[a - start:b - start]
    span = torch.tensor([a, b], dtype=torch.int64)
    spans = [torch.empty_like(span) for _ in range(world)]
    dist.all_gather(spans, span, group=group)
    buf = torch.from_numpy(slots)
    bufs = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(bufs, buf, group=group)
    tail = np.empty_like(slots)
    covered = 0
    for sp, bf in zip(spans, bufs):
        ra, rb = int(sp[0]), int(sp[1])
        if ra < rb:
            tail[ra - first:rb - first] = bf.numpy()[ra - first:rb - first]
            covered += rb - ra
    if covered != count:
        raise ValueError("the ranks' shares do not cover the batch tail exactly once")
    return numpy_mean0_f32(tail)


def max_over_ranks(value: float, group=None) -> float:
    """Largest value over all ranks (the step time the whole job waited for)."""
    import torch

    dist = _dist()
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def register_batches(batches: Sequence, w_init: np.ndarray, flow_fn: Callable, last: int = 20,
                     group=None, update_initialization_w: bool = True):
    """Runs pyflowreg's batch loop (compensate_recording.py:773-806) with every
    batch sharded over the ranks of `group`.

    batches: sequence of (T_b, H, W, K) arrays, identical on every rank.
    flow_fn(frames, w_init) -> (t, H, W, 2) flows of a contiguous shard.
    Returns this rank's flows per batch and the final w_init.
    """
    dist = _dist()
    world = dist.get_world_size(group) if dist.is_available() and dist.is_initialized() else 1
    rank = dist.get_rank(group) if world > 1 else 0
    out = []
    w = np.asarray(w_init, dtype=np.float32)
    for batch in batches:
        n = len(batch)
        a, b = shard_range(n, rank, world)
        flows = np.asarray(flow_fn(batch[a:b], w), dtype=np.float32)
        out.append(flows)
        if update_initialization_w:
            w = next_w_init(flows, a, n, last=last, group=group)
    return out, w


def default_group() -> Optional[object]:
    dist = _dist()
    return None if not (dist.is_available() and dist.is_initialized()) else dist.group.WORLD
