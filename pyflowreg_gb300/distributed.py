"""Frame sharding over ranks (one process per GPU) and the only cross-frame
exchange of pyflowreg's batch loop.

Frames of a batch are independent once ``w_init`` is fixed
(motion_correction/parallelization/sequential.py:97-163), so ranks take
contiguous frame ranges and register them with no communication.  Between
batches pyflowreg sets the next initial field to the mean of the last (up to
20) flows of the batch (motion_correction/compensate_recording.py:801-806);
with frames sharded, that mean is an all-reduce of per-rank partial sums.
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


def next_w_init(local_flows, start: int, n_total: int, last: int = 20, group=None) -> np.ndarray:
    """Mean of the last `last` flows of the whole batch (all of them when the
    batch has no more than `last` frames), from each rank's contiguous share.

    local_flows: (t, H, W, 2) flows of global frames [start, start + t).
    Returns (H, W, 2) float32 on every rank, as the reference stores w_init.
    The partial sums are float64, so the result may differ from numpy's
    float32 mean by one float32 rounding.
    """
    import torch

    flows = np.asarray(local_flows, dtype=np.float64)
    first = n_total - last if n_total > last else 0
    t = flows.shape[0]
    lo = max(first - start, 0)
    part = flows[lo:t].sum(axis=0) if lo < t else np.zeros(flows.shape[1:], np.float64)
    count = max(t - lo, 0)
    dist = _dist()
    if dist.is_available() and dist.is_initialized():
        buf = torch.from_numpy(np.concatenate([part.ravel(), [float(count)]]))
        dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
        part = buf[:-1].numpy().reshape(part.shape)
        count = int(round(float(buf[-1])))
    if count == 0:
        raise ValueError("empty batch")
    return (part / count).astype(np.float32)


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
