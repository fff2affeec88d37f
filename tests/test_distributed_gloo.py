"""Multi-rank host logic on CPU: two gloo ranks shard frames and reproduce the
single-process batch loop of pyflowreg (w_init = mean of the last 20 flows,
motion_correction/compensate_recording.py:801-806)."""
import os
import socket

import numpy as np
import pytest

from pyflowreg_gb300.distributed import next_w_init, register_batches, shard_range


@pytest.mark.parametrize("n,world", [(400, 2), (401, 2), (7, 3), (1, 2), (20, 4), (152, 8)])
def test_shard_range_partitions(n, world):
    ranges = [shard_range(n, r, world) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == n
    for (a0, b0), (a1, _) in zip(ranges, ranges[1:]):
        assert b0 == a1
    sizes = [b - a for a, b in ranges]
    assert max(sizes) - min(sizes) <= 1


def _fake_flow(frames, w_init):
    # a deterministic stand-in for the device registration: depends on the frame and on w_init
    return frames[..., :2] * 0.5 + w_init[None] * 0.25


def _reference_loop(batches, w0):
    w = w0
    outs = []
    for b in batches:
        f = _fake_flow(b, w).astype(np.float32)
        outs.append(f)
        w = (np.mean(f[-20:], axis=0) if f.shape[0] > 20 else np.mean(f, axis=0)).astype(np.float32)
    return outs, w


def _batches():
    rng = np.random.default_rng(0)
    return [rng.standard_normal((n, 6, 5, 2)).astype(np.float32) for n in (45, 13, 30)]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        outs, w = register_batches(_batches(), np.zeros((6, 5, 2), np.float32), _fake_flow)
        q.put((rank, [o for o in outs], w))
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_gloo_ranks_match_single_process():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict()
    for _ in range(2):
        rank, outs, w = q.get(timeout=120)
        results[rank] = (outs, w)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref_outs, ref_w = _reference_loop(_batches(), np.zeros((6, 5, 2), np.float32))
    for bi, ref in enumerate(ref_outs):
        merged = np.concatenate([results[0][0][bi], results[1][0][bi]], axis=0)
        np.testing.assert_allclose(merged, ref, rtol=1e-6, atol=1e-6)
    np.testing.assert_array_equal(results[0][1], ref_w)
    np.testing.assert_array_equal(results[0][1], results[1][1])


def test_next_w_init_single_process_matches_reference():
    rng = np.random.default_rng(1)
    flows = rng.standard_normal((33, 4, 3, 2)).astype(np.float32)
    np.testing.assert_array_equal(next_w_init(flows, 0, 33), np.mean(flows[-20:], axis=0))
    np.testing.assert_array_equal(next_w_init(flows[:12], 0, 12), np.mean(flows[:12], axis=0))
