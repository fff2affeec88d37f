"""StreamCompensator (compensate_recording's batch loop on the GPU, streamed)
against the numpy/scipy/oracle restatement of the same loop
(motion_correction/compensate_recording.py:773-830).

Each batch is checked on its own, from the initial field the pipeline used:
preprocessing bit for bit, flows within the parity bar (fp64 plan), the next
initial field bit for bit from the batch's own flows (numpy's mean), the
compensated frames against the oracle's warp with the same flows, the
statistics against numpy's."""
import numpy as np
import pytest
import torch

from oracle import prep_oracle as P
from pyflowreg_gb300.synthetic import Video

pytestmark = pytest.mark.gpu

MAX_TOL = 1e-3
EPE_TOL = 1e-4


class ListReader:
    """The sequential part of the VideoReader interface (util/io/_base.py)."""

    def __init__(self, frames, buffer_size):
        self.frames, self.buffer_size, self.t = frames, buffer_size, 0

    def has_batch(self):
        return self.t < len(self.frames)

    def read_batch(self):
        out = self.frames[self.t:self.t + self.buffer_size]
        self.t += len(out)
        return out


class ListWriter:
    def __init__(self):
        self.batches = []

    def write_frames(self, frames):
        self.batches.append(np.array(frames))


def _video(dtype, T=26, h=40, w=48, K=2):
    frames, _ = Video(seed=5, h=h, w=w, K=K, n_blobs=8, shift_std=1.0).frames(0, T)
    return frames.astype(dtype)


@pytest.mark.parametrize("dtype", [np.uint16, np.float32])
def test_stream_compensator_follows_the_reference_loop(oracle, dtype):
    from pyflowreg_gb300.pipeline import StreamCompensator

    raw = _video(dtype)
    ref_raw = raw[:8].astype(np.float64).mean(0)
    opts = dict(alpha=(1.5, 1.5), iterations=20, levels=50, eta=0.8)
    B = 10
    sc = StreamCompensator(ref_raw, batch=B, precision="fp64", **opts)
    writer = ListWriter()
    flows = {}
    res = sc.run(ListReader(raw, B), writer, flow_sink=lambda t0, f: flows.__setitem__(t0, f))
    sc.close()
    assert res["frames"] == len(raw) and len(writer.batches) == 3
    assert all(b.dtype == raw.dtype for b in writer.batches)

    ref_proc = P.preprocess(ref_raw, None, np.array([1.0, 1.0, 0.1])).astype(np.float32)
    w_inits = res["w_init"]
    all_flows = np.concatenate([flows[t0] for t0 in sorted(flows)])
    for b, t0 in enumerate(range(0, len(raw), B)):
        batch = raw[t0:t0 + B]
        proc = P.preprocess(batch, ref_raw, np.array([1.0, 1.0, 0.1])).astype(np.float32)
        got = flows[t0]
        for t in range(len(batch)):
            want = oracle.get_displacement(ref_proc, proc[t], uv=w_inits[b], **opts)
            d = got[t].astype(np.float64) - want
            assert np.abs(d).max() <= MAX_TOL and np.sqrt((d ** 2).sum(-1)).mean() <= EPE_TOL, (b, t)
        # next initial field: np.mean of the batch's last (up to) 20 float32 flows
        if b + 1 < len(w_inits):
            np.testing.assert_array_equal(w_inits[b + 1], np.mean(got[-20:], axis=0))
        # compensation warp of the raw frames with these flows, stored into the source dtype
        reg = writer.batches[b]
        for t in range(len(batch)):
            want = np.empty(batch.shape[1:], np.float32)
            for k in range(batch.shape[3]):
                want[..., k] = oracle.warp(batch[t, ..., k].astype(np.float64), got[t, ..., 0].astype(np.float64),
                                           got[t, ..., 1].astype(np.float64),
                                           ref_raw[..., k].astype(np.float32).astype(np.float64), True)
            if np.issubdtype(raw.dtype, np.integer):
                info = np.iinfo(raw.dtype)
                want = np.clip(np.trunc(want), info.min, info.max).astype(raw.dtype)
                assert np.abs(reg[t].astype(np.int64) - want.astype(np.int64)).max() <= 1
                assert np.mean(reg[t] != want) < 1e-3
            else:
                np.testing.assert_allclose(reg[t], want, rtol=0, atol=2e-4 * max(1.0, np.abs(want).max()))
    # first batch's initial field: the mean flow of its first min(22, B) frames from zero
    proc0 = P.preprocess(raw[:B], ref_raw, np.array([1.0, 1.0, 0.1])).astype(np.float32)
    init = np.mean([oracle.get_displacement(ref_proc, proc0[t], **opts).astype(np.float32) for t in range(B)], axis=0)
    assert np.abs(w_inits[0] - init).max() <= MAX_TOL
    stats = P.statistics(all_flows.astype(np.float64))
    np.testing.assert_allclose(res["mean_disp"], stats[:, 0], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(res["max_disp"], stats[:, 1], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(res["mean_div"], stats[:, 2], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(res["mean_translation"], stats[:, 3], rtol=1e-9, atol=1e-9)


def test_stream_compensator_fp32_and_no_w_update():
    """fp32 plan, update_initialization_w off (every batch from zero), an
    in-memory array as the source: flows equal the batched plan's own."""
    import pyflowreg_gb300 as G
    from pyflowreg_gb300.pipeline import StreamCompensator

    raw = _video(np.uint16, T=12)
    ref_raw = raw[:4].astype(np.float64).mean(0)
    sc = StreamCompensator(ref_raw, batch=5, update_initialization_w=False, alpha=(1.5, 1.5), iterations=20,
                          precision="fp32")
    flows = {}
    res = sc.run(raw, None, flow_sink=lambda t0, f: flows.__setitem__(t0, f))
    sc.close()
    assert all(np.all(w == 0) for w in res["w_init"])
    ref_proc = P.preprocess(ref_raw, None, np.array([1.0, 1.0, 0.1])).astype(np.float32)
    for t0 in sorted(flows):
        proc = P.preprocess(raw[t0:t0 + 5], ref_raw, np.array([1.0, 1.0, 0.1])).astype(np.float32)
        want = G.get_displacement_batch(ref_proc, proc, alpha=(1.5, 1.5), iterations=20, precision="fp32")
        np.testing.assert_array_equal(flows[t0], want)
    assert res["h2d_bytes"] == raw.nbytes  # uint16 travels as 2 bytes per value


def test_stream_compensator_rejects_oversized_batches():
    from pyflowreg_gb300.pipeline import StreamCompensator

    raw = _video(np.float32, T=6)
    sc = StreamCompensator(raw[0], batch=2, iterations=5)
    with pytest.raises(ValueError):
        sc.run(ListReader(raw, 3))
    sc.close()
    torch.cuda.synchronize()
