"""Streaming registration of long recordings with overlapped host<->device copies.

The reference reads a recording in batches (motion_correction/compensate_recording.py:773-806,
batch size OFOptions.buffer_size) and hands each batch to the executor.
StreamRegistrar does the same on the GPU: batches pass through two pinned host
staging buffers; while batch i is registered on the compute stream, batch i+1
is copied in and batch i-1's flows are copied out on a copy stream, and the
host fills the next staging buffer from the source.  Between batches the
initial field for the next batch is the mean of the last (up to 20) flows
(compensate_recording.py:801-806), computed on the device.
"""

from __future__ import annotations

from typing import Callable, Optional

import numpy as np
import torch

from . import api


class StreamRegistrar:
    """source(t0, n) -> frames (n, H, W, K) float32: a numpy array (copied into a
    pinned staging buffer) or a pinned torch tensor (copied to the device from
    where it lies); sink(t0, flows (n, H, W, 2) float32 numpy array)."""

    def __init__(self, reference: torch.Tensor, batch: int = 32, weight: Optional[torch.Tensor] = None,
                 update_initialization_w: bool = True, **options):
        self.ref = reference.contiguous()
        self.H, self.W, self.K = (int(s) for s in reference.shape)
        self.B = int(batch)
        self.weight = weight
        self.update_w = update_initialization_w
        self.plan = api.Plan(api.make_params(K=self.K, **options), self.H, self.W, self.K, self.B)
        self.plan.set_reference(self.ref, weight)
        dev = reference.device
        shape_in, shape_out = (self.B, self.H, self.W, self.K), (self.B, self.H, self.W, 2)
        self.h_in = [torch.empty(shape_in, dtype=torch.float32).pin_memory() for _ in range(2)]
        self.h_out = [torch.empty(shape_out, dtype=torch.float32).pin_memory() for _ in range(2)]
        self.d_in = [torch.empty(shape_in, dtype=torch.float32, device=dev) for _ in range(2)]
        self.d_out = [torch.empty(shape_out, dtype=torch.float32, device=dev) for _ in range(2)]
        self.w_init = torch.zeros((self.H, self.W, 2), dtype=torch.float32, device=dev)
        self.compute = torch.cuda.Stream(device=dev)
        self.copy = torch.cuda.Stream(device=dev)

    def run(self, source: Callable[[int, int], np.ndarray], n_frames: int,
            sink: Callable[[int, np.ndarray], None]) -> dict:
        """Registers frames [0, n_frames); returns {"frames", "h2d_bytes", "d2h_bytes"}."""
        B = self.B
        starts = list(range(0, n_frames, B))
        h2d_done = [torch.cuda.Event() for _ in range(2)]
        comp_done = [torch.cuda.Event() for _ in range(2)]
        d2h_done = [torch.cuda.Event() for _ in range(2)]
        pending = []  # (slot, t0, n) waiting to be handed to the sink
        keep = [None, None]  # host sources of the copies in flight
        h2d = d2h = 0

        def stage(i):
            t0 = starts[i]
            n = min(B, n_frames - t0)
            slot = i & 1
            if i >= 2:
                h2d_done[slot].synchronize()  # the copy out of h_in[slot] two batches ago has finished
            src = source(t0, n)
            if torch.is_tensor(src) and src.is_pinned() and src.dtype == torch.float32 and src.is_contiguous():
                host = src
            else:
                self.h_in[slot][:n].copy_(torch.from_numpy(np.ascontiguousarray(src, dtype=np.float32)))
                host = self.h_in[slot][:n]
            keep[slot] = host
            with torch.cuda.stream(self.copy):
                if i >= 2:
                    self.copy.wait_event(comp_done[slot])  # d_in[slot] no longer read
                self.d_in[slot][:n].copy_(host, non_blocking=True)
                h2d_done[slot].record(self.copy)
            return slot, t0, n

        def flush(entry):
            slot, t0, n = entry
            d2h_done[slot].synchronize()
            sink(t0, self.h_out[slot][:n].numpy().copy())

        staged = stage(0) if starts else None
        for i in range(len(starts)):
            slot, t0, n = staged
            with torch.cuda.stream(self.compute):
                self.compute.wait_event(h2d_done[slot])
                if i >= 2:
                    self.compute.wait_event(d2h_done[slot])  # d_out[slot] copied out
                w = self.w_init if self.update_w else None
                self.plan.displacement(self.d_in[slot][:n], w, self.d_out[slot][:n], stream=self.compute)
                if self.update_w:
                    # next initial field: mean of the last (up to) 20 flows of this batch
                    self.w_init = self.d_out[slot][max(0, n - 20):n].mean(0).contiguous()
                comp_done[slot].record(self.compute)
            with torch.cuda.stream(self.copy):
                self.copy.wait_event(comp_done[slot])
                self.h_out[slot][:n].copy_(self.d_out[slot][:n], non_blocking=True)
                d2h_done[slot].record(self.copy)
            h2d += n * self.H * self.W * self.K * 4
            d2h += n * self.H * self.W * 2 * 4
            if pending:
                flush(pending.pop(0))
            pending.append((slot, t0, n))
            staged = stage(i + 1) if i + 1 < len(starts) else None
        while pending:
            flush(pending.pop(0))
        return {"frames": n_frames, "h2d_bytes": h2d, "d2h_bytes": d2h}

    def close(self):
        self.plan.close()
