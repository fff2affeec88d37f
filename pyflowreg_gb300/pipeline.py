"""compensate_recording's batch loop on the GPU, streamed from a reader.

``StreamCompensator.run(reader, writer)`` follows
CompensateRecording.run (motion_correction/compensate_recording.py:773-830)
batch by batch:

* ``reader.read_batch()`` while ``reader.has_batch()`` (util/io/_base.py:
  VideoReader.read_batch / has_batch), or consecutive slices of an array;
* preprocessing against the raw reference, normalize + Gaussian
  (compensate_recording.py:521-561), on the device;
* on the first batch, the initial field: the mean flow of its first
  min(22, T) frames from a zero start (compensate_recording.py:645-678);
* the flows of the batch from w_init, then the compensation warp of the raw
  frames against the raw reference (parallelization/sequential.py:141-163),
  cast back to an integer source dtype as the executors' stores do;
* w_init <- mean of the batch's last (up to) 20 flows
  (compensate_recording.py:801-806), on the device;
* the per-frame statistics mean_disp, max_disp, mean_div, mean_translation
  (compensate_recording.py:808-821), on the device;
* ``writer.write_frames(registered)`` (the VideoWriter interface).

Batches pass through two pinned host staging slots: while batch i is
registered on the compute stream, batch i + 1 is read by the host and copied
in, and batch i - 1's registered frames and flows are copied out, on a copy
stream.  Integer sources travel in their own dtype (uint16 is half the bytes
of float32) and are widened on the device.
"""

from __future__ import annotations

from typing import Callable, Optional

import numpy as np
import torch

from . import api
from .prep import flow_statistics_device, preprocess_device


def _wire(dt: np.dtype):
    """(torch dtype the frames travel in, numpy view of the source with that
    layout): uint8 and int16 as themselves, uint16 as the bits of int16, the
    rest as float32 (float64 sources are rounded to float32 on the host)."""
    dt = np.dtype(dt)
    if dt == np.uint8:
        return torch.uint8, np.uint8
    if dt == np.int16:
        return torch.int16, np.int16
    if dt == np.uint16:
        return torch.int16, np.int16
    return torch.float32, np.float32


def _widen(src, dt: np.dtype, out):
    """Frames in their wire dtype -> float32 values (out), on the current stream."""
    if np.dtype(dt) == np.uint16:
        out.copy_(torch.bitwise_and(src.to(torch.int32), 0xFFFF))
    else:
        out.copy_(src)
    return out


def _narrow(x, dt: np.dtype, out):
    """Registered float32 frames -> the source dtype's values in the wire dtype.
    The executors store into np.empty_like(batch) (parallelization/sequential.py:
    82, 159-163), numpy's unsafe cast: in-range values truncate toward zero;
    out-of-range ones (cubic overshoot), which numpy leaves to the platform,
    saturate here."""
    dt = np.dtype(dt)
    if not np.issubdtype(dt, np.integer):
        out.copy_(x)
        return out
    info = np.iinfo(dt)
    v = torch.clamp(torch.trunc(x), info.min, info.max)
    if dt == np.uint16:
        v = v.to(torch.int32)
        v = torch.where(v > 32767, v - 65536, v)
    out.copy_(v)
    return out


def _mean_frames(x):
    """np.mean(x, axis=0) of float32 frames: float32 sums in frame order, then
    the division by the count in float32 (numpy reduces a leading axis
    element-wise, one frame after another)."""
    acc = x[0].clone()
    for t in range(1, x.shape[0]):
        acc.add_(x[t])
    # a tensor divisor: torch turns division by a Python scalar into a multiplication by its reciprocal
    return acc.div_(torch.full_like(acc, float(x.shape[0])))


class _ArraySource:
    """(T, H, W, C) array as a sequential reader with batches of ``batch`` frames."""

    def __init__(self, array, batch):
        self.a = array
        self.B = batch
        self.t = 0

    def has_batch(self):
        return self.t < self.a.shape[0]

    def read_batch(self):
        out = self.a[self.t:self.t + self.B]
        self.t += out.shape[0]
        return out


class StreamCompensator:
    """reference_raw (H, W, C) numpy array; ``batch`` = the largest batch the
    reader returns (OFOptions.buffer_size); flow options as
    ``get_displacement`` takes them (alpha, iterations, ..., precision)."""

    def __init__(self, reference_raw, batch: int = 32, sigma=((1.0, 1.0, 0.1),),
                 channel_normalization: str = "together", weight=None, update_initialization_w: bool = True,
                 interpolation_method: str = "cubic", device=None, **flow_options):
        # the raw reference is held in float64 (compensate_recording.py:491-498)
        ref = np.asarray(reference_raw).astype(np.float64)
        if ref.ndim == 2:
            ref = ref[:, :, None]
        self.ref_raw = ref
        self.H, self.W, self.K = ref.shape
        self.B = int(batch)
        self.sigma = sigma
        self.norm = channel_normalization
        self.update_w = update_initialization_w
        self.method = interpolation_method
        self.dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        flow_options.setdefault("precision", "fp64")
        self.plan = api.Plan(api.make_params(K=self.K, **flow_options), self.H, self.W, self.K, self.B)
        self.fp64 = self.plan.fp64
        self.ref_raw_t = torch.from_numpy(np.ascontiguousarray(ref, dtype=np.float32)).to(self.dev)
        self.ref_raw64_t = torch.from_numpy(np.ascontiguousarray(ref)).to(self.dev)
        self.weight_t = None
        if weight is not None:
            w = api.normalize_weight(weight, self.H, self.W, self.K)
            self.weight_t = torch.from_numpy(np.ascontiguousarray(w, dtype=np.float32)).to(self.dev)
        self.compute = torch.cuda.Stream(device=self.dev)
        self.copy = torch.cuda.Stream(device=self.dev)
        self._slots_dtype = None

    # ------------------------------------------------------------------ buffers
    def _alloc(self, src_dtype):
        wire, _ = _wire(src_dtype)
        if self._slots_dtype == (wire, np.dtype(src_dtype)):
            return
        B, H, W, K = self.B, self.H, self.W, self.K
        self._slots_dtype = (wire, np.dtype(src_dtype))
        self.h_in = [torch.empty((B, H, W, K), dtype=wire).pin_memory() for _ in range(2)]
        self.h_reg = [torch.empty((B, H, W, K), dtype=wire).pin_memory() for _ in range(2)]
        self.h_flow = [torch.empty((B, H, W, 2), dtype=torch.float32).pin_memory() for _ in range(2)]
        self.h_stats = [torch.empty((B, 4), dtype=torch.float64).pin_memory() for _ in range(2)]
        self.d_in = [torch.empty((B, H, W, K), dtype=wire, device=self.dev) for _ in range(2)]
        self.d_reg = [torch.empty((B, H, W, K), dtype=wire, device=self.dev) for _ in range(2)]
        self.d_flow = [torch.empty((B, H, W, 2), dtype=torch.float32, device=self.dev) for _ in range(2)]
        self.d_stats = [torch.empty((B, 4), dtype=torch.float64, device=self.dev) for _ in range(2)]
        self.d_raw = torch.empty((B, H, W, K), dtype=torch.float32, device=self.dev)
        self.d_proc = torch.empty((B, H, W, K), dtype=torch.float32, device=self.dev)
        self.d_warp = torch.empty((B, H, W, K), dtype=torch.float32, device=self.dev)
        self.d_flow64 = (torch.empty((B, H, W, 2), dtype=torch.float64, device=self.dev) if self.fp64 else None)

    def _flows(self, proc, uv, out32):
        """Flows of proc (n, H, W, K) from uv into out32 (float32), on the current stream."""
        s = torch.cuda.current_stream()
        if self.fp64:
            f64 = self.plan.displacement(proc, uv, self.d_flow64[:proc.shape[0]], stream=s)
            out32.copy_(f64)
        else:
            self.plan.displacement(proc, uv, out32, stream=s)
        return out32

    # --------------------------------------------------------------------- run
    def run(self, reader, writer=None, flow_sink: Optional[Callable[[int, np.ndarray], None]] = None) -> dict:
        """Registers everything the reader yields.  writer.write_frames(registered)
        receives each batch in the source dtype; flow_sink(t0, flows) the float32
        flows.  Returns the statistics lists, the w_init used by each batch and
        the byte counts of the copies."""
        if isinstance(reader, np.ndarray):
            arr = reader if reader.ndim == 4 else reader[..., None]
            reader = _ArraySource(arr, self.B)
        B, H, W, K = self.B, self.H, self.W, self.K
        h2d_done = [torch.cuda.Event() for _ in range(2)]
        comp_done = [torch.cuda.Event() for _ in range(2)]
        d2h_done = [torch.cuda.Event() for _ in range(2)]
        out = {"mean_disp": [], "max_disp": [], "mean_div": [], "mean_translation": [], "w_init": [],
               "frames": 0, "h2d_bytes": 0, "d2h_bytes": 0}
        pending = []
        keep = [None, None]
        state = {"i": 0, "t0": 0, "src_dtype": None}
        ref_proc = None
        w_init = torch.zeros((H, W, 2), dtype=torch.float32, device=self.dev)

        def stage():
            """Reads the next batch into a staging slot and queues its upload."""
            if not reader.has_batch():
                return None
            batch = np.asarray(reader.read_batch())
            if batch.ndim == 3:
                batch = batch[..., None]
            n = batch.shape[0]
            if n == 0:
                return None
            if n > B or batch.shape[1:] != (H, W, K):
                raise ValueError(f"reader batch {batch.shape} does not fit the plan ({B}, {H}, {W}, {K})")
            if state["src_dtype"] is None:
                state["src_dtype"] = batch.dtype
                self._alloc(batch.dtype)
            elif batch.dtype != state["src_dtype"]:
                raise ValueError("the reader changed its dtype between batches")
            i = state["i"]
            slot = i & 1
            if i >= 2:
                h2d_done[slot].synchronize()
            host = self.h_in[slot][:n]
            view = _wire(batch.dtype)[1]
            if view == np.float32:
                host.copy_(torch.from_numpy(np.ascontiguousarray(batch, dtype=np.float32)))
            else:
                host.copy_(torch.from_numpy(np.ascontiguousarray(batch).view(view)))
            keep[slot] = host
            with torch.cuda.stream(self.copy):
                if i >= 2:
                    self.copy.wait_event(comp_done[slot])
                self.d_in[slot][:n].copy_(host, non_blocking=True)
                h2d_done[slot].record(self.copy)
            entry = (slot, state["t0"], n)
            state["i"] += 1
            state["t0"] += n
            out["h2d_bytes"] += host.numel() * host.element_size()
            return entry

        def flush(entry):
            slot, t0, n = entry
            d2h_done[slot].synchronize()
            st = self.h_stats[slot][:n].numpy()
            out["mean_disp"].extend(st[:, 0].tolist())
            out["max_disp"].extend(st[:, 1].tolist())
            out["mean_div"].extend(st[:, 2].tolist())
            out["mean_translation"].extend(st[:, 3].tolist())
            if writer is not None:
                reg = self.h_reg[slot][:n].numpy()
                if state["src_dtype"] == np.uint16:
                    reg = reg.view(np.uint16)
                writer.write_frames(reg.astype(state["src_dtype"], copy=False))
            if flow_sink is not None:
                flow_sink(t0, self.h_flow[slot][:n].numpy().copy())
            out["frames"] += n

        staged = stage()
        first = True
        while staged is not None:
            slot, t0, n = staged
            with torch.cuda.stream(self.compute):
                self.compute.wait_event(h2d_done[slot])
                if state["i"] > 2:
                    self.compute.wait_event(d2h_done[slot])
                raw = _widen(self.d_in[slot][:n], state["src_dtype"], self.d_raw[:n])
                proc = self.d_proc[:n]
                if ref_proc is None:
                    ref_proc = preprocess_device(self.ref_raw64_t, self.ref_raw, self.sigma, self.norm,
                                                 stream=self.compute)
                    self.plan.set_reference(ref_proc, self.weight_t, stream=self.compute)
                preprocess_device(raw, self.ref_raw, self.sigma, self.norm, frames_dtype=state["src_dtype"],
                                  out=proc, stream=self.compute)
                flow = self.d_flow[slot][:n]
                if first and self.update_w:
                    # initial field: mean flow of the first min(22, n) frames from zero (the
                    # reference also computes it when it then starts every batch from zero)
                    n_init = min(22, n)
                    self._flows(proc[:n_init], None, flow[:n_init])
                    w_init = _mean_frames(flow[:n_init])
                    first = False
                uv = w_init if self.update_w else torch.zeros_like(w_init)
                out["w_init"].append(uv.detach().clone())
                self._flows(proc, uv, flow)
                if self.update_w:
                    w_init = _mean_frames(flow[max(0, n - 20):n])
                api.imregister_device(raw, flow, self.ref_raw_t, self.method, out_t=self.d_warp[:n],
                                      stream=self.compute)
                _narrow(self.d_warp[:n], state["src_dtype"], self.d_reg[slot][:n])
                _, stats = flow_statistics_device(flow, valid_masks=False, stream=self.compute)
                self.d_stats[slot][:n].copy_(stats)
                comp_done[slot].record(self.compute)
            with torch.cuda.stream(self.copy):
                self.copy.wait_event(comp_done[slot])
                self.h_reg[slot][:n].copy_(self.d_reg[slot][:n], non_blocking=True)
                self.h_flow[slot][:n].copy_(self.d_flow[slot][:n], non_blocking=True)
                self.h_stats[slot][:n].copy_(self.d_stats[slot][:n], non_blocking=True)
                d2h_done[slot].record(self.copy)
            out["d2h_bytes"] += (self.h_reg[slot][:n].numel() * self.h_reg[slot].element_size()
                                 + n * H * W * 2 * 4 + n * 4 * 8)
            if pending:
                flush(pending.pop(0))
            pending.append((slot, t0, n))
            staged = stage()
        while pending:
            flush(pending.pop(0))
        torch.cuda.current_stream(self.dev).wait_stream(self.compute)
        out["w_init"] = [w.cpu().numpy() for w in out["w_init"]]
        return out

    def close(self):
        self.plan.close()
