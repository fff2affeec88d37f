"""``GB300Executor``: pyflowreg batch executor that registers a whole batch in
one device pass.

Implements ``BaseExecutor.process_batch`` (motion_correction/parallelization/
base.py:76-110) with the semantics of ``SequentialExecutor.process_batch``
(sequential.py:27-169, no cross-correlation pre-alignment): flow of every
frame against the preprocessed reference starting from ``w_init``, then the
compensation warp of the raw frame against the raw reference.  The batch is
uploaded once, all flows are computed by the batched plan, the warp runs on
the device, and the results come back once.

The batch logic is :func:`process_batch`, which needs no pyflowreg import;
:class:`GB300Executor` (defined when pyflowreg is importable) subclasses
pyflowreg's ``BaseExecutor`` around it.
"""

from __future__ import annotations

from typing import Callable, Optional

import numpy as np

from . import api

_CC_KEYS = ("cc_initialization", "cc_hw", "cc_up")


def process_batch(batch, batch_proc, reference_raw, reference_proc, w_init, interpolation_method="cubic",
                  flow_params=None, precision="fp64"):
    """One batch as ``SequentialExecutor.process_batch`` computes it, in one
    device pass.  Arrays as pyflowreg's ``BaseExecutor._normalize_inputs``
    leaves them: batch, batch_proc (T, H, W, C); reference_raw,
    reference_proc (H, W, C); w_init (H, W, 2).  Returns (registered (T, H, W,
    C) in the batch's dtype, flow (T, H, W, 2) float32).

    * flow[t] = get_displacement(reference_proc, batch_proc[t], uv=w_init,
      **flow_params), stored as float32 (sequential.py:141-145, 296-298);
    * registered[t] = imregister_wrapper(batch[t], flow[t, ..., 0],
      flow[t, ..., 1], reference_raw, interpolation_method) (:300-307),
      stored into ``np.empty_like(batch)``: integer batches truncate toward
      zero (numpy's cast); out-of-range values, which numpy leaves to the
      platform, saturate here.
    """
    T = batch.shape[0]
    flow_params = dict(flow_params or {})
    if flow_params.get("cc_initialization", False):
        raise NotImplementedError("cross-correlation pre-alignment is not implemented by the gb300 executor")
    flow_params = {k: v for k, v in flow_params.items() if k not in _CC_KEYS}
    flow = api.get_displacement_batch(reference_proc, batch_proc, uv=w_init, precision=precision, **flow_params)
    flow32 = np.ascontiguousarray(flow, dtype=np.float32)
    reg = _warp_frames(batch, flow32, reference_raw, interpolation_method)
    if np.issubdtype(batch.dtype, np.integer):
        info = np.iinfo(batch.dtype)
        reg = np.clip(np.trunc(reg), info.min, info.max)
    registered = reg.astype(batch.dtype, copy=False).reshape(batch.shape)
    assert registered.shape[0] == T
    return registered, flow32


def _warp_frames(batch, flow32, reference_raw, interpolation_method):
    """imregister_wrapper of every frame on the device: (T, H, W, C) float32."""
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    frames_t = torch.from_numpy(np.ascontiguousarray(batch, dtype=np.float32)).to(dev)
    flow_t = torch.from_numpy(flow32).to(dev)
    ref_t = torch.from_numpy(np.ascontiguousarray(reference_raw, dtype=np.float32)).to(dev)
    return api.imregister_device(frames_t, flow_t, ref_t, interpolation_method).cpu().numpy()


def _precision_of(get_displacement_func) -> str:
    """The precision the registered backend was configured with (its factory
    returns a partial of api.get_displacement), "fp64" otherwise."""
    kw = getattr(get_displacement_func, "keywords", None) or {}
    return kw.get("precision", "fp64")


try:
    from pyflowreg.motion_correction.parallelization.base import BaseExecutor
except ImportError:  # pyflowreg absent: process_batch stays usable on its own
    BaseExecutor = None

if BaseExecutor is not None:

    class GB300Executor(BaseExecutor):
        def __init__(self, n_workers: Optional[int] = None):
            super().__init__(n_workers=1)

        def process_batch(self, batch, batch_proc, reference_raw, reference_proc, w_init,
                          get_displacement_func: Callable, imregister_func: Callable,
                          interpolation_method: str = "cubic",
                          progress_callback: Optional[Callable[[int], None]] = None, **kwargs):
            batch, batch_proc, reference_raw, reference_proc, w_init = self._normalize_inputs(
                batch, batch_proc, reference_raw, reference_proc, w_init)
            registered, flow = process_batch(batch, batch_proc, reference_raw, reference_proc, w_init,
                                             interpolation_method, kwargs.get("flow_params", {}),
                                             _precision_of(get_displacement_func))
            if progress_callback is not None:
                progress_callback(batch.shape[0])
            return registered, flow

        def get_info(self) -> dict:
            info = super().get_info()
            info.update({"parallel": True, "description": "Batched GB300 device registration"})
            return info
