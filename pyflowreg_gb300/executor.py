"""``GB300Executor``: pyflowreg batch executor that registers a whole batch in
one device pass.

Implements ``BaseExecutor.process_batch`` (motion_correction/parallelization/
base.py:76-110) with the semantics of ``SequentialExecutor.process_batch``
(sequential.py:27-169, no cross-correlation pre-alignment): flow of every
frame against the preprocessed reference starting from ``w_init``, then the
compensation warp of the raw frame against the raw reference.  The batch is
uploaded once, all flows are computed by the batched plan, the warp runs on
the device, and the results come back once.

Importing this module requires pyflowreg (it subclasses its BaseExecutor).
"""

from __future__ import annotations

from typing import Callable, Optional

import numpy as np
from pyflowreg.motion_correction.parallelization.base import BaseExecutor

from . import api

_CC_KEYS = ("cc_initialization", "cc_hw", "cc_up")


class GB300Executor(BaseExecutor):
    def __init__(self, n_workers: Optional[int] = None):
        super().__init__(n_workers=1)

    def process_batch(self, batch, batch_proc, reference_raw, reference_proc, w_init,
                      get_displacement_func: Callable, imregister_func: Callable,
                      interpolation_method: str = "cubic",
                      progress_callback: Optional[Callable[[int], None]] = None, **kwargs):
        import torch

        batch, batch_proc, reference_raw, reference_proc, w_init = self._normalize_inputs(
            batch, batch_proc, reference_raw, reference_proc, w_init)
        T, H, W, C = batch.shape
        flow_params_all = dict(kwargs.get("flow_params", {}))
        if flow_params_all.get("cc_initialization", False):
            raise NotImplementedError("cross-correlation pre-alignment is not implemented by the gb300 executor")
        flow_params = {k: v for k, v in flow_params_all.items() if k not in _CC_KEYS}
        flow = api.get_displacement_batch(reference_proc, batch_proc, uv=w_init, **flow_params)

        dev = torch.device("cuda", torch.cuda.current_device())
        frames_t = torch.from_numpy(np.ascontiguousarray(batch, dtype=np.float32)).to(dev)
        flow_t = torch.from_numpy(np.ascontiguousarray(flow, dtype=np.float32)).to(dev)
        ref_t = torch.from_numpy(np.ascontiguousarray(reference_raw, dtype=np.float32)).to(dev)
        reg = api.imregister_device(frames_t, flow_t, ref_t, interpolation_method).cpu().numpy()
        if np.issubdtype(batch.dtype, np.integer):
            # registered[t] = reg_frame into np.empty_like(batch) (sequential.py:82, 159-163) casts
            # unsafely: in-range values truncate toward zero; out-of-range ones (cubic overshoot),
            # which numpy leaves to the platform, saturate here
            info = np.iinfo(batch.dtype)
            reg = np.clip(np.trunc(reg), info.min, info.max)
        registered = reg.astype(batch.dtype, copy=False)
        if progress_callback is not None:
            progress_callback(T)
        return registered, flow.astype(np.float32, copy=False)

    def get_info(self) -> dict:
        info = super().get_info()
        info.update({"parallel": True, "description": "Batched GB300 device registration"})
        return info
