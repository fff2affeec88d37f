"""Registration of the GB300 backend with pyflowreg.

``register()`` adds, without modifying pyflowreg:

* the flow backend ``"flowreg_gb300"`` through
  ``pyflowreg.core.backend_registry.register_backend``
  (core/backend_registry.py:19-47).  Its factory returns
  :func:`pyflowreg_gb300.api.get_displacement`, so
  ``OFOptions(flow_backend="flowreg_gb300")`` resolves to it through
  ``OFOptions.resolve_get_displacement`` (motion_correction/OF_options.py:1021-1082).
  It declares ``{"sequential", "gb300"}``: multiprocessing workers call
  pyflowreg's own solver directly (parallelization/multiprocessing.py:70, 151),
  so they must not be offered.
* the batch executor ``"gb300"`` through
  ``RuntimeContext.register_parallelization_executor`` (_runtime.py:151-171);
  it registers a whole batch in one device pass (see ``executor.py``).  Select
  it with ``RegistrationConfig(parallelization="gb300")``: pyflowreg's
  automatic executor choice only knows its built-in names
  (motion_correction/compensate_recording.py:283-287).
"""

from __future__ import annotations

BACKEND_NAME = "flowreg_gb300"
EXECUTOR_NAME = "gb300"
SUPPORTED_EXECUTORS = {"sequential", EXECUTOR_NAME}


def _factory(**backend_params):
    """Backend factory, called with ``OFOptions.backend_params``: ``device``
    selects the CUDA device, ``precision`` is "fp64" (default: the reference's
    precision, flows within 1e-3 px of pyflowreg's) or "fp32" (faster, up to
    ~0.7 px away), ``max_frames`` bounds the device batch of one call."""
    from functools import partial

    from . import api

    unknown = set(backend_params) - {"max_frames", "device", "precision"}
    if unknown:
        raise ValueError(f"unknown backend_params for {BACKEND_NAME}: {sorted(unknown)}")
    dev = backend_params.get("device")
    if dev is not None:
        import torch

        torch.cuda.set_device(torch.device(dev))
    precision = backend_params.get("precision", "fp64")
    if precision not in api.PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(api.PRECISIONS)}")
    return partial(api.get_displacement, precision=precision)


def register(executor: bool = True) -> None:
    """Registers the backend (and the batch executor) with pyflowreg."""
    from pyflowreg.core.backend_registry import register_backend

    register_backend(BACKEND_NAME, _factory, supported_executors=set(SUPPORTED_EXECUTORS))
    if executor:
        from pyflowreg._runtime import RuntimeContext

        from .executor import GB300Executor

        RuntimeContext.register_parallelization_executor(EXECUTOR_NAME, GB300Executor)
