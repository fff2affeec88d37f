"""The drop-in boundary, driven by pyflowreg itself (unmodified, imported by
tests/pyflowreg_env.py):

* the backend registers in pyflowreg's own registry
  (core/backend_registry.py:19-68) and ``OFOptions(flow_backend=...)``
  resolves to it through ``OFOptions.resolve_get_displacement``
  (motion_correction/OF_options.py:1021-1082), fp64 (the parity precision)
  by default;
* the ``"gb300"`` executor registers with pyflowreg's RuntimeContext and its
  ``process_batch`` returns what pyflowreg's ``SequentialExecutor``
  (parallelization/sequential.py:27-169) returns for the same batch;
* ``compensate_arr`` (motion_correction/compensate_arr.py:16-231) with
  ``RegistrationConfig(parallelization="gb300")`` runs pyflowreg's own batch
  loop through that executor and gives the sequential executor's result.

These run on the CPU: the device steps (the backend's per-frame flow, the
executor's batched flow and its compensation warp) are replaced by the
oracle and by pyflowreg's own imregister_wrapper, so what is checked is the
executor's host logic (input normalisation, w_init and option forwarding,
float32 flow storage, the integer cast of registered frames) inside
pyflowreg's real pipeline.  The
device steps themselves are checked against the oracle on the GPU
(tests/test_gpu_boundary.py).
"""
import numpy as np
import pytest

from pyflowreg_env import import_motion_correction, import_pyflowreg

KW = dict(alpha=(1.5, 1.5), iterations=6, update_lag=3, levels=100, eta=0.8, min_level=0)


def _video(T=5, H=40, W=36, C=2, dtype=np.uint16, seed=0):
    from pyflowreg_gb300.synthetic import pair_256

    frames = []
    for t in range(T):
        _, mv, _ = pair_256(seed + t, h=H, w=W)
        mv = np.asarray(mv, np.float64)
        fr = np.stack([mv * (1000 + 200 * c) + 50 for c in range(C)], axis=2)
        frames.append(fr)
    v = np.stack(frames)
    return v.astype(dtype) if np.issubdtype(dtype, np.integer) else v.astype(dtype)


@pytest.fixture()
def oracle_device(monkeypatch, oracle):
    """Replaces the device steps by CPU equivalents: the backend's per-frame
    flow and the executor's batched flow by the oracle (pyflowreg's
    get_displacement semantics), the warp by pyflowreg's own
    imregister_wrapper."""
    import_pyflowreg()
    from pyflowreg.core.warping import imregister_wrapper

    from pyflowreg_gb300 import api, executor

    calls = {"flow": 0, "warp": 0, "single": 0}

    def flow_single(fixed, moving, precision="fp64", **kw):
        calls["single"] += 1
        assert precision == "fp64"
        return oracle.get_displacement(fixed, moving, **kw)

    def flow_batch(fixed, moving, uv=None, precision="fp64", **kw):
        calls["flow"] += 1
        assert precision == "fp64"
        return np.stack([oracle.get_displacement(fixed, moving[t], uv=None if uv is None else np.array(uv), **kw)
                         for t in range(moving.shape[0])])

    def warp(batch, flow32, reference_raw, method):
        calls["warp"] += 1
        out = []
        for t in range(batch.shape[0]):
            r = imregister_wrapper(batch[t], flow32[t, ..., 0], flow32[t, ..., 1], reference_raw,
                                   interpolation_method=method)
            out.append(r[..., None] if r.ndim == 2 else r)
        return np.stack(out).astype(np.float32)

    monkeypatch.setattr(api, "get_displacement", flow_single)
    monkeypatch.setattr(api, "get_displacement_batch", flow_batch)
    monkeypatch.setattr(executor, "_warp_frames", warp)
    return calls


def test_backend_resolves_through_pyflowreg_options():
    import_motion_correction()
    from functools import partial

    from pyflowreg.core.backend_registry import get_backend
    from pyflowreg.motion_correction.OF_options import OFOptions

    from pyflowreg_gb300 import api, backend

    backend.register()
    assert get_backend(backend.BACKEND_NAME) is backend._factory
    fn = OFOptions(flow_backend=backend.BACKEND_NAME).resolve_get_displacement()
    assert isinstance(fn, partial) and fn.func is api.get_displacement
    assert fn.keywords == {"precision": "fp64"}
    fn32 = OFOptions(flow_backend=backend.BACKEND_NAME, backend_params={"precision": "fp32"}).resolve_get_displacement()
    assert fn32.keywords == {"precision": "fp32"}
    with pytest.raises(ValueError):
        OFOptions(flow_backend=backend.BACKEND_NAME, backend_params={"precision": "fp16"}).resolve_get_displacement()
    with pytest.raises(ValueError):
        OFOptions(flow_backend=backend.BACKEND_NAME, backend_params={"threads": 4}).resolve_get_displacement()


def test_executor_registers_with_pyflowreg_runtime():
    import_motion_correction()
    from pyflowreg._runtime import RuntimeContext

    from pyflowreg_gb300 import backend
    from pyflowreg_gb300.executor import GB300Executor

    backend.register()
    assert RuntimeContext.get_parallelization_executor(backend.EXECUTOR_NAME) is GB300Executor
    assert GB300Executor().get_info()["parallel"] is True


@pytest.mark.parametrize("dtype", [np.uint16, np.float32])
def test_executor_matches_sequential_executor(oracle, oracle_device, dtype):
    import_motion_correction()
    from functools import partial

    from pyflowreg.core.warping import imregister_wrapper
    from pyflowreg.motion_correction.parallelization.sequential import SequentialExecutor

    from pyflowreg_gb300.executor import GB300Executor

    batch = _video(T=4, dtype=dtype)
    ref_raw = batch[:2].astype(np.float64).mean(0)
    lo, hi = ref_raw.min(), ref_raw.max()
    batch_proc = ((batch.astype(np.float64) - lo) / (hi - lo)).astype(np.float32)
    ref_proc = ((ref_raw - lo) / (hi - lo)).astype(np.float32)
    rng = np.random.default_rng(3)
    w_init = (0.3 * rng.standard_normal((batch.shape[1], batch.shape[2], 2))).astype(np.float32)
    weight = np.full(batch.shape[1:], 0.5)
    flow_params = dict(KW, weight=weight, a_data=0.45, a_smooth=1.0, const_assumption="gc", gnc_schedule=None,
                       warping_steps=None, cc_initialization=False)
    seq_reg, seq_flow = SequentialExecutor().process_batch(
        batch, batch_proc, ref_raw, ref_proc, w_init, partial(oracle.get_displacement), imregister_wrapper,
        "cubic", flow_params={k: v for k, v in flow_params.items() if k != "cc_initialization"})
    seen = []
    gb_reg, gb_flow = GB300Executor().process_batch(
        batch, batch_proc, ref_raw, ref_proc, w_init, partial(oracle.get_displacement, precision="fp64"),
        imregister_wrapper, "cubic", progress_callback=seen.append, flow_params=flow_params)
    assert oracle_device == {"flow": 1, "warp": 1, "single": 0}
    assert seen == [batch.shape[0]]
    assert gb_flow.dtype == np.float32 and gb_reg.dtype == batch.dtype
    np.testing.assert_array_equal(gb_flow, seq_flow)
    np.testing.assert_array_equal(gb_reg, seq_reg)


def test_executor_rejects_cross_correlation_prealignment(oracle_device):
    import_motion_correction()
    from pyflowreg_gb300.executor import GB300Executor

    batch = _video(T=2, dtype=np.float32)
    with pytest.raises(NotImplementedError):
        GB300Executor().process_batch(batch, batch, batch[0], batch[0], np.zeros(batch.shape[1:3] + (2,), np.float32),
                                      None, None, flow_params=dict(KW, cc_initialization=True))


def test_compensate_arr_through_the_gb300_executor(oracle, oracle_device):
    """pyflowreg's compensate_arr batch loop (preprocessing, w_init chain,
    batching) with the gb300 executor gives the sequential executor's result."""
    mc = import_motion_correction()
    from pyflowreg.motion_correction.compensate_recording import RegistrationConfig
    from pyflowreg.motion_correction.OF_options import OFOptions

    from pyflowreg_gb300 import backend

    backend.register()
    video = _video(T=7, dtype=np.uint16, seed=10)
    ref = video[:3].astype(np.float64).mean(0)
    opts = dict(alpha=(1.5, 1.5), iterations=6, update_lag=3, levels=100, min_level=0, buffer_size=3)
    out_gb = mc.compensate_arr(video, ref, OFOptions(flow_backend=backend.BACKEND_NAME, **opts),
                               registration_config=RegistrationConfig(parallelization=backend.EXECUTOR_NAME))
    out_seq = mc.compensate_arr(video, ref, OFOptions(**opts), get_displacement=oracle.get_displacement,
                                registration_config=RegistrationConfig(parallelization="sequential"))
    assert oracle_device["flow"] == 3  # batches of 3 frames: 3 + 3 + 1
    assert oracle_device["single"] > 0  # the initial field, frame by frame through the backend
    for a, b in zip(out_gb, out_seq):
        np.testing.assert_array_equal(a, b)
