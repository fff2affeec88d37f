"""The drop-in boundary on the GPU: the executor's batch (one device pass)
against what pyflowreg's SequentialExecutor computes frame by frame
(parallelization/sequential.py:141-163) with the oracle's get_displacement
and warp; and the backend as pyflowreg's core registry hands it out
(core/backend_registry.py:19-68), against the oracle.  Default precision:
fp64, within the parity bar (max |delta flow| <= 1e-3 px, mean EPE <= 1e-4 px).
"""
import numpy as np
import pytest

from pyflowreg_env import import_pyflowreg

pytestmark = pytest.mark.gpu

KW = dict(alpha=(1.5, 1.5), iterations=20, update_lag=5, levels=100, eta=0.8, min_level=0, a_data=0.45,
          a_smooth=1.0, const_assumption="gc")


def _batch(dtype, T=4, H=72, W=64, C=2):
    from pyflowreg_gb300.synthetic import pair_256

    fr = []
    for t in range(T):
        _, mv, _ = pair_256(40 + t, h=H, w=W)
        mv = np.asarray(mv, np.float64)
        fr.append(np.stack([mv * (900 + 300 * c) + 40 for c in range(C)], axis=2))
    v = np.stack(fr)
    return v.astype(dtype)


def _flow_diff(a, b):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return float(np.abs(d).max()), float(np.sqrt((d ** 2).sum(-1)).mean())


@pytest.mark.parametrize("dtype", [np.uint16, np.float32])
def test_executor_batch_matches_sequential_semantics(oracle, dtype):
    from pyflowreg_gb300.executor import process_batch

    batch = _batch(dtype)
    ref_raw = batch[:2].astype(np.float64).mean(0)
    lo, hi = ref_raw.min(), ref_raw.max()
    batch_proc = ((batch.astype(np.float64) - lo) / (hi - lo)).astype(np.float32)
    ref_proc = ((ref_raw - lo) / (hi - lo)).astype(np.float32)
    w_init = (0.4 * np.random.default_rng(9).standard_normal(batch.shape[1:3] + (2,))).astype(np.float32)
    weight = np.full(batch.shape[1:], 0.5)
    reg, flow = process_batch(batch, batch_proc, ref_raw, ref_proc, w_init, "cubic",
                              dict(KW, weight=weight, gnc_schedule=None, warping_steps=None,
                                   cc_initialization=False))
    assert flow.dtype == np.float32 and reg.dtype == batch.dtype and reg.shape == batch.shape
    for t in range(batch.shape[0]):
        want = oracle.get_displacement(ref_proc, batch_proc[t], uv=w_init.copy(), weight=weight,
                                       **KW).astype(np.float32)
        mx, ep = _flow_diff(flow[t], want)
        assert mx <= 1e-3 and ep <= 1e-4, (t, mx, ep)
        # imregister_wrapper of the raw frame with the stored float32 flow, cast as the executors cast
        for c in range(batch.shape[3]):
            w = oracle.warp(batch[t, :, :, c].astype(np.float64), flow[t, :, :, 0].astype(np.float64),
                            flow[t, :, :, 1].astype(np.float64), ref_raw[:, :, c])
            if np.issubdtype(dtype, np.integer):
                info = np.iinfo(dtype)
                w = np.clip(np.trunc(w.astype(np.float32)), info.min, info.max).astype(dtype)
                # float32 warps that agree to a few ulp can truncate to neighbouring integers
                assert np.abs(reg[t, :, :, c].astype(np.int64) - w.astype(np.int64)).max() <= 1
                assert np.mean(reg[t, :, :, c] == w) > 0.99
            else:
                np.testing.assert_allclose(reg[t, :, :, c], w, rtol=0, atol=2e-6 * np.abs(w).max())


def test_backend_from_pyflowreg_registry_matches_oracle(oracle):
    import_pyflowreg()
    from pyflowreg.core.backend_registry import get_backend

    from pyflowreg_gb300 import backend

    backend.register(executor=False)
    fn = get_backend(backend.BACKEND_NAME)()  # OFOptions.resolve_get_displacement with no backend_params
    fixed = _batch(np.float32, T=1)[0] / 1000.0
    moving = _batch(np.float32, T=2)[1] / 1000.0
    got = fn(fixed, moving, **KW)
    assert got.dtype == np.float64 and got.shape == fixed.shape[:2] + (2,)
    mx, ep = _flow_diff(got, oracle.get_displacement(fixed, moving, **KW))
    assert mx <= 1e-3 and ep <= 1e-4, (mx, ep)
