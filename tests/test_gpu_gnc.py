"""Graduated non-convexity stages (core/optical_flow.py:620-770, 887-929) on
the GPU against the oracle.

Parity bar as for the plain pyramid (fp64 reference-order mode against the
fp64 oracle with numba typing): max |delta flow| <= 1e-3 px and mean
endpoint error <= 1e-4 px.  GNC runs on the reference-order kernels in both
precisions, so the fp32 plan's flow is the fp64 flow rounded to float32.
"""
import numpy as np
import pytest

import pyflowreg_gb300 as G
from pyflowreg_gb300.synthetic import pair_256

pytestmark = pytest.mark.gpu

MAX_TOL = 1e-3
EPE_TOL = 1e-4
GOLDEN_KW = dict(alpha=(1.5, 1.5), gnc_schedule=(0.0, 0.5, 1.0), warping_steps=2, iterations=6, a_smooth=0.7)


def flow_diff(got, ref):
    d = np.asarray(got, np.float64) - np.asarray(ref, np.float64)
    return float(np.abs(d).max()), float(np.sqrt((d ** 2).sum(-1)).mean())


def assert_parity(got, ref):
    maxd, epe = flow_diff(got, ref)
    assert maxd <= MAX_TOL and epe <= EPE_TOL, f"max {maxd:.3e} px, mean EPE {epe:.3e} px"


def test_gnc_golden(oracle, golden_dir):
    f = np.load(f"{golden_dir}/full.npz")
    got = G.get_displacement(f["b_fixed"], f["b_moving"], precision="fp64", **GOLDEN_KW)
    assert got.shape == f["g_flow"].shape
    assert_parity(got, oracle.get_displacement(f["b_fixed"], f["b_moving"], **GOLDEN_KW))
    # the committed vector comes from the reference source run without numba
    assert flow_diff(got, f["g_flow"])[0] < 1e-3
    got32 = G.get_displacement(f["b_fixed"], f["b_moving"], precision="fp32", **GOLDEN_KW)
    np.testing.assert_array_equal(got32, got.astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("kw", [
    dict(alpha=(1.5, 1.5), gnc_schedule=(0.0, 0.5, 1.0), warping_steps=2, iterations=8),
    dict(alpha=(2.0, 1.0), gnc_schedule=(0.0, 0.25, 0.75, 1.0), warping_steps=3, iterations=7, update_lag=3,
         a_smooth=0.6, a_data=0.3),
    dict(alpha=(1.5, 1.5), gnc_schedule=(0.0, 1.0), warping_steps=2, iterations=6, const_assumption="cs"),
    dict(alpha=(1.5, 1.5), gnc_schedule=(0.0, 0.5, 1.0), warping_steps=2, iterations=6, const_assumption="gray",
         eta=0.7),
    dict(alpha=(1.5, 1.5), gnc_schedule=(0.0, 1.0), warping_steps=2, iterations=6, min_level=2),
    # a_data = 1 is outside (0, 1): the data weights keep the plain robust form
    dict(alpha=(1.5, 1.5), gnc_schedule=(0.0, 0.5, 1.0), warping_steps=1, iterations=5, a_data=1.0, update_lag=1),
])
def test_fp64_gnc_options(oracle, kw):
    fixed, moving, _ = pair_256(3, h=40, w=56)
    got = G.get_displacement(fixed, moving, precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(fixed, moving, **kw))


def test_fp64_gnc_initial_flow_and_weights(oracle):
    fixed, moving, truth = pair_256(8, h=48, w=40)
    fixed2 = np.stack([fixed, 0.5 * fixed + 0.2], -1)
    moving2 = np.stack([moving, 0.5 * moving + 0.2], -1)
    kw = dict(alpha=(1.5, 1.5), gnc_schedule=(0.0, 0.5, 1.0), warping_steps=2, iterations=6,
              uv=(truth * 0.5).astype(np.float32), weight=np.array([0.7, 0.3]), a_data=np.array([0.45, 0.6]))
    got = G.get_displacement(fixed2, moving2, precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(fixed2, moving2, **kw))


@pytest.mark.parametrize("shape", [(12, 40, 0.5), (10, 30, 0.4)])
def test_fp64_gnc_small_levels_without_median(oracle, shape):
    """Levels with min(h, w) <= 5 skip the median; the state's border is then
    u + du with du's border as set_boundary_2d left it."""
    h, w, eta = shape
    fixed, moving, _ = pair_256(9, h=h, w=w)
    kw = dict(alpha=(1.5, 1.5), gnc_schedule=(0.0, 0.5, 1.0), warping_steps=3, iterations=7, eta=eta)
    got = G.get_displacement(fixed, moving, precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(fixed, moving, **kw))
    kw["a_smooth"] = 0.8
    got = G.get_displacement(fixed, moving, precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(fixed, moving, **kw))


def test_fp64_gnc_default_warping_steps(oracle):
    fixed, moving, _ = pair_256(10, h=32, w=32)
    kw = dict(alpha=(1.5, 1.5), gnc_schedule=(0.0, 1.0), iterations=4)  # 10 warping steps per level
    got = G.get_displacement(fixed, moving, precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(fixed, moving, **kw))


def test_gnc_batch_frames_independent(oracle):
    fixed, _, _ = pair_256(11, h=36, w=44)
    frames = np.stack([pair_256(s, h=36, w=44)[1] for s in (12, 13, 14)])
    kw = dict(alpha=(1.5, 1.5), gnc_schedule=(0.0, 0.5, 1.0), warping_steps=2, iterations=6)
    got = G.get_displacement_batch(fixed, frames, precision="fp64", **kw)
    for t in range(frames.shape[0]):
        assert_parity(got[t], oracle.get_displacement(fixed, frames[t], **kw))


def test_gnc_invalid_schedules_raise():
    fixed, moving, _ = pair_256(4, h=32, w=32)
    for bad in [(0.5, 1.0), (0.0,), (0.0, 0.7, 0.5, 1.0), (0.0, 1.2)]:
        with pytest.raises(ValueError):
            G.get_displacement(fixed, moving, gnc_schedule=bad)
    with pytest.raises(ValueError):
        G.get_displacement(fixed, moving, gnc_schedule=(0.0, 1.0), warping_steps=0)
