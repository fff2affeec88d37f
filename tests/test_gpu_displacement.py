"""Full get_displacement on the GPU against the oracle (numba-equivalent,
lexicographic fp64) and the golden vectors of the reference itself.

Tolerance (fp32 device arithmetic vs the fp64 reference):
max |delta flow| <= 1e-3 px and mean endpoint error <= 1e-4 px.
"""
import numpy as np
import pytest

import pyflowreg_gb300 as G
from pyflowreg_gb300.synthetic import Video, pair_256

pytestmark = pytest.mark.gpu

MAX_TOL = 1e-3
EPE_TOL = 1e-4


def assert_flow_close(got, ref):
    d = got - ref
    maxd = np.abs(d).max()
    epe = np.sqrt((d ** 2).sum(-1)).mean()
    assert maxd <= MAX_TOL and epe <= EPE_TOL, f"max {maxd:.3e} px, mean EPE {epe:.3e} px"


def test_golden_single_channel(golden_dir):
    f = np.load(f"{golden_dir}/full.npz")
    got = G.get_displacement(f["a_fixed"], f["a_moving"], alpha=(1.5, 1.5))
    assert got.shape == f["a_flow"].shape and got.dtype == np.float64
    assert_flow_close(got, f["a_flow"])


def test_golden_two_channels_uv_weight(golden_dir):
    f = np.load(f"{golden_dir}/full.npz")
    got = G.get_displacement(f["b_fixed"], f["b_moving"], alpha=(1.5, 1.5), uv=f["b_uv"], weight=f["b_weight"],
                             iterations=20, update_lag=4)
    assert_flow_close(got, f["b_flow"])


def test_golden_gray_value_constancy(golden_dir):
    f = np.load(f"{golden_dir}/full.npz")
    got = G.get_displacement(f["b_fixed"], f["b_moving"], const_assumption="gray", iterations=12, eta=0.7)
    assert_flow_close(got, f["d_flow"])


def test_pair_256_default_options(oracle):
    """Single 256x256 pair with pyflowreg's default OFOptions flow settings."""
    fixed, moving, _ = pair_256(0)
    kw = dict(alpha=(1.5, 1.5), levels=100, iterations=50, update_lag=5, a_data=0.45, eta=0.8)
    ref = oracle.get_displacement(fixed, moving, **kw)
    got = G.get_displacement(fixed, moving, **kw)
    assert_flow_close(got, ref)


@pytest.mark.slow
def test_video_512x2_frames(oracle):
    vid = Video(seed=1, h=512, w=512, K=2)
    frames, _ = vid.frames(0, 3)
    fixed = frames.mean(axis=0)
    fixed = fixed / fixed.max()
    mov = frames / frames.max()
    kw = dict(alpha=(1.5, 1.5), levels=100, weight=np.array([0.5, 0.5]))
    ref = oracle.get_displacement_batch(fixed, mov[:2], **kw)
    got = G.get_displacement_batch(fixed, mov[:2], **kw)
    for t in range(2):
        assert_flow_close(got[t].astype(np.float64), ref[t])


def test_batch_equals_single_frames():
    rng = np.random.default_rng(5)
    fixed, moving, _ = pair_256(1, h=96, w=80)
    frames = np.stack([moving, np.roll(moving, 1, axis=0), np.roll(moving, -2, axis=1)])
    batch = G.get_displacement_batch(fixed, frames, alpha=(1.5, 1.5))
    for t in range(3):
        single = G.get_displacement(fixed, frames[t], alpha=(1.5, 1.5))
        np.testing.assert_array_equal(batch[t], single.astype(np.float32))


def test_uv_init_and_nonsquare(oracle):
    fixed, moving, truth = pair_256(2, h=72, w=120)
    uv = (truth * 0.7).astype(np.float32)
    kw = dict(alpha=(2.0, 1.0), iterations=30, update_lag=4, uv=uv)
    assert_flow_close(G.get_displacement(fixed, moving, **kw), oracle.get_displacement(fixed, moving, **kw))


def test_tall_frame(oracle):
    fixed, moving, _ = pair_256(3, h=160, w=64)
    kw = dict(alpha=(1.5, 1.5), iterations=20)
    assert_flow_close(G.get_displacement(fixed, moving, **kw), oracle.get_displacement(fixed, moving, **kw))


def test_unsupported_options_raise():
    fixed, moving, _ = pair_256(4, h=32, w=32)
    with pytest.raises(NotImplementedError):
        G.get_displacement(fixed, moving, const_assumption="cs")
    with pytest.raises(NotImplementedError):
        G.get_displacement(fixed, moving, gnc_schedule=(0.0, 1.0))
    with pytest.raises(ValueError):
        G.get_displacement(fixed, moving, const_assumption="nope")
