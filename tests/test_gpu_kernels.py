"""GPU kernels against the CPU oracle, one building block at a time."""
import numpy as np
import pytest

import pyflowreg_gb300 as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ih,iw,oh,ow", [(37, 45, 30, 36), (37, 45, 9, 11), (64, 64, 64, 64), (20, 24, 25, 30),
                                         (512, 512, 9, 9), (512, 512, 410, 410), (256, 300, 137, 160)])
def test_resize(oracle, ih, iw, oh, ow):
    rng = np.random.default_rng(ih * 1000 + ow)
    img = rng.random((ih, iw, 2)).astype(np.float32)
    got = G.imresize_fused_gauss_cubic(img, (oh, ow))
    ref = oracle.resize(img, (oh, ow))
    np.testing.assert_allclose(got, ref, rtol=0, atol=2e-6)


@pytest.mark.parametrize("cubic", [True, False])
def test_warp(oracle, golden_dir, cubic):
    g = np.load(f"{golden_dir}/warp.npz")
    f2 = g["f2"].astype(np.float32)
    f1 = g["f1"].astype(np.float32)
    got = G.imregister_wrapper(f2, g["u"], g["v"], f1, "cubic" if cubic else "linear")
    ref = oracle.warp(f2.astype(np.float64), g["u"], g["v"], f1.astype(np.float64), cubic)
    np.testing.assert_allclose(got, ref, rtol=0, atol=2e-6)
    oob = ((np.arange(27)[None, :] + g["u"]) < 0) | ((np.arange(27)[None, :] + g["u"]) >= 27) | \
          ((np.arange(31)[:, None] + g["v"]) < 0) | ((np.arange(31)[:, None] + g["v"]) >= 31)
    assert oob.any()
    np.testing.assert_array_equal(got[oob], f1[oob])


def test_warp_integer_shift_content():
    """Reference warp test (tests/core/test_warping.py:250-300): a constant
    integer shift reproduces shifted content; out-of-bounds pixels take the
    reference value."""
    H, W, sx, sy = 64, 64, 10, 5
    yy, xx = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    frame = (yy * 1000 + xx).astype(np.float32)
    u = np.full((H, W), sx, np.float64)
    v = np.full((H, W), sy, np.float64)
    ref = np.zeros((H, W), np.float32)
    out = G.imregister_wrapper(frame, u, v, ref)
    np.testing.assert_allclose(out[: H - sy, : W - sx], frame[sy:, sx:], atol=1e-2)
    assert np.all(out[:, W - sx:] == 0) and np.all(out[H - sy:, :] == 0)


@pytest.mark.parametrize("gray", [0, 1])
def test_motion_tensor(oracle, golden_dir, gray):
    g = np.load(f"{golden_dir}/tensor.npz")
    f1 = g["f1"].astype(np.float32).astype(np.float64)
    f2 = g["f2"].astype(np.float32).astype(np.float64)
    hy, hx = float(g["hy"]), float(g["hx"])
    fn = G.get_motion_tensor_gray if gray else G.get_motion_tensor_gc
    got = np.stack(fn(f1, f2, hy, hx))
    ref = np.stack(oracle.motion_tensor(f1, f2, hy, hx, 0, gray))
    scale = np.abs(ref).max(axis=(1, 2), keepdims=True) + 1e-30
    assert np.isfinite(got).all()
    np.testing.assert_allclose(got / scale, ref / scale, rtol=0, atol=2e-5)


def test_motion_tensor_known_answer():
    hy, hx = 1.0, 2.0
    x = np.arange(23, dtype=np.float64) * hx
    f = np.tile(1e-3 * x**2, (17, 1))
    J = G.get_motion_tensor_gc(f, f, hy, hx)
    np.testing.assert_allclose(J[0][8, 11], 0.8, atol=0.01)
    assert J[2][8, 11] == 0 and J[4][8, 11] == 0


@pytest.mark.parametrize("h,w", [(6, 6), (7, 13), (40, 33), (128, 96)])
def test_median(oracle, h, w):
    rng = np.random.default_rng(h * w)
    a = rng.standard_normal((h, w)).astype(np.float32)
    a[::3, ::2] = a[0, 0]  # ties
    got = G.median_filter5(a)
    ref = oracle.median5(a.astype(np.float64)).astype(np.float32)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("h,w", [(5, 5), (9, 17), (64, 48), (131, 77)])
def test_median_f64_exact(h, w):
    """The float64 median (float32-key selection with a float64 tie-break) equals
    scipy's median_filter(size=(5, 5), mode="mirror") bit for bit, including
    values that agree in their top 20 fraction bits, exact ties, signed zeros
    and large magnitudes."""
    import ctypes

    import scipy.ndimage as ndi
    import torch

    from pyflowreg_gb300 import _lib

    rng = np.random.default_rng(h * 1000 + w)
    a = rng.standard_normal((h, w))
    # a smooth ramp (values 1e-7 apart share their top 20 fraction bits, as in a
    # smooth flow field), positive on the left half, negative on the right
    yy, xx = np.mgrid[:h, :w]
    ramp = 0.3 + 1e-7 * (yy * 3 + xx) + 2.0 ** -44 * rng.integers(0, 64, (h, w))
    a[: h // 2 + 1] = np.where(xx < w // 2, ramp, -ramp)[: h // 2 + 1]
    # blocks whose values all share one high word (every tie rank occurs)
    a[-4:, : w // 3] = 1.7 * (1 + 2.0 ** -45 * rng.integers(-40, 40, a[-4:, : w // 3].shape))
    a[-4:, -(w // 3):] = -1.7 * (1 + 2.0 ** -45 * rng.integers(-40, 40, a[-4:, -(w // 3):].shape))
    a[::3, ::2] = a[0, 0]                                   # exact ties
    a[1::4, 1::3] = a[1, 1] * (1 + 2.0 ** -40 * rng.integers(-3, 4, a[1::4, 1::3].shape))  # same top bits
    a[2::5, ::4] = 0.0
    a[3::6, 2::5] = -0.0
    a[0, :] *= 1e200
    src = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dst = torch.empty_like(src)
    rc = _lib.load().frg_median5_f64(h, w, ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
                                     ctypes.c_void_p(0))
    _lib.check(rc, "frg_median5_f64")
    torch.cuda.synchronize()
    ref = ndi.median_filter(a, size=(5, 5), mode="mirror")
    np.testing.assert_array_equal(dst.cpu().numpy(), ref)
