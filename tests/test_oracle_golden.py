"""Pins the CPU oracle against golden vectors produced by pyflowreg's own
Python source (tests/golden/make_golden.py).

semantics="python" reproduces the reference source executed without numba
bit for bit; semantics="numba" (the deployed typing: float64 resize
accumulators) must stay within float32 rounding of it.
"""
import numpy as np
import pytest


def load(golden_dir, name):
    import os

    return np.load(os.path.join(golden_dir, f"{name}.npz"))


def test_resize_tables_and_passes(oracle, golden_dir):
    g = load(golden_dir, "resize")
    for q, (ih, iw, oh, ow) in enumerate(g["cases"]):
        sig = oracle.sigma_for((ih, iw), (oh, ow))
        ix, wx = oracle.resize_tables(iw, ow, sig, "python")
        np.testing.assert_array_equal(ix, g[f"ix{q}"])
        np.testing.assert_array_equal(wx, g[f"wx{q}"])
        np.testing.assert_array_equal(oracle.resize(g[f"in{q}"], (oh, ow), "python"), g[f"out{q}"])
        ixn, wxn = oracle.resize_tables(iw, ow, sig, "numba")
        np.testing.assert_array_equal(ixn, g[f"ix{q}"])
        np.testing.assert_allclose(wxn, g[f"wx{q}"], rtol=0, atol=2e-7)
        np.testing.assert_allclose(oracle.resize(g[f"in{q}"], (oh, ow), "numba"), g[f"out{q}"], rtol=0, atol=1e-6)


def test_warp(oracle, golden_dir):
    g = load(golden_dir, "warp")
    np.testing.assert_array_equal(oracle.warp(g["f2"], g["u"], g["v"], g["f1"], True), g["cubic"])
    np.testing.assert_array_equal(oracle.warp(g["f2"], g["u"], g["v"], g["f1"], False), g["linear"])
    np.testing.assert_array_equal(oracle.warp(g["f2_3c"], g["u"], g["v"], g["f1_3c"], True), g["cubic_2c"])


@pytest.mark.parametrize("name,f32,gray", [("gc", 0, 0), ("gc_f32", 1, 0), ("gray", 0, 1), ("gray_f32", 1, 1),
                                           ("cs", 0, 2), ("cs_f32", 1, 2)])
def test_motion_tensor(oracle, golden_dir, name, f32, gray):
    g = load(golden_dir, "tensor")
    f2 = g["f2"].astype(np.float32).astype(np.float64) if f32 else g["f2"]
    J = np.stack(oracle.motion_tensor(g["f1"], f2, float(g["hy"]), float(g["hx"]), f32, gray))
    np.testing.assert_array_equal(J, g[name])


@pytest.mark.parametrize("name,a_s,lag", [("smooth1", 1.0, 5), ("smooth05", 0.5, 3)])
def test_level_solver(oracle, golden_dir, name, a_s, lag):
    g = load(golden_dir, "solver")
    J = g["J"]
    r = oracle.compute_flow(*J, g["weight"], g["u"], g["v"], 1.7, 2.3, 23, lag, np.array([0.45, 0.6]), a_s, 1.25, 0.8)
    np.testing.assert_array_equal(r, g[name])


@pytest.mark.parametrize("name,a_s,lag,beta", [("gnc0_smooth05", 0.5, 3, 0.0), ("gnc05_smooth1", 1.0, 5, 0.5),
                                               ("gnc05_smooth05", 0.5, 3, 0.5)])
def test_level_solver_gnc(oracle, golden_dir, name, a_s, lag, beta):
    g = load(golden_dir, "solver")
    r = oracle.compute_flow(*g["J"], g["weight"], g["u"], g["v"], 1.7, 2.3, 23, lag, np.array([0.45, 0.6]), a_s,
                            1.25, 0.8, gnc_beta=beta)
    np.testing.assert_array_equal(r, g[name])
    # beta = 1 is the plain solver
    plain = oracle.compute_flow(*g["J"], g["weight"], g["u"], g["v"], 1.7, 2.3, 23, lag, np.array([0.45, 0.6]),
                                a_s, 1.25, 0.8)
    np.testing.assert_array_equal(oracle.compute_flow(*g["J"], g["weight"], g["u"], g["v"], 1.7, 2.3, 23, lag,
                                                      np.array([0.45, 0.6]), a_s, 1.25, 0.8, gnc_beta=1.0), plain)


def test_full_displacement(oracle, golden_dir):
    f = load(golden_dir, "full")
    a = oracle.get_displacement(f["a_fixed"], f["a_moving"], alpha=(1.5, 1.5), semantics="python")
    np.testing.assert_array_equal(a, f["a_flow"])
    b = oracle.get_displacement(f["b_fixed"], f["b_moving"], alpha=(1.5, 1.5), uv=f["b_uv"], weight=f["b_weight"],
                                iterations=20, update_lag=4, semantics="python")
    np.testing.assert_array_equal(b, f["b_flow"])
    c = oracle.get_displacement(f["b_fixed"], f["b_moving"], alpha=(2.0, 1.0), a_smooth=0.7,
                                weight=np.array([0.8, 0.2]), iterations=15, semantics="python")
    np.testing.assert_array_equal(c, f["c_flow"])
    d = oracle.get_displacement(f["b_fixed"], f["b_moving"], const_assumption="gray", iterations=12, eta=0.7,
                                semantics="python")
    np.testing.assert_array_equal(d, f["d_flow"])
    e = oracle.get_displacement(f["b_fixed"], f["b_moving"], alpha=(1.5, 1.5), min_level=2, iterations=10,
                                semantics="python")
    np.testing.assert_array_equal(e, f["e_flow"])
    cs = oracle.get_displacement(f["b_fixed"], f["b_moving"], const_assumption="cs", iterations=12, semantics="python")
    np.testing.assert_array_equal(cs, f["f_flow"])
    # graduated non-convexity: three stages, two warping steps per level
    gnc = oracle.get_displacement(f["b_fixed"], f["b_moving"], alpha=(1.5, 1.5), gnc_schedule=(0.0, 0.5, 1.0),
                                  warping_steps=2, iterations=6, a_smooth=0.7, semantics="python")
    np.testing.assert_array_equal(gnc, f["g_flow"])
    an = oracle.get_displacement(f["a_fixed"], f["a_moving"], alpha=(1.5, 1.5), semantics="numba")
    assert np.abs(an - f["a_flow"]).max() < 1e-4


def test_known_answer_gc_tensor(oracle):
    """tests/core/test_optical_flow.py:529-551 of the reference: f = 1e-3 x^2 on
    a grid with hx = 2 gives J11 = 0.8 at interior pixels, zero temporal terms."""
    hy, hx = 1.0, 2.0
    H, W = 17, 23
    x = np.arange(W, dtype=np.float64) * hx
    f = np.tile(1e-3 * x**2, (H, 1))
    J11, J22, J33, J12, J13, J23 = oracle.motion_tensor(f, f, hy, hx)
    c = (H // 2, W // 2)
    np.testing.assert_allclose(J11[c], 0.8, atol=0.01)
    np.testing.assert_allclose(J33[c], 0.0, atol=1e-12)
    np.testing.assert_allclose(J13[c], 0.0, atol=1e-12)


def test_schedule_matches_reference_level_counts(oracle):
    """Level counts of the pyramid schedule (16 levels at 256^2, 19 at 512^2)."""
    assert len(oracle.level_schedule(256, 256, 100, 0.8, 0)[0]) == 16
    assert len(oracle.level_schedule(512, 512, 100, 0.8, 0)[0]) == 19
    assert len(oracle.level_schedule(1024, 1024, 100, 0.8, 0)[0]) == 22


def test_native_timed_build_returns_the_checkers_bits(oracle):
    """The CPU baseline is timed on the -O3 -march=native build; it has the
    checker's float semantics (no contraction, no fast-math), so its flows are
    bit-identical to the portable build's."""
    from pyflowreg_gb300.synthetic import pair_256

    fixed, moving, _ = pair_256(5, h=48, w=40)
    kw = dict(alpha=(1.5, 1.5), iterations=12, update_lag=5, weight=None)
    mv = np.stack([moving, moving[::-1]]).astype(np.float64)
    a = oracle.get_displacement_batch(fixed, mv, n_threads=2, **kw)
    b = oracle.get_displacement_batch(fixed, mv, n_threads=2, variant="native", **kw)
    np.testing.assert_array_equal(a, b)
    flags = oracle.build_flags()
    assert "-O3" in flags["native"] and "-ffp-contract=off" in flags["native"]
