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


def test_o3_timed_build_returns_the_checkers_bits(oracle):
    """The CPU baseline is timed on the -O3 build; it has the
    checker's float semantics (no contraction, no fast-math), so its flows are
    bit-identical to the portable build's."""
    from pyflowreg_gb300.synthetic import pair_256

    fixed, moving, _ = pair_256(5, h=48, w=40)
    kw = dict(alpha=(1.5, 1.5), iterations=12, update_lag=5, weight=None)
    mv = np.stack([moving, moving[::-1]]).astype(np.float64)
    a = oracle.get_displacement_batch(fixed, mv, n_threads=2, **kw)
    b = oracle.get_displacement_batch(fixed, mv, n_threads=2, variant="o3", **kw)
    np.testing.assert_array_equal(a, b)
    flags = oracle.build_flags()
    assert "-O3" in flags["o3"] and "-ffp-contract=off" in flags["o3"]


def _compute_flow_numpy_f32(J, wgt, u, v, ax, ay, iterations, update_lag, a_data, omega):
    """compute_flow (core/level_solver.py:158-369, a_smooth = 1) as the
    reference writes it, loop by loop, on numpy float32 scalars, with the C
    library's powf for the power (numpy's own float32 power may take a SIMD
    routine with other last-bit rounding)."""
    import ctypes
    import ctypes.util

    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    libm.powf.argtypes = [ctypes.c_float, ctypes.c_float]
    libm.powf.restype = ctypes.c_float
    f = np.float32
    J11, J22, J33, J12, J13, J23 = [x.astype(f) for x in J]
    wgt, u, v = wgt.astype(f), u.astype(f), v.astype(f)
    m, n, K = J11.shape
    du = np.zeros((m, n), f)
    dv = np.zeros((m, n), f)
    psi = np.ones((m, n, K), f)
    ax, ay, omega = f(ax), f(ay), f(omega)
    for it in range(iterations):
        if (it + 1) % update_lag == 0:
            for k in range(K):
                ak = f(a_data)
                for i in range(m):
                    for j in range(n):
                        a, b = du[i, j], dv[i, j]
                        val = (J11[i, j, k] * a * a + J22[i, j, k] * b * b + J23[i, j, k] * b
                               + f(2) * J12[i, j, k] * a * b + f(2) * J13[i, j, k] * a + J23[i, j, k] * b
                               + J33[i, j, k])
                        val = max(val, f(0))
                        psi[i, j, k] = ak * f(libm.powf(val + f(0.00001), ak - f(1)))
        for x in (du, dv):
            x[0, :] = x[1, :]
            x[-1, :] = x[-2, :]
            x[:, 0] = x[:, 1]
            x[:, -1] = x[:, -2]
        for j in range(1, n - 1):
            for i in range(1, m - 1):
                num_u = num_v = den_u = den_v = f(0)
                for (ii, jj, t) in ((i, j - 1, ax), (i, j + 1, ax), (i + 1, j, ay), (i - 1, j, ay)):
                    num_u += t * (u[ii, jj] + du[ii, jj] - u[i, j])
                    num_v += t * (v[ii, jj] + dv[ii, jj] - v[i, j])
                    den_u += t
                    den_v += t
                for k in range(K):
                    wp = wgt[i, j, k] * psi[i, j, k]
                    num_u -= wp * (J13[i, j, k] + J12[i, j, k] * dv[i, j])
                    den_u += wp * J11[i, j, k]
                    den_v += wp * J22[i, j, k]
                du_kp1 = num_u / den_u if den_u != 0 else f(0)
                du[i, j] = (f(1) - omega) * du[i, j] + omega * du_kp1
                num_v2 = num_v
                for k in range(K):
                    num_v2 -= wgt[i, j, k] * psi[i, j, k] * (J23[i, j, k] + J12[i, j, k] * du[i, j])
                dv_kp1 = num_v2 / den_v if den_v != 0 else f(0)
                dv[i, j] = (f(1) - omega) * dv[i, j] + omega * dv_kp1
    return np.stack([du, dv], axis=2)


def test_float32_solver_is_the_reference_loop_in_numpy_float32(oracle):
    """The float32 level solver (the rounding envelope of the float32 path)
    equals the reference's loops evaluated on numpy float32 scalars, bit for
    bit, and stays near the float64 solver."""
    rng = np.random.default_rng(11)
    m, n, K = 9, 8, 2
    J = [np.abs(rng.standard_normal((m, n, K))) for _ in range(3)] + \
        [0.3 * rng.standard_normal((m, n, K)) for _ in range(3)]
    wgt = np.full((m, n, K), 0.5)
    u = 0.2 * rng.standard_normal((m, n))
    v = 0.2 * rng.standard_normal((m, n))
    hx, hy = 1.3, 0.9
    ax, ay = 1.5 / (hx * hx), 1.5 / (hy * hy)
    got = oracle.compute_flow_f32(*J, wgt, u, v, 1.5, 1.5, 10, 5, 0.45, hx, hy)
    ref = _compute_flow_numpy_f32(J, wgt, u, v, ax, ay, 10, 5, 0.45, 1.95)
    np.testing.assert_array_equal(got, ref.astype(np.float64))
    f64 = oracle.compute_flow(*J, wgt, u, v, 1.5, 1.5, 10, 5, 0.45, 1.0, hx, hy)
    assert 0 < np.abs(got - f64).max() <= 1e-6 * np.abs(f64).max()
