"""Full get_displacement on the GPU against the oracle.

Parity bar (fp64 reference-order mode against the fp64 oracle with numba
typing): max |delta flow| <= 1e-3 px and mean endpoint error <= 1e-4 px.

The fp32 fast path cannot meet that bar against any fp64 run, because the
reference algorithm amplifies rounding: perturbing the input by one float32
ulp moves the oracle's own output by ~0.1 px.  Its test
therefore measures that envelope on the same case -- the oracle re-run on
inputs perturbed at the float32 rounding level -- and requires the fp32
deviation to stay within twice it, and its accuracy against the known
displacement to match the oracle's.
"""
import numpy as np
import pytest

import pyflowreg_gb300 as G
from pyflowreg_gb300.synthetic import Video, pair_256

pytestmark = pytest.mark.gpu

MAX_TOL = 1e-3
EPE_TOL = 1e-4


def flow_diff(got, ref):
    d = np.asarray(got, np.float64) - np.asarray(ref, np.float64)
    return float(np.abs(d).max()), float(np.sqrt((d ** 2).sum(-1)).mean())


def assert_parity(got, ref):
    maxd, epe = flow_diff(got, ref)
    assert maxd <= MAX_TOL and epe <= EPE_TOL, f"max {maxd:.3e} px, mean EPE {epe:.3e} px"


def envelope(oracle, fixed, moving, kw, seeds=(1, 2)):
    """How far the reference's own result moves without any change to its
    algorithm: the oracle on the moving frame perturbed at the float32
    rounding level (1e-7 and 1e-6 relative), and the reference source run as
    plain Python instead of numba (float32 instead of float64 resize
    accumulators).  Returns (numba-typed result, worst max, worst mean EPE)."""
    base = oracle.get_displacement(fixed, moving, **kw)
    worst_max, worst_epe = flow_diff(oracle.get_displacement(fixed, moving, semantics="python", **kw), base)
    for s in seeds:
        for eps in (1e-7, 1e-6):
            rng = np.random.default_rng(s)
            m2 = (np.asarray(moving, np.float64) * (1 + eps * rng.standard_normal(np.shape(moving))))
            mx, ep = flow_diff(oracle.get_displacement(fixed, m2.astype(np.float32), **kw), base)
            worst_max, worst_epe = max(worst_max, mx), max(worst_epe, ep)
    return base, worst_max, worst_epe


# ---------------------------------------------------------------- fp64 parity
def test_fp64_golden_single_channel(oracle, golden_dir):
    f = np.load(f"{golden_dir}/full.npz")
    kw = dict(alpha=(1.5, 1.5))
    got = G.get_displacement(f["a_fixed"], f["a_moving"], precision="fp64", **kw)
    assert got.shape == f["a_flow"].shape and got.dtype == np.float64
    assert_parity(got, oracle.get_displacement(f["a_fixed"], f["a_moving"], **kw))
    # the committed vectors come from the reference source run without numba
    # (float32 resize accumulators); the numba typing differs from them only by
    # that rounding
    assert flow_diff(got, f["a_flow"])[0] < 1e-3


def test_fp64_golden_two_channels_uv_weight(oracle, golden_dir):
    f = np.load(f"{golden_dir}/full.npz")
    kw = dict(alpha=(1.5, 1.5), uv=f["b_uv"], weight=f["b_weight"], iterations=20, update_lag=4)
    got = G.get_displacement(f["b_fixed"], f["b_moving"], precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(f["b_fixed"], f["b_moving"], **kw))


def test_fp64_gray_value_constancy(oracle, golden_dir):
    f = np.load(f"{golden_dir}/full.npz")
    kw = dict(const_assumption="gray", iterations=12, eta=0.7)
    got = G.get_displacement(f["b_fixed"], f["b_moving"], precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(f["b_fixed"], f["b_moving"], **kw))


@pytest.mark.parametrize("a_smooth,lag,its", [(0.7, 4, 20), (0.5, 5, 50), (0.6, 1, 7), (1.3, 3, 11)])
def test_fp64_nonlinear_smoothness(oracle, golden_dir, a_smooth, lag, its):
    """a_smooth != 1 (core/level_solver.py:69-155): psi_s at every tick,
    including its border that lags one iteration behind the interior."""
    f = np.load(f"{golden_dir}/full.npz")
    kw = dict(alpha=(2.0, 1.0), a_smooth=a_smooth, weight=np.array([0.8, 0.2]), update_lag=lag, iterations=its)
    got = G.get_displacement(f["b_fixed"], f["b_moving"], precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(f["b_fixed"], f["b_moving"], **kw))


def test_nonlinear_smoothness_golden_and_fp32_rounding(oracle, golden_dir):
    """The reference's own a_smooth = 0.7 result (golden c_flow); the float32
    API runs the same reference-order kernels and rounds their flow."""
    f = np.load(f"{golden_dir}/full.npz")
    kw = dict(alpha=(2.0, 1.0), a_smooth=0.7, weight=np.array([0.8, 0.2]), iterations=15)
    got = G.get_displacement(f["b_fixed"], f["b_moving"], precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(f["b_fixed"], f["b_moving"], **kw))
    # the committed vector comes from the reference source run without numba
    assert flow_diff(got, f["c_flow"])[0] < 1e-3
    got32 = G.get_displacement(f["b_fixed"], f["b_moving"], precision="fp32", **kw)
    np.testing.assert_array_equal(got32, got.astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("kw", [dict(iterations=12), dict(iterations=30, update_lag=3, a_smooth=0.8),
                                dict(iterations=20, alpha=(2.0, 1.0), weight=np.array([0.8, 0.2]))])
def test_fp64_census(oracle, golden_dir, kw):
    """Census data term (core/optical_flow.py:231-345), float32 arithmetic on
    the warped frame below the top level as numpy does it."""
    f = np.load(f"{golden_dir}/full.npz")
    kw = dict(const_assumption="cs", **kw)
    got = G.get_displacement(f["b_fixed"], f["b_moving"], precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(f["b_fixed"], f["b_moving"], **kw))
    got32 = G.get_displacement(f["b_fixed"], f["b_moving"], precision="fp32", **kw)
    np.testing.assert_array_equal(got32, got.astype(np.float32).astype(np.float64))


def test_census_golden(golden_dir):
    f = np.load(f"{golden_dir}/full.npz")
    got = G.get_displacement(f["b_fixed"], f["b_moving"], const_assumption="cs", iterations=12, precision="fp64")
    # the committed vector comes from the reference source run without numba
    assert flow_diff(got, f["f_flow"])[0] < 1e-3


def test_fp64_pair_256_default_options(oracle):
    """Single 256x256 pair with pyflowreg's default OFOptions flow settings."""
    fixed, moving, _ = pair_256(0)
    kw = dict(alpha=(1.5, 1.5), levels=100, iterations=50, update_lag=5, a_data=0.45, eta=0.8)
    got = G.get_displacement(fixed, moving, precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(fixed, moving, **kw))


@pytest.mark.parametrize("lag,its", [(1, 6), (3, 23), (7, 30)])
def test_fp64_update_lag_and_shapes(oracle, lag, its):
    fixed, moving, truth = pair_256(2, h=72, w=120)
    uv = (truth * 0.7).astype(np.float32)
    kw = dict(alpha=(2.0, 1.0), iterations=its, update_lag=lag, uv=uv)
    got = G.get_displacement(fixed, moving, precision="fp64", **kw)
    assert_parity(got, oracle.get_displacement(fixed, moving, **kw))


@pytest.mark.parametrize("min_level", [2, 4, 6])
def test_fp64_min_level_cubic_upsampling(oracle, golden_dir, min_level):
    """Quality presets 'balanced' (4) and 'fast' (6) stop above full resolution
    and upsample with cv2.resize INTER_CUBIC (core/optical_flow.py:615-616)."""
    fixed, moving, _ = pair_256(5, h=96, w=120)
    kw = dict(alpha=(1.5, 1.5), min_level=min_level, iterations=15)
    ref = oracle.get_displacement(fixed, moving, **kw)
    got = G.get_displacement(fixed, moving, precision="fp64", **kw)
    assert got.shape == (96, 120, 2)
    assert_parity(got, ref)
    if min_level == 2:
        f = np.load(f"{golden_dir}/full.npz")
        kw2 = dict(alpha=(1.5, 1.5), min_level=2, iterations=10)
        g2 = G.get_displacement(f["b_fixed"], f["b_moving"], precision="fp64", **kw2)
        assert flow_diff(g2, f["e_flow"])[0] < 1e-3


def test_fp32_min_level_runs_and_stays_close(oracle):
    fixed, moving, _ = pair_256(5, h=96, w=120)
    kw = dict(alpha=(1.5, 1.5), min_level=4, iterations=15)
    base, env_max, env_epe = envelope(oracle, fixed, moving, kw)
    mx, ep = flow_diff(G.get_displacement(fixed, moving, precision="fp32", **kw), base)
    assert mx <= 2 * env_max + 1e-3 and ep <= 2 * env_epe + 1e-4, (mx, ep, env_max, env_epe)


@pytest.mark.parametrize("h,w", [(700, 96), (1100, 72)])
def test_frames_taller_than_512_rows(oracle, h, w):
    """Levels over 512 rows use the 1024-thread ring (up to 1024 rows) and the
    global-memory wavefront (taller); fp64 parity, fp32 within the envelope."""
    fixed, moving, _ = pair_256(10 + h, h=h, w=w)
    kw = dict(alpha=(1.5, 1.5), iterations=10, levels=100)
    base, env_max, env_epe = envelope(oracle, fixed, moving, kw, seeds=(1,))
    assert_parity(G.get_displacement(fixed, moving, precision="fp64", **kw), base)
    mx, ep = flow_diff(G.get_displacement(fixed, moving, precision="fp32", **kw), base)
    assert mx <= 2 * env_max + 1e-3 and ep <= 2 * env_epe + 1e-4, (mx, ep, env_max, env_epe)


def test_fp64_tall_frame(oracle):
    fixed, moving, _ = pair_256(3, h=160, w=64)
    kw = dict(alpha=(1.5, 1.5), iterations=20)
    assert_parity(G.get_displacement(fixed, moving, precision="fp64", **kw),
                  oracle.get_displacement(fixed, moving, **kw))


@pytest.mark.slow
def test_fp64_video_512x2(oracle):
    vid = Video(seed=1, h=512, w=512, K=2)
    frames, _ = vid.frames(0, 3)
    fixed = frames.mean(axis=0) / frames.max()
    mov = frames / frames.max()
    kw = dict(alpha=(1.5, 1.5), levels=100, weight=np.array([0.5, 0.5]))
    ref = oracle.get_displacement_batch(fixed, mov[:2], **kw)
    got = G.get_displacement_batch(fixed, mov[:2], precision="fp64", **kw)
    for t in range(2):
        assert_parity(got[t], ref[t])


# ---------------------------------------------------------------- fp32 fast path
def test_fp32_pair_256_within_reference_envelope(oracle):
    fixed, moving, truth = pair_256(0)
    kw = dict(alpha=(1.5, 1.5), levels=100)
    base, env_max, env_epe = envelope(oracle, fixed, moving, kw)
    got = G.get_displacement(fixed, moving, precision="fp32", **kw)
    mx, ep = flow_diff(got, base)
    assert mx <= 2 * env_max and ep <= 2 * env_epe, (mx, ep, env_max, env_epe)
    # accuracy against the known displacement matches the oracle's
    core = (slice(16, -16), slice(16, -16))
    e_gpu = np.sqrt(((got - truth) ** 2).sum(-1))[core].mean()
    e_ref = np.sqrt(((base - truth) ** 2).sum(-1))[core].mean()
    assert abs(e_gpu - e_ref) <= 0.02 * e_ref + 2 * env_epe, (e_gpu, e_ref)


def test_fp32_matches_fp64_small(oracle, golden_dir):
    """On small frames the amplification is weak: fp32 stays close."""
    f = np.load(f"{golden_dir}/full.npz")
    kw = dict(alpha=(1.5, 1.5))
    got = G.get_displacement(f["a_fixed"], f["a_moving"], precision="fp32", **kw)
    mx, ep = flow_diff(got, oracle.get_displacement(f["a_fixed"], f["a_moving"], **kw))
    assert mx <= 2e-2 and ep <= 2e-3, (mx, ep)


def test_batch_equals_single_frames():
    fixed, moving, _ = pair_256(1, h=96, w=80)
    frames = np.stack([moving, np.roll(moving, 1, axis=0), np.roll(moving, -2, axis=1)])
    for precision in ("fp32", "fp64"):
        batch = G.get_displacement_batch(fixed, frames, alpha=(1.5, 1.5), precision=precision)
        for t in range(3):
            single = G.get_displacement(fixed, frames[t], alpha=(1.5, 1.5), precision=precision)
            np.testing.assert_array_equal(batch[t], single.astype(batch.dtype))


def test_many_channels_generic_path(oracle):
    """K = 5 runs the generic kernels (separate fold, row-per-thread SOR,
    diagonal-major median); fp64 parity still holds and fp32 stays close."""
    rng = np.random.default_rng(9)
    fixed, moving, _ = pair_256(8, h=48, w=56)
    f5 = np.stack([fixed * (1 + 0.1 * k) for k in range(5)], axis=2)
    m5 = np.stack([moving * (1 + 0.1 * k) for k in range(5)], axis=2) + 0.001 * rng.standard_normal((48, 56, 5))
    kw = dict(alpha=(1.5, 1.5), iterations=20)
    ref, env_max, env_epe = envelope(oracle, f5, m5.astype(np.float32), kw)
    assert_parity(G.get_displacement(f5, m5.astype(np.float32), precision="fp64", **kw), ref)
    mx, ep = flow_diff(G.get_displacement(f5, m5.astype(np.float32), precision="fp32", **kw), ref)
    assert mx <= 2 * env_max and ep <= 2 * env_epe, (mx, ep, env_max, env_epe)


@pytest.mark.parametrize("K", [3, 4])
def test_fp64_three_and_four_channels(oracle, K):
    """K = 3 and 4 run the float64 chained SOR's largest instantiations (their
    fold inputs spill a few registers): parity with the oracle, per-channel
    weights included."""
    rng = np.random.default_rng(10 + K)
    fixed, moving, _ = pair_256(3 + K, h=70, w=58)
    fk = np.stack([fixed * (1 + 0.2 * k) for k in range(K)], axis=2)
    mk = (np.stack([moving * (1 + 0.2 * k) for k in range(K)], axis=2)
          + 0.001 * rng.standard_normal((70, 58, K))).astype(np.float32)
    weight = np.linspace(1.0, 2.0, K)
    kw = dict(alpha=(1.5, 1.5), iterations=25, weight=weight)
    assert_parity(G.get_displacement(fk, mk, precision="fp64", **kw), oracle.get_displacement(fk, mk, **kw))


def test_deterministic():
    fixed, moving, _ = pair_256(6, h=128, w=128)
    a = G.get_displacement(fixed, moving, alpha=(1.5, 1.5))
    b = G.get_displacement(fixed, moving, alpha=(1.5, 1.5))
    np.testing.assert_array_equal(a, b)


def test_caller_level_solver_matches_the_oracle(oracle):
    """get_displacement with a caller-supplied level_solver_backend
    (core/optical_flow.py:579-606): the device pyramid, warp and tensor hand
    the solver the arrays the reference passes -- here the oracle's
    restatement of compute_flow behind the reference's signature -- and the
    flow matches the oracle's own get_displacement.  A solver's exception
    reaches the caller."""
    f1, m1, _ = pair_256(5, h=48, w=56)
    f2, m2, _ = pair_256(6, h=48, w=56)
    fixed, moving = np.stack([f1, f2 * 0.9], axis=2), np.stack([m1, m2 * 0.9], axis=2)
    kw = dict(alpha=(1.5, 2.0), iterations=20)
    shapes = []

    def solver(J11, J22, J33, J12, J13, J23, weight, u, v, alpha, iterations, update_lag, verbose, a_data,
               a_smooth, hx, hy, gnc_beta=None):
        shapes.append((J11.shape, weight.shape, u.shape))
        out = oracle.compute_flow(J11, J22, J33, J12, J13, J23, weight, u, v, alpha[0], alpha[1], iterations,
                                  update_lag, a_data, a_smooth, hx, hy, gnc_beta=gnc_beta)
        return out[..., 0], out[..., 1]

    got = G.get_displacement(fixed, moving, level_solver_backend=solver, **kw)
    want = oracle.get_displacement(fixed, moving, **kw)
    assert shapes and all(j[2] == 2 and w[2] == 2 and len(u) == 2 and j[:2] == u for j, w, u in shapes)
    assert_parity(got, want)

    def bad(*args, **kwargs):
        raise KeyError("solver failed")

    with pytest.raises(KeyError):
        G.get_displacement(fixed, moving, level_solver_backend=bad, **kw)


def test_unsupported_options_raise():
    fixed, moving, _ = pair_256(4, h=32, w=32)
    with pytest.raises(NotImplementedError):
        G.get_displacement(fixed, moving, level_solver_backend=lambda *a, **k: None, precision="fp32")
    with pytest.raises(ValueError):
        G.get_displacement(fixed, moving, const_assumption="nope")
    with pytest.raises(ValueError):
        G.get_displacement(fixed, moving, gnc_schedule=(0.5, 1.0))
