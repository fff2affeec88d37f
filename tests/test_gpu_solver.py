"""The exact-order wavefront SOR against the oracle's lexicographic
compute_flow (core/level_solver.py:158-369) on identical inputs."""
import numpy as np
import pytest

import pyflowreg_gb300 as G

pytestmark = pytest.mark.gpu


def level_inputs(rng, h, w, K, oracle):
    from pyflowreg_gb300.synthetic import Blobs

    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    J = np.zeros((6, h + 2, w + 2, K))
    for k in range(K):
        f1 = Blobs(rng, h, w, n=max(4, h * w // 200))(yy, xx)
        f2 = Blobs(rng, h, w, n=max(4, h * w // 200))(yy, xx) * 0.2 + f1 * 0.8
        f1 = f1.astype(np.float32).astype(np.float64)
        f2 = f2.astype(np.float32).astype(np.float64)
        for q, a in enumerate(oracle.motion_tensor(f1, f2, 1.1, 0.9)):
            J[q, :, :, k] = a
    J = J.astype(np.float32).astype(np.float64)
    wgt = np.zeros((h + 2, w + 2, K))
    wgt[1:-1, 1:-1, :] = rng.uniform(0.2, 1.0, K)
    u = np.pad(rng.standard_normal((h, w)) * 0.5, 1, mode="edge").astype(np.float32).astype(np.float64)
    v = np.pad(rng.standard_normal((h, w)) * 0.5, 1, mode="edge").astype(np.float32).astype(np.float64)
    return J, wgt, u, v


@pytest.mark.parametrize("h,w,K,its,lag", [
    (9, 9, 1, 50, 5), (21, 17, 2, 23, 3), (40, 64, 1, 50, 5), (64, 40, 2, 50, 5), (33, 35, 1, 12, 1),
    (50, 70, 2, 30, 7), (100, 120, 1, 50, 5), (250, 300, 2, 50, 5), (512, 512, 1, 10, 5),
    (30, 40, 4, 20, 5), (30, 40, 5, 20, 5), (45, 38, 6, 17, 7), (64, 64, 3, 24, 12),
    # taller than 512 rows: 1024-thread ring with shorter passes, then the global-memory wavefront
    (600, 80, 2, 20, 5), (900, 60, 1, 23, 5), (1030, 50, 2, 12, 5), (700, 30, 6, 10, 5),
])
def test_level_solve_matches_lexicographic_oracle(oracle, h, w, K, its, lag):
    rng = np.random.default_rng(h * 7 + w)
    J, wgt, u, v = level_inputs(rng, h, w, K, oracle)
    a_data = np.linspace(0.45, 0.6, K)
    ref = oracle.compute_flow(*J, wgt, u, v, 1.7, 2.3, its, lag, a_data, 1.0, 1.25, 0.8)
    du, dv = G.level_solver(*J, wgt, u, v, (1.7, 2.3), its, lag, 0, a_data, 1.0, 1.25, 0.8, precision="fp32")
    got = np.stack([du, dv], axis=2)
    err = np.abs(got[1:-1, 1:-1] - ref[1:-1, 1:-1]).max()
    scale = np.abs(ref).max()
    assert err <= 2e-4 * max(scale, 1.0), (err, scale)


def test_red_black_order_is_not_the_reference(oracle):
    """Guard for the design choice: a red-black sweep does not reproduce the
    lexicographic result the reference computes, the GPU result does."""
    rng = np.random.default_rng(3)
    J, wgt, u, v = level_inputs(rng, 48, 56, 1, oracle)
    a = np.array([0.45])
    lex = oracle.compute_flow(*J, wgt, u, v, 1.5, 1.5, 50, 5, a, 1.0, 1.0, 1.0)
    rb = oracle.compute_flow(*J, wgt, u, v, 1.5, 1.5, 50, 5, a, 1.0, 1.0, 1.0, order=oracle.ORDER_RED_BLACK)
    du, dv = G.level_solver(*J, wgt, u, v, (1.5, 1.5), 50, 5, 0, a, 1.0, 1.0, 1.0, precision="fp32")
    gpu = np.stack([du, dv], axis=2)
    e_gpu = np.abs(gpu - lex)[1:-1, 1:-1].max()
    e_rb = np.abs(rb - lex)[1:-1, 1:-1].max()
    assert e_gpu < 1e-4 < e_rb


@pytest.mark.parametrize("name,a_s,lag,beta", [("smooth1", 1.0, 5, None), ("smooth05", 0.5, 3, None),
                                               ("gnc0_smooth05", 0.5, 3, 0.0), ("gnc05_smooth1", 1.0, 5, 0.5),
                                               ("gnc05_smooth05", 0.5, 3, 0.5)])
def test_level_solve_f64_golden(golden_dir, name, a_s, lag, beta):
    """The float64 seam (compute_flow / compute_flow_gnc) against the
    reference's own solver output, rings included."""
    g = np.load(f"{golden_dir}/solver.npz")
    du, dv = G.level_solver(*g["J"], g["weight"], g["u"], g["v"], (1.7, 2.3), 23, lag, 0, np.array([0.45, 0.6]),
                            a_s, 1.25, 0.8, gnc_beta=beta, precision="fp64")
    got = np.stack([du, dv], axis=2)
    assert got.dtype == np.float64
    np.testing.assert_allclose(got, g[name], rtol=0, atol=1e-9)


@pytest.mark.parametrize("h,w,K,its,lag,a_s,beta", [
    (21, 17, 2, 23, 3, 1.0, 0.25), (40, 64, 1, 30, 5, 0.6, 0.75), (64, 40, 3, 17, 1, 0.8, 0.0),
    (33, 35, 1, 12, 4, 1.0, 1.0), (5, 4, 1, 9, 2, 0.7, 0.5),
])
def test_level_solve_f64_gnc_matches_oracle(oracle, h, w, K, its, lag, a_s, beta):
    rng = np.random.default_rng(h * 11 + w)
    J, wgt, u, v = level_inputs(rng, h, w, K, oracle)
    a_data = np.linspace(0.45, 0.6, K)
    ref = oracle.compute_flow(*J, wgt, u, v, 1.7, 2.3, its, lag, a_data, a_s, 1.25, 0.8, gnc_beta=beta)
    du, dv = G.level_solver(*J, wgt, u, v, (1.7, 2.3), its, lag, 0, a_data, a_s, 1.25, 0.8, gnc_beta=beta)
    got = np.stack([du, dv], axis=2)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9 * max(1.0, np.abs(ref).max()))
