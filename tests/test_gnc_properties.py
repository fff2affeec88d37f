"""Stage-weight properties of compute_flow_gnc (core/level_solver.py:372-555),
the cases of the reference's tests/core/test_level_solver_gnc.py:63-106:
the data weights change only on a psi tick; beta orders the one-pixel
response; exponents of 1 ignore beta; a sublinear smoothness exponent does
not.  Checked on the oracle (CPU) and on the float64 GPU seam."""
import numpy as np
import pytest


def one_pixel_data_case(a_data=0.45):
    """3x3 padded level, one interior pixel with J11 = 1, J13 = -1, J33 = 4."""
    J = np.zeros((6, 3, 3, 1))
    J[0, 1, 1, 0] = 1.0   # J11
    J[2, 1, 1, 0] = 4.0   # J33
    J[4, 1, 1, 0] = -1.0  # J13
    return dict(J=J, weight=np.ones((3, 3, 1)), u=np.zeros((3, 3)), v=np.zeros((3, 3)), a_data=a_data,
                a_smooth=1.0)


def bump_smoothness_case(a_smooth):
    """5x5 padded level with no data term and a unit bump in u."""
    u = np.zeros((5, 5))
    u[2, 2] = 1.0
    return dict(J=np.zeros((6, 5, 5, 1)), weight=np.ones((5, 5, 1)), u=u, v=np.zeros((5, 5)), a_data=1.0,
                a_smooth=a_smooth)


def _oracle_solve(case, lag, beta):
    from oracle import oracle as O

    O.build()
    return O.compute_flow(*case["J"], case["weight"], case["u"], case["v"], 1.0, 1.0, 1, lag,
                          np.array([case["a_data"]]), case["a_smooth"], 1.0, 1.0, gnc_beta=beta)


def _gpu_solve(case, lag, beta):
    import pyflowreg_gb300 as G

    du, dv = G.level_solver(*case["J"], case["weight"], case["u"], case["v"], (1.0, 1.0), 1, lag, 0,
                            np.array([case["a_data"]]), case["a_smooth"], 1.0, 1.0, gnc_beta=beta, precision="fp64")
    return np.stack([du, dv], axis=2)


SOLVERS = [pytest.param(_oracle_solve, id="oracle"), pytest.param(_gpu_solve, id="gpu", marks=pytest.mark.gpu)]


@pytest.mark.parametrize("solve", SOLVERS)
def test_data_weights_follow_the_tick_and_beta_orders_the_response(solve):
    case = one_pixel_data_case()
    # update_lag 2 with one iteration: no tick, psi = 1 whatever beta
    np.testing.assert_allclose(solve(case, 2, 0.0), solve(case, 2, 1.0))
    # a tick in the first iteration: the quadratic stage pulls hardest
    q, mid, r = (solve(case, 1, b)[1, 1, 0] for b in (0.0, 0.5, 1.0))
    assert q > mid > r


@pytest.mark.parametrize("solve", SOLVERS)
def test_quadratic_data_exponent_ignores_beta(solve):
    case = one_pixel_data_case(a_data=1.0)
    np.testing.assert_allclose(solve(case, 1, 0.0), solve(case, 1, 1.0))


@pytest.mark.parametrize("solve", SOLVERS)
def test_smoothness_weights_blend_only_when_sublinear(solve):
    assert not np.allclose(solve(bump_smoothness_case(0.5), 1, 0.0), solve(bump_smoothness_case(0.5), 1, 1.0))
    np.testing.assert_allclose(solve(bump_smoothness_case(1.0), 1, 0.0), solve(bump_smoothness_case(1.0), 1, 1.0))


@pytest.mark.gpu
@pytest.mark.parametrize("lag,beta,a_s", [(1, 0.0, 1.0), (1, 0.5, 1.0), (2, 1.0, 1.0), (1, 0.0, 0.5), (1, 0.7, 0.5)])
def test_gpu_equals_oracle_on_the_small_cases(lag, beta, a_s):
    for case in (one_pixel_data_case(), bump_smoothness_case(a_s)):
        np.testing.assert_allclose(_gpu_solve(case, lag, beta), _oracle_solve(case, lag, beta), rtol=0, atol=1e-12)
