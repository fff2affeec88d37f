"""Accuracy of the float64 solver's power function (frg_pow_f64), the
nonlinearity psi = a (E + 1e-5)^(a - 1) of core/level_solver.py:247.

The reference evaluates it with the platform's pow, within an ulp of the
exact power.  The solver's power (a table of 2^(e b) c_j^b per exponent with a
binomial series for |b| <= 1, table-driven log2 / exp2 otherwise) must stay
within a few ulp of it over the arguments the solver produces
(E + 1e-5 >= 1e-5), over exponents a - 1 for a in (0, 2] and beyond, plus the
special cases pow handles.
"""
import ctypes

import numpy as np
import pytest

from pyflowreg_gb300 import _lib

pytestmark = pytest.mark.gpu


def _pow_gpu(x, b):
    import torch

    xt = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    out = torch.empty_like(xt)
    rc = _lib.load().frg_pow_f64(xt.numel(), ctypes.c_void_p(xt.data_ptr()), float(b),
                                 ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(0))
    _lib.check(rc, "frg_pow_f64")
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("b", [-0.55, -0.5, -0.3, -0.95, -1.0, 0.0, 0.25, 0.7, 1.0, 1.5, -1.2])
def test_pow_within_a_few_ulp(b):
    rng = np.random.default_rng(11)
    # the solver's range (1e-5 up to large residuals), log-uniform, plus values near
    # powers of two and table boundaries
    x = 10.0 ** rng.uniform(-5, 16, 200_000)
    edges = np.ldexp(1.0 + np.arange(257) / 256.0, rng.integers(-17, 50, 257))
    x = np.concatenate([x, edges, np.nextafter(edges, 0), np.nextafter(edges, np.inf), [1e-5, 1.0, 2.0]])
    got = _pow_gpu(x, b)
    ref = np.power(x, b)
    ulp = np.spacing(np.abs(ref))
    err = np.abs(got - ref) / ulp
    assert err.max() <= 4.0, (b, float(err.max()), float(x[np.argmax(err)]))


def test_pow_special_values_follow_pow():
    x = np.array([0.0, 5e-324, 1e-310, np.inf, np.nan, 1e300, -1.0])
    for b in (-0.55, 0.7):
        got = _pow_gpu(x, b)
        with np.errstate(all="ignore"):
            ref = np.power(x, b)
        assert np.allclose(got, ref, rtol=1e-15, equal_nan=True), (b, got, ref)
