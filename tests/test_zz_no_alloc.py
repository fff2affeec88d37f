"""frg_level_solve_noalloc: the level solver for callers that cannot allocate
device memory (inside a CUDA graph capture, or when another framework has
reserved the device memory up front).  It uses a fixed scratch array inside
the library instead of cudaMallocAsync.

The test calls it through the C ABI several times in a row on different
levels and checks each result against frg_level_solve.  Both run the same
kernels on the same inputs, so the results must be equal bit for bit.  The
cases cover the chained SOR (K <= 4) and the fold + row-per-thread SOR
(K = 6), the latter after a larger level has left other data in the shared
scratch array.  This file is collected last so that a failure here leaves
every other test already run.
"""
import ctypes

import numpy as np
import pytest

from pyflowreg_gb300 import _lib

pytestmark = pytest.mark.gpu


def _level(seed, h, w, K):
    """A gray-value-constancy style tensor (positive semi-definite) with weights and flow."""
    rng = np.random.default_rng(seed)
    m, n = h + 2, w + 2
    fx, fy, ft = (rng.standard_normal((3, m, n, K)) * np.array([0.3, 0.3, 0.1])[:, None, None, None])
    J = np.stack([fx * fx, fy * fy, ft * ft, fx * fy, fx * ft, fy * ft]).astype(np.float32)
    J[:, [0, -1], :, :] = 0
    J[:, :, [0, -1], :] = 0
    wgt = np.zeros((m, n, K), np.float32)
    wgt[1:-1, 1:-1, :] = rng.uniform(0.2, 1.0, K)
    u = np.pad(rng.standard_normal((h, w)) * 0.5, 1, mode="edge").astype(np.float32)
    v = np.pad(rng.standard_normal((h, w)) * 0.5, 1, mode="edge").astype(np.float32)
    return J, wgt, u, v


def _solve(fn, J, wgt, u, v, its, lag, a_data):
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    _, m, n, K = J.shape
    Jt, Wt = torch.from_numpy(J).to(dev), torch.from_numpy(wgt).to(dev)
    ut, vt = torch.from_numpy(u).to(dev), torch.from_numpy(v).to(dev)
    du = torch.empty((m, n), dtype=torch.float32, device=dev)
    dv = torch.empty((m, n), dtype=torch.float32, device=dev)
    ad = np.ascontiguousarray(a_data, dtype=np.float64)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = fn(m, n, K, ctypes.c_void_p(Jt.data_ptr()), ctypes.c_void_p(Wt.data_ptr()), ctypes.c_void_p(ut.data_ptr()),
            ctypes.c_void_p(vt.data_ptr()), 1.7, 2.3, its, lag, ad.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            1.0, 1.25, 0.8, 1.95, ctypes.c_void_p(du.data_ptr()), ctypes.c_void_p(dv.data_ptr()), stream)
    _lib.check(rc, "level solve")
    torch.cuda.synchronize()
    return np.stack([du.cpu().numpy(), dv.cpu().numpy()], axis=2).astype(np.float64)


def test_noalloc_matches_allocating_entry_point_calls_in_a_row():
    lib = _lib.load()
    assert lib.frg_level_solve_noalloc_capacity() == 8 << 20
    # (seed, h, w, K, iterations, update_lag): chained SOR, chained SOR with
    # split groups, then K = 6 (fold kernel + row SOR) after the larger level
    cases = [(101, 96, 120, 2, 50, 5), (102, 63, 41, 1, 23, 3), (104, 40, 50, 6, 20, 5)]
    for seed, h, w, K, its, lag in cases:
        J, wgt, u, v = _level(seed, h, w, K)
        a_data = np.linspace(0.45, 0.6, K)
        ref = _solve(lib.frg_level_solve, J, wgt, u, v, its, lag, a_data)
        got = _solve(lib.frg_level_solve_noalloc, J, wgt, u, v, its, lag, a_data)
        assert np.isfinite(ref).all()
        assert np.array_equal(got, ref), (seed, float(np.abs(got - ref).max()))


def test_noalloc_rejects_levels_beyond_its_scratch():
    lib = _lib.load()
    J, wgt, u, v = _level(103, 300, 300, 2)
    with pytest.raises(ValueError, match="8 MiB"):
        _solve(lib.frg_level_solve_noalloc, J, wgt, u, v, 5, 5, np.array([0.45, 0.45]))
