"""Host-side tap tables of the fused Gauss-cubic resize.

pyflowreg builds these tables on the host with numpy and numba
(util/resize_util.py:68-76, 182-229).  The float32 Gaussian taps come from
numpy's float32 ``exp``, whose last bit differs between CPU builds, and the
variational solver amplifies table differences of one ulp to ~0.1 px in the
final flow.  The plan therefore takes its tables from this module -- the
reference's own construction with numpy on the host that runs it -- instead of
the C++ fallback inside the library.

Typing follows numba's compilation of the reference: float32 taps ``g``,
float64 ``acc``/``ssum``/``inv``, float32 stores.
"""

from __future__ import annotations

import functools

import numpy as np

_A = -0.75


def _cubic(x: np.ndarray) -> np.ndarray:
    """Keys cubic, A = -0.75 (util/resize_util.py:68-76), float64."""
    ax = np.abs(x)
    inner = (_A + 2.0) * np.power(ax, 3.0) - (_A + 3.0) * (ax * ax) + 1.0
    outer = _A * np.power(ax, 3.0) - 5.0 * _A * (ax * ax) + 8.0 * _A * ax - 4.0 * _A
    return np.where(ax < 1.0, inner, np.where(ax < 2.0, outer, 0.0))


def _reflect(j: np.ndarray, n: int) -> np.ndarray:
    """_reflect_idx (util/resize_util.py:182-191) on an index array."""
    if n <= 1:
        return np.zeros_like(j)
    j = j.copy()
    while True:
        lo = j < 0
        if not (lo.any() or (j >= n).any()):
            return j
        j = np.where(lo, -j - 1, j)
        j = np.where(j >= n, 2 * n - 1 - j, j)


def sigma_for(in_hw, out_hw, sigma_coeff: float = 0.6) -> float:
    """sigma of imresize_fused_gauss_cubic (util/resize_util.py:235-242)."""
    sy = int(out_hw[0]) / int(in_hw[0])
    sx = int(out_hw[1]) / int(in_hw[1])
    s = sy if sy < sx else sx
    return (sigma_coeff / s) if s < 1.0 else 0.0


@functools.lru_cache(maxsize=1024)
def resize_tables(in_len: int, out_len: int, sigma: float):
    """(idx int32 (out_len, P), wt float32 (out_len, P)) for one axis
    (_precompute_fused_gauss_cubic, util/resize_util.py:216-229).  Arguments are
    taken as Python int/float, as the reference passes them."""
    in_len, out_len, sigma = int(in_len), int(out_len), float(sigma)
    scale = out_len / in_len
    if sigma <= 0.0:
        R = 0
        g = np.array([1.0], dtype=np.float32)
    else:
        R = int(np.ceil(2.0 * sigma))
        xs = np.arange(-R, R + 1, dtype=np.float32)
        g = np.exp(-0.5 * (xs / sigma) ** 2).astype(np.float32)
        g /= g.sum()
    P = 2 * R + 4
    x = (np.arange(out_len, dtype=np.float64) + 0.5) / scale - 0.5
    left = np.floor(x - 2.0).astype(np.int64) - R
    j = left[:, None] + np.arange(P)[None, :]
    idx = np.ascontiguousarray(_reflect(j, in_len).astype(np.int32))
    d = x[:, None] - j.astype(np.float64)
    acc = np.zeros((out_len, P), dtype=np.float64)
    for u in range(-R, R + 1):
        acc = acc + np.float64(g[u + R]) * _cubic(d - u)
    wt32 = acc.astype(np.float32)
    ssum = np.zeros(out_len, dtype=np.float64)
    for p in range(P):
        ssum = ssum + acc[:, p]
    wt = np.ascontiguousarray((wt32.astype(np.float64) * (1.0 / ssum)[:, None]).astype(np.float32))
    idx.setflags(write=False)
    wt.setflags(write=False)
    return idx, wt


def level_tables(in_hw, out_hw):
    """Tables (ix, wx, iy, wy) resizing an in_hw image to out_hw."""
    sig = sigma_for(in_hw, out_hw)
    ix, wx = resize_tables(in_hw[1], out_hw[1], sig)
    iy, wy = resize_tables(in_hw[0], out_hw[0], sig)
    return ix, wx, iy, wy
