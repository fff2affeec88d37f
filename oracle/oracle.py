"""CPU oracle for pyflowreg's variational optical-flow path -- TEST INFRASTRUCTURE.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker or the timed CPU
baseline; the product (``pyflowreg_gb300``) never does.

It restates, without importing pyflowreg:
  * ``warpingDepth`` and the level schedule   core/warping.py:237-277,
    core/optical_flow.py:497-518, 572-577
  * the fused Gauss-cubic tap tables           util/resize_util.py:68-76, 182-229
  * input normalisation of ``get_displacement`` core/optical_flow.py:842-885
and drives the C restatement in ``flowreg_oracle.c`` (resize passes, cv2-style
warp, motion tensors, level solver, 5x5 median) through ctypes.

Parity pin: ``tests/golden/make_golden.py`` runs pyflowreg's own Python source
(numba/cv2 replaced by the shims in ``oracle/_shims``) and stores its outputs;
``tests/test_oracle_golden.py`` checks this oracle against them.  OpenCV's
``remap`` itself is restated from its documentation (the shim); agreement
with real OpenCV at single-precision rounding level is unpinned.
"""

from __future__ import annotations

import ctypes
import functools
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

ORDER_LEXICOGRAPHIC = 0
ORDER_RED_BLACK = 1


_VARIANTS = {"portable": _LIB_PATH,
             "o3": os.path.join(_HERE, "_build", "liboracle_o3.so"),
             "fastmath": os.path.join(_HERE, "_build", "liboracle_fastmath.so")}
_variant_libs = {}


def build(force: bool = False) -> str:
    """Compile the C oracle (gcc) and return the path of the shared library."""
    src = os.path.join(_HERE, "flowreg_oracle.c")
    script = os.path.join(_HERE, "build_oracle.sh")
    stale = any(not os.path.exists(p) or os.path.getmtime(p) < max(os.path.getmtime(src), os.path.getmtime(script))
                for p in _VARIANTS.values())
    if force or stale:
        subprocess.check_call(["bash", script])
    return _LIB_PATH


def build_flags() -> dict:
    """Compiler and flags of the timed builds ("o3", "fastmath")."""
    build()
    out = {}
    with open(os.path.join(_HERE, "_build", "flags.txt")) as f:
        for line in f:
            k, _, v = line.partition(":")
            out[k.strip()] = v.strip()
    return out


class _Level(ctypes.Structure):
    _fields_ = [
        ("h", ctypes.c_int), ("w", ctypes.c_int),
        ("p_img", ctypes.c_int),
        ("ix_img", ctypes.c_void_p), ("iy_img", ctypes.c_void_p),
        ("wx_img", ctypes.c_void_p), ("wy_img", ctypes.c_void_p),
        ("fh", ctypes.c_int), ("fw", ctypes.c_int),
        ("p_flow", ctypes.c_int),
        ("ix_flow", ctypes.c_void_p), ("iy_flow", ctypes.c_void_p),
        ("wx_flow", ctypes.c_void_p), ("wy_flow", ctypes.c_void_p),
        ("alpha_x", ctypes.c_double), ("alpha_y", ctypes.c_double),
        ("top", ctypes.c_int),
    ]


class _Params(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int), ("update_lag", ctypes.c_int),
        ("a_smooth", ctypes.c_double), ("gray", ctypes.c_int),
        ("order", ctypes.c_int), ("omega", ctypes.c_double),
        ("acc_f32", ctypes.c_int), ("gnc_beta", ctypes.c_double),
        ("warping_steps", ctypes.c_int), ("solver_f32", ctypes.c_int),
    ]


def lib(variant: str = "portable"):
    """The checker ("portable") or one of the timed builds ("o3",
    "fastmath"), see build_oracle.sh."""
    global _lib
    if variant != "portable":
        if variant not in _variant_libs:
            build()
            v = ctypes.CDLL(_VARIANTS[variant])
            _declare(v)
            _variant_libs[variant] = v
        return _variant_libs[variant]
    if _lib is None:
        path = build()
        _lib = ctypes.CDLL(path)
        _declare(_lib)
    return _lib


def _declare(lib_):
    """ctypes signatures of the oracle's C entry points."""
    P = ctypes.c_void_p
    I, D = ctypes.c_int, ctypes.c_double
    lib_.orc_displacement.argtypes = [I, I, I, P, P, P, P, I, P, P, P, P]
    lib_.orc_displacement_gnc.argtypes = [I, I, I, P, P, P, P, I, P, P, P, P]
    lib_.orc_displacement_batch.argtypes = [I, I, I, I, P, P, P, P, I, P, P, P, I, I, P, I]
    lib_.orc_resize_plane.argtypes = [P, I, I, P, I, I, P, P, I, P, P, I, P, I]
    lib_.orc_resize_plane.restype = None
    lib_.orc_warp_plane.argtypes = [P, P, P, P, I, I, I, P]
    lib_.orc_warp_plane.restype = None
    lib_.orc_motion_tensor.argtypes = [P, P, I, I, D, D, I, I, P, P, P, P, P, P]
    lib_.orc_compute_flow.argtypes = [P, P, P, P, P, P, P, P, P, I, I, I, D, D, I, I, P, D,
                                      D, D, I, D, D, P, P]
    lib_.orc_compute_flow_f32.argtypes = [P, P, P, P, P, P, P, P, P, I, I, I, D, D, I, I, P, D, D, D, P, P]
    lib_.orc_median5_plane.argtypes = [P, I, I, P]
    lib_.orc_median5_plane.restype = None
    lib_.orc_cubic_table.argtypes = [P]
    lib_.orc_cubic_table.restype = None


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


# --------------------------------------------------------------------------
# Schedule: core/warping.py:237-277 and core/optical_flow.py:494-518, 572-577
# --------------------------------------------------------------------------
def warping_depth(eta: float, levels: int, m: int, n: int) -> int:
    min_dim = min(m, n)
    depth = 0
    for _ in range(levels):
        depth += 1
        min_dim *= eta
        if round(min_dim) < 10:
            break
    return depth


def level_schedule(m: int, n: int, levels: int, eta: float, min_level: int):
    """Returns (list of (i, (h, w)) from coarse to fine, effective min_level)."""
    max_level_y = warping_depth(eta, levels, m, m)
    max_level_x = warping_depth(eta, levels, n, n)
    max_level = min(max_level_x, max_level_y) * 4
    max_level_y = min(max_level_y, max_level)
    max_level_x = min(max_level_x, max_level)
    top = max(max_level_x, max_level_y)
    if top <= min_level:
        min_level = top - 1
    if min_level < 0:
        min_level = 0
    out = []
    for i in range(top, min_level - 1, -1):
        size = (int(round(m * eta ** (min(i, max_level_y)))),
                int(round(n * eta ** (min(i, max_level_x)))))
        out.append((i, size))
    return out, min_level


# --------------------------------------------------------------------------
# Fused Gauss-cubic tables: util/resize_util.py:68-76, 182-229
# --------------------------------------------------------------------------
_A = -0.75


def _cubic(x: np.ndarray) -> np.ndarray:
    ax = np.abs(x)
    inner = (_A + 2.0) * np.power(ax, 3.0) - (_A + 3.0) * (ax * ax) + 1.0
    outer = _A * np.power(ax, 3.0) - 5.0 * _A * (ax * ax) + 8.0 * _A * ax - 4.0 * _A
    return np.where(ax < 1.0, inner, np.where(ax < 2.0, outer, 0.0))


def _reflect_idx(j: np.ndarray, n: int) -> np.ndarray:
    if n <= 1:
        return np.zeros_like(j)
    j = j.copy()
    while True:
        lo, hi = j < 0, j >= n
        if not (lo.any() or hi.any()):
            return j
        j = np.where(lo, -j - 1, j)
        j = np.where(j >= n, 2 * n - 1 - j, j)


@functools.lru_cache(maxsize=512)
def resize_tables(in_len: int, out_len: int, sigma: float, semantics: str = "numba"):
    """(idx int32 (out_len, P), wt float32 (out_len, P)) as the reference builds them.

    semantics="numba": the typing numba gives util/resize_util.py:194-213
    (float64 ``acc``/``ssum``/``inv``, float32 stores).  semantics="python":
    the same source run as plain Python under numpy 2 promotion, where
    ``float32 * python_float`` and ``python_float + float32`` stay float32.
    Arguments are coerced to Python int/float: under numpy 2 promotion a
    numpy-typed sigma would change the float32 Gaussian taps.
    """
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
    i = np.arange(out_len, dtype=np.float64)
    x = (i + 0.5) / scale - 0.5
    left = np.floor(x - 2.0).astype(np.int64) - R
    j = left[:, None] + np.arange(P)[None, :]
    idx = _reflect_idx(j, in_len).astype(np.int32)
    d = x[:, None] - j.astype(np.float64)
    if semantics == "numba":
        acc = np.zeros((out_len, P), dtype=np.float64)
        for uu in range(-R, R + 1):
            acc = acc + np.float64(g[uu + R]) * _cubic(d - uu)
        wt32 = acc.astype(np.float32)
        ssum = np.zeros(out_len, dtype=np.float64)
        for p in range(P):
            ssum = ssum + acc[:, p]
        inv = 1.0 / ssum
        wt = (wt32.astype(np.float64) * inv[:, None]).astype(np.float32)
    elif semantics == "python":
        acc = np.zeros((out_len, P), dtype=np.float32)
        for uu in range(-R, R + 1):
            acc = (acc + (g[uu + R] * _cubic(d - uu).astype(np.float32))).astype(np.float32)
        ssum = np.zeros(out_len, dtype=np.float32)
        for p in range(P):
            ssum = (ssum + acc[:, p]).astype(np.float32)
        inv = (np.float32(1.0) / ssum).astype(np.float32)
        wt = (acc * inv[:, None]).astype(np.float32)
    else:
        raise ValueError(semantics)
    idx.setflags(write=False)
    wt.setflags(write=False)
    return idx, wt


def sigma_for(in_hw, out_hw, sigma_coeff: float = 0.6) -> float:
    sy = int(out_hw[0]) / int(in_hw[0])
    sx = int(out_hw[1]) / int(in_hw[1])
    s = sy if sy < sx else sx
    return (sigma_coeff / s) if s < 1.0 else 0.0


def resize(img: np.ndarray, size, semantics: str = "numba") -> np.ndarray:
    """imresize_fused_gauss_cubic (util/resize_util.py:232-254) via the C passes."""
    oh, ow = int(size[0]), int(size[1])
    x = np.asarray(img).astype(np.float32, copy=False)
    sig = sigma_for(x.shape[:2], (oh, ow))
    ix, wx = resize_tables(x.shape[1], ow, sig, semantics)
    iy, wy = resize_tables(x.shape[0], oh, sig, semantics)
    L = lib()
    planes = [x] if x.ndim == 2 else [x[:, :, k] for k in range(x.shape[2])]
    outs = []
    for pl in planes:
        pl = np.ascontiguousarray(pl, dtype=np.float32)
        out = np.empty((oh, ow), np.float32)
        tmp = np.empty((pl.shape[0], ow), np.float32)
        L.orc_resize_plane(_p(pl), pl.shape[0], pl.shape[1], _p(out), oh, ow, _p(ix), _p(wx),
                           ix.shape[1], _p(iy), _p(wy), iy.shape[1], _p(tmp),
                           1 if semantics == "python" else 0)
        outs.append(out)
    y = outs[0] if x.ndim == 2 else np.stack(outs, axis=2)
    return y.astype(np.asarray(img).dtype, copy=False)


def warp(f2: np.ndarray, u: np.ndarray, v: np.ndarray, f1: np.ndarray, cubic: bool = True) -> np.ndarray:
    """imregister_wrapper (core/warping.py:160-234) for (H, W) or (H, W, C) inputs."""
    f2 = np.asarray(f2, dtype=np.float64)
    f1 = np.asarray(f1, dtype=np.float64)
    squeeze = f2.ndim == 2
    if squeeze:
        f2, f1 = f2[:, :, None], f1[:, :, None]
    H, W, C = f2.shape
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    out = np.empty((H, W, C), np.float32)
    L = lib()
    for c in range(C):
        a = np.ascontiguousarray(f2[:, :, c])
        b = np.ascontiguousarray(f1[:, :, c])
        o = np.empty((H, W), np.float32)
        L.orc_warp_plane(_p(a), _p(b), _p(u), _p(v), H, W, 1 if cubic else 0, _p(o))
        out[:, :, c] = o
    return out[:, :, 0] if squeeze and C == 1 else out


def _const_mode(const_assumption) -> int:
    """0 gradient constancy, 1 gray value, 2 census (core/optical_flow.py:466-473)."""
    key = str(getattr(const_assumption, "value", const_assumption)).strip().lower()
    modes = {"gc": 0, "gradient": 0, "gray": 1, "brightness": 1, "cs": 2, "census": 2}
    if key not in modes:
        raise ValueError(f"oracle: unsupported constancy assumption '{const_assumption}'")
    return modes[key]


def motion_tensor(f1, f2, hy, hx, f2_is_f32=False, gray=False):
    """get_motion_tensor_gc / _gray / _cs (core/optical_flow.py:73-345) on one channel;
    gray: False/0 gradient constancy, True/1 gray value, 2 census."""
    f1 = np.ascontiguousarray(f1, dtype=np.float64)
    f2 = np.ascontiguousarray(f2, dtype=np.float64)
    h, w = f1.shape
    J = [np.empty((h + 2, w + 2), np.float64) for _ in range(6)]
    rc = lib().orc_motion_tensor(_p(f1), _p(f2), h, w, float(hy), float(hx), int(f2_is_f32),
                                 int(gray), *[_p(a) for a in J])
    if rc:
        raise MemoryError("oracle motion tensor")
    return tuple(J)


def compute_flow(J11, J22, J33, J12, J13, J23, weight, u, v, alpha_x, alpha_y, iterations,
                 update_lag, a_data, a_smooth, hx, hy, order=ORDER_LEXICOGRAPHIC, omega=1.95,
                 gnc_beta=None):
    """compute_flow (core/level_solver.py:158-369), or compute_flow_gnc
    (core/level_solver.py:372-555) when gnc_beta is given; returns (m, n, 2)."""
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (J11, J22, J33, J12, J13, J23, weight)]
    if arrs[0].ndim == 2:
        arrs = [a[:, :, None] for a in arrs]
    m, n, K = arrs[0].shape
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    ad = np.ascontiguousarray(np.broadcast_to(np.asarray(a_data, dtype=np.float64), (K,)))
    du = np.empty((m, n), np.float64)
    dv = np.empty((m, n), np.float64)
    rc = lib().orc_compute_flow(*[_p(a) for a in arrs], _p(u), _p(v), m, n, K, float(alpha_x),
                                float(alpha_y), int(iterations), int(update_lag), _p(ad),
                                float(a_smooth), float(hx), float(hy), int(order), float(omega),
                                -1.0 if gnc_beta is None else float(gnc_beta), _p(du), _p(dv))
    if rc:
        raise MemoryError("oracle level solver")
    return np.stack([du, dv], axis=2)


def compute_flow_f32(J11, J22, J33, J12, J13, J23, weight, u, v, alpha_x, alpha_y, iterations,
                     update_lag, a_data, hx, hy, omega=1.95):
    """compute_flow (core/level_solver.py:158-369, a_smooth = 1, lexicographic)
    in float32 arithmetic; returns (m, n, 2) float64 holding float32 values."""
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (J11, J22, J33, J12, J13, J23, weight)]
    if arrs[0].ndim == 2:
        arrs = [a[:, :, None] for a in arrs]
    m, n, K = arrs[0].shape
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    ad = np.ascontiguousarray(np.broadcast_to(np.asarray(a_data, dtype=np.float64), (K,)))
    du = np.empty((m, n), np.float64)
    dv = np.empty((m, n), np.float64)
    rc = lib().orc_compute_flow_f32(*[_p(a) for a in arrs], _p(u), _p(v), m, n, K, float(alpha_x),
                                    float(alpha_y), int(iterations), int(update_lag), _p(ad), float(hx),
                                    float(hy), float(omega), _p(du), _p(dv))
    if rc:
        raise MemoryError("oracle level solver")
    return np.stack([du, dv], axis=2)


def median5(a: np.ndarray) -> np.ndarray:
    """scipy.ndimage.median_filter(a, size=(5, 5), mode='mirror')."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    out = np.empty_like(a)
    lib().orc_median5_plane(_p(a), a.shape[0], a.shape[1], _p(out))
    return out


# --------------------------------------------------------------------------
# get_displacement: core/optical_flow.py:476-617, 773-929 (single stage)
# --------------------------------------------------------------------------
def normalize_inputs(fixed, moving, weight, a_data):
    """Input handling of get_displacement (core/optical_flow.py:842-885)."""
    assert fixed.ndim == moving.ndim
    fixed = np.asarray(fixed).astype(np.float64)
    moving = np.asarray(moving).astype(np.float64)
    if fixed.ndim == 3:
        m, n, K = fixed.shape
    else:
        m, n = fixed.shape
        K = 1
        fixed = fixed[:, :, None]
        moving = moving[:, :, None]
    if weight is None:
        weight = np.ones((m, n, K), dtype=np.float64) / K
    else:
        weight = np.asarray(weight).astype(np.float64)
        if weight.ndim < 3:
            if weight.ndim == 1:
                if len(weight) < K:
                    ex = np.full(K, 1.0 / K, dtype=np.float64)
                    ex[: len(weight)] = weight
                    weight = ex
                elif len(weight) > K:
                    weight = weight[:K]
                weight = weight / weight.sum()
                weight = np.ones((m, n, K), dtype=np.float64) * weight.reshape(1, 1, -1)
            else:
                weight = np.ones((m, n, K), dtype=np.float64) * weight[..., None]
    if not isinstance(a_data, np.ndarray):
        a_data_arr = np.full(K, a_data, dtype=np.float64)
    else:
        a_data_arr = a_data
    return fixed, moving, np.ascontiguousarray(weight), np.ascontiguousarray(a_data_arr, dtype=np.float64)


class _Plan:
    """Level structs and the arrays they point to (kept alive together)."""

    def __init__(self, m, n, alpha, levels, eta, min_level, semantics="numba"):
        sched, self.min_level = level_schedule(m, n, levels, eta, min_level)
        self.sched = sched
        self.keep = []
        self.levels = (_Level * len(sched))()
        prev = None
        for li, (i, (h, w)) in enumerate(sched):
            L = self.levels[li]
            L.h, L.w = h, w
            sig = sigma_for((m, n), (h, w))
            ix, wx = resize_tables(n, w, sig, semantics)
            iy, wy = resize_tables(m, h, sig, semantics)
            L.p_img = ix.shape[1]
            L.ix_img, L.wx_img, L.iy_img, L.wy_img = self._ptrs(ix, wx, iy, wy)
            src = (m, n) if prev is None else prev
            sig_f = sigma_for(src, (h, w))
            fix, fwx = resize_tables(src[1], w, sig_f, semantics)
            fiy, fwy = resize_tables(src[0], h, sig_f, semantics)
            L.fh, L.fw = src
            L.p_flow = fix.shape[1]
            L.ix_flow, L.wx_flow, L.iy_flow, L.wy_flow = self._ptrs(fix, fwx, fiy, fwy)
            scale = 1.0 if i == self.min_level else eta ** (-0.5 * i)
            L.alpha_x = scale * alpha[0]
            L.alpha_y = scale * alpha[1]
            L.top = 1 if prev is None else 0
            prev = (h, w)
        self.out_hw = prev

    def _ptrs(self, *arrs):
        out = []
        for a in arrs:
            a = np.ascontiguousarray(a)
            self.keep.append(a)
            out.append(a.ctypes.data)
        return out


def _alpha_pair(alpha):
    if np.isscalar(alpha):
        return (float(alpha), float(alpha))
    alpha = list(alpha)
    return (float(alpha[0]), float(alpha[1] if len(alpha) > 1 else alpha[0]))


def _upsample_final(w, m, n):
    # cv2.resize(w, (n, m), INTER_CUBIC) (core/optical_flow.py:615-616): restated in the shim
    import importlib.util

    spec = importlib.util.spec_from_file_location("_orc_cv2", os.path.join(_HERE, "_shims", "cv2", "__init__.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.resize(w, (n, m), interpolation=mod.INTER_CUBIC)


def gnc_stages(gnc_schedule, warping_steps):
    """normalize_gnc_schedule / normalize_warping_steps (core/optical_flow.py:414-443)
    and the default of 10 steps (core/optical_flow.py:911): (betas or None, steps)."""
    if gnc_schedule is None:
        return None, None
    sched = np.asarray(gnc_schedule, dtype=np.float64)
    if sched.ndim != 1:
        raise ValueError("gnc_schedule must be a 1D sequence of stage weights")
    if sched.size < 2:
        raise ValueError("gnc_schedule must contain at least two stages")
    if np.any(sched < 0.0) or np.any(sched > 1.0):
        raise ValueError("gnc_schedule entries must lie in [0, 1]")
    if not np.all(np.diff(sched) >= 0.0):
        raise ValueError("gnc_schedule must be monotone nondecreasing")
    if not np.isclose(sched[0], 0.0) or not np.isclose(sched[-1], 1.0):
        raise ValueError("gnc_schedule must start at 0.0 and end at 1.0")
    steps = 10 if warping_steps is None else int(warping_steps)
    if steps < 1:
        raise ValueError("warping_steps must be a positive integer")
    return [float(b) for b in sched], steps


def get_displacement(fixed, moving, alpha=(2, 2), update_lag=5, iterations=50, min_level=0,
                     levels=50, eta=0.8, a_smooth=1.0, a_data=0.45, const_assumption="gc",
                     uv=None, weight=None, order=ORDER_LEXICOGRAPHIC, omega=1.95,
                     semantics="numba", gnc_schedule=None, warping_steps=None):
    """Oracle of pyflowreg.core.optical_flow.get_displacement
    (core/optical_flow.py:773-929), GNC stages included (620-770).

    semantics="numba" follows the deployed (numba-compiled) reference;
    "python" reproduces the reference source run without numba (see
    resize_tables), which is what the committed golden vectors hold.
    """
    mode = _const_mode(const_assumption)
    betas, steps = gnc_stages(gnc_schedule, warping_steps)
    fixed, moving, weight, a_data_arr = normalize_inputs(fixed, moving, weight, a_data)
    m, n, K = fixed.shape
    plan = _Plan(m, n, _alpha_pair(alpha), levels, eta, min_level, semantics)
    oh, ow = plan.out_hw
    flow = uv
    for beta in (betas if betas is not None else [None]):
        prm = _Params(int(iterations), int(update_lag), float(a_smooth), mode, int(order), float(omega),
                      1 if semantics == "python" else 0, -1.0 if beta is None else beta,
                      0 if steps is None else steps)
        uvd = None if flow is None else np.ascontiguousarray(np.asarray(flow, dtype=np.float64)[:, :, :2])
        out = np.empty((oh, ow, 2), np.float64)
        fn = lib().orc_displacement if beta is None else lib().orc_displacement_gnc
        rc = fn(m, n, K, _p(np.ascontiguousarray(fixed)), _p(np.ascontiguousarray(moving)),
                _p(weight), None if uvd is None else _p(uvd), len(plan.sched),
                ctypes.byref(plan.levels), _p(a_data_arr), ctypes.byref(prm), _p(out))
        if rc:
            raise RuntimeError(f"oracle failed with status {rc}")
        if plan.min_level > 0:
            out = _upsample_final(out, m, n)
        flow = out
    return flow


def get_displacement_batch(fixed, moving_frames, n_threads=None, alpha=(2, 2), update_lag=5,
                           iterations=50, min_level=0, levels=50, eta=0.8, a_smooth=1.0,
                           a_data=0.45, const_assumption="gc", uv=None, weight=None,
                           order=ORDER_LEXICOGRAPHIC, omega=1.95, variant="portable", solver_f32=False):
    """Many moving frames (T, H, W[, K]) against one fixed frame, OpenMP over
    frames.  variant: "portable" (the checker), or a timed build ("o3",
    "fastmath"; see build_oracle.sh).  solver_f32: every level solve in
    float32 arithmetic (the reference algorithm in single precision, for the
    rounding envelope of a float32 implementation; a_smooth = 1 only)."""
    moving_frames = np.asarray(moving_frames)
    fixed3, m0, weight, a_data_arr = normalize_inputs(fixed, moving_frames[0], weight, a_data)
    m, n, K = fixed3.shape
    T = moving_frames.shape[0]
    mov = np.ascontiguousarray(moving_frames.astype(np.float64).reshape(T, m, n, K))
    plan = _Plan(m, n, _alpha_pair(alpha), levels, eta, min_level)
    prm = _Params(int(iterations), int(update_lag), float(a_smooth), _const_mode(const_assumption),
                  int(order), float(omega), 0, -1.0, 0, 1 if solver_f32 else 0)
    uvd = None if uv is None else np.ascontiguousarray(np.asarray(uv, dtype=np.float64)[:, :, :2])
    oh, ow = plan.out_hw
    out = np.empty((T, oh, ow, 2), np.float64)
    nt = int(n_threads or os.cpu_count() or 1)
    rc = lib(variant).orc_displacement_batch(T, m, n, K, _p(np.ascontiguousarray(fixed3)), _p(mov), _p(weight),
                                      None if uvd is None else _p(uvd), len(plan.sched),
                                      ctypes.byref(plan.levels), _p(a_data_arr), ctypes.byref(prm),
                                      oh, ow, _p(out), nt)
    if rc:
        raise RuntimeError(f"oracle failed with status {rc}")
    if plan.min_level > 0:
        out = np.stack([_upsample_final(o, m, n) for o in out])
    return out
