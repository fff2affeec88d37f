"""Test-infrastructure shim: the subset of OpenCV that pyflowreg's optical-flow
path calls, restated from OpenCV's documented behaviour (OpenCV is absent in
this image and cannot be installed).

Call sites it serves (pyflowreg):
  * ``cv2.remap``          core/warping.py:222-228 (imregister_wrapper)
  * ``cv2.copyMakeBorder`` core/optical_flow.py:566-568, 691-693
  * ``cv2.resize``         core/optical_flow.py:616, 769 (only when min_level > 0)

Documented semantics restated here:
  * ``remap`` with floating-point maps and bilinear/bicubic interpolation
    quantises each map coordinate to a 1/32-pixel grid (``INTER_BITS = 5``):
    ``X = round_half_even(x * 32)``, integer part ``X >> 5`` (floor), fraction
    index ``X & 31``.  Bicubic uses the Keys kernel with ``A = -0.75`` on the
    four taps at distances ``1+t, t, 1-t, 2-t``; the fourth weight is one minus
    the other three.  Weights are single precision; the 2-D weight is the
    single-precision product of the row and column weights.  A float64 source
    is accumulated in double, a float32 source in single precision.
    ``BORDER_REPLICATE`` clamps tap indices into the image,
    ``BORDER_CONSTANT`` reads ``borderValue`` outside it.
  * ``copyMakeBorder`` with ``BORDER_CONSTANT`` pads rows/columns only.
  * ``resize`` with ``INTER_CUBIC``: source coordinate
    ``(d + 0.5) * (src/dst) - 0.5``, Keys ``A = -0.75`` weights, clamped taps.

Only ``tests/golden/make_golden.py`` (fixture generation, run where the
reference source is present) puts this directory on ``sys.path``.  Parity
against real OpenCV at the level of single-precision rounding is unpinned
because OpenCV cannot run here.
"""

import numpy as np

INTER_NEAREST = 0
INTER_LINEAR = 1
INTER_CUBIC = 2
INTER_AREA = 3
INTER_LANCZOS4 = 4
BORDER_CONSTANT = 0
BORDER_REPLICATE = 1
BORDER_REFLECT = 2
BORDER_WRAP = 3
BORDER_REFLECT_101 = 4
BORDER_REFLECT101 = 4
BORDER_DEFAULT = 4
BORDER_TRANSPARENT = 5

_INTER_BITS = 5
_TAB = 1 << _INTER_BITS
_A = np.float32(-0.75)


def _keys_inner(x):
    # |x| < 1 branch, single precision, fixed operation order
    x = np.float32(x)
    return np.float32(
        np.float32(np.float32(np.float32(_A + np.float32(2.0)) * x) - np.float32(_A + np.float32(3.0)))
        * np.float32(x * x)
    ) + np.float32(1.0)


def _keys_outer(x):
    # 1 <= |x| < 2 branch, single precision, fixed operation order
    x = np.float32(x)
    a = _A
    t = np.float32(np.float32(a * x) - np.float32(np.float32(5.0) * a))
    t = np.float32(np.float32(t * x) + np.float32(np.float32(8.0) * a))
    return np.float32(np.float32(t * x) - np.float32(np.float32(4.0) * a))


def cubic_coeffs(t):
    """Four single-precision Keys (A=-0.75) weights for fractional offset t."""
    t = np.float32(t)
    one = np.float32(1.0)
    w0 = np.float32(_keys_outer(one + t))
    w1 = np.float32(_keys_inner(t))
    w2 = np.float32(_keys_inner(one - t))
    w3 = np.float32(np.float32(np.float32(one - w0) - w1) - w2)
    return np.array([w0, w1, w2, w3], dtype=np.float32)


def cubic_table():
    """(32, 4) float32 table of bicubic weights at the 1/32 positions."""
    return np.stack([cubic_coeffs(np.float32(k) / np.float32(_TAB)) for k in range(_TAB)])


def linear_table():
    """(32, 2) float32 table of bilinear weights at the 1/32 positions."""
    t = np.arange(_TAB, dtype=np.float32) / np.float32(_TAB)
    return np.stack([np.float32(1.0) - t, t], axis=1).astype(np.float32)


def _gather(src, yy, xx, border, cval):
    H, W = src.shape
    if border == BORDER_CONSTANT:
        inside = (yy >= 0) & (yy < H) & (xx >= 0) & (xx < W)
        v = src[np.clip(yy, 0, H - 1), np.clip(xx, 0, W - 1)]
        return np.where(inside, v, src.dtype.type(cval))
    return src[np.clip(yy, 0, H - 1), np.clip(xx, 0, W - 1)]


def remap(src, map1, map2, interpolation, borderMode=BORDER_CONSTANT, borderValue=0.0):
    src = np.asarray(src)
    if src.ndim != 2:
        raise NotImplementedError("remap shim supports single-channel 2-D sources")
    if src.dtype not in (np.float32, np.float64):
        src = src.astype(np.float32)
    acc_t = np.float64 if src.dtype == np.float64 else np.float32
    mx = np.asarray(map1, dtype=np.float32)
    my = np.asarray(map2, dtype=np.float32)
    if interpolation == INTER_NEAREST:
        ix = np.rint(mx.astype(np.float64)).astype(np.int64)
        iy = np.rint(my.astype(np.float64)).astype(np.int64)
        return _gather(src, iy, ix, borderMode, borderValue).astype(src.dtype)
    X = np.rint(mx.astype(np.float64) * _TAB).astype(np.int64)
    Y = np.rint(my.astype(np.float64) * _TAB).astype(np.int64)
    ix, fx = X >> _INTER_BITS, X & (_TAB - 1)
    iy, fy = Y >> _INTER_BITS, Y & (_TAB - 1)
    if interpolation == INTER_CUBIC:
        tab, off = cubic_table(), -1
    elif interpolation == INTER_LINEAR:
        tab, off = linear_table(), 0
    else:
        raise NotImplementedError(f"interpolation {interpolation}")
    ntap = tab.shape[1]
    wx = tab[fx]
    wy = tab[fy]
    acc = np.zeros(mx.shape, dtype=acc_t)
    for i in range(ntap):
        for j in range(ntap):
            w2d = (wy[..., i] * wx[..., j]).astype(np.float32)
            s = _gather(src, iy + off + i, ix + off + j, borderMode, borderValue)
            acc = (acc + (s.astype(acc_t) * w2d.astype(acc_t))).astype(acc_t)
    return acc.astype(src.dtype)


def copyMakeBorder(src, top, bottom, left, right, borderType, dst=None, value=0.0):
    src = np.asarray(src)
    pad = [(top, bottom), (left, right)] + [(0, 0)] * (src.ndim - 2)
    if borderType == BORDER_CONSTANT:
        return np.pad(src, pad, mode="constant", constant_values=value)
    if borderType == BORDER_REPLICATE:
        return np.pad(src, pad, mode="edge")
    raise NotImplementedError(f"copyMakeBorder border {borderType}")


def _resize_axis_cubic(a, out_len, axis):
    in_len = a.shape[axis]
    scale = in_len / out_len
    d = np.arange(out_len, dtype=np.float64)
    f = (d + 0.5) * scale - 0.5
    s = np.floor(f).astype(np.int64)
    t = (f - s).astype(np.float32)
    w = np.stack([cubic_coeffs(tt) for tt in t])  # (out_len, 4)
    out = np.zeros(a.shape[:axis] + (out_len,) + a.shape[axis + 1:], dtype=np.float64)
    for k in range(4):
        idx = np.clip(s - 1 + k, 0, in_len - 1)
        taken = np.take(a, idx, axis=axis).astype(np.float64)
        shape = [1] * a.ndim
        shape[axis] = out_len
        out += taken * w[:, k].astype(np.float64).reshape(shape)
    return out


def resize(src, dsize, dst=None, fx=None, fy=None, interpolation=INTER_LINEAR):
    src = np.asarray(src)
    if interpolation != INTER_CUBIC:
        raise NotImplementedError("resize shim supports INTER_CUBIC only")
    out_w, out_h = int(dsize[0]), int(dsize[1])
    tmp = _resize_axis_cubic(src.astype(np.float64), out_w, 1)
    out = _resize_axis_cubic(tmp, out_h, 0)
    return out.astype(src.dtype)


def __getattr__(name):
    def _unavailable(*args, **kwargs):
        raise NotImplementedError(f"cv2.{name} is not provided by the oracle shim")

    return _unavailable
