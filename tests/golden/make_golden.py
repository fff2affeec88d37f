"""Generates the golden vectors in tests/golden/*.npz by running pyflowreg's
own Python source on small seeded inputs.

numba, OpenCV and scikit-image are not installed here, so the directory
``oracle/_shims`` supplies stand-ins: an identity ``numba.njit`` (the
reference's loops then run as plain Python), a ``cv2`` subset restated from
OpenCV's documentation, and a ``skimage`` stub that is never called on this
path.  Everything else -- pyramid schedule, resize tables and passes, motion
tensors, level solver, median filter (real scipy), level loop -- is the
reference's own code.

Run it where the reference source is available:

    python tests/golden/make_golden.py <path/to/pyflowreg/src>

The outputs are small (< 100 KB each) and are committed; tests never import
the reference.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_golden.py <path/to/pyflowreg/src>")
REF_SRC = sys.argv[1]


def blobs(rng, h, w, n=12, bg=0.05):
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.full((h, w), bg)
    for _ in range(n):
        cy, cx = rng.uniform(0, h), rng.uniform(0, w)
        s = rng.uniform(1.5, 4.0)
        a = rng.uniform(0.3, 1.0)
        img += a * np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * s * s))
    return img


def smooth_field(rng, h, w, amp):
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    u = np.zeros((h, w))
    v = np.zeros((h, w))
    for _ in range(3):
        k = rng.uniform(0.05, 0.2, size=2)
        ph = rng.uniform(0, 2 * np.pi, size=2)
        u += np.sin(k[0] * yy + k[1] * xx + ph[0])
        v += np.cos(k[1] * yy - k[0] * xx + ph[1])
    s = amp / max(np.abs(u).max(), np.abs(v).max())
    return u * s, v * s


def pair(rng, h, w, K, amp=1.5, noise=0.01):
    """fixed/moving (h, w, K) where moving(x + w(x)) ~ fixed(x), plus noise."""
    u, v = smooth_field(rng, h, w, amp)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    fixed = np.zeros((h, w, K))
    moving = np.zeros((h, w, K))
    for k in range(K):
        f = blobs(rng, h, w)
        fixed[:, :, k] = f + noise * rng.standard_normal((h, w))
        # moving(y, x) = f(y - v, x - u) evaluated by bilinear sampling
        ys = np.clip(yy - v, 0, h - 1.001)
        xs = np.clip(xx - u, 0, w - 1.001)
        y0, x0 = np.floor(ys).astype(int), np.floor(xs).astype(int)
        ty, tx = ys - y0, xs - x0
        g = (f[y0, x0] * (1 - ty) * (1 - tx) + f[y0 + 1, x0] * ty * (1 - tx)
             + f[y0, x0 + 1] * (1 - ty) * tx + f[y0 + 1, x0 + 1] * ty * tx)
        moving[:, :, k] = g + noise * rng.standard_normal((h, w))
    return fixed, moving, np.stack([u, v], axis=2)


def main():
    sys.path[:0] = [os.path.join(REPO, "oracle", "_shims"), REF_SRC]
    from pyflowreg.core import optical_flow as of
    from pyflowreg.core import level_solver as ls
    from pyflowreg.core import warping as wp
    from pyflowreg.util import resize_util as ru

    out = {}

    # 1) resize tables and resize results (util/resize_util.py:216-254)
    rng = np.random.default_rng(11)
    img = rng.random((37, 45)).astype(np.float64)
    cases = [(37, 45, 30, 36), (37, 45, 9, 11), (37, 45, 37, 45), (20, 24, 25, 30), (37, 45, 29, 45)]
    rz = {}
    for q, (ih, iw, oh, ow) in enumerate(cases):
        src = img[:ih, :iw]
        rz[f"in{q}"] = src
        rz[f"out{q}"] = ru.imresize_fused_gauss_cubic(src, (oh, ow))
        sy, sx = oh / ih, ow / iw
        s = min(sy, sx)
        sig = 0.6 / s if s < 1.0 else 0.0
        ix, wx = ru._precompute_fused_gauss_cubic(iw, ow, sig)
        rz[f"ix{q}"], rz[f"wx{q}"] = ix, wx
    rz["cases"] = np.array(cases, dtype=np.int32)
    out["resize"] = rz

    # 2) warp (core/warping.py:160-234), fractional and out-of-bounds shifts
    rng = np.random.default_rng(12)
    f2 = blobs(rng, 31, 27)
    f1 = blobs(rng, 31, 27)
    u, v = smooth_field(rng, 31, 27, 3.0)
    u = u + 0.37
    v = v - 1.61
    out["warp"] = {
        "f2": f2, "f1": f1, "u": u, "v": v,
        "cubic": wp.imregister_wrapper(f2, u, v, f1, "cubic"),
        "linear": wp.imregister_wrapper(f2, u, v, f1, "linear"),
        "f2_3c": np.stack([f2, f1 * 0.5], axis=2), "f1_3c": np.stack([f1, f2 * 0.5], axis=2),
        "cubic_2c": wp.imregister_wrapper(np.stack([f2, f1 * 0.5], axis=2), u, v,
                                          np.stack([f1, f2 * 0.5], axis=2), "cubic"),
    }

    # 3) motion tensors (core/optical_flow.py:73-228)
    rng = np.random.default_rng(13)
    f1 = blobs(rng, 23, 19)
    f2 = blobs(rng, 23, 19)
    mt = {"f1": f1, "f2": f2, "hy": 1.3, "hx": 1.7}
    mt["gc"] = np.stack(of.get_motion_tensor_gc(f1, f2, 1.3, 1.7))
    mt["gc_f32"] = np.stack(of.get_motion_tensor_gc(f1, f2.astype(np.float32), 1.3, 1.7))
    mt["gray"] = np.stack(of.get_motion_tensor_gray(f1, f2, 1.3, 1.7))
    mt["gray_f32"] = np.stack(of.get_motion_tensor_gray(f1, f2.astype(np.float32), 1.3, 1.7))
    # census (core/optical_flow.py:231-345)
    mt["cs"] = np.stack(of.get_motion_tensor_cs(f1, f2, 1.3, 1.7))
    mt["cs_f32"] = np.stack(of.get_motion_tensor_cs(f1, f2.astype(np.float32), 1.3, 1.7))
    out["tensor"] = mt

    # 4) level solver (core/level_solver.py:158-369)
    rng = np.random.default_rng(14)
    h, w, K = 21, 17, 2
    fx, mv, _ = pair(rng, h, w, K)
    Js = [np.zeros((h + 2, w + 2, K)) for _ in range(6)]
    for k in range(K):
        for q, a in enumerate(of.get_motion_tensor_gc(fx[:, :, k], mv[:, :, k], 1.0, 1.0)):
            Js[q][:, :, k] = a
    wgt = np.zeros((h + 2, w + 2, K))
    wgt[1:-1, 1:-1, 0] = 0.7
    wgt[1:-1, 1:-1, 1] = 0.3
    uu = np.pad(rng.standard_normal((h, w)) * 0.3, 1, mode="edge")
    vv = np.pad(rng.standard_normal((h, w)) * 0.3, 1, mode="edge")
    sol = {"J": np.stack(Js), "weight": wgt, "u": uu, "v": vv}
    for name, a_s, lag in (("smooth1", 1.0, 5), ("smooth05", 0.5, 3)):
        res = ls.compute_flow(*[np.ascontiguousarray(a) for a in Js], wgt, uu, vv, 1.7, 2.3, 23, lag,
                              np.array([0.45, 0.6]), a_s, 1.25, 0.8)
        sol[name] = res
    # compute_flow_gnc (core/level_solver.py:372-555): the GNC stage weight mixes psi and psi_s
    for name, a_s, lag, beta in (("gnc0_smooth05", 0.5, 3, 0.0), ("gnc05_smooth1", 1.0, 5, 0.5),
                                 ("gnc05_smooth05", 0.5, 3, 0.5)):
        sol[name] = ls.compute_flow_gnc(*[np.ascontiguousarray(a) for a in Js], wgt, uu, vv, 1.7, 2.3, 23, lag,
                                        np.array([0.45, 0.6]), a_s, 1.25, 0.8, beta)
    out["solver"] = sol

    # 5) full get_displacement (core/optical_flow.py:773-929)
    full = {}
    rng = np.random.default_rng(15)
    fx, mv, truth = pair(rng, 30, 36, 1, amp=2.0)
    full["a_fixed"], full["a_moving"], full["a_truth"] = fx[:, :, 0], mv[:, :, 0], truth
    full["a_flow"] = of.get_displacement(fx[:, :, 0], mv[:, :, 0], alpha=(1.5, 1.5))
    rng = np.random.default_rng(16)
    fx, mv, truth = pair(rng, 34, 28, 2, amp=2.0)
    uv0 = (truth * 0.5).astype(np.float32)
    wgt = np.ones((34, 28, 2))
    wgt[:, :, 0] = 0.5
    wgt[:, :, 1] = 0.5
    full["b_fixed"], full["b_moving"], full["b_uv"], full["b_weight"] = fx, mv, uv0, wgt
    full["b_flow"] = of.get_displacement(fx, mv, alpha=(1.5, 1.5), uv=uv0, weight=wgt, iterations=20,
                                         update_lag=4)
    full["c_flow"] = of.get_displacement(fx, mv, alpha=(2.0, 1.0), a_smooth=0.7, weight=np.array([0.8, 0.2]),
                                         iterations=15)
    full["d_flow"] = of.get_displacement(fx, mv, const_assumption="gray", iterations=12, eta=0.7)
    # min_level > 0: the finest levels are skipped and the flow is upsampled by cv2.resize (cubic)
    full["e_flow"] = of.get_displacement(fx, mv, alpha=(1.5, 1.5), min_level=2, iterations=10)
    # census data term and a graduated non-convexity schedule (core/optical_flow.py:620-770, 887-929)
    full["f_flow"] = of.get_displacement(fx, mv, const_assumption="cs", iterations=12)
    full["g_flow"] = of.get_displacement(fx, mv, alpha=(1.5, 1.5), gnc_schedule=(0.0, 0.5, 1.0), warping_steps=2,
                                         iterations=6, a_smooth=0.7)
    out["full"] = full

    for name, d in out.items():
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in d.items()})
        print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()
