"""Differentiable CPU oracle (torch, float64) for the differentiable mode -- TEST
INFRASTRUCTURE.

Only the tests may import this module, as the checker; the product never does.

The differentiable mode is pyflowreg's flow path with the reference torch
backend's level solver (``flowreg_torch``; torch/core/level_solver.py:11-199,
registered at core/__init__.py:140-197), with ONE deliberate change: the
per-level warp and the compensation warp interpolate continuously.  The
reference warp rounds map coordinates to 1/32 px (cv2.remap), which makes
the flow piecewise constant in its inputs and its derivative zero; here the
map is used as is with the Keys cubic (A = -0.75, the kernel cv2 documents for
INTER_CUBIC), BORDER_REPLICATE taps and the reference's out-of-bounds rule
(core/warping.py:160-234).  Everything else follows the reference:

  * level schedule and alpha scaling        core/optical_flow.py:497-577
  * Gauss-cubic resize with the reference's tap tables (used in float64)
                                            util/resize_util.py:68-76,182-254
  * gradient-constancy motion tensor        core/optical_flow.py:73-160
  * red-black lagged-psi SOR, torch semantics (eps = 1e-6, psi tick when
    it % update_lag == 0, clamped denominators, both colours read the old
    du/dv of the pixel)                     torch/core/level_solver.py:11-199
  * 5x5 mirror median of du, dv interiors   core/optical_flow.py:607-609

Gradients come from torch autograd, i.e. unrolled through every iteration.
``rbgs_solve`` is pinned to the reference solver by tests/golden/rbgs_torch.npz
(forward values and forward-mode directional derivatives of the reference's
own code); the rest is a restatement checked by finite differences.
"""

from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

from . import oracle as O

A_KEYS = -0.75


# ---------------------------------------------------------------- resize
def resize(x: torch.Tensor, size) -> torch.Tensor:
    """(..., H, W) -> (..., oh, ow): horizontal then vertical pass with the
    reference tap tables (util/resize_util.py:232-254), in float64."""
    H, W = x.shape[-2:]
    oh, ow = int(size[0]), int(size[1])
    sig = O.sigma_for((H, W), (oh, ow))
    ix, wx = O.resize_tables(W, ow, sig)
    iy, wy = O.resize_tables(H, oh, sig)
    ix_t = torch.as_tensor(ix.astype(np.int64))
    iy_t = torch.as_tensor(iy.astype(np.int64))
    wx_t = torch.as_tensor(wx.astype(np.float64))
    wy_t = torch.as_tensor(wy.astype(np.float64))
    t = (x[..., ix_t] * wx_t).sum(-1)                       # (..., H, ow)
    t = t.transpose(-1, -2)                                 # (..., ow, H)
    t = (t[..., iy_t] * wy_t).sum(-1)                       # (..., ow, oh)
    return t.transpose(-1, -2)


# ---------------------------------------------------------------- warp
def keys_weights(t: torch.Tensor):
    """Keys cubic-convolution weights of the taps at offsets -1, 0, 1, 2 for a
    fractional position t in [0, 1) (R. Keys, 1981; A = -0.75)."""
    a = A_KEYS
    s = t + 1.0
    w0 = ((a * s - 5 * a) * s + 8 * a) * s - 4 * a
    w1 = ((a + 2) * t - (a + 3)) * t * t + 1
    r = 1.0 - t
    w2 = ((a + 2) * r - (a + 3)) * r * r + 1
    q = 2.0 - t
    w3 = ((a * q - 5 * a) * q + 8 * a) * q - 4 * a
    return w0, w1, w2, w3


def warp(f2: torch.Tensor, u: torch.Tensor, v: torch.Tensor, f1: torch.Tensor, oob_fill: bool = True) -> torch.Tensor:
    """Continuous backward warp: out(y, x) = f2(y + v, x + u), Keys cubic with
    replicated borders; pixels whose map leaves [0, W) x [0, H) take f1.
    f2, f1: (K, h, w); u, v: (h, w) in pixels of this level.  oob_fill=False
    (oracle-only, for finite-difference checks) keeps the clamped sample."""
    K, h, w = f2.shape
    gy, gx = torch.meshgrid(torch.arange(h, dtype=u.dtype), torch.arange(w, dtype=u.dtype), indexing="ij")
    mx = gx + u
    my = gy + v
    oob = (mx < 0) | (mx >= w) | (my < 0) | (my >= h)
    mxc = mx.clamp(0, w - 1)
    myc = my.clamp(0, h - 1)
    x0 = torch.floor(mxc)
    y0 = torch.floor(myc)
    tx = mxc - x0
    ty = myc - y0
    wxs = keys_weights(tx)
    wys = keys_weights(ty)
    x0i = x0.long()
    y0i = y0.long()
    out = torch.zeros_like(f2)
    flat = f2.reshape(K, h * w)
    for i in range(4):
        yi = (y0i + i - 1).clamp(0, h - 1)
        for j in range(4):
            xj = (x0i + j - 1).clamp(0, w - 1)
            out = out + (wys[i] * wxs[j]) * flat[:, (yi * w + xj).reshape(-1)].reshape(K, h, w)
    return torch.where(oob.unsqueeze(0), f1, out) if oob_fill else out


# ---------------------------------------------------------------- motion tensor
def motion_tensor_gc(f1: torch.Tensor, f2: torch.Tensor, hy: float, hx: float):
    """Gradient-constancy tensor (core/optical_flow.py:73-160) of one channel
    pair (h, w), written through S = (f1 + f2) / 2 and D = f2 - f1: the
    reference's symmetric pads become clamped neighbour indices.  Returns the
    six interior components (h, w) each (the reference's zero ring is implicit)."""
    h, w = f1.shape
    S = 0.5 * (f1 + f2)
    D = f2 - f1
    xm = torch.clamp(torch.arange(w) - 1, 0, w - 1)
    xp = torch.clamp(torch.arange(w) + 1, 0, w - 1)
    ym = torch.clamp(torch.arange(h) - 1, 0, h - 1)
    yp = torch.clamp(torch.arange(h) + 1, 0, h - 1)
    fxx = (S[:, xm] - 2 * S + S[:, xp]) / (hx * hx)
    fyy = (S[ym, :] - 2 * S + S[yp, :]) / (hy * hy)
    FX = (S[:, xp] - S[:, xm]) / (2 * hx)
    fxy = (FX[yp, :] - FX[ym, :]) / (2 * hy)
    fxt = (D[:, xp] - D[:, xm]) / (2 * hx)
    fyt = (D[yp, :] - D[ym, :]) / (2 * hy)
    rx = 1.0 / (fxx * fxx + fxy * fxy + 1e-6)
    ry = 1.0 / (fxy * fxy + fyy * fyy + 1e-6)
    J11 = rx * fxx * fxx + ry * fxy * fxy
    J22 = rx * fxy * fxy + ry * fyy * fyy
    J33 = rx * fxt * fxt + ry * fyt * fyt
    J12 = rx * fxx * fxy + ry * fxy * fyy
    J13 = rx * fxx * fxt + ry * fxy * fyt
    J23 = rx * fxy * fxt + ry * fyy * fyt
    return J11, J22, J33, J12, J13, J23


# ---------------------------------------------------------------- level solver
def _bnd(a: torch.Tensor) -> torch.Tensor:
    """Out-of-place set_boundary_2d: columns, then rows, copied from the inside."""
    a = torch.cat([a[:, 1:2], a[:, 1:-1], a[:, -2:-1]], dim=1)
    return torch.cat([a[1:2, :], a[1:-1, :], a[-2:-1, :]], dim=0)


def rbgs_solve(J11, J22, J33, J12, J13, J23, W, u, v, alpha, iterations, update_lag, a_data,
               hx, hy, omega=1.95, eps=1e-6, pixel_order="torch", psi_grad=True):
    """The reference torch solver (torch/core/level_solver.py:11-199, a_smooth
    = 1, no GNC) written without in-place updates so autograd can unroll it.
    J*, W: (m, n, K); u, v: (m, n) padded; alpha: 2-element tensor.

    pixel_order="torch": du and dv of a moving pixel both from the old values
    (the reference torch backend).  "gauss_seidel": dv from the new du, the
    within-pixel order of the numba solver (core/level_solver.py:355-364).
    psi_grad=False holds psi fixed for autograd (the lagged adjoint)."""
    m, n, K = J11.shape
    du = torch.zeros_like(u)
    dv = torch.zeros_like(v)
    ax = alpha[0] / (hx * hx)
    ay = alpha[1] / (hy * hy)
    A = torch.as_tensor(a_data, dtype=J11.dtype).reshape(1, 1, -1)
    ii = torch.arange(1, m - 1).view(-1, 1)
    jj = torch.arange(1, n - 1).view(1, -1)
    red = ((ii + jj) % 2 == 0)
    psi = None
    den_ud = den_vd = None
    for it in range(iterations):
        if it % update_lag == 0:
            d3, e3 = du.unsqueeze(-1), dv.unsqueeze(-1)
            E = (J11 * (d3 * d3) + J22 * (e3 * e3) + 2 * J12 * (d3 * e3) + 2 * J13 * d3 + 2 * J23 * e3
                 + J33)
            E = E.clamp_min(0)
            if not psi_grad:
                E = E.detach()
            psi = A * (E + eps) ** (A - 1)
            den_ud = torch.maximum(torch.sum(W * psi * J11, dim=2), torch.as_tensor(eps, dtype=u.dtype))
            den_vd = torch.maximum(torch.sum(W * psi * J22, dim=2), torch.as_tensor(eps, dtype=u.dtype))
        for mask in (red, ~red):
            du = _bnd(du)
            dv = _bnd(dv)
            c = (slice(1, m - 1), slice(1, n - 1))
            nu = (-torch.sum(W * psi * (J13 + J12 * dv.unsqueeze(-1)), dim=2)[c]
                  + ax * (u[1:-1, 0:-2] + du[1:-1, 0:-2] - u[c])
                  + ax * (u[1:-1, 2:] + du[1:-1, 2:] - u[c])
                  + ay * (u[0:-2, 1:-1] + du[0:-2, 1:-1] - u[c])
                  + ay * (u[2:, 1:-1] + du[2:, 1:-1] - u[c]))
            den_u = den_ud[c] + (ax + ax + ay + ay)
            epsv = torch.as_tensor(eps, dtype=u.dtype)
            new_u = (1 - omega) * du[c] + omega * (nu / torch.maximum(den_u, epsv))
            du_v = du
            if pixel_order == "gauss_seidel":
                du_v = F.pad(torch.where(mask, new_u, du[c]), (1, 1, 1, 1))
            nv = (-torch.sum(W * psi * (J23 + J12 * du_v.unsqueeze(-1)), dim=2)[c]
                  + ax * (v[1:-1, 0:-2] + dv[1:-1, 0:-2] - v[c])
                  + ax * (v[1:-1, 2:] + dv[1:-1, 2:] - v[c])
                  + ay * (v[0:-2, 1:-1] + dv[0:-2, 1:-1] - v[c])
                  + ay * (v[2:, 1:-1] + dv[2:, 1:-1] - v[c]))
            den_v = den_vd[c] + (ax + ax + ay + ay)
            new_v = (1 - omega) * dv[c] + omega * (nv / torch.maximum(den_v, epsv))
            iu = torch.where(mask, new_u, du[c])
            iv = torch.where(mask, new_v, dv[c])
            du = F.pad(iu, (1, 1, 1, 1))
            dv = F.pad(iv, (1, 1, 1, 1))
        du = _bnd(du)
        dv = _bnd(dv)
    return du, dv


# ---------------------------------------------------------------- median
def median5(a: torch.Tensor) -> torch.Tensor:
    """scipy.ndimage.median_filter(size=5, mode='mirror') of a 2-D plane."""
    p = F.pad(a[None, None], (2, 2, 2, 2), mode="reflect")
    cols = F.unfold(p, 5)                        # (1, 25, h*w)
    return cols.median(dim=1).values.reshape(a.shape)


# ---------------------------------------------------------------- level loop
def flow(fixed, moving, alpha, weight, levels=100, eta=0.8, iterations=50, update_lag=5,
         a_data=0.45, min_level=0, uv=None, smooth_only=False, pixel_order="torch", psi_grad=True):
    """Differentiable-mode flow of one pair.  fixed, moving: (K, H, W) float64
    tensors; alpha: tensor (2,); weight: (K,) or (K, H, W).  Returns (u, v),
    each (H, W).  min_level must resolve to 0 (no final upsampling).

    The function has jumps (a pixel whose map crosses the frame edge switches
    from the warped sample to f1) and kinks (the 5x5 median), which central
    differences at small sizes straddle.  smooth_only=True (oracle-only) drops
    both so finite differences can check the rest of the chain tightly."""
    K, H, W = fixed.shape
    a_data = np.broadcast_to(np.asarray(a_data, np.float64), (K,)).copy()
    sched, min_level = O.level_schedule(H, W, levels, eta, min_level)
    if min_level != 0:
        raise NotImplementedError("the differentiable mode computes down to level 0")
    wt = torch.as_tensor(np.asarray(weight, np.float64))
    if wt.dim() == 1:
        wt = wt.view(K, 1, 1).expand(K, H, W)
    u0 = torch.zeros(H, W, dtype=torch.float64) if uv is None else torch.as_tensor(uv[..., 0])
    v0 = torch.zeros(H, W, dtype=torch.float64) if uv is None else torch.as_tensor(uv[..., 1])
    u = v = None
    top = sched[0][0]
    for i, (h, w) in sched:
        f1 = resize(fixed, (h, w))
        f2 = resize(moving, (h, w))
        hrow, hcol = H / h, W / w
        if i == top:
            u = resize(u0, (h, w))
            v = resize(v0, (h, w))
            f2w = f2
        else:
            u = resize(u, (h, w))
            v = resize(v, (h, w))
            f2w = warp(f2, u / hcol, v / hrow, f1, oob_fill=not smooth_only)
        Js = [motion_tensor_gc(f1[k], f2w[k], hrow, hcol) for k in range(K)]
        Jp = [F.pad(torch.stack([Js[k][q] for k in range(K)], dim=-1).permute(2, 0, 1), (1, 1, 1, 1))
              .permute(1, 2, 0) for q in range(6)]
        Wl = F.pad(resize(wt, (h, w)), (1, 1, 1, 1)).permute(1, 2, 0)
        scale = 1.0 if i == min_level else eta ** (-0.5 * i)
        up = F.pad(u[None], (1, 1, 1, 1), mode="replicate")[0]
        vp = F.pad(v[None], (1, 1, 1, 1), mode="replicate")[0]
        du, dv = rbgs_solve(*Jp, Wl, up, vp, alpha * scale, iterations, update_lag, a_data, hcol, hrow,
                            pixel_order=pixel_order, psi_grad=psi_grad)
        du, dv = du[1:-1, 1:-1], dv[1:-1, 1:-1]
        if min(h, w) > 5 and not smooth_only:
            du = median5(du)
            dv = median5(dv)
        u = u + du
        v = v + dv
    return u, v


def loss(fixed, moving, truth, w_true, alpha, weight, lam=0.1, **opts):
    """MSE(warp(moving, flow), truth) + lam * mean(|flow - w_true|^2) for one
    pair (K, H, W); the compensation warp uses the continuous warp with the
    reference frame for out-of-bounds pixels (motion_correction/parallelization/
    sequential.py:148-154)."""
    u, v = flow(fixed, moving, alpha, weight, **opts)
    reg = warp(moving, u, v, fixed, oob_fill=not opts.get("smooth_only", False))
    return ((reg - truth) ** 2).mean() + lam * ((u - w_true[0]) ** 2 + (v - w_true[1]) ** 2).mean()
