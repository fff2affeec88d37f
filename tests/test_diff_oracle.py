"""The differentiable-mode oracle on CPU: its solver against the reference
torch backend's own values and forward-mode derivatives (golden fixture), and
its unrolled autograd gradient against float64 central differences."""
import os

import numpy as np
import pytest
import torch

from oracle import diff_oracle as D

NAMES = ("J11", "J22", "J33", "J12", "J13", "J23")


def _case(z, c):
    g = {k[len(c) + 1:]: z[k] for k in z.files if k.startswith(c + "_")}
    return g


@pytest.mark.parametrize("c", ["a", "b", "c"])
def test_rbgs_solver_matches_reference_values_and_derivatives(golden_dir, c):
    z = np.load(os.path.join(golden_dir, "rbgs_torch.npz"))
    g = _case(z, c)
    t = lambda a: torch.tensor(a, dtype=torch.float64, requires_grad=True)  # noqa: E731
    ins = {k: t(g[k]) for k in NAMES + ("u", "v", "alpha")}
    du, dv = D.rbgs_solve(*(ins[k] for k in NAMES), torch.tensor(g["W"]), ins["u"], ins["v"], ins["alpha"],
                          int(g["iterations"]), int(g["lag"]), g["a_data"], float(g["hx"]), float(g["hy"]))
    np.testing.assert_allclose(du.detach().numpy(), g["du"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(dv.detach().numpy(), g["dv"], rtol=0, atol=1e-12)
    rng = np.random.default_rng(5)
    cu = rng.standard_normal(g["du"].shape)
    cv = rng.standard_normal(g["dv"].shape)
    L = (du * torch.tensor(cu)).sum() + (dv * torch.tensor(cv)).sum()
    L.backward()
    for d in range(1, int(g["n_dir"]) + 1):
        lhs = sum(float((ins[k].grad * torch.tensor(g[f"dir{d}_{k}"])).sum()) for k in ins)
        rhs = float((cu * g[f"dir{d}_du_dot"]).sum() + (cv * g[f"dir{d}_dv_dot"]).sum())
        assert abs(lhs - rhs) <= 1e-9 * max(1.0, abs(rhs)), (d, lhs, rhs)


def synthetic_pair(seed, K, h, w, amp=1.2):
    """fixed (K,h,w), moving (K,h,w), truth (K,h,w), w_true (2,h,w) with
    moving(x + w(x)) = truth(x), built analytically from blobs."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    n = max(6, h * w // 100)
    cy, cx = rng.uniform(0, h, (K, n)), rng.uniform(0, w, (K, n))
    s = rng.uniform(1.5, 3.5, (K, n))
    a = rng.uniform(0.3, 1.0, (K, n))

    def img(k, Y, X):
        out = np.full(Y.shape, 0.05)
        for i in range(n):
            out += a[k, i] * np.exp(-((Y - cy[k, i]) ** 2 + (X - cx[k, i]) ** 2) / (2 * s[k, i] ** 2))
        return out

    kx, ky = rng.uniform(0.02, 0.08, 2)
    ph = rng.uniform(0, 2 * np.pi, 2)
    wu = lambda Y, X: amp * np.sin(kx * X + ky * Y + ph[0])  # noqa: E731
    wv = lambda Y, X: amp * np.cos(ky * X - kx * Y + ph[1])  # noqa: E731
    # moving(y, x) = truth(p) where p + w(p) = (y, x): fixed point p <- (y, x) - w(p)
    py, px = yy.copy(), xx.copy()
    for _ in range(60):
        py, px = yy - wv(py, px), xx - wu(py, px)
    truth = np.stack([img(k, yy, xx) for k in range(K)])
    moving = np.stack([img(k, py, px) for k in range(K)])
    fixed = truth + rng.normal(0, 0.01, truth.shape)
    moving = moving + rng.normal(0, 0.01, moving.shape)
    w_true = np.stack([wu(yy, xx), wv(yy, xx)])
    return fixed, moving, truth, w_true


@pytest.mark.parametrize("seed,order", [(3, "torch"), (4, "torch"), (3, "gauss_seidel"), (5, "gauss_seidel")])
def test_diff_mode_gradient_matches_central_differences(seed, order):
    """Autograd through the whole chain (resize, warp, tensor, red-black solve,
    flow upsampling, compensation warp, loss) against central differences, on
    the smooth part of the function (no out-of-bounds switch, no median)."""
    K, h, w = 1, 20, 24
    fixed, moving, truth, w_true = synthetic_pair(seed, K, h, w)
    opts = dict(levels=100, eta=0.8, iterations=10, update_lag=5, a_data=0.45, smooth_only=True, pixel_order=order)
    weight = np.full(K, 1.0 / K)
    f = torch.tensor(fixed, requires_grad=True)
    m = torch.tensor(moving, requires_grad=True)
    al = torch.tensor([1.5, 1.5], dtype=torch.float64, requires_grad=True)
    L = D.loss(f, m, torch.tensor(truth), torch.tensor(w_true), al, weight, **opts)
    L.backward()
    rng = np.random.default_rng(11)
    step = 1e-7
    for _ in range(3):
        df = rng.standard_normal(fixed.shape)
        dm = rng.standard_normal(moving.shape)
        da = rng.standard_normal(2)
        nrm = np.sqrt((df ** 2).sum() + (dm ** 2).sum() + (da ** 2).sum())
        df, dm, da = df / nrm, dm / nrm, da / nrm

        def at(sgn):
            with torch.no_grad():
                return float(D.loss(torch.tensor(fixed + sgn * step * df), torch.tensor(moving + sgn * step * dm),
                                    torch.tensor(truth), torch.tensor(w_true),
                                    torch.tensor([1.5, 1.5]) + sgn * step * torch.tensor(da), weight, **opts))

        fd = (at(1) - at(-1)) / (2 * step)
        an = float((f.grad * torch.tensor(df)).sum() + (m.grad * torch.tensor(dm)).sum()
                   + (al.grad * torch.tensor(da)).sum())
        assert abs(fd - an) <= 1e-4 * max(abs(fd), 1e-2), (fd, an)
