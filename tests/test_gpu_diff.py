"""Differentiable mode on the GPU against the differentiable oracle: forward
flow, and gradients with respect to both frames and alpha against autograd
unrolled through the restated torch-backend solver (float64), plus central
differences of the CUDA forward itself."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from test_diff_oracle import synthetic_pair  # noqa: E402


def _frames(seeds, K, h, w):
    f, m, t, wt = zip(*(synthetic_pair(s, K, h, w) for s in seeds))
    return np.stack(f), np.stack(m), np.stack(t), np.stack(wt)


GS = "gauss_seidel"


def _plan(h, w, K, F, dtype, **opts):
    from pyflowreg_gb300.diff import DiffPlan

    p = DiffPlan(h, w, K, F, dtype=dtype, **opts)
    p.set_weight(np.full(K, 1.0 / K))
    return p


def _oracle_flow(fixed, moving, alpha, K, **opts):
    from oracle import diff_oracle as D

    u, v = D.flow(fixed, moving, alpha, np.full(K, 1.0 / K), **opts)
    return torch.stack([u, v])


# The torch backend's within-pixel order diverges after a few tens of
# iterations (its flow reaches 1e50 px at 50 iterations on these frames), so
# it is compared only where it has not yet diverged.
@pytest.mark.parametrize("K,h,w,its,lag,order", [
    (1, 24, 28, 10, 5, GS), (2, 30, 26, 12, 5, GS), (1, 40, 48, 50, 5, GS), (1, 33, 21, 7, 3, GS),
    (2, 64, 48, 50, 5, GS), (1, 24, 28, 10, 5, "torch"), (1, 33, 21, 7, 3, "torch")])
def test_forward_matches_oracle_fp64(K, h, w, its, lag, order):
    from pyflowreg_gb300.diff import flow

    fixed, moving, _, _ = _frames([1, 2], K, h, w)
    opts = dict(iterations=its, update_lag=lag, pixel_order=order)
    plan = _plan(h, w, K, 2, torch.float64, **opts)
    dev = torch.device("cuda")
    got = flow(torch.tensor(fixed, device=dev), torch.tensor(moving, device=dev),
               torch.tensor([1.5, 1.2], dtype=torch.float64), plan).cpu()
    for f in range(2):
        ref = _oracle_flow(torch.tensor(fixed[f]), torch.tensor(moving[f]),
                           torch.tensor([1.5, 1.2], dtype=torch.float64), K, **opts)
        # float64 on both sides; the pyramid amplifies rounding differences by
        # ~1e7 (a 4e-8 change of alpha moves this flow by 0.05 px), so the
        # bound is 1e-6 px, three orders below the 1e-3 px parity bar.
        err = float((got[f] - ref).abs().max())
        assert err <= 1e-6, err


@pytest.mark.parametrize("K,h,w,its,lag,order,ckpt,psi", [
    (1, 24, 28, 10, 5, GS, "ticks", "exact"), (2, 26, 30, 12, 5, GS, "ticks", "exact"),
    (1, 36, 40, 50, 5, GS, "ticks", "exact"), (1, 30, 30, 9, 1, GS, "ticks", "exact"),
    (1, 36, 40, 50, 5, GS, "sweeps", "exact"), (2, 26, 30, 23, 5, GS, "sweeps", "exact"),
    (1, 36, 40, 50, 5, GS, "ticks", "lagged"), (2, 26, 30, 12, 3, GS, "sweeps", "lagged"),
    (1, 24, 28, 10, 5, "torch", "ticks", "exact"), (2, 26, 30, 12, 5, "torch", "sweeps", "exact")])
def test_gradients_match_unrolled_autograd_fp64(K, h, w, its, lag, order, ckpt, psi):
    from pyflowreg_gb300.diff import flow

    fixed, moving, _, _ = _frames([7], K, h, w)
    opts = dict(iterations=its, update_lag=lag, pixel_order=order)
    rng = np.random.default_rng(2)
    r = rng.standard_normal((1, 2, h, w))
    dev = torch.device("cuda")
    plan = _plan(h, w, K, 1, torch.float64, checkpoint=ckpt, psi_gradient=psi, **opts)
    f_t = torch.tensor(fixed, device=dev, requires_grad=True)
    m_t = torch.tensor(moving, device=dev, requires_grad=True)
    a_t = torch.tensor([1.5, 1.2], dtype=torch.float64, device=dev, requires_grad=True)
    (flow(f_t, m_t, a_t, plan) * torch.tensor(r, device=dev)).sum().backward()

    fo = torch.tensor(fixed[0], requires_grad=True)
    mo = torch.tensor(moving[0], requires_grad=True)
    ao = torch.tensor([1.5, 1.2], dtype=torch.float64, requires_grad=True)
    (_oracle_flow(fo, mo, ao, K, psi_grad=(psi == "exact"), **opts) * torch.tensor(r[0])).sum().backward()
    for got, ref in ((f_t.grad[0].cpu(), fo.grad), (m_t.grad[0].cpu(), mo.grad), (a_t.grad.cpu(), ao.grad)):
        scale = float(ref.abs().max())
        err = float((got - ref).abs().max())
        assert err <= 1e-5 * max(scale, 1e-12), (err, scale)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("K,h,w,its,lag,order,ckpt", [
    (1, 75, 100, 23, 5, GS, "ticks"), (2, 70, 66, 12, 3, GS, "sweeps"), (1, 97, 41, 9, 1, GS, "ticks"),
    (1, 64, 130, 50, 5, GS, "sweeps"), (1, 50, 70, 10, 5, "torch", "ticks")])
def test_tiled_window_adjoint_equals_stepwise(dtype, K, h, w, its, lag, order, ckpt):
    """The tiled window adjoint (one launch per tick window, tiles of 32 with
    halos in shared memory) against the one-launch-per-half-sweep adjoint:
    both run the same per-pixel arithmetic, so the frame gradients agree to
    the last bits and the alpha gradients to the rounding of their sums.
    Shapes span several tiles, with ragged edges, short last windows and
    update_lag 1, 3 and 5."""
    from pyflowreg_gb300.diff import flow

    fixed, moving, _, _ = _frames([21, 22], K, h, w)
    dev = torch.device("cuda")
    rng = np.random.default_rng(5)
    r = torch.tensor(rng.standard_normal((2, 2, h, w)), device=dev, dtype=dtype)
    grads = {}
    for adj in ("stepwise", "tiled"):
        plan = _plan(h, w, K, 2, dtype, iterations=its, update_lag=lag, pixel_order=order, checkpoint=ckpt,
                     adjoint=adj)
        f_t = torch.tensor(fixed, device=dev, dtype=dtype, requires_grad=True)
        m_t = torch.tensor(moving, device=dev, dtype=dtype, requires_grad=True)
        a_t = torch.tensor([1.5, 1.2], dtype=torch.float64, device=dev, requires_grad=True)
        (flow(f_t, m_t, a_t, plan) * r).sum().backward()
        grads[adj] = (f_t.grad.double().cpu(), m_t.grad.double().cpu(), a_t.grad.cpu())
    tol = 1e-12 if dtype == torch.float64 else 1e-5
    for name, gs, gt in zip(("fixed", "moving", "alpha"), grads["stepwise"], grads["tiled"]):
        scale = float(gs.abs().max())
        err = float((gs - gt).abs().max())
        assert scale > 0 and err <= tol * scale, (name, err, scale)


@pytest.mark.parametrize("K,h,w,ckpt", [(1, 32, 36, "ticks"), (2, 30, 26, "sweeps")])
def test_implicit_gradient_equals_unrolled_at_convergence_fp64(K, h, w, ckpt):
    """With the forward converged (400 sweeps, psi computed once), the
    fixed-point adjoint (one SOR solve of M lam = g on the level's operator)
    equals the unrolled lagged-psi gradient."""
    from pyflowreg_gb300.diff import flow

    fixed, moving, _, _ = _frames([13], K, h, w)
    dev = torch.device("cuda")
    rng = np.random.default_rng(3)
    r = torch.tensor(rng.standard_normal((1, 2, h, w)), device=dev)
    grads = {}
    for mode in ("unrolled", "implicit"):
        plan = _plan(h, w, K, 1, torch.float64, iterations=400, update_lag=400, psi_gradient="lagged",
                     gradient=mode, checkpoint=ckpt)
        m_t = torch.tensor(moving, device=dev, requires_grad=True)
        f_t = torch.tensor(fixed, device=dev, requires_grad=True)
        a_t = torch.tensor([1.5, 1.2], dtype=torch.float64, device=dev, requires_grad=True)
        (flow(f_t, m_t, a_t, plan) * r).sum().backward()
        grads[mode] = (m_t.grad.cpu(), f_t.grad.cpu(), a_t.grad.cpu())
    for gu, gi in zip(grads["unrolled"], grads["implicit"]):
        scale = float(gu.abs().max())
        assert float((gu - gi).abs().max()) <= 1e-6 * scale, (float((gu - gi).abs().max()), scale)


def test_implicit_gradient_tracks_unrolled_at_default_iterations_fp64():
    """At the default 50 sweeps per level the forward is not converged; the
    implicit gradient then approximates the unrolled lagged one (measured
    cosine over the moving-frame gradient: 0.81 on these frames)."""
    from pyflowreg_gb300.diff import flow

    K, h, w = 1, 64, 64
    fixed, moving, _, _ = _frames([17], K, h, w)
    dev = torch.device("cuda")
    rng = np.random.default_rng(4)
    r = torch.tensor(rng.standard_normal((1, 2, h, w)), device=dev)
    grads = {}
    for mode in ("unrolled", "implicit"):
        plan = _plan(h, w, K, 1, torch.float64, psi_gradient="lagged", gradient=mode)
        m_t = torch.tensor(moving, device=dev, requires_grad=True)
        (flow(torch.tensor(fixed, device=dev), m_t, torch.tensor(1.5), plan) * r).sum().backward()
        grads[mode] = m_t.grad.cpu()
    gu, gi = grads["unrolled"], grads["implicit"]
    cos = float((gu * gi).sum() / (gu.norm() * gi.norm()))
    assert cos >= 0.7, cos


def test_registration_loss_gradient_matches_oracle_fp64():
    from oracle import diff_oracle as D
    from pyflowreg_gb300.diff import registration_loss

    K, h, w = 1, 32, 36
    fixed, moving, truth, w_true = _frames([11], K, h, w)
    opts = dict(iterations=50, update_lag=5, pixel_order=GS)
    dev = torch.device("cuda")
    plan = _plan(h, w, K, 1, torch.float64, **opts)
    m_t = torch.tensor(moving, device=dev, requires_grad=True)
    f_t = torch.tensor(fixed, device=dev, requires_grad=True)
    a_t = torch.tensor(1.5, dtype=torch.float64, device=dev, requires_grad=True)
    L = registration_loss(f_t, m_t, torch.tensor(truth, device=dev), torch.tensor(w_true, device=dev), a_t, plan)
    L.backward()
    mo = torch.tensor(moving[0], requires_grad=True)
    fo = torch.tensor(fixed[0], requires_grad=True)
    ao = torch.tensor(1.5, dtype=torch.float64, requires_grad=True)
    Lo = D.loss(fo, mo, torch.tensor(truth[0]), torch.tensor(w_true[0]), torch.stack([ao, ao]), np.full(K, 1.0),
                **opts)
    Lo.backward()
    Lv, Lov = float(L.detach()), float(Lo.detach())
    assert abs(Lv - Lov) <= 1e-8 * abs(Lov), (Lv, Lov)
    for got, ref in ((m_t.grad[0].cpu(), mo.grad), (f_t.grad[0].cpu(), fo.grad), (a_t.grad.cpu(), ao.grad)):
        scale = float(ref.abs().max())
        err = float((got - ref).abs().max())
        assert err <= 1e-5 * max(scale, 1e-12), (err, scale)


def test_warp_adjoint_matches_autograd():
    from oracle import diff_oracle as D
    from pyflowreg_gb300.diff import warp

    rng = np.random.default_rng(4)
    F, K, H, W = 2, 2, 20, 23
    src = rng.standard_normal((F, K, H, W))
    fill = rng.standard_normal((F, K, H, W))
    flw = rng.uniform(-3, 3, (F, 2, H, W))
    dev = torch.device("cuda")
    s_t = torch.tensor(src, device=dev, requires_grad=True)
    f_t = torch.tensor(flw, device=dev, requires_grad=True)
    l_t = torch.tensor(fill, device=dev, requires_grad=True)
    out = warp(s_t, f_t, l_t)
    g = rng.standard_normal(out.shape)
    (out * torch.tensor(g, device=dev)).sum().backward()
    for f in range(F):
        so = torch.tensor(src[f], requires_grad=True)
        fo = torch.tensor(flw[f], requires_grad=True)
        lo = torch.tensor(fill[f], requires_grad=True)
        oo = D.warp(so, fo[0], fo[1], lo)
        assert float((out[f].detach().cpu() - oo.detach()).abs().max()) <= 1e-12
        (oo * torch.tensor(g[f])).sum().backward()
        for got, ref in ((s_t.grad[f], so.grad), (f_t.grad[f], fo.grad), (l_t.grad[f], lo.grad)):
            assert float((got.cpu() - ref).abs().max()) <= 1e-10 * max(1.0, float(ref.abs().max()))


def test_central_differences_of_the_cuda_forward_fp64():
    """Directional derivatives of the registration loss from the adjoint
    against central differences of the CUDA forward (float64), on unit-norm
    directions in (moving, fixed, alpha).  The function is stiff: psi =
    a (E + 1e-6)^(a - 1) and the tensor's 1 / (fxx^2 + fxy^2 + 1e-6) change
    over tiny input changes, so differences at steps 1e-4 .. 1e-6 are still
    dominated by curvature (and by the median's kinks and the out-of-bounds
    switch); at 1e-8 they have converged to the derivative."""
    from pyflowreg_gb300.diff import registration_loss

    K, h, w, F = 1, 64, 64, 2
    fixed, moving, truth, w_true = _frames([21, 22], K, h, w)
    dev = torch.device("cuda")
    plan = _plan(h, w, K, F, torch.float64)
    tr, wt = torch.tensor(truth, device=dev), torch.tensor(w_true, device=dev)
    m_t = torch.tensor(moving, device=dev, requires_grad=True)
    f_t = torch.tensor(fixed, device=dev, requires_grad=True)
    a_t = torch.tensor(1.5, dtype=torch.float64, device=dev, requires_grad=True)
    registration_loss(f_t, m_t, tr, wt, a_t, plan).backward()
    rng = np.random.default_rng(9)
    report = []
    for _ in range(8):
        dm, df, da = rng.standard_normal(moving.shape), rng.standard_normal(fixed.shape), rng.standard_normal()
        nrm = np.sqrt((dm ** 2).sum() + (df ** 2).sum() + da * da)
        dm, df, da = dm / nrm, df / nrm, da / nrm

        def at(s):
            with torch.no_grad():
                return float(registration_loss(torch.tensor(fixed + s * df, device=dev),
                                               torch.tensor(moving + s * dm, device=dev), tr, wt,
                                               torch.tensor(1.5 + s * da, dtype=torch.float64), plan))

        fd = (at(1e-8) - at(-1e-8)) / 2e-8
        an = float((m_t.grad.cpu() * torch.tensor(dm)).sum() + (f_t.grad.cpu() * torch.tensor(df)).sum()
                   + a_t.grad.cpu() * da)
        report.append((fd, an))
    for fd, an in report:
        assert abs(fd - an) <= 1e-3 * max(abs(an), 1e-3), report


@pytest.mark.parametrize("a_data,psi", [(1.0, "exact"), (1.0, "lagged")])
def test_fp32_plan_tracks_fp64(a_data, psi):
    """float32 against float64 where the gradient is well conditioned (a
    quadratic data term).  With a < 1 the float32 flow still agrees to a few
    hundredths of a pixel, but psi = a (E + 1e-6)^(a - 1) takes values up to
    ~2000x its typical size at pixels whose linearised residual E is near 0,
    so the float32 gradient there (exact or lagged) follows a different
    coefficient field; gradient work with a < 1 uses float64."""
    from pyflowreg_gb300.diff import flow

    K, h, w = 2, 48, 40
    fixed, moving, _, _ = _frames([5, 6, 7], K, h, w)
    dev = torch.device("cuda")
    out = {}
    for dt in (torch.float32, torch.float64):
        plan = _plan(h, w, K, 3, dt, iterations=20, a_data=a_data, psi_gradient=psi)
        m_t = torch.tensor(moving, device=dev, dtype=dt, requires_grad=True)
        fl = flow(torch.tensor(fixed, device=dev, dtype=dt), m_t, torch.tensor(1.5), plan)
        fl.pow(2).sum().backward()
        out[dt] = (fl.detach().double().cpu(), m_t.grad.double().cpu())
    # float32 rounding, amplified by the pyramid like any other perturbation
    e_flow = float((out[torch.float32][0] - out[torch.float64][0]).abs().max())
    assert e_flow <= 0.1, e_flow
    g32, g64 = out[torch.float32][1], out[torch.float64][1]
    cos = float((g32 * g64).sum() / (g32.norm() * g64.norm()))
    assert cos >= 0.999, (cos, e_flow)


def test_plan_rejects_out_of_order_backward():
    from pyflowreg_gb300.diff import flow

    K, h, w = 1, 24, 24
    fixed, moving, _, _ = _frames([3], K, h, w)
    dev = torch.device("cuda")
    plan = _plan(h, w, K, 1, torch.float64, iterations=4)
    m_t = torch.tensor(moving, device=dev, requires_grad=True)
    y1 = flow(torch.tensor(fixed, device=dev), m_t, torch.tensor(1.5), plan)
    flow(torch.tensor(fixed, device=dev), torch.tensor(moving, device=dev), torch.tensor(1.5), plan)
    with pytest.raises(RuntimeError):
        y1.sum().backward()


def test_auto_checkpoint_keeps_sweeps_when_they_fit():
    """checkpoint="auto" keeps every half-sweep (the faster backward) when the
    checkpoints fit in half the free device memory, which a small plan does;
    its gradients are those of an explicit "sweeps" plan (to the rounding of
    the warp adjoint's atomic scatter, whose order varies from run to run)."""
    from pyflowreg_gb300.diff import flow

    K, h, w = 1, 40, 36
    fixed, moving, _, _ = _frames([9], K, h, w)
    dev = torch.device("cuda")
    grads = {}
    for ckpt in ("auto", "sweeps"):
        plan = _plan(h, w, K, 1, torch.float64, iterations=12, checkpoint=ckpt)
        assert plan.checkpoint == "sweeps"
        m_t = torch.tensor(moving, device=dev, requires_grad=True)
        flow(torch.tensor(fixed, device=dev), m_t, torch.tensor(1.5), plan).pow(2).sum().backward()
        grads[ckpt] = m_t.grad.cpu()
    scale = float(grads["sweeps"].abs().max())
    assert float((grads["auto"] - grads["sweeps"]).abs().max()) <= 1e-12 * scale
