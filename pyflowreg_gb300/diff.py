"""Differentiable mode: the flow as a differentiable function of both frames
and alpha, with hand-written CUDA adjoints.

The function is pyflowreg's flow path with the level solver of its torch
backend ("flowreg_torch": red-black order, eps = 1e-6, psi tick when
it % update_lag == 0; torch/core/level_solver.py:11-199, registered at
core/__init__.py:140-197), by default with the numba solver's within-pixel
order (see DiffPlan), and a continuous warp: the reference's cv2.remap
rounds map coordinates to 1/32 px (core/warping.py:160-234), which makes the
flow piecewise constant in its inputs, so here the map is used unrounded
(Keys cubic, replicated borders, out-of-bounds pixels from the reference).
The reference runs that backend under ``torch.no_grad()``; this module adds
the gradient.

``flow(fixed, moving, alpha)`` is a ``torch.autograd.Function``: its forward
stores per-level checkpoints on the device (resized frames, the level's input
flow, the solver state at every psi tick) and its backward recomputes each
level from them and runs the exact adjoint of every step, unrolled through all
SOR iterations.  ``warp(src, flow, fill)`` is the compensation warp with its
adjoint (an atomic scatter-add of the cubic weights).
"""

from __future__ import annotations

import ctypes
import threading

import numpy as np
import torch

from . import _lib
from .api import make_params

_PREC = {torch.float32: _lib.FRG_FP32, torch.float64: _lib.FRG_FP64_REFERENCE}
# Plan flags (frg_diff_plan_create) and backward flags (frg_diff_backward).
PIXEL_ORDERS = {"gauss_seidel": 0, "torch": 1}
CHECKPOINTS = {"ticks": 0, "sweeps": 2}
LAGGED_PSI = 1
IMPLICIT = 2
STEPWISE_ADJOINT = 4


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class DiffPlan:
    """One frg_diff_plan: frame shape, options, element type, maximum batch.

    pixel_order "gauss_seidel" (default) updates dv of a moving pixel from its
    new du, the numba solver's order (core/level_solver.py:355-364): the sweep
    is SOR on a symmetric positive definite system and converges.  "torch" is
    the torch backend's order (both from the old values): a Jacobi step on the
    2x2 pixel block that diverges with omega = 1.95 wherever
    |A12| / sqrt(A11 A22) > 2 / omega - 1, so its flow and gradients blow up
    after a few tens of iterations on gradient-constancy tensors.

    checkpoint "ticks" keeps per level the resized frames, the level's input
    flow and the solver state at every psi tick, and the backward recomputes
    each tick window; "sweeps" also keeps the pixels every half-sweep moves
    (2 * iterations half-planes per level) and each window's coefficients, so
    the backward recomputes no sweep and no tick (about 2.1x the forward for
    the exact gradient, against 3.1x with "ticks", at about 3.5x the memory).
    "auto" (default) takes "sweeps" when its checkpoints need at most half of
    the device's free memory, else "ticks".

    gradient "unrolled" (default) is the exact derivative of the computed
    flow: every half-sweep is reversed.  psi_gradient "exact" (default)
    differentiates through the psi ticks too; "lagged" holds psi fixed.  The
    exact derivative of psi = a (E + 1e-6)^(a - 1) is ~1e9 where the
    linearised residual E is near 0, so with a < 1 exact gradients are stiff
    and need float64 to be resolved; lagged gradients are well conditioned.

    gradient "implicit" differentiates each level's fixed point with psi held
    at its last tick: one red-black SOR solve of M lam = dL/dx on the level's
    symmetric operator M, then dL/db = lam, dL/dM = -lam x^T.  It costs about
    one forward solve, equals the unrolled lagged gradient when the forward
    has converged, and approximates it otherwise.

    adjoint "tiled" (default) runs each tick window's unrolled adjoint in one
    launch over tiles whose halos live in shared memory; "stepwise" runs one
    launch per half-sweep.  Both do the same per-pixel arithmetic.

    A plan keeps the checkpoints of its last forward only, so the backward of
    a forward must run before the next forward on the same plan (checked)."""

    def __init__(self, H: int, W: int, K: int, max_frames: int, dtype=torch.float32, *, levels=100, eta=0.8,
                 iterations=50, update_lag=5, a_data=0.45, omega=1.95, pixel_order="gauss_seidel",
                 checkpoint="auto", psi_gradient="exact", gradient="unrolled", adjoint="tiled", device=None):
        if dtype not in _PREC:
            raise ValueError("dtype must be torch.float32 or torch.float64")
        if pixel_order not in PIXEL_ORDERS:
            raise ValueError(f"pixel_order must be one of {sorted(PIXEL_ORDERS)}")
        if checkpoint not in CHECKPOINTS and checkpoint != "auto":
            raise ValueError(f"checkpoint must be 'auto' or one of {sorted(CHECKPOINTS)}")
        if psi_gradient not in ("exact", "lagged"):
            raise ValueError("psi_gradient must be 'exact' or 'lagged'")
        if gradient not in ("unrolled", "implicit"):
            raise ValueError("gradient must be 'unrolled' or 'implicit'")
        if adjoint not in ("tiled", "stepwise"):
            raise ValueError("adjoint must be 'tiled' or 'stepwise'")
        self.backward_flags = (LAGGED_PSI if psi_gradient == "lagged" else 0) | (
            IMPLICIT if gradient == "implicit" else 0) | (STEPWISE_ADJOINT if adjoint == "stepwise" else 0)
        self.lib = _lib.load()
        self.H, self.W, self.K, self.max_frames, self.dtype = int(H), int(W), int(K), int(max_frames), dtype
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.params = make_params((1.0, 1.0), update_lag, iterations, 0, levels, eta, 1.0, a_data, "gc", self.K,
                                  omega, precision="fp32" if dtype == torch.float32 else "fp64")
        if checkpoint == "auto":
            checkpoint = self._auto_checkpoint(iterations, update_lag)
        self.checkpoint = checkpoint
        self.handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.frg_diff_plan_create(ctypes.byref(self.params), self.H, self.W, self.K,
                                                     self.max_frames,
                                                     PIXEL_ORDERS[pixel_order] | CHECKPOINTS[checkpoint],
                                                     ctypes.byref(self.handle)),
                       "frg_diff_plan_create")
        self._load_tables()
        self.generation = 0
        self._pending = None
        self._weight_set = False
        self._lock = threading.Lock()

    def _auto_checkpoint(self, iterations: int, update_lag: int) -> str:
        """"sweeps" when its extra checkpoints (per level: 2 * iterations
        half-planes of moved pixels, the final state and each tick window's five
        coefficient planes, for every frame) take at most half of the free
        device memory, else "ticks"."""
        es = 4 if self.dtype == torch.float32 else 8
        n_ticks = -(-int(iterations) // int(update_lag))
        px = sum(h * w for (h, w) in self.schedule())
        extra = self.max_frames * px * es * (2 * int(iterations) + 2 + 5 * n_ticks)
        with torch.cuda.device(self.device):
            free, _ = torch.cuda.mem_get_info()
        return "sweeps" if extra <= free // 2 else "ticks"

    def schedule(self):
        n = 64
        h = (ctypes.c_int * n)()
        w = (ctypes.c_int * n)()
        ax = (ctypes.c_double * n)()
        ay = (ctypes.c_double * n)()
        cnt = self.lib.frg_schedule(ctypes.byref(self.params), self.H, self.W, n, h, w, ax, ay)
        if cnt < 0:
            _lib.check(-cnt, "frg_schedule")
        return [(h[i], w[i]) for i in range(cnt)]

    def _load_tables(self):
        """Uploads the reference's numpy-built tap tables for every level."""
        from . import tables

        pI = ctypes.POINTER(ctypes.c_int)
        pF = ctypes.POINTER(ctypes.c_float)
        prev = None
        for i, (h, w) in enumerate(self.schedule()):
            for kind, src in ((0, (self.H, self.W)), (1, prev if prev is not None else (self.H, self.W))):
                ix, wx, iy, wy = tables.level_tables(src, (h, w))
                _lib.check(self.lib.frg_diff_set_level_tables(
                    self.handle, i, kind, ix.shape[1], ix.ctypes.data_as(pI), wx.ctypes.data_as(pF),
                    iy.ctypes.data_as(pI), wy.ctypes.data_as(pF)), "frg_diff_set_level_tables")
            prev = (h, w)

    def device_bytes(self) -> int:
        return int(self.lib.frg_diff_plan_device_bytes(self.handle))

    def set_weight(self, weight) -> None:
        """weight: per-channel (K,) or per-pixel (K, H, W) data-term weights."""
        wt = torch.as_tensor(weight, dtype=self.dtype, device=self.device)
        if wt.dim() == 1:
            wt = wt.view(self.K, 1, 1).expand(self.K, self.H, self.W)
        wt = wt.contiguous()
        if wt.shape != (self.K, self.H, self.W):
            raise ValueError(f"weight must be ({self.K},) or ({self.K}, {self.H}, {self.W})")
        _lib.check(self.lib.frg_diff_set_weight(self.handle, _ptr(wt), _stream(self.device)), "frg_diff_set_weight")
        self._weight_keep = wt
        self._weight_set = True

    def _check_frames(self, t, name):
        if t.dtype != self.dtype or t.device != self.device or not t.is_contiguous():
            raise ValueError(f"{name} must be a contiguous {self.dtype} tensor on {self.device}")
        if t.dim() != 4 or tuple(t.shape[1:]) != (self.K, self.H, self.W):
            raise ValueError(f"{name} must be (F, {self.K}, {self.H}, {self.W})")
        if not 1 <= t.shape[0] <= self.max_frames:
            raise ValueError(f"{name}: batch of {t.shape[0]} frames exceeds the plan's {self.max_frames}")

    def forward(self, fixed, moving, alpha_x: float, alpha_y: float, uv_init=None):
        """Flow (F, 2, H, W) of each (fixed[f], moving[f]) pair; stores the checkpoints."""
        if not self._weight_set:
            self.set_weight(torch.full((self.K,), 1.0 / self.K))
        self._check_frames(fixed, "fixed")
        self._check_frames(moving, "moving")
        F = moving.shape[0]
        if fixed.shape[0] != F:
            raise ValueError("fixed and moving must have the same number of frames")
        if uv_init is not None:
            uv_init = uv_init.to(device=self.device, dtype=self.dtype).contiguous()
            if tuple(uv_init.shape) != (F, 2, self.H, self.W):
                raise ValueError(f"uv_init must be ({F}, 2, {self.H}, {self.W})")
        out = torch.empty((F, 2, self.H, self.W), dtype=self.dtype, device=self.device)
        _lib.check(self.lib.frg_diff_forward(self.handle, F, float(alpha_x), float(alpha_y), _ptr(fixed),
                                             _ptr(moving), _ptr(uv_init), _ptr(out), _stream(self.device)),
                   "frg_diff_forward")
        self.generation += 1
        self._pending = (F, self.generation)
        return out

    def backward(self, g_flow, need_fixed=True, need_moving=True, need_alpha=True):
        """(g_fixed, g_moving, g_alpha (F, 2) float64) of the last forward."""
        if self._pending is None:
            raise RuntimeError("no forward pass to differentiate on this plan")
        F = self._pending[0]
        g_flow = g_flow.to(device=self.device, dtype=self.dtype).contiguous()
        if tuple(g_flow.shape) != (F, 2, self.H, self.W):
            raise ValueError(f"g_flow must be ({F}, 2, {self.H}, {self.W})")
        shape = (F, self.K, self.H, self.W)
        gf = torch.empty(shape, dtype=self.dtype, device=self.device) if need_fixed else None
        gm = torch.empty(shape, dtype=self.dtype, device=self.device) if need_moving else None
        ga = torch.empty((F, 2), dtype=torch.float64, device=self.device) if need_alpha else None
        _lib.check(self.lib.frg_diff_backward(self.handle, _ptr(g_flow), _ptr(gf), _ptr(gm), _ptr(ga),
                                              self.backward_flags, _stream(self.device)), "frg_diff_backward")
        return gf, gm, ga

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            self.lib.frg_diff_plan_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _alpha_pair(alpha):
    a = torch.as_tensor(alpha)
    if a.numel() == 1:
        v = float(a.reshape(()))
        return v, v
    if a.numel() == 2:
        return float(a.reshape(-1)[0]), float(a.reshape(-1)[1])
    raise ValueError("alpha must be a scalar or a pair")


class _FlowFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, fixed, moving, alpha, plan, uv_init):
        ax, ay = _alpha_pair(alpha.detach())
        out = plan.forward(fixed.detach().contiguous(), moving.detach().contiguous(), ax, ay, uv_init)
        ctx.plan = plan
        ctx.generation = plan.generation
        ctx.alpha_numel = alpha.numel()
        ctx.alpha_shape = alpha.shape
        ctx.alpha_dtype = alpha.dtype
        return out

    @staticmethod
    def backward(ctx, g_flow):
        plan = ctx.plan
        if plan.generation != ctx.generation:
            raise RuntimeError("the plan ran another forward before this backward; use one plan per pending graph")
        need = ctx.needs_input_grad
        gf, gm, ga = plan.backward(g_flow, need_fixed=need[0], need_moving=need[1], need_alpha=need[2])
        g_alpha = None
        if ga is not None:
            tot = ga.sum(0)
            g_alpha = (tot.sum() if ctx.alpha_numel == 1 else tot).to(ctx.alpha_dtype).reshape(ctx.alpha_shape)
        return gf, gm, g_alpha, None, None


def flow(fixed, moving, alpha, plan: DiffPlan, uv_init=None):
    """Differentiable flow (F, 2, H, W) of frames (F, K, H, W).

    fixed may be (K, H, W) (one reference for all frames; its gradient is then
    the sum over frames).  alpha: scalar (alpha_x = alpha_y) or pair tensor."""
    alpha = torch.as_tensor(alpha, dtype=torch.float64, device=moving.device) if not torch.is_tensor(alpha) else alpha
    if fixed.dim() == 3:
        fixed = fixed.unsqueeze(0).expand(moving.shape[0], *fixed.shape)
    return _FlowFn.apply(fixed.contiguous(), moving.contiguous(), alpha, plan, uv_init)


class _WarpFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, src, flw, fill):
        src, flw, fill = src.detach().contiguous(), flw.detach().contiguous(), fill.detach().contiguous()
        F, K, H, W = src.shape
        out = torch.empty_like(src)
        lib = _lib.load()
        _lib.check(lib.frg_diff_warp(_PREC[src.dtype], F, K, H, W, _ptr(src), _ptr(flw), _ptr(fill), _ptr(out),
                                     _stream(src.device)), "frg_diff_warp")
        ctx.save_for_backward(src, flw)
        return out

    @staticmethod
    def backward(ctx, g_out):
        src, flw = ctx.saved_tensors
        F, K, H, W = src.shape
        g_out = g_out.contiguous()
        g_src = torch.empty_like(src)
        g_fill = torch.empty_like(src) if ctx.needs_input_grad[2] else None
        g_flow = torch.empty_like(flw) if ctx.needs_input_grad[1] else None
        lib = _lib.load()
        _lib.check(lib.frg_diff_warp_backward(_PREC[src.dtype], F, K, H, W, _ptr(src), _ptr(flw), _ptr(g_out),
                                              _ptr(g_src), _ptr(g_fill), _ptr(g_flow), _stream(src.device)),
                   "frg_diff_warp_backward")
        return g_src, g_flow, g_fill


def warp(src, flw, fill):
    """Continuous compensation warp out = src(x + flow), out-of-bounds pixels
    from fill (motion_correction/parallelization/sequential.py:148-154);
    src, fill (F, K, H, W), flow (F, 2, H, W); differentiable in all three."""
    if fill.dim() == 3:
        fill = fill.unsqueeze(0).expand_as(src)
    return _WarpFn.apply(src, flw, fill)


def registration_loss(fixed, moving, truth, w_true, alpha, plan: DiffPlan, lam: float = 0.1):
    """MSE(warp(moving, flow), truth) + lam * mean |flow - w_true|^2, the
    differentiation workload's loss; flow = flow(fixed, moving, alpha)."""
    w = flow(fixed, moving, alpha, plan)
    reg = warp(moving, w, fixed if fixed.dim() == 4 else fixed.unsqueeze(0).expand_as(moving))
    return ((reg - truth) ** 2).mean() + lam * ((w - w_true) ** 2).sum(1).mean()
