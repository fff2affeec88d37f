"""Reference-facing API of the GB300 backend.

Each public function mirrors a pyflowreg function on the optical-flow path --
same name, arguments, argument meaning, return type and error behaviour -- and
runs on the GPU through the C ABI (``include/flowreg_gb300.h``):

* ``get_displacement``      core/optical_flow.py:773-929
* ``imregister_wrapper``    core/warping.py:160-234
* ``level_solver``          core/optical_flow.py:348-411 (the ``level_solver_backend`` seam)
* ``imresize_fused_gauss_cubic`` util/resize_util.py:232-254
* ``get_motion_tensor_gc`` / ``get_motion_tensor_gray`` core/optical_flow.py:73-228

plus batched/device entry points (``get_displacement_batch``,
``get_displacement_device``, ``imregister_device``) that register many frames
in one call.  There is no CPU fallback: without a CUDA device these raise.
"""

from __future__ import annotations

import ctypes
import os
import threading
from typing import Optional

import numpy as np

from . import _lib

try:  # torch provides device memory and streams
    import torch
except ImportError:  # pragma: no cover - torch is a hard dependency of the package
    torch = None

_CONST = {"gc": 0, "gradient": 0, "gray": 1, "brightness": 1, "cs": 2, "census": 2}


def _require_cuda():
    if torch is None or not torch.cuda.is_available():
        raise RuntimeError("pyflowreg_gb300 needs a CUDA GPU (sm_103a); there is no CPU fallback")


def _stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


# --------------------------------------------------------------------------
# Option handling (core/optical_flow.py:414-473, 842-885)
# --------------------------------------------------------------------------
def resolve_const_assumption(const_assumption) -> int:
    if hasattr(const_assumption, "value"):
        const_assumption = const_assumption.value
    key = str(const_assumption).strip().lower()
    if key not in _CONST:
        supported = "', '".join(sorted(_CONST))
        raise ValueError(
            f"Unknown constancy assumption: '{const_assumption}'. Supported values are: '{supported}'."
        )
    return _CONST[key]


def normalize_gnc_schedule(gnc_schedule):
    """Validation of core/optical_flow.py:414-432."""
    if gnc_schedule is None:
        return None
    schedule = np.asarray(gnc_schedule, dtype=np.float64)
    if schedule.ndim != 1:
        raise ValueError("gnc_schedule must be a 1D sequence of stage weights")
    if schedule.size < 2:
        raise ValueError("gnc_schedule must contain at least two stages")
    if np.any(schedule < 0.0) or np.any(schedule > 1.0):
        raise ValueError("gnc_schedule entries must lie in [0, 1]")
    if not np.all(np.diff(schedule) >= 0.0):
        raise ValueError("gnc_schedule must be monotone nondecreasing")
    if not np.isclose(schedule[0], 0.0):
        raise ValueError("gnc_schedule must start at 0.0")
    if not np.isclose(schedule[-1], 1.0):
        raise ValueError("gnc_schedule must end at 1.0")
    return schedule


def normalize_warping_steps(warping_steps):
    if warping_steps is None:
        return None
    steps = int(warping_steps)
    if steps < 1:
        raise ValueError("warping_steps must be a positive integer")
    return steps


def normalize_weight(weight, m: int, n: int, K: int) -> np.ndarray:
    """(m, n, K) float64 weight exactly as get_displacement builds it (:856-879)."""
    if weight is None:
        return np.ones((m, n, K), dtype=np.float64) / K
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
            weight = np.ones((m, n, K), dtype=np.float64) * weight[..., np.newaxis]
    return weight


def normalize_a_data(a_data, K: int) -> np.ndarray:
    if not isinstance(a_data, np.ndarray):
        return np.full(K, a_data, dtype=np.float64)
    return np.ascontiguousarray(a_data, dtype=np.float64)


def alpha_pair(alpha):
    if np.isscalar(alpha):
        return float(alpha), float(alpha)
    alpha = list(alpha)
    return float(alpha[0]), float(alpha[1] if len(alpha) > 1 else alpha[0])


PRECISIONS = {"fp32": _lib.FRG_FP32, "fp64": _lib.FRG_FP64_REFERENCE}


def make_params(alpha=(2, 2), update_lag=5, iterations=50, min_level=0, levels=50, eta=0.8,
                a_smooth=1.0, a_data=0.45, const_assumption="gc", K=1, omega=1.95,
                precision="fp32", gnc_schedule=None, warping_steps=None) -> "_lib.FrgParams":
    """Options as a frg_params struct.  precision "fp32" is the fast path;
    "fp64" computes in the reference's precision and operation order (the
    parity mode).  gnc_schedule / warping_steps select the graduated
    non-convexity stages (core/optical_flow.py:887-929; 10 warping steps
    per level when warping_steps is None)."""
    if K > _lib.FRG_MAX_CHANNELS:
        raise ValueError(f"at most {_lib.FRG_MAX_CHANNELS} channels are supported")
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
    p = _lib.FrgParams()
    p.precision = PRECISIONS[precision]
    p.alpha_x, p.alpha_y = alpha_pair(alpha)
    p.eta = float(eta)
    p.levels = int(levels)
    p.min_level = int(min_level)
    p.iterations = int(iterations)
    p.update_lag = int(update_lag)
    p.a_smooth = float(a_smooth)
    ad = normalize_a_data(a_data, K)
    if ad.shape != (K,):
        raise ValueError(f"a_data must have one entry per channel ({K})")
    for k in range(K):
        p.a_data[k] = float(ad[k])
    p.const_assumption = resolve_const_assumption(const_assumption)
    p.omega = float(omega)
    sched = normalize_gnc_schedule(gnc_schedule)
    steps = normalize_warping_steps(warping_steps)
    if sched is not None:
        if sched.size > _lib.FRG_MAX_GNC_STAGES:
            raise ValueError(f"at most {_lib.FRG_MAX_GNC_STAGES} GNC stages are supported")
        p.gnc_stages = int(sched.size)
        for i, b in enumerate(sched):
            p.gnc_schedule[i] = float(b)
        p.warping_steps = 10 if steps is None else steps
    return p


def _params_key(p) -> tuple:
    return (p.alpha_x, p.alpha_y, p.eta, p.levels, p.min_level, p.iterations, p.update_lag, p.a_smooth,
            tuple(p.a_data), p.const_assumption, p.omega, p.precision, p.gnc_stages,
            tuple(p.gnc_schedule[:p.gnc_stages]), p.warping_steps)


# --------------------------------------------------------------------------
# Plans
# --------------------------------------------------------------------------
class Plan:
    """Owns one frg_plan: fixed frame shape, options and maximum batch."""

    def __init__(self, params, H: int, W: int, K: int, max_frames: int):
        _require_cuda()
        self.lib = _lib.load()
        self.H, self.W, self.K, self.max_frames = H, W, K, max_frames
        self.params = params
        self.device = torch.cuda.current_device()
        h = ctypes.c_void_p()
        _lib.check(self.lib.frg_plan_create(ctypes.byref(params), H, W, K, max_frames, ctypes.byref(h)),
                   "frg_plan_create")
        self.handle = h
        self._ref_key = None
        self._load_tables()

    def _load_tables(self):
        """Uploads the reference's numpy-built resize tables for every level."""
        from . import tables

        pI = ctypes.POINTER(ctypes.c_int)
        pF = ctypes.POINTER(ctypes.c_float)
        prev = None
        for i, (h, w, _, _) in enumerate(self.levels()):
            srcs = ((0, (self.H, self.W)), (1, prev if prev is not None else (self.H, self.W)))
            for kind, src in srcs:
                ix, wx, iy, wy = tables.level_tables(src, (h, w))
                _lib.check(self.lib.frg_plan_set_level_tables(
                    self.handle, i, kind, ix.shape[1], ix.ctypes.data_as(pI), wx.ctypes.data_as(pF),
                    iy.ctypes.data_as(pI), wy.ctypes.data_as(pF)), "frg_plan_set_level_tables")
            prev = (h, w)

    def levels(self):
        out = []
        for i in range(self.lib.frg_plan_num_levels(self.handle)):
            h, w = ctypes.c_int(), ctypes.c_int()
            ax, ay = ctypes.c_double(), ctypes.c_double()
            _lib.check(self.lib.frg_plan_level_info(self.handle, i, ctypes.byref(h), ctypes.byref(w),
                                                    ctypes.byref(ax), ctypes.byref(ay)))
            out.append((h.value, w.value, ax.value, ay.value))
        return out

    def device_bytes(self) -> int:
        return int(self.lib.frg_plan_device_bytes(self.handle))

    def set_profiling(self, enable: bool) -> None:
        _lib.check(self.lib.frg_plan_set_profiling(self.handle, 1 if enable else 0))

    def profile(self):
        """(SOR launches, summed SOR device ms, SOR algorithmic bytes) since set_profiling."""
        n = ctypes.c_longlong()
        ms, b = ctypes.c_double(), ctypes.c_double()
        _lib.check(self.lib.frg_plan_profile(self.handle, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(b)))
        return n.value, ms.value, b.value

    def level_tuning(self):
        """[(sor_G, sor_threads, gmax, rows)] per level, coarsest first (gmax 0:
        the level does not use the fused SOR kernel)."""
        out = []
        for i in range(self.lib.frg_plan_num_levels(self.handle)):
            v = [ctypes.c_int() for _ in range(4)]
            _lib.check(self.lib.frg_plan_level_tuning(self.handle, i, *[ctypes.byref(x) for x in v]))
            out.append(tuple(x.value for x in v))
        return out

    def set_level_tuning(self, level: int, sor_G: int = 0, sor_threads: int = 0) -> None:
        _lib.check(self.lib.frg_plan_set_level_tuning(self.handle, level, sor_G, sor_threads),
                   "frg_plan_set_level_tuning")

    def level_variant(self, level: int):
        """(variant, n_variants) of a level's fused SOR kernel: 0 the diagonal
        ring, 1 rows with the state in registers (one launch per pass), 2 the
        same with all passes of the level chained in one launch; n_variants
        counts the variants that serve the level."""
        v, n = ctypes.c_int(), ctypes.c_int()
        _lib.check(self.lib.frg_plan_level_variant(self.handle, level, ctypes.byref(v), ctypes.byref(n)))
        return v.value, n.value

    def set_level_variant(self, level: int, variant: int) -> None:
        _lib.check(self.lib.frg_plan_set_level_variant(self.handle, level, variant), "frg_plan_set_level_variant")

    def autotune(self, moving_t, n_levels: int = 5, reps: int = 2):
        """Launch-shape tuning on `moving_t` (a representative device batch);
        the flows do not depend on the choice.  fp32 plans: see
        _autotune_fp32.  fp64 plans: for the `n_levels` finest levels, the
        rows per CTA strip of the float64 SOR (256, 128 or 64; 0 = chosen
        from the batch size), each candidate timed with CUDA events on full
        calls (best of `reps`), coordinate descent from the finest level.
        Returns {level: (variant, sor_G, sor_threads, ms)}."""
        if self.fp64:
            return self._autotune_fp64(moving_t, n_levels, reps)
        return self._autotune_fp32(moving_t, n_levels, reps)

    def _timer(self, moving_t, reps):
        odt = torch.float64 if self.fp64 else torch.float32
        out_t = torch.empty((moving_t.shape[0], self.H, self.W, 2), dtype=odt, device=moving_t.device)

        def timed():
            best = float("inf")
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                self.displacement(moving_t, None, out_t)
                e1.record()
                torch.cuda.synchronize()
                best = min(best, e0.elapsed_time(e1))
            return best

        self.displacement(moving_t, None, out_t)
        torch.cuda.synchronize()
        return timed

    def _autotune_fp64(self, moving_t, n_levels, reps):
        timed = self._timer(moving_t, reps)
        tun = self.level_tuning()
        chosen = {}
        for i in list(range(len(tun) - 1, -1, -1))[:n_levels]:
            best = None
            for rows in (0, 256, 128, 64):
                try:
                    self.set_level_tuning(i, 0, rows)
                except ValueError:
                    continue
                ms = timed()
                if best is None or ms < best[3]:
                    best = (0, 0, rows, ms)
            if best is not None:
                self.set_level_tuning(i, 0, best[2])
                chosen[i] = best
        return chosen

    def _autotune_fp32(self, moving_t, n_levels: int = 5, reps: int = 2):
        """Picks, for the `n_levels` finest levels that use a fused SOR kernel,
        the kernel variant, the iterations per wavefront pass and (ring variant)
        the threads per CTA that make full calls on `moving_t` (a
        representative device batch) fastest: coordinate descent from the
        finest level, each candidate timed with CUDA events (best of `reps`).
        The flows do not depend on the choice.
        Returns {level: (variant, sor_G, sor_threads, ms)}."""
        tun = self.level_tuning()
        timed = self._timer(moving_t, reps)
        chosen = {}
        levels = [i for i in range(len(tun) - 1, -1, -1) if tun[i][2] > 0][:n_levels]
        for i in levels:
            _, _, gmax, rows = tun[i]
            # every pass length: short passes free shared memory for a second CTA per SM
            gs = list(range(gmax, 0, -1))
            ths = sorted({t for t in (rows, ((rows * 3 // 2) + 31) // 32 * 32, 1024) if rows <= t <= 1024})
            cands = [(0, g, t) for g in gs for t in ths]
            nv = self.level_variant(i)[1]
            cands += [(v, g, 0) for v in range(1, nv) for g in gs]
            best = None
            for var, g, t in cands:
                self.set_level_variant(i, var)
                self.set_level_tuning(i, g, t)
                ms = timed()
                if best is None or ms < best[3]:
                    best = (var, g, t, ms)
            self.set_level_variant(i, best[0])
            self.set_level_tuning(i, best[1], best[2])
            chosen[i] = best
        return chosen

    def set_reference(self, fixed_t, weight_t=None, stream=None, key=None):
        """fixed_t (H, W, K) float32 CUDA tensor; weight_t the same shape or None."""
        if key is not None and key == self._ref_key:
            return
        self._check(fixed_t, (self.H, self.W, self.K))
        if weight_t is not None:
            self._check(weight_t, (self.H, self.W, self.K))
        _lib.check(self.lib.frg_set_reference(self.handle, _ptr(fixed_t),
                                              None if weight_t is None else _ptr(weight_t),
                                              _stream_ptr(stream)), "frg_set_reference")
        self._ref_key = key

    @property
    def fp64(self) -> bool:
        return self.params.precision == _lib.FRG_FP64_REFERENCE

    def displacement(self, moving_t, uv_t=None, out_t=None, stream=None):
        """moving_t (T, H, W, K) float32 CUDA tensor -> flow (T, H, W, 2), float32
        (float64 for an fp64 plan)."""
        T = moving_t.shape[0]
        self._check(moving_t, (T, self.H, self.W, self.K))
        if uv_t is not None:
            self._check(uv_t, (self.H, self.W, 2))
        odt = torch.float64 if self.fp64 else torch.float32
        if out_t is None:
            out_t = torch.empty((T, self.H, self.W, 2), dtype=odt, device=moving_t.device)
        self._check(out_t, (T, self.H, self.W, 2), odt)
        fn = self.lib.frg_get_displacement_f64 if self.fp64 else self.lib.frg_get_displacement
        for t0 in range(0, T, self.max_frames):
            t1 = min(T, t0 + self.max_frames)
            _lib.check(fn(self.handle, t1 - t0, _ptr(moving_t[t0:t1]), None if uv_t is None else _ptr(uv_t),
                          _ptr(out_t[t0:t1]), _stream_ptr(stream)), "frg_get_displacement")
        return out_t

    @staticmethod
    def _check(t, shape, dtype=None):
        dtype = dtype or torch.float32
        if not (t.is_cuda and t.dtype == dtype and t.is_contiguous()):
            raise ValueError(f"expected a contiguous {dtype} CUDA tensor")
        if tuple(t.shape) != tuple(shape):
            raise ValueError(f"expected shape {tuple(shape)}, got {tuple(t.shape)}")

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.frg_plan_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lanes_for(n_frames: int) -> int:
    """Lanes of a batched plan: one frame's level runs as one CTA (or one cluster),
    so a batch of a few hundred frames leaves the last wave of every level part
    empty; independent lanes on their own streams fill those gaps."""
    return 4 if n_frames >= 256 else (2 if n_frames >= 128 else 1)


class LanePlan:
    """Several plans over contiguous frame ranges of one batch, each on its own
    stream, joined to the caller's stream by events: the same flows as one
    plan (every frame is independent), with the levels of different lanes
    overlapping on the GPU.  Tuning, kernel variants and profiling apply to
    every lane."""

    def __init__(self, params, H: int, W: int, K: int, max_frames: int, lanes: int):
        _require_cuda()
        self.H, self.W, self.K, self.params = H, W, K, params
        self.device = torch.cuda.current_device()
        self.lane_frames = -(-int(max_frames) // int(lanes))
        self.plans = [Plan(params, H, W, K, self.lane_frames) for _ in range(int(lanes))]
        self.max_frames = self.lane_frames * len(self.plans)
        self.streams = [torch.cuda.Stream() for _ in self.plans]

    @property
    def fp64(self) -> bool:
        return self.plans[0].fp64

    def levels(self):
        return self.plans[0].levels()

    def level_tuning(self):
        return self.plans[0].level_tuning()

    def level_variant(self, level: int):
        return self.plans[0].level_variant(level)

    def set_level_tuning(self, level: int, sor_G: int = 0, sor_threads: int = 0) -> None:
        for p in self.plans:
            p.set_level_tuning(level, sor_G, sor_threads)

    def set_level_variant(self, level: int, variant: int) -> None:
        for p in self.plans:
            p.set_level_variant(level, variant)

    def device_bytes(self) -> int:
        return sum(p.device_bytes() for p in self.plans)

    def set_profiling(self, enable: bool) -> None:
        for p in self.plans:
            p.set_profiling(enable)

    def profile(self):
        """Summed over the lanes (their launches overlap in time)."""
        n = ms = b = 0
        for p in self.plans:
            pn, pms, pb = p.profile()
            n, ms, b = n + pn, ms + pms, b + pb
        return n, ms, b

    def autotune(self, moving_t, n_levels: int = 5, reps: int = 2):
        """Plan.autotune on the first lane with a lane-sized slice of the batch;
        the other lanes take its choice."""
        chosen = self.plans[0].autotune(moving_t[:self.lane_frames], n_levels, reps)
        for i, (v, g, t, _) in chosen.items():
            for p in self.plans[1:]:
                p.set_level_variant(i, v)
                p.set_level_tuning(i, g, t)
        return chosen

    def set_reference(self, fixed_t, weight_t=None, stream=None, key=None):
        for p in self.plans:
            p.set_reference(fixed_t, weight_t, stream=stream, key=key)

    def displacement(self, moving_t, uv_t=None, out_t=None, stream=None):
        T = moving_t.shape[0]
        odt = torch.float64 if self.fp64 else torch.float32
        if out_t is None:
            out_t = torch.empty((T, self.H, self.W, 2), dtype=odt, device=moving_t.device)
        n = self.lane_frames
        if T <= n:
            return self.plans[0].displacement(moving_t, uv_t, out_t, stream=stream)
        s = stream if stream is not None else torch.cuda.current_stream()
        start = torch.cuda.Event()
        start.record(s)
        per = -(-T // len(self.plans))
        for i, (p, ls) in enumerate(zip(self.plans, self.streams)):
            t0, t1 = i * per, min(T, (i + 1) * per)
            if t0 >= t1:
                break
            ls.wait_event(start)
            p.displacement(moving_t[t0:t1], uv_t, out_t[t0:t1], stream=ls)
            done = torch.cuda.Event()
            done.record(ls)
            s.wait_event(done)
        return out_t

    def close(self):
        for p in self.plans:
            p.close()


_plans: dict = {}
_plans_lock = threading.Lock()


def get_plan(params, H: int, W: int, K: int, n_frames: int, max_frames: Optional[int] = None):
    """Cached plan for (shape, options, device); grown when a larger batch
    arrives.  Batches of 128 frames and more get a LanePlan."""
    _require_cuda()
    key = (H, W, K, _params_key(params), torch.cuda.current_device())
    want = max(1, int(max_frames or n_frames))
    with _plans_lock:
        plan = _plans.get(key)
        if plan is None or plan.max_frames < want:
            if plan is not None:
                plan.close()
            lanes = lanes_for(want)
            plan = LanePlan(params, H, W, K, want, lanes) if lanes > 1 else Plan(params, H, W, K, want)
            _plans[key] = plan
        return plan


def clear_plans():
    with _plans_lock:
        for p in _plans.values():
            p.close()
        _plans.clear()


# --------------------------------------------------------------------------
# get_displacement (core/optical_flow.py:773-929)
# --------------------------------------------------------------------------
def _prepare(fixed, moving, weight, a_data, alpha, update_lag, iterations, min_level, levels, eta, a_smooth,
             const_assumption, gnc_schedule, warping_steps, level_solver_backend, precision="fp64"):
    const = resolve_const_assumption(const_assumption)
    if level_solver_backend is not None:
        if not callable(level_solver_backend):
            raise TypeError("level_solver_backend must be callable")
        if precision != "fp64":
            raise NotImplementedError("a caller-supplied level solver runs on the float64 path (precision='fp64')")
        if gnc_schedule is not None:
            raise NotImplementedError("a caller-supplied level solver is supported without a GNC schedule")
    fixed = np.asarray(fixed)
    moving = np.asarray(moving)
    K = fixed.shape[2] if fixed.ndim == 3 else 1
    m, n = fixed.shape[:2]
    w = normalize_weight(weight, m, n, K)
    params = make_params(alpha, update_lag, iterations, min_level, levels, eta, a_smooth, a_data,
                         ["gc", "gray", "cs"][const], K, precision=precision, gnc_schedule=gnc_schedule,
                         warping_steps=warping_steps)
    return fixed, moving, w, params, m, n, K


def get_displacement(fixed, moving, alpha=(2, 2), update_lag=5, iterations=50, min_level=0, levels=50, eta=0.8,
                     a_smooth=1.0, a_data=0.45, const_assumption="gc", uv=None, weight=None,
                     level_solver_backend=None, gnc_schedule=None, warping_steps=None, precision="fp64"):
    """Drop-in for pyflowreg.core.optical_flow.get_displacement on the GPU.

    Returns the (H, W, 2) float64 displacement, [..., 0] = u (columns),
    [..., 1] = v (rows), like the reference.  ``precision`` is the only
    argument the reference does not have: "fp64" (default) computes in the
    reference's float64 precision and operation order and matches it within
    1e-3 px; "fp32" is faster, but the algorithm amplifies float32 rounding to
    deviations of up to ~0.7 px from the reference's flow.
    """
    assert fixed.ndim == moving.ndim, (
        f"Fixed and moving must have same dimensions: fixed.shape={fixed.shape}, moving.shape={moving.shape}"
    )
    fixed, moving, w, params, m, n, K = _prepare(fixed, moving, weight, a_data, alpha, update_lag, iterations,
                                                 min_level, levels, eta, a_smooth, const_assumption, gnc_schedule,
                                                 warping_steps, level_solver_backend, precision)
    if level_solver_backend is not None:
        return _run_with_solver(level_solver_backend, params, fixed.reshape(m, n, K), moving.reshape(1, m, n, K), w,
                                uv, normalize_a_data(a_data, K), float(a_smooth), int(iterations), int(update_lag))
    flow = _run_host(params, fixed.reshape(m, n, K), moving.reshape(1, m, n, K), w, uv)
    return flow[0].astype(np.float64)


class _DeviceF64:
    """A float64 device buffer given by pointer and shape, viewed by torch
    through the CUDA array interface (no copy)."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": tuple(int(s) for s in shape), "typestr": "<f8",
                                         "data": (int(ptr), False), "version": 3, "strides": None}


def _device_f64(ptr, shape):
    return torch.as_tensor(_DeviceF64(ptr, shape), device=torch.device("cuda", torch.cuda.current_device()))


def _run_with_solver(solver, params, fixed, moving, weight, uv, a_data, a_smooth, iterations, update_lag):
    """get_displacement with the caller's level solver (core/optical_flow.py:579-606):
    the float64 path computes each level's pyramid, warp and motion tensor on
    the device and, in place of its own SOR, hands the solver the arrays the
    reference passes (J11..J23 and the weight as padded (m, n, K) float64, u, v
    as padded (m, n), alpha, iterations, update_lag, verbose 0, a_data,
    a_smooth, hx, hy, gnc_beta None); the returned du, dv go through the
    median and accumulation on the device."""
    _require_cuda()
    m, n, K = fixed.shape
    dev = torch.device("cuda", torch.cuda.current_device())
    errors = []

    def call(user, level, frame, mm, nn, kk, J, W, u, v, ax, ay, hx, hy, du, dv):
        try:
            Jh = _device_f64(J, (6, kk, mm, nn)).cpu().numpy()
            Wh = _device_f64(W, (kk, mm, nn)).cpu().numpy()
            uh = _device_f64(u, (mm, nn)).cpu().numpy()
            vh = _device_f64(v, (mm, nn)).cpu().numpy()
            planes = [np.ascontiguousarray(Jh[q].transpose(1, 2, 0)) for q in range(6)]
            d_u, d_v = solver(*planes, np.ascontiguousarray(Wh.transpose(1, 2, 0)), uh, vh, [ax, ay], iterations,
                              update_lag, 0, a_data.copy(), a_smooth, hx, hy, None)
            for ptr, arr in ((du, d_u), (dv, d_v)):
                a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64))
                if a.shape != (mm, nn):
                    raise ValueError(f"the level solver returned shape {a.shape}, expected {(mm, nn)}")
                _device_f64(ptr, (mm, nn)).copy_(torch.from_numpy(a))
            torch.cuda.synchronize()
            return 0
        except BaseException as e:  # reported after the call returns
            errors.append(e)
            return 1

    fn = _lib.LEVEL_SOLVER_FN(call)
    plan = Plan(params, m, n, K, 1)
    try:
        _lib.check(plan.lib.frg_plan_set_level_solver(plan.handle, fn, None), "frg_plan_set_level_solver")
        plan.set_reference(torch.from_numpy(np.ascontiguousarray(fixed, dtype=np.float32)).to(dev),
                           torch.from_numpy(np.ascontiguousarray(weight, dtype=np.float32)).to(dev))
        uv_t = None
        if uv is not None:
            uv_t = torch.from_numpy(np.ascontiguousarray(np.asarray(uv)[:, :, :2], dtype=np.float32)).to(dev)
        try:
            flow = plan.displacement(torch.from_numpy(np.ascontiguousarray(moving, dtype=np.float32)).to(dev), uv_t)
        except _lib.FrgError:
            if errors:
                raise errors[0]
            raise
        torch.cuda.synchronize()
        return flow[0].cpu().numpy().astype(np.float64)
    finally:
        plan.close()


def get_displacement_batch(fixed, moving_frames, alpha=(2, 2), update_lag=5, iterations=50, min_level=0,
                           levels=50, eta=0.8, a_smooth=1.0, a_data=0.45, const_assumption="gc", uv=None,
                           weight=None, gnc_schedule=None, warping_steps=None, max_frames=None, precision="fp64"):
    """Many moving frames (T, H, W[, K]) against one fixed frame in one device
    pass; returns (T, H, W, 2) float64 for precision="fp64" (default), float32
    for "fp32"."""
    moving_frames = np.asarray(moving_frames)
    fixed, _, w, params, m, n, K = _prepare(fixed, moving_frames[0], weight, a_data, alpha, update_lag,
                                            iterations, min_level, levels, eta, a_smooth, const_assumption,
                                            gnc_schedule, warping_steps, None, precision)
    T = moving_frames.shape[0]
    return _run_host(params, fixed.reshape(m, n, K), moving_frames.reshape(T, m, n, K), w, uv, max_frames)


class _HostIO:
    """Per-lane staging of the host-buffer calls, kept with the plan (pinning
    memory is slow, so it is done once): device input and output slots of a
    lane's frames, their pinned host copies, and the copy streams."""

    def __init__(self, H, W, K, frames, fp64, dev):
        odt = torch.float64 if fp64 else torch.float32
        self.frames = frames
        self.dev_in = torch.empty((frames, H, W, K), dtype=torch.float32, device=dev)
        self.dev_out = torch.empty((frames, H, W, 2), dtype=odt, device=dev)
        self.pin_in = torch.empty((frames, H, W, K), dtype=torch.float32).pin_memory()
        self.pin_out = torch.empty((frames, H, W, 2), dtype=odt).pin_memory()
        self.up_done = None  # event: pin_in consumed by the upload


def _host_io(plan, key, H, W, K, frames, fp64, dev):
    cache = plan.__dict__.setdefault("_host_io", {})
    io = cache.get(key)
    if io is None or io.frames < frames:
        io = cache[key] = _HostIO(H, W, K, frames, fp64, dev)
    return io


_copy_pool = None
_copy_pool_lock = threading.Lock()


def _host_copy(dst: np.ndarray, src) -> None:
    """dst[...] = src for large frame stacks, split over host threads along the
    first axis (numpy releases the GIL while it copies), so pinned staging
    keeps up with the transfers.  src = None writes zeros: it touches fresh
    pages of dst ahead of a later copy."""
    global _copy_pool
    n = dst.shape[0]
    if n < 8 or dst.nbytes < (64 << 20):
        dst[...] = 0 if src is None else src
        return
    with _copy_pool_lock:
        if _copy_pool is None:
            from concurrent.futures import ThreadPoolExecutor

            _copy_pool = ThreadPoolExecutor(max_workers=max(1, min(8, (os.cpu_count() or 1))))
        pool = _copy_pool
    parts = min(pool._max_workers, n)
    step = -(-n // parts)

    def part(i):
        a, b = i * step, min(n, (i + 1) * step)
        if a < b:
            dst[a:b] = 0 if src is None else src[a:b]

    for f in [pool.submit(part, i) for i in range(parts)]:
        f.result()


def _run_host(params, fixed, moving, weight, uv, max_frames=None):
    """Host arrays in, host array out.  The batch goes to the plan's lanes in
    contiguous parts; each part is copied into pinned memory, uploaded on a
    copy stream and registered on its lane's stream, so the host copies and
    transfers of one part overlap the device work of the others.  A part whose
    lane takes another part is read back through pinned memory before the lane
    moves on; the last part of every lane is read back straight into the output
    array, which is page-locked for the copies while the lanes compute."""
    _require_cuda()
    T, m, n, K = moving.shape
    dev = torch.device("cuda", torch.cuda.current_device())
    plan = get_plan(params, m, n, K, T, max_frames)
    fixed32 = np.ascontiguousarray(fixed, dtype=np.float32)
    w32 = np.ascontiguousarray(weight, dtype=np.float32)
    key = (fixed32.tobytes().__hash__(), w32.tobytes().__hash__())
    fixed_t = torch.from_numpy(fixed32).to(dev)
    w_t = torch.from_numpy(w32).to(dev)
    plan.set_reference(fixed_t, w_t, key=key)
    uv_t = None
    if uv is not None:
        uv_t = torch.from_numpy(np.ascontiguousarray(np.asarray(uv)[:, :, :2], dtype=np.float32)).to(dev)
    lanes = list(getattr(plan, "plans", [plan]))
    streams = list(getattr(plan, "streams", [torch.cuda.current_stream()]))
    per = -(-T // len(lanes))
    if len(lanes) > 1:
        per = min(per, plan.lane_frames)
    else:
        per = min(T, plan.max_frames)
    parts = [(t0, min(T, t0 + per)) for t0 in range(0, T, per)]
    cache_owner = plan
    st_up = cache_owner.__dict__.get("_st_up")
    if st_up is None:
        st_up = cache_owner.__dict__["_st_up"] = torch.cuda.Stream(device=dev)
        cache_owner.__dict__["_st_down"] = torch.cuda.Stream(device=dev)
    st_down = cache_owner.__dict__["_st_down"]
    main = torch.cuda.current_stream()
    st_up.wait_stream(main)  # the reference and uv uploads above precede the lanes' work
    out = np.empty((T, m, n, 2), np.float64 if plan.fp64 else np.float32)
    pending = {}  # lane -> (io, t0, t1) awaiting its copy into `out`
    mov = np.asarray(moving)

    def drain(li):
        io, a, b, done = pending.pop(li)
        with torch.cuda.stream(st_down):
            st_down.wait_event(done)
            io.pin_out[:b - a].copy_(io.dev_out[:b - a], non_blocking=True)
        st_down.synchronize()
        _host_copy(out[a:b], io.pin_out[:b - a].numpy())

    for pi, (t0, t1) in enumerate(parts):
        li = pi % len(lanes)
        if li in pending:
            drain(li)
        io = _host_io(plan, li, m, n, K, t1 - t0, plan.fp64, dev)
        if io.up_done is not None:
            io.up_done.synchronize()
        k = t1 - t0
        _host_copy(io.pin_in[:k].numpy(), mov[t0:t1])
        ls = streams[li]
        with torch.cuda.stream(st_up):
            io.dev_in[:k].copy_(io.pin_in[:k], non_blocking=True)
            io.up_done = torch.cuda.Event()
            io.up_done.record(st_up)
        ls.wait_event(io.up_done)
        ls.wait_stream(main)
        lanes[li].displacement(io.dev_in[:k], uv_t, io.dev_out[:k], stream=ls)
        done = torch.cuda.Event()
        done.record(ls)
        pending[li] = (io, t0, t1, done)
    # the lanes' last parts: while they compute, the output rows they fill are first touched
    # (page faults) and page-locked, so each is read back by one device-to-host copy
    a0 = min(a for _, a, _, _ in pending.values())
    tail = out[a0:]
    _host_copy(tail, None)
    locked = _page_lock(tail)
    try:
        with torch.cuda.stream(st_down):
            for io, a, b, done in pending.values():
                st_down.wait_event(done)
                if locked:
                    torch.from_numpy(out[a:b]).copy_(io.dev_out[:b - a], non_blocking=True)
                else:
                    io.pin_out[:b - a].copy_(io.dev_out[:b - a], non_blocking=True)
        st_down.synchronize()
        if not locked:
            for io, a, b, _ in pending.values():
                _host_copy(out[a:b], io.pin_out[:b - a].numpy())
    finally:
        if locked:
            _lib.check(_lib.load().frg_host_unregister(ctypes.c_void_p(tail.ctypes.data)), "frg_host_unregister")
    pending.clear()
    return out


def _page_lock(arr: np.ndarray) -> bool:
    """Page-locks a host array of at least 64 MiB for asynchronous
    device-to-host copies; False for a smaller array or when the runtime
    refuses (the caller then copies through its pinned buffers)."""
    if arr.nbytes < (64 << 20):
        return False
    return _lib.load().frg_host_register(ctypes.c_void_p(arr.ctypes.data), arr.nbytes) == 0


def get_displacement_device(fixed_t, moving_t, uv_t=None, weight_t=None, out_t=None, stream=None,
                            max_frames=None, **options):
    """Device-resident form: fixed_t (H, W, K), moving_t (T, H, W, K) and
    optional uv_t (H, W, 2) / weight_t (H, W, K) are float32 CUDA tensors;
    returns flow (T, H, W, 2) on the device, float64 for precision="fp64"
    (default) and float32 for "fp32", enqueued on `stream`."""
    _require_cuda()
    T, H, W, K = moving_t.shape
    options.setdefault("precision", "fp64")
    params = make_params(K=K, **options)
    plan = get_plan(params, H, W, K, T, max_frames)
    key = ("device", fixed_t.data_ptr(), fixed_t._version,
           None if weight_t is None else (weight_t.data_ptr(), weight_t._version))
    plan.set_reference(fixed_t, weight_t, stream=stream, key=key)
    return plan.displacement(moving_t, uv_t, out_t, stream=stream)


# --------------------------------------------------------------------------
# imregister_wrapper (core/warping.py:160-234)
# --------------------------------------------------------------------------
def imregister_device(frames_t, flow_t, reference_t, interpolation_method="cubic", out_t=None, stream=None):
    """frames_t (T, H, W, K), flow_t (T, H, W, 2), reference_t (H, W, K): float32 CUDA."""
    _require_cuda()
    method = str(interpolation_method).lower()
    if method not in ("cubic", "linear"):
        raise ValueError("Unsupported interpolation method. Use 'linear' or 'cubic'.")
    T, H, W, K = frames_t.shape
    for t, shp in ((frames_t, (T, H, W, K)), (flow_t, (T, H, W, 2)), (reference_t, (H, W, K))):
        Plan._check(t, shp)
    if out_t is None:
        out_t = torch.empty_like(frames_t)
    lib = _lib.load()
    _lib.check(lib.frg_imregister(T, H, W, K, _ptr(frames_t), _ptr(flow_t), _ptr(reference_t),
                                  1 if method == "cubic" else 0, _ptr(out_t), _stream_ptr(stream)),
               "frg_imregister")
    return out_t


def imregister_wrapper(f2_level, u, v, f1_level, interpolation_method="cubic"):
    """Drop-in for pyflowreg.core.warping.imregister_wrapper (float32 result,
    channel axis squeezed when single-channel, like the reference)."""
    _require_cuda()
    f2 = np.asarray(f2_level)
    f1 = np.asarray(f1_level)
    if f2.ndim == 2:
        f2 = f2[:, :, None]
        f1 = f1[:, :, None]
    H, W, C = f2.shape
    dev = torch.device("cuda", torch.cuda.current_device())
    fr = torch.from_numpy(np.ascontiguousarray(f2, dtype=np.float32)[None]).to(dev)
    ref = torch.from_numpy(np.ascontiguousarray(f1, dtype=np.float32)).to(dev)
    fl = torch.from_numpy(np.ascontiguousarray(np.stack([u, v], axis=-1), dtype=np.float32)[None]).to(dev)
    out = imregister_device(fr, fl, ref, interpolation_method)[0].cpu().numpy()
    return out[:, :, 0] if out.shape[2] == 1 else out


# --------------------------------------------------------------------------
# level_solver seam (core/optical_flow.py:348-411)
# --------------------------------------------------------------------------
def level_solver(J11, J22, J33, J12, J13, J23, weight, u, v, alpha, iterations, update_lag, verbose, a_data,
                 a_smooth, hx, hy, gnc_beta=None, precision="fp64"):
    """GPU level solver with the signature of ``level_solver_backend``
    (core/optical_flow.py:348-411).

    Runs compute_flow's exact update order on the device and returns (du, dv)
    as float64 (m, n) arrays.  precision "fp64" (default; taken as well
    whenever a_smooth != 1 or gnc_beta is given) computes in the reference's
    float64 arithmetic, compute_flow_gnc when gnc_beta is not None; "fp32" is
    the float32 solver (a_smooth = 1, no GNC).
    """
    _require_cuda()
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
    if precision == "fp64" or gnc_beta is not None or float(a_smooth) != 1.0:
        return _level_solver_f64(J11, J22, J33, J12, J13, J23, weight, u, v, alpha, iterations, update_lag,
                                 a_data, a_smooth, hx, hy, gnc_beta)
    J = np.stack([np.asarray(a, dtype=np.float32) for a in (J11, J22, J33, J12, J13, J23)])
    if J.ndim == 3:
        J = J[..., None]
    _, m, n, K = J.shape
    wgt = np.asarray(weight, dtype=np.float32)
    if wgt.ndim == 2:
        wgt = wgt[..., None]
    wgt = np.array(np.broadcast_to(wgt, (m, n, K)), order="C")
    ad = np.ascontiguousarray(normalize_a_data(a_data, K))
    dev = torch.device("cuda", torch.cuda.current_device())
    Jt = torch.from_numpy(np.ascontiguousarray(J)).to(dev)
    Wt = torch.from_numpy(wgt).to(dev)
    ut = torch.from_numpy(np.ascontiguousarray(u, dtype=np.float32)).to(dev)
    vt = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float32)).to(dev)
    du = torch.empty((m, n), dtype=torch.float32, device=dev)
    dv = torch.empty((m, n), dtype=torch.float32, device=dev)
    ax, ay = alpha_pair(alpha)
    lib = _lib.load()
    _lib.check(lib.frg_level_solve(m, n, K, _ptr(Jt), _ptr(Wt), _ptr(ut), _ptr(vt), ax, ay, int(iterations),
                                   int(update_lag), ad.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   float(a_smooth), float(hx), float(hy), 1.95, _ptr(du), _ptr(dv),
                                   _stream_ptr()), "frg_level_solve")
    torch.cuda.current_stream().synchronize()
    return du.cpu().numpy().astype(np.float64), dv.cpu().numpy().astype(np.float64)


def _level_solver_f64(J11, J22, J33, J12, J13, J23, weight, u, v, alpha, iterations, update_lag, a_data,
                     a_smooth, hx, hy, gnc_beta):
    J = np.stack([np.asarray(a, dtype=np.float64) for a in (J11, J22, J33, J12, J13, J23)])
    if J.ndim == 3:
        J = J[..., None]
    _, m, n, K = J.shape
    wgt = np.asarray(weight, dtype=np.float64)
    if wgt.ndim == 2:
        wgt = wgt[..., None]
    wgt = np.array(np.broadcast_to(wgt, (m, n, K)), order="C")
    ad = np.ascontiguousarray(normalize_a_data(a_data, K))
    dev = torch.device("cuda", torch.cuda.current_device())
    Jt = torch.from_numpy(np.ascontiguousarray(J)).to(dev)
    Wt = torch.from_numpy(wgt).to(dev)
    ut = torch.from_numpy(np.ascontiguousarray(u, dtype=np.float64)).to(dev)
    vt = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).to(dev)
    du = torch.empty((m, n), dtype=torch.float64, device=dev)
    dv = torch.empty((m, n), dtype=torch.float64, device=dev)
    ax, ay = alpha_pair(alpha)
    beta = -1.0 if gnc_beta is None else float(gnc_beta)
    if not (beta < 0.0 or 0.0 <= beta <= 1.0):
        raise ValueError("gnc_beta must lie in [0, 1]")
    lib = _lib.load()
    _lib.check(lib.frg_level_solve_f64(m, n, K, _ptr(Jt), _ptr(Wt), _ptr(ut), _ptr(vt), ax, ay, int(iterations),
                                       int(update_lag), ad.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       float(a_smooth), float(hx), float(hy), 1.95, beta, _ptr(du), _ptr(dv),
                                       _stream_ptr()), "frg_level_solve_f64")
    torch.cuda.current_stream().synchronize()
    return du.cpu().numpy(), dv.cpu().numpy()


# --------------------------------------------------------------------------
# Building blocks with the reference's signatures
# --------------------------------------------------------------------------
def imresize_fused_gauss_cubic(img, size, sigma_coeff=0.6, per_axis=False):
    """Drop-in for util/resize_util.py:232-254 (sigma_coeff 0.6, per_axis False)."""
    _require_cuda()
    if sigma_coeff != 0.6 or per_axis:
        raise NotImplementedError("only sigma_coeff=0.6, per_axis=False are implemented")
    x = np.asarray(img)
    oh, ow = int(size[0]), int(size[1])
    planes = x[None] if x.ndim == 2 else np.moveaxis(x, 2, 0)
    dev = torch.device("cuda", torch.cuda.current_device())
    src = torch.from_numpy(np.ascontiguousarray(planes, dtype=np.float32)).to(dev)
    dst = torch.empty((planes.shape[0], oh, ow), dtype=torch.float32, device=dev)
    lib = _lib.load()
    _lib.check(lib.frg_resize(planes.shape[0], planes.shape[1], planes.shape[2], _ptr(src), oh, ow, _ptr(dst),
                              _stream_ptr()), "frg_resize")
    y = dst.cpu().numpy()
    y = y[0] if x.ndim == 2 else np.moveaxis(y, 0, 2)
    return y.astype(x.dtype, copy=False)


def _tensor(f1, f2, hy, hx, gray):
    _require_cuda()
    f1 = np.asarray(f1, dtype=np.float32)
    f2 = np.asarray(f2, dtype=np.float32)
    h, w = f1.shape
    dev = torch.device("cuda", torch.cuda.current_device())
    a = torch.from_numpy(np.ascontiguousarray(f1)).to(dev)
    b = torch.from_numpy(np.ascontiguousarray(f2)).to(dev)
    out = torch.empty((6, h + 2, w + 2), dtype=torch.float32, device=dev)
    lib = _lib.load()
    _lib.check(lib.frg_motion_tensor(h, w, _ptr(a), _ptr(b), float(hy), float(hx), int(gray), _ptr(out),
                                     _stream_ptr()), "frg_motion_tensor")
    o = out.cpu().numpy().astype(np.float64)
    return tuple(o[i] for i in range(6))


def get_motion_tensor_gc(f1, f2, hy, hx):
    return _tensor(f1, f2, hy, hx, 0)


def get_motion_tensor_gray(f1, f2, hy, hx):
    return _tensor(f1, f2, hy, hx, 1)


def median_filter5(a):
    """scipy.ndimage.median_filter(a, size=(5, 5), mode='mirror') of a 2-D array."""
    _require_cuda()
    a = np.asarray(a, dtype=np.float32)
    h, w = a.shape
    dev = torch.device("cuda", torch.cuda.current_device())
    src = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    dst = torch.empty_like(src)
    lib = _lib.load()
    _lib.check(lib.frg_median5(h, w, _ptr(src), _ptr(dst), _stream_ptr()), "frg_median5")
    return dst.cpu().numpy()
