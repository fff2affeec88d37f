"""Seeded synthetic workloads for benchmarking and tests.

No public data set ships with this project, so frames are rendered from
closed-form images with a known displacement field:

* ``blob_image``: isotropic Gaussian blobs (centres uniform in the frame,
  sigma U[2, 6] px, amplitude U[0.3, 1]) on a background of 0.05.
* ``sinusoid_field``: a sum of random plane-wave sinusoids per component
  (wavelength U[64, 256] px, random direction and phase) scaled to a
  maximum magnitude.
* Moving frames are rendered analytically: ``moving(x + w(x)) = fixed(x)``,
  i.e. each output pixel ``y`` evaluates the blobs at ``x`` solving
  ``x = y - w(x)`` by fixed-point iteration (it contracts because
  ``|grad w| < 1`` for these fields).  There is no interpolation error in the
  ground truth.  This matches the convention of ``imregister_wrapper``:
  ``warped(x) = moving(x + w(x))``.

``pair_256`` is the single-pair 256x256x1 workload; ``video_512x2`` produces
frames of the 512x512x2 photon-count video (Poisson counts with a per-frame
mean in [50, 2000], rigid shift N(0, 3) px plus a drifting sinusoid field).
"""

from __future__ import annotations

import numpy as np


class Blobs:
    def __init__(self, rng: np.random.Generator, h: int, w: int, n: int = 40, bg: float = 0.05):
        self.cy = rng.uniform(0, h, n)
        self.cx = rng.uniform(0, w, n)
        self.s = rng.uniform(2.0, 6.0, n)
        self.a = rng.uniform(0.3, 1.0, n)
        self.bg = bg

    def __call__(self, yy: np.ndarray, xx: np.ndarray) -> np.ndarray:
        out = np.full(yy.shape, self.bg, dtype=np.float64)
        for cy, cx, s, a in zip(self.cy, self.cx, self.s, self.a):
            out += a * np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2.0 * s * s))
        return out


class SinusoidField:
    def __init__(self, rng: np.random.Generator, amp: float, n: int = 4):
        self.k = []
        for _ in range(2):
            lam = rng.uniform(64.0, 256.0, n)
            th = rng.uniform(0.0, 2.0 * np.pi, n)
            ph = rng.uniform(0.0, 2.0 * np.pi, n)
            self.k.append((2 * np.pi / lam * np.cos(th), 2 * np.pi / lam * np.sin(th), ph))
        self.amp = amp
        self.scale = None

    def raw(self, yy, xx, phase_shift=0.0):
        comps = []
        for ky, kx, ph in self.k:
            c = np.zeros(np.broadcast(yy, xx).shape)
            for a, b, p in zip(ky, kx, ph):
                c += np.sin(a * yy + b * xx + p + phase_shift)
            comps.append(c)
        return comps

    def calibrate(self, h, w):
        yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
        u, v = self.raw(yy, xx)
        self.scale = self.amp / max(np.sqrt(u * u + v * v).max(), 1e-12)

    def __call__(self, yy, xx, phase_shift=0.0):
        u, v = self.raw(yy, xx, phase_shift)
        return u * self.scale, v * self.scale


def render_moving(img_fn, field_fn, h, w, shift=(0.0, 0.0), iters=30):
    """moving(y) = img(x) with y = x + w(x) + shift; returns (moving, u, v at x grid)."""
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    px, py = xx.copy(), yy.copy()
    for _ in range(iters):
        u, v = field_fn(py, px)
        px = xx - u - shift[0]
        py = yy - v - shift[1]
    moving = img_fn(py, px)
    u, v = field_fn(yy, xx)
    return moving, u + shift[0], v + shift[1]


def pair_256(seed: int = 0, h: int = 256, w: int = 256, noise: float = 0.02, max_disp: float = 4.0):
    """Single 2-D pair: (fixed (h, w) float32, moving (h, w) float32, truth (h, w, 2))."""
    rng = np.random.default_rng(seed)
    img = Blobs(rng, h, w)
    field = SinusoidField(rng, max_disp)
    field.calibrate(h, w)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    fixed = img(yy, xx) + noise * rng.standard_normal((h, w))
    moving, u, v = render_moving(img, field, h, w)
    moving = moving + noise * rng.standard_normal((h, w))
    return fixed.astype(np.float32), moving.astype(np.float32), np.stack([u, v], axis=2)


class Video:
    """Photon-count video (T, h, w, K) registered against the mean of its first frames."""

    def __init__(self, seed: int = 1, h: int = 512, w: int = 512, K: int = 2, n_blobs: int = 40,
                 sinus_amp: float = 2.0, shift_std: float = 3.0, drift_period: float = 250.0):
        self.rng = np.random.default_rng(seed)
        self.h, self.w, self.K = h, w, K
        self.imgs = [Blobs(self.rng, h, w, n_blobs) for _ in range(K)]
        self.field = SinusoidField(self.rng, sinus_amp)
        self.field.calibrate(h, w)
        self.shift_std = shift_std
        self.period = drift_period
        self.seed = seed

    def frame(self, t: int):
        rng = np.random.default_rng(1000 * self.seed + t)
        shift = rng.normal(0.0, self.shift_std, 2)
        phase = 2.0 * np.pi * t / self.period
        lam = rng.uniform(50.0, 2000.0)

        def fld(yy, xx):
            return self.field(yy, xx, phase)

        out = np.empty((self.h, self.w, self.K), np.float32)
        truth = None
        for k, img in enumerate(self.imgs):
            mov, u, v = render_moving(img, fld, self.h, self.w, shift=tuple(shift))
            norm = mov / 2.0
            out[:, :, k] = rng.poisson(lam * np.clip(norm, 0, None)).astype(np.float32)
            truth = np.stack([u, v], axis=2)
        return out, truth

    def frames(self, t0: int, n: int):
        fr = np.empty((n, self.h, self.w, self.K), np.float32)
        tr = np.empty((n, self.h, self.w, 2), np.float64)
        for i in range(n):
            fr[i], tr[i] = self.frame(t0 + i)
        return fr, tr


# --------------------------------------------------------------------------
# Device-side renderer for large batches (torch; CPU or CUDA)
# --------------------------------------------------------------------------
class TorchVideo:
    """The photon-count video above rendered with torch on `device`.

    Per channel a fixed set of blobs; per frame t a rigid shift N(0, shift_std)
    plus a sinusoid field whose phases drift as 2*pi*t/period, Poisson counts
    with a per-frame mean in [50, 2000].  Seeds are per frame, so any frame can
    be rendered independently and every call is reproducible.
    """

    def __init__(self, seed=1, h=512, w=512, K=2, n_blobs=40, sinus_amp=2.0, shift_std=3.0, period=250.0,
                 device="cpu"):
        import torch

        self.torch = torch
        self.h, self.w, self.K = h, w, K
        self.device = torch.device(device)
        rng = np.random.default_rng(seed)
        self.blobs = []
        for _ in range(K):
            b = Blobs(rng, h, w, n_blobs)
            self.blobs.append([torch.tensor(a, dtype=torch.float32, device=self.device)
                               for a in (b.cy, b.cx, b.s, b.a)])
        self.field = SinusoidField(rng, sinus_amp)
        self.field.calibrate(h, w)
        self.fk = [[torch.tensor(np.asarray(a), dtype=torch.float32, device=self.device) for a in comp]
                   for comp in self.field.k]
        self.shift_std, self.period, self.seed = shift_std, period, seed
        yy, xx = torch.meshgrid(torch.arange(h, dtype=torch.float32, device=self.device),
                                torch.arange(w, dtype=torch.float32, device=self.device), indexing="ij")
        self.yy, self.xx = yy, xx

    def _field(self, yy, xx, phase):
        out = []
        for ky, kx, ph in self.fk:
            arg = ky[:, None, None] * yy[None] + kx[:, None, None] * xx[None] + ph[:, None, None] + phase
            out.append(self.torch.sin(arg).sum(0) * float(self.field.scale))
        return out

    def _blobs(self, k, yy, xx):
        cy, cx, s, a = self.blobs[k]
        out = self.torch.full_like(yy, 0.05)
        for i in range(cy.shape[0]):
            out = out + a[i] * self.torch.exp(-((yy - cy[i]) ** 2 + (xx - cx[i]) ** 2) / (2.0 * s[i] * s[i]))
        return out

    def frame(self, t: int):
        torch = self.torch
        rng = np.random.default_rng(1000 * self.seed + t)
        shift = rng.normal(0.0, self.shift_std, 2)
        lam = float(rng.uniform(50.0, 2000.0))
        phase = 2.0 * np.pi * t / self.period
        px, py = self.xx.clone(), self.yy.clone()
        for _ in range(30):
            u, v = self._field(py, px, phase)
            px = self.xx - u - float(shift[0])
            py = self.yy - v - float(shift[1])
        gen = torch.Generator(device=self.device)
        gen.manual_seed(int(1000 * self.seed + t))
        out = torch.empty((self.h, self.w, self.K), dtype=torch.float32, device=self.device)
        for k in range(self.K):
            img = self._blobs(k, py, px)
            out[:, :, k] = torch.poisson(lam * torch.clamp(img / 2.0, min=0.0), generator=gen)
        return out

    def frames(self, t0: int, n: int):
        out = self.torch.empty((n, self.h, self.w, self.K), dtype=self.torch.float32, device=self.device)
        for i in range(n):
            out[i] = self.frame(t0 + i)
        return out

    def truth(self, t: int):
        """(unwarped noise-free frame (h, w, K) at frame t's mean count, true
        flow (h, w, 2) with moving(x + flow(x)) = unwarped(x))."""
        torch = self.torch
        rng = np.random.default_rng(1000 * self.seed + t)
        shift = rng.normal(0.0, self.shift_std, 2)
        lam = float(rng.uniform(50.0, 2000.0))
        phase = 2.0 * np.pi * t / self.period
        img = torch.stack([lam * torch.clamp(self._blobs(k, self.yy, self.xx) / 2.0, min=0.0) for k in range(self.K)],
                          dim=2)
        u, v = self._field(self.yy, self.xx, phase)
        flow = torch.stack([u + float(shift[0]), v + float(shift[1])], dim=2)
        return img, flow


def preprocess_torch(frames, ref_raw, sigma=1.0, truncate=4.0):
    """Normalise by the raw reference's joint min/max and blur each channel with
    a spatial Gaussian (sigma 1, truncate 4, reflect) -- the input preparation
    compensate_recording applies before get_displacement
    (motion_correction/compensate_recording.py:521-561), used here only to give
    the synthetic workload the value range the flow path sees."""
    import torch
    import torch.nn.functional as F

    lo, hi = float(ref_raw.min()), float(ref_raw.max())
    x = (frames - lo) / max(hi - lo, 1e-12)
    r = int(truncate * sigma + 0.5)
    g = torch.exp(-0.5 * (torch.arange(-r, r + 1, dtype=torch.float32, device=frames.device) / sigma) ** 2)
    g = g / g.sum()
    single = x.ndim == 3
    if single:
        x = x[None]
    T, H, W, K = x.shape
    y = x.permute(0, 3, 1, 2).reshape(T * K, 1, H, W)
    y = F.pad(y, (r, r, 0, 0), mode="reflect")
    y = F.conv2d(y, g.view(1, 1, 1, -1))
    y = F.pad(y, (0, 0, r, r), mode="reflect")
    y = F.conv2d(y, g.view(1, 1, -1, 1))
    y = y.reshape(T, K, H, W).permute(0, 2, 3, 1).contiguous()
    return y[0] if single else y
