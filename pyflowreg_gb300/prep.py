"""Per-frame work around the flow, on the device: input preprocessing and
post-registration statistics.

* ``preprocess_device`` -- CompensateRecording._preprocess_frames
  (motion_correction/compensate_recording.py:521-561): ``normalize`` then
  ``apply_gaussian_filter`` (util/image_processing.py:12-165), for a batch
  (T, H, W, K) spatio-temporally or a single frame (H, W, K) spatially.
* ``flow_statistics_device`` -- the statistics compensate_recording collects
  per batch (compensate_recording.py:808-821) and the valid masks of the
  backward warp (core/warping.py:14-60, compute_batch_valid_masks).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


def gaussian_taps(sigma: float, truncate: float = 4.0) -> np.ndarray:
    """Taps w[0..r] (centre outwards) of scipy.ndimage.gaussian_filter1d:
    radius int(truncate * sigma + 0.5), exp(-0.5 / sigma^2 * x^2) normalised
    in float64; sigma <= 1e-15 (an axis scipy skips) gives [1.0]."""
    sigma = float(sigma)
    if sigma <= 1e-15:
        return np.ones(1)
    radius = int(truncate * sigma + 0.5)
    x = np.arange(-radius, radius + 1)
    phi = np.exp(-0.5 / (sigma * sigma) * x ** 2)
    phi = phi / phi.sum()
    return np.ascontiguousarray(phi[radius:])


def _sigmas(sigma, K):
    s = np.asarray(sigma, dtype=np.float64)
    if s.ndim == 1:
        s = np.broadcast_to(s, (K, s.shape[0]))
    return [s[min(k, len(s) - 1)] for k in range(K)]


def _taps_tensor(per_channel, device):
    """Taps of every channel at stride (largest radius + 1), and the radius per channel."""
    radii = [len(t) - 1 for t in per_channel]
    stride = max(radii) + 1
    buf = np.zeros((len(per_channel), stride))
    for k, t in enumerate(per_channel):
        buf[k, :len(t)] = t
    return torch.tensor(buf.ravel(), dtype=torch.float64, device=device), (ctypes.c_int * len(radii))(*radii)


def normalization(ref, K, channel_normalization="together", frames_dtype=np.float32):
    """(lo, den, float32_storage) as normalize() computes them
    (util/image_processing.py:12-103): the reference's min and max, jointly or
    per channel, den = max - min + 1e-8, in the dtype numpy's promotion gives
    frames - ref.min()."""
    ref = np.asarray(ref)
    res = np.result_type(np.dtype(frames_dtype), ref.dtype)
    f32 = res == np.float32
    if channel_normalization == "separate" and ref.ndim >= 3:
        mins = [ref[..., k].min() for k in range(K)]
        maxs = [ref[..., k].max() for k in range(K)]
    else:
        mins = [ref.min()] * K
        maxs = [ref.max()] * K
    if f32:
        den = [float(np.float32(np.float32(mx) - np.float32(mn)) + np.float32(1e-8)) for mn, mx in zip(mins, maxs)]
        lo = [float(np.float32(mn)) for mn in mins]
    else:
        den = [float(np.float64(mx) - np.float64(mn) + 1e-8) for mn, mx in zip(mins, maxs)]
        lo = [float(mn) for mn in mins]
    return np.asarray(lo), np.asarray(den), bool(f32)


def preprocess_device(frames, ref_raw, sigma=((1.0, 1.0, 0.1),), channel_normalization="together",
                      truncate: float = 4.0, frames_dtype=np.float32, out=None, stream=None):
    """frames: (T, H, W, K) or (H, W, K) float32 CUDA tensor holding the raw
    values (exact for uint16 sources), or float64 (then numpy's arithmetic is
    float64 whatever frames_dtype says); ref_raw: the raw reference (numpy or
    tensor) whose min/max normalise.  sigma: (3,) or (K, 3) as (sy, sx, st).
    frames_dtype: the dtype the frames had in the reference pipeline (it
    decides float32 or float64 arithmetic as numpy would).  Returns float32."""
    single = frames.dim() == 3
    x = frames.unsqueeze(0) if single else frames
    if not (x.is_cuda and x.dtype in (torch.float32, torch.float64)):
        raise ValueError("frames must be a float32 or float64 CUDA tensor")
    if x.dtype == torch.float64:
        frames_dtype = np.float64
    x = x.contiguous()
    T, H, W, K = x.shape
    ref_np = ref_raw.detach().cpu().numpy() if torch.is_tensor(ref_raw) else np.asarray(ref_raw)
    lo, den, f32 = normalization(ref_np, K, channel_normalization, frames_dtype)
    # per-channel normalisation stores into a float64 array (util/image_processing.py:51-78)
    f32_store = f32 and not (channel_normalization == "separate")
    sig = _sigmas(sigma, K)
    # a single frame is filtered spatially only; a batch along time too (sigma order sy, sx, st)
    wt, rt = _taps_tensor([gaussian_taps(0.0 if single else s[2], truncate) for s in sig], x.device)
    wy, ry = _taps_tensor([gaussian_taps(s[0], truncate) for s in sig], x.device)
    wx, rx = _taps_tensor([gaussian_taps(s[1], truncate) for s in sig], x.device)
    tmp = torch.empty((T * K * H * W,), dtype=torch.float32 if f32_store else torch.float64, device=x.device)
    out_t = out if out is not None else torch.empty(x.shape, dtype=torch.float32, device=x.device)
    lib = _lib.load()
    pD = ctypes.POINTER(ctypes.c_double)
    lo_c = (ctypes.c_double * K)(*lo)
    den_c = (ctypes.c_double * K)(*den)
    s = stream if stream is not None else torch.cuda.current_stream()
    pI = ctypes.POINTER(ctypes.c_int)
    common = (ctypes.cast(lo_c, pD), ctypes.cast(den_c, pD), ctypes.c_void_p(wt.data_ptr()), ctypes.cast(rt, pI),
              ctypes.c_void_p(wy.data_ptr()), ctypes.cast(ry, pI), ctypes.c_void_p(wx.data_ptr()),
              ctypes.cast(rx, pI))
    tail = (ctypes.c_void_p(tmp.data_ptr()), ctypes.c_void_p(out_t.data_ptr()), ctypes.c_void_p(s.cuda_stream))
    if x.dtype == torch.float64:
        _lib.check(lib.frg_preprocess_f64(T, H, W, K, ctypes.c_void_p(x.data_ptr()), *common, 0, *tail),
                   "frg_preprocess_f64")
    else:
        _lib.check(lib.frg_preprocess(T, H, W, K, ctypes.c_void_p(x.data_ptr()), *common, 1 if f32 else 0,
                                      1 if f32_store else 0, *tail), "frg_preprocess")
    return out_t[0] if single else out_t


def flow_statistics_device(flow, valid_masks: bool = True, stream=None):
    """flow (T, H, W, 2) float32 CUDA tensor -> (valid (T, H, W) uint8 0/255 or
    None, stats (T, 4) float64 tensor: mean |w|, max |w|, mean divergence,
    |mean w|), the lists compensate_recording keeps as mean_disp, max_disp,
    mean_div and mean_translation."""
    if not (flow.is_cuda and flow.dtype == torch.float32 and flow.dim() == 4 and flow.shape[-1] == 2):
        raise ValueError("flow must be a (T, H, W, 2) float32 CUDA tensor")
    f = flow.contiguous()
    T, H, W, _ = f.shape
    lib = _lib.load()
    ws = torch.empty((int(lib.frg_flow_post_workspace(T, H, W)),), dtype=torch.uint8, device=f.device)
    valid = torch.empty((T, H, W), dtype=torch.uint8, device=f.device) if valid_masks else None
    stats = torch.empty((T, 4), dtype=torch.float64, device=f.device)
    s = stream if stream is not None else torch.cuda.current_stream()
    _lib.check(lib.frg_flow_post(T, H, W, ctypes.c_void_p(f.data_ptr()),
                                 ctypes.c_void_p(valid.data_ptr()) if valid is not None else None,
                                 ctypes.c_void_p(ws.data_ptr()), ctypes.c_void_p(stats.data_ptr()),
                                 ctypes.c_void_p(s.cuda_stream)), "frg_flow_post")
    return valid, stats
