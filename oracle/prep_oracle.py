"""CPU oracle for the per-frame work around the flow -- TEST INFRASTRUCTURE.

Only the tests may import this module, as the checker.  It restates, with
numpy and scipy (the reference's own dependencies), without importing
pyflowreg:
  * normalize                util/image_processing.py:12-103
  * apply_gaussian_filter    util/image_processing.py:106-165
  * the preprocessing order  motion_correction/compensate_recording.py:521-561
  * backward_valid_mask / compute_batch_valid_masks  core/warping.py:14-60, 128-157
  * the per-batch statistics motion_correction/compensate_recording.py:808-821
"""

from __future__ import annotations

import numpy as np
from scipy.ndimage import gaussian_filter


def normalize(arr, ref=None, channel_normalization="together", eps=1e-8):
    if channel_normalization == "separate" and arr.ndim in (3, 4):
        result = np.zeros_like(arr, dtype=np.float64)
        for c in range(arr.shape[-1]):
            src = ref[..., c] if (ref is not None and ref.ndim >= 3) else arr[..., c]
            mn, mx = src.min(), src.max()
            result[..., c] = (arr[..., c] - mn) / (mx - mn + eps)
        return result
    src = ref if ref is not None else arr
    mn, mx = src.min(), src.max()
    return (arr - mn) / (mx - mn + eps)


def apply_gaussian_filter(arr, sigma, mode="reflect", truncate=4.0):
    sigma = np.asarray(sigma)
    if arr.ndim == 3:
        result = np.zeros_like(arr, dtype=np.float64)
        for c in range(arr.shape[2]):
            s = sigma[min(c, len(sigma) - 1), :2] if sigma.ndim == 2 else sigma[:2]
            result[..., c] = gaussian_filter(arr[..., c], sigma=s, mode=mode, truncate=truncate)
        return result
    if arr.ndim == 4:
        result = np.zeros_like(arr, dtype=np.float64)
        for c in range(arr.shape[3]):
            s = sigma[min(c, len(sigma) - 1)] if sigma.ndim == 2 else sigma
            result[..., c] = gaussian_filter(arr[..., c], sigma=(s[2], s[0], s[1]), mode=mode, truncate=truncate)
        return result
    return arr


def preprocess(frames, normalization_ref=None, sigma=((1.0, 1.0, 0.1),), channel_normalization="together"):
    """normalize then filter, as CompensateRecording._preprocess_frames; float64."""
    normalized = normalize(frames, ref=normalization_ref, channel_normalization=channel_normalization)
    return apply_gaussian_filter(normalized, sigma=np.asarray(sigma), mode="reflect", truncate=4.0).astype(np.float64)


def valid_masks(w):
    T, H, W = w.shape[:3]
    gy, gx = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    out = np.empty((T, H, W), np.uint8)
    for t in range(T):
        mx = gx + w[t, ..., 0]
        my = gy + w[t, ..., 1]
        out[t] = (((mx >= 0) & (mx < W) & (my >= 0) & (my < H)).astype(np.uint8) * 255)
    return out


def statistics(w):
    """(T, 4): mean |w|, max |w|, mean divergence, |mean w| per frame."""
    out = []
    mag = np.sqrt(w[..., 0] ** 2 + w[..., 1] ** 2)
    for t in range(w.shape[0]):
        div = np.gradient(w[t, :, :, 0], axis=1) + np.gradient(w[t, :, :, 1], axis=0)
        mu, mv = float(np.mean(w[t, :, :, 0])), float(np.mean(w[t, :, :, 1]))
        out.append((float(np.mean(mag[t])), float(np.max(mag[t])), float(np.mean(div)), float(np.sqrt(mu * mu + mv * mv))))
    return np.asarray(out)
