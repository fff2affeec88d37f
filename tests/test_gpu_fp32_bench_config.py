"""The float32 path at the configuration the benchmark runs (512x512x2, the
photon-count video, pyflowreg's default options), on two frame pairs whose
true displacement is known (the noise-free unwarped frame against the Poisson
frame warped by the known field):

* the float32 flow stays within twice the distance between the oracle's
  float32 and float64 level solvers (the reference algorithm computed in
  single precision: the algorithm amplifies float32 rounding to ~0.1 px,
  which bounds how close any float32 implementation can come);
* its end-point error against the true displacement equals the oracle's
  within 5 %: float32 costs no accuracy against the truth;
* the float64 path meets the parity bar on the same pairs.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

OPTS = dict(alpha=(1.5, 1.5), levels=100, eta=0.8, min_level=0, iterations=50, update_lag=5, a_data=0.45,
            a_smooth=1.0, const_assumption="gc")


def _pairs(ts):
    from pyflowreg_gb300.synthetic import TorchVideo, preprocess_torch

    vid = TorchVideo(seed=1, h=512, w=512, K=2, device="cuda")
    fixed, moving, truth = [], [], []
    for t in ts:
        img, flow = vid.truth(t)
        fixed.append(preprocess_torch(img, img))
        moving.append(preprocess_torch(vid.frame(t), img))
        truth.append(flow.cpu().numpy().astype(np.float64))
    return fixed, moving, truth


def _diff(a, b):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return float(np.abs(d).max()), float(np.sqrt((d ** 2).sum(-1)).mean())


def test_fp32_at_bench_config_within_reference_envelope(oracle):
    import pyflowreg_gb300 as G

    fixed, moving, truth = _pairs([50, 51])
    wt = np.full((512, 512, 2), 0.5)
    wt_t = torch.full((512, 512, 2), 0.5, device="cuda")
    for f, m, tr in zip(fixed, moving, truth):
        fx = f.cpu().numpy().astype(np.float64)
        mv = m.cpu().numpy().astype(np.float64)
        base = oracle.get_displacement_batch(fx, mv[None], n_threads=1, weight=wt, **OPTS)[0]
        single = oracle.get_displacement_batch(fx, mv[None], n_threads=1, weight=wt, solver_f32=True, **OPTS)[0]
        env_max, env_epe = _diff(single, base)
        got32 = G.get_displacement_device(f, m[None], None, wt_t, precision="fp32", **OPTS)[0].cpu().numpy()
        got64 = G.get_displacement_device(f, m[None], None, wt_t, **OPTS)[0].cpu().numpy()
        mx, ep = _diff(got32, base)
        assert mx <= 2 * env_max and ep <= 2 * env_epe, (mx, ep, env_max, env_epe)
        e_or = _diff(base, tr)[1]
        e_32 = _diff(got32, tr)[1]
        assert abs(e_32 - e_or) <= 0.05 * e_or, (e_32, e_or)
        mx64, ep64 = _diff(got64, base)
        assert mx64 <= 1e-3 and ep64 <= 1e-4, (mx64, ep64)
