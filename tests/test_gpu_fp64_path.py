"""The float64 path's launch choices do not change its results: every strip
height of the float64 chained SOR (256, 128 or 64 rows per CTA, levels over
the strip height as clusters of strips, up to 16 CTAs for levels over 1024
rows in 128-row strips) gives the same bits, and the plan's automatic choice
agrees with each explicit one."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

OPTS = dict(alpha=(1.5, 1.5), levels=100, eta=0.8, iterations=20, update_lag=5, a_data=0.45, precision="fp64")


def _frames(H, W, K, n, seed):
    from pyflowreg_gb300.synthetic import TorchVideo, preprocess_torch

    vid = TorchVideo(seed=seed, h=H, w=W, K=K, n_blobs=12, device="cuda")
    raw = vid.frames(0, n + 4)
    ref_raw = raw[:4].mean(0)
    return preprocess_torch(ref_raw, ref_raw).contiguous(), preprocess_torch(raw[4:], ref_raw).contiguous()


@pytest.mark.parametrize("H,W,K", [(300, 96, 2), (160, 144, 1), (1100, 48, 1), (1700, 40, 2)])
def test_strip_heights_give_identical_flows(H, W, K):
    from pyflowreg_gb300 import api

    ref, fr = _frames(H, W, K, 3, 31)
    plan = api.Plan(api.make_params(K=K, **OPTS), H, W, K, 3)
    plan.set_reference(ref)
    base = plan.displacement(fr).clone()
    torch.cuda.synchronize()
    n = len(plan.level_tuning())
    tried = 0
    for rows in (256, 128, 64):
        ok = []
        for i in range(n):
            try:
                plan.set_level_tuning(i, 0, rows)
                ok.append(i)
            except ValueError:
                plan.set_level_tuning(i, 0, 0)
        got = plan.displacement(fr)
        torch.cuda.synchronize()
        assert torch.equal(got, base), rows
        tried += len(ok)
    assert tried > n
    with pytest.raises(ValueError):
        plan.set_level_tuning(n - 1, 1, 0)
    plan.close()
