"""Preprocessing and post-registration statistics on the device against the
numpy/scipy restatement of compensate_recording's own steps."""
import numpy as np
import pytest
import torch

from oracle import prep_oracle as P

pytestmark = pytest.mark.gpu


def _raw(seed, T, H, W, K, integer=False):
    rng = np.random.default_rng(seed)
    base = rng.gamma(2.0, 300.0, (T, H, W, K))
    if integer:
        return np.round(base).astype(np.uint16)
    return base.astype(np.float32)


@pytest.mark.parametrize("integer,norm,sigma", [
    (False, "together", ((1.0, 1.0, 0.1),)),
    (False, "separate", ((1.0, 1.5, 0.1), (2.0, 1.0, 0.1))),
    (True, "together", ((1.0, 1.0, 0.1),)),
    (False, "together", ((1.2, 0.8, 0.8),)),  # temporal radius 3: frames of the batch mix
])
def test_batch_preprocessing_bit_exact(integer, norm, sigma):
    from pyflowreg_gb300.prep import preprocess_device

    T, H, W, K = 6, 37, 53, 2
    raw = _raw(1, T, H, W, K, integer)
    ref = raw[:4].mean(0)  # float32 mean for float32 frames, float64 for uint16
    sig = np.asarray(sigma, dtype=np.float64)
    if sig.shape[0] == 1:
        sig = sig[0]
    want = P.preprocess(raw, ref, sig, norm).astype(np.float32)
    got = preprocess_device(torch.tensor(raw.astype(np.float32), device="cuda"), ref, sig, norm,
                            frames_dtype=raw.dtype).cpu().numpy()
    assert np.array_equal(got, want), np.abs(got.astype(np.float64) - want).max()


def test_reference_preprocessing_bit_exact():
    from pyflowreg_gb300.prep import preprocess_device

    raw = _raw(2, 8, 41, 29, 2)
    ref = raw.mean(0)
    want = P.preprocess(ref, None, np.array([1.0, 1.0, 0.1])).astype(np.float32)
    got = preprocess_device(torch.tensor(ref, device="cuda"), ref, (1.0, 1.0, 0.1), frames_dtype=ref.dtype)
    assert np.array_equal(got.cpu().numpy(), want)


def test_flow_statistics_and_valid_masks():
    from pyflowreg_gb300.prep import flow_statistics_device

    rng = np.random.default_rng(3)
    w = (rng.standard_normal((5, 33, 47, 2)) * 4).astype(np.float32)
    w[1] += 30.0  # mostly out of bounds
    valid, stats = flow_statistics_device(torch.tensor(w, device="cuda"))
    np.testing.assert_array_equal(valid.cpu().numpy(), P.valid_masks(w))
    np.testing.assert_allclose(stats.cpu().numpy(), P.statistics(w.astype(np.float64)), rtol=1e-9, atol=1e-9)
