"""Uneven batches (frames of several sizes in one call, optionally replayed as
CUDA graphs) and streaming registration with overlapped copies: both must give
exactly the flows of direct per-group calls."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

OPTS = dict(alpha=(1.5, 1.5), levels=100, eta=0.8, iterations=20, update_lag=5, a_data=0.45)


def _frames(key, n, seed):
    from pyflowreg_gb300.synthetic import TorchVideo, preprocess_torch

    H, W, K = key
    vid = TorchVideo(seed=seed, h=H, w=W, K=K, n_blobs=12, device="cuda")
    raw = vid.frames(0, n + 4)
    ref_raw = raw[:4].mean(0)
    return preprocess_torch(ref_raw, ref_raw).contiguous(), preprocess_torch(raw[4:], ref_raw).contiguous()


@pytest.mark.parametrize("graphs,precision", [(False, "fp32"), (True, "fp32"), (True, "fp64")])
def test_uneven_batch_equals_per_group_calls(graphs, precision):
    from pyflowreg_gb300 import api
    from pyflowreg_gb300.batch import UnevenBatch

    shapes = [(64, 64, 1), (80, 96, 2), (128, 112, 1), (72, 48, 2)]
    counts = [5, 3, 4, 2]
    refs, frames, keys = {}, [], []
    for i, (key, n) in enumerate(zip(shapes, counts)):
        ref, fr = _frames(key, n, 10 + i)
        refs[key] = ref
        frames += [fr[j] for j in range(n)]
        keys += [key] * n
    order = np.random.default_rng(0).permutation(len(frames))
    frames = [frames[i] for i in order]
    keys = [keys[i] for i in order]
    ub = UnevenBatch(refs, graphs=graphs, precision=precision, **OPTS)
    for _ in range(2):  # the second call replays the captured graphs
        got = ub.register(frames)
    torch.cuda.synchronize()
    for key in shapes:
        idx = [i for i, k in enumerate(keys) if k == key]
        plan = api.Plan(api.make_params(K=key[2], precision=precision, **OPTS), *key, len(idx))
        plan.set_reference(refs[key])
        ref = plan.displacement(torch.stack([frames[i] for i in idx]))
        torch.cuda.synchronize()
        for j, i in enumerate(idx):
            assert torch.equal(got[i], ref[j]), key
        plan.close()
    ub.close()


def test_stream_registrar_equals_batch_loop():
    from pyflowreg_gb300 import api
    from pyflowreg_gb300.stream import StreamRegistrar

    key = (96, 80, 2)
    ref, fr = _frames(key, 45, 3)
    host = fr.cpu().numpy()
    out = np.zeros((45, key[0], key[1], 2), np.float32)

    def sink(t0, flows):
        out[t0:t0 + len(flows)] = flows

    sr = StreamRegistrar(ref, batch=16, **OPTS)
    info = sr.run(lambda t0, n: host[t0:t0 + n], 45, sink)
    sr.close()
    assert info["frames"] == 45
    plan = api.Plan(api.make_params(K=2, **OPTS), *key, 16)
    plan.set_reference(ref)
    w = torch.zeros((key[0], key[1], 2), dtype=torch.float32, device="cuda")
    for t0 in range(0, 45, 16):
        n = min(16, 45 - t0)
        f = plan.displacement(fr[t0:t0 + n].contiguous(), w)
        np.testing.assert_array_equal(out[t0:t0 + n], f.cpu().numpy())
        w = f[max(0, n - 20):n].mean(0).contiguous()
    plan.close()


def test_autotuned_plan_gives_identical_flows():
    """The launch-shape tuning (iterations per wavefront pass, threads per CTA)
    changes no result bit."""
    from pyflowreg_gb300 import api

    key = (200, 168, 2)
    ref, fr = _frames(key, 6, 5)
    plan = api.Plan(api.make_params(K=2, **OPTS), *key, 6)
    plan.set_reference(ref)
    base = plan.displacement(fr).clone()
    chosen = plan.autotune(fr, n_levels=3, reps=1)
    assert chosen
    tuned = plan.displacement(fr)
    assert torch.equal(base, tuned)
    for i, (v, g, t, ms) in chosen.items():
        plan.set_level_variant(i, 0)
        plan.set_level_tuning(i, max(1, g - 1), 1024)
    assert torch.equal(base, plan.displacement(fr))
    plan.close()


@pytest.mark.parametrize("key,frames", [((200, 168, 2), 3), ((96, 130, 1), 2), ((150, 90, 3), 2),
                                        ((70, 64, 4), 2), ((600, 96, 2), 2), ((900, 60, 1), 2)])
def test_sor_variants_give_identical_flows(key, frames):
    """The rows-in-registers SOR (one CTA, or a cluster of row strips above 512
    rows; one launch per pass, or every pass of a level chained in one launch)
    and the diagonal-ring SOR give the same bits on every level they serve,
    for every pass length (G = 3 splits the windows between psi ticks, so
    passes that store and read back the folded coefficients are chained too)."""
    from pyflowreg_gb300 import api

    ref, fr = _frames(key, frames, 7)
    plan = api.Plan(api.make_params(K=key[2], **OPTS), *key, frames)
    plan.set_reference(ref)
    tun = plan.level_tuning()
    both = [i for i in range(len(tun)) if tun[i][2] > 0 and plan.level_variant(i)[1] > 1]
    assert both
    for i in both:
        plan.set_level_variant(i, 0)
    base = plan.displacement(fr).clone()
    for var in (1, 2):
        for G in (5, 3, 1):
            served = [i for i in both if plan.level_variant(i)[1] > var]
            for i in served:
                plan.set_level_variant(i, var)
                plan.set_level_tuning(i, min(G, tun[i][2]), 0)
            assert torch.equal(base, plan.displacement(fr)), (var, G)
    assert all(plan.level_variant(i)[1] == 3 for i in both)
    plan.close()


@pytest.mark.parametrize("key", [(1100, 72, 1), (1060, 40, 2), (640, 200, 2)])
def test_cluster_sor_on_tall_levels_matches_the_other_kernels(oracle, key):
    """Levels over 512 rows run as clusters of row strips (all passes chained in
    one launch).  Over 1024 rows the alternative is the global-memory wavefront
    with a separate fold, whose rounding differs: the two stay within float32
    rounding of each other, and the cluster result within the fp32 bound of the
    fp64 oracle."""
    from pyflowreg_gb300 import api

    ref, fr = _frames(key, 1, 9)
    opts = dict(OPTS, iterations=10)
    plan = api.Plan(api.make_params(K=key[2], **opts), *key, 1)
    plan.set_reference(ref)
    tall = [i for i in range(len(plan.level_tuning())) if plan.level_tuning()[i][3] > 512]
    assert tall and all(plan.level_variant(i) == (2, 3) for i in tall)
    got = plan.displacement(fr).cpu().numpy()
    for i in tall:
        plan.set_level_variant(i, 0)
    other = plan.displacement(fr).cpu().numpy()
    plan.close()
    # the reference amplifies rounding (a 1e-7 input change moves its flow by ~0.1 px at
    # single pixels), so the comparisons are on the mean, and the fp32 result is held to
    # the accuracy of the kernel it replaces
    assert np.abs(got - other).mean() < 0.01, np.abs(got - other).mean()
    want = oracle.get_displacement(ref.cpu().numpy(), fr[0].cpu().numpy(), **opts)
    e_got, e_other = np.abs(got[0] - want).mean(), np.abs(other[0] - want).mean()
    assert e_got <= 1.25 * e_other + 1e-3, (e_got, e_other)


@pytest.mark.parametrize("T", [130, 261])
def test_lane_plan_equals_one_plan(T):
    """Large batches run as lanes (plans over contiguous frame ranges on their
    own streams): the flows are exactly those of one plan, also for a batch
    that the lanes do not divide evenly and for a call smaller than a lane."""
    from pyflowreg_gb300 import api

    key = (48, 56, 2)
    ref, fr = _frames(key, T, 11)
    params = api.make_params(K=2, **OPTS)
    one = api.Plan(params, *key, T)
    one.set_reference(ref)
    want = one.displacement(fr).clone()
    one.close()
    lanes = api.LanePlan(params, *key, T, api.lanes_for(T))
    assert len(lanes.plans) == (4 if T >= 256 else 2)
    lanes.set_reference(ref)
    assert torch.equal(lanes.displacement(fr), want)
    assert torch.equal(lanes.displacement(fr[:7]), want[:7])
    lanes.close()


def test_host_batch_read_back_paths_equal_device_call():
    """The host-array batch call reads a part back through pinned memory when its
    lane takes another part, and the lanes' last parts (over 64 MiB here)
    straight into the page-locked output array: both give the flows of the
    device-resident call."""
    import pyflowreg_gb300 as G
    from pyflowreg_gb300 import api

    key = (256, 256, 2)
    ref, fr = _frames(key, 300, 21)
    wt = np.full(key, 0.5)
    want = G.get_displacement_device(ref, fr, None, torch.full(key, 0.5, device="cuda"), **OPTS).cpu().numpy()
    api.clear_plans()
    # a 128-frame plan runs two lanes of 64 frames: parts 0-2 are read back while
    # their lane moves on, parts 3 and 4 (frames 192-299) into the locked output
    got = G.get_displacement_batch(ref.cpu().numpy(), fr.cpu().numpy(), weight=wt, max_frames=128, **OPTS)
    assert got.dtype == np.float64 and got[192:].nbytes >= 64 << 20
    np.testing.assert_array_equal(got, want)
    api.clear_plans()
