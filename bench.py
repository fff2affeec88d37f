"""Benchmark of the GB300 optical-flow path on the 512x512x2 photon-count video.

One step = one pass of get_displacement over one batch of frames (default
400, pyflowreg's OFOptions.buffer_size) against the reference frame (mean of
the first 50 frames), with pyflowreg's default flow options (alpha 1.5,
eta 0.8, 50 iterations, update_lag 5, a_data 0.45, gradient constancy,
quality preset -> min_level 0, channel weights 0.5/0.5), in the reference's
float64 precision (the parity path; --precision fp32 times the float32 path).

Prints one JSON line.  ``value`` is frames/s with the batch resident in HBM
(the batch's frame ranges on the lanes of the cached plan, each lane running
the steps on its own stream); ``e2e`` is the same batch through the
reference-facing call with host arrays (numpy frames in, numpy flows out,
host<->device copies inside the timed region).  ``parity`` compares the timed
flows with the CPU oracle on a sample; ``fp32_fast_path`` is the float32
path on the same batch; ``reference_gpu`` times pyflowreg's own GPU level
solver on the same frame size.
``--impl reference`` times the CPU oracle (a restatement of pyflowreg's
numba path; pyflowreg itself cannot run here) on the host cores instead.

Multi-GPU (torchrun): frames are sharded, every rank registers its own batch
(weak scaling, no data-path collective); the step time is the max over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

METRIC = "frames/s 512²×2ch batched vs per-frame GPU at ≤1e-3 px vs ref; bwd/fwd ratio"
H = W = 512
K = 2
OPTIONS = dict(alpha=(1.5, 1.5), eta=0.8, levels=100, min_level=0, iterations=50, update_lag=5, a_smooth=1.0,
               a_data=0.45, const_assumption="gc")
WEIGHT = (0.5, 0.5)
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"],
                    help="the timed path: fp64 (the reference's precision, within the parity tolerance) or fp32")
    ap.add_argument("--no-fp32-secondary", dest="fp32_secondary", action="store_false",
                    help="skip the secondary float32 measurement")
    ap.add_argument("--reference-gpu-frames", type=int, default=2,
                    help="frames of pyflowreg's own GPU level solver timed beside the CPU baseline; 0 skips")
    ap.add_argument("--cpu-fastmath", action="store_true",
                    help="also time the -ffast-math build of the oracle (numba fastmath analogue)")
    ap.add_argument("--frames", type=int, default=400, help="frames per step and rank")
    ap.add_argument("--plain-frames", type=int, default=8, help="frames timed in the one-frame-per-call form")
    ap.add_argument("--cpu-sample", type=int, default=0, help="frames of the CPU baseline sample (0: one per core)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--diff-frames", type=int, default=64,
                    help="frames of the differentiation workload (512x512x1); 0 skips it")
    ap.add_argument("--diff-modes", default="unrolled_store_sweeps,unrolled,implicit",
                    help="gradient modes timed in the differentiation workload")
    ap.add_argument("--compensate-frames", type=int, default=800,
                    help="frames of the 512x512x2 compensate loop in float64 (batches of 400); 0 skips it")
    ap.add_argument("--no-config0", dest="config0", action="store_false",
                    help="skip the single 256x256x1 pair through get_displacement")
    ap.add_argument("--uneven-frames", type=int, default=256,
                    help="frames of the uneven-size batch (sizes 256^2, 512^2, 796x512, 1024^2; 1-2 channels); 0 skips")
    ap.add_argument("--stream-epe-frames", type=int, default=0,
                    help="frames of the 2048x2048x2 stream compared with the CPU oracle (about a minute of host "
                         "time per frame, one core each); 0 skips")
    ap.add_argument("--stream-only", action="store_true",
                    help="run only the 2048x2048x2 streaming workloads; prints their JSON object")
    ap.add_argument("--stream-frames", type=int, default=128,
                    help="frames of the 2048x2048x2 streaming workload (batches of 32); 0 skips")
    ap.add_argument("--autotune-levels", type=int, default=4,
                    help="finest levels whose SOR launch shape the autotuner times on the workload")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default SOR launch shape instead of tuning it on the workload first")
    ap.add_argument("--only-diff", action="store_true",
                    help="run only the differentiation workload (for profiling); prints its JSON object")
    return ap.parse_args()


# --------------------------------------------------------------------------
# workload
# --------------------------------------------------------------------------
def make_workload(n_frames: int, device, seed: int = 1, frame0: int = 50):
    """(reference (H, W, K), frames (T, H, W, K)) preprocessed, float32, on device."""
    import torch

    from pyflowreg_gb300.synthetic import TorchVideo, preprocess_torch

    vid = TorchVideo(seed=seed, h=H, w=W, K=K, device=device)
    with torch.no_grad():
        first = vid.frames(0, 50)
        ref_raw = first.mean(0)
        distinct = min(n_frames, 64)
        raw = vid.frames(frame0, distinct)
        proc = preprocess_torch(raw, ref_raw)
        ref = preprocess_torch(ref_raw, ref_raw)
        reps = (n_frames + distinct - 1) // distinct
        frames = proc.repeat(reps, 1, 1, 1)[:n_frames].contiguous()
    return ref.contiguous(), frames


def run_diff(args, dev):
    """Differentiation workload: 64 frames of 512x512x1 from the same video
    generator, loss = MSE(warp(moving, flow), unwarped truth) + 0.1 * mean
    |flow - true flow|^2, gradients with respect to the moving frames, the
    reference and alpha through the hand-written adjoint (per-level
    checkpoints, recomputation of each level).  Times the forward (flow +
    compensation warp + loss) and the backward separately on the device."""
    import torch

    from pyflowreg_gb300 import diff
    from pyflowreg_gb300.synthetic import TorchVideo, preprocess_torch

    F = args.diff_frames
    vid = TorchVideo(seed=3, h=H, w=W, K=1, device=dev)
    with torch.no_grad():
        ref_raw = vid.frames(0, 50).mean(0)
        lo, hi = float(ref_raw.min()), float(ref_raw.max())
        moving = preprocess_torch(vid.frames(50, F), ref_raw).permute(0, 3, 1, 2).contiguous()
        fixed = preprocess_torch(ref_raw, ref_raw).permute(2, 0, 1).contiguous()
        tr = [vid.truth(50 + i) for i in range(F)]
        truth = torch.stack([(t[0] - lo) / (hi - lo) for t in tr]).permute(0, 3, 1, 2).contiguous()
        w_true = torch.stack([t[1] for t in tr]).permute(0, 3, 1, 2).contiguous()
    opts = {k: OPTIONS[k] for k in ("levels", "eta", "iterations", "update_lag")}
    stream = torch.cuda.current_stream()
    modes = {}
    all_modes = {"implicit": dict(checkpoint="ticks", gradient="implicit"),
                 "unrolled": dict(checkpoint="ticks", gradient="unrolled"),
                 "unrolled_store_sweeps": dict(checkpoint="sweeps", gradient="unrolled"),
                 "unrolled_stepwise": dict(checkpoint="ticks", gradient="unrolled", adjoint="stepwise"),
                 "unrolled_store_sweeps_stepwise": dict(checkpoint="sweeps", gradient="unrolled",
                                                        adjoint="stepwise")}
    for name in args.diff_modes.split(","):
        kw = all_modes[name]
        plan = diff.DiffPlan(H, W, 1, F, dtype=torch.float32, **kw, **opts)
        plan.set_weight([1.0])
        fwd_ms, bwd_ms, loss_v = [], [], None
        for rep in range(1 + max(args.steps, 1)):
            m = moving.clone().requires_grad_(True)
            f = fixed.clone().requires_grad_(True)
            a = torch.tensor(float(OPTIONS["alpha"][0]), dtype=torch.float32, device=dev, requires_grad=True)
            torch.cuda.synchronize()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            loss = diff.registration_loss(f, m, truth, w_true, a, plan)
            e1.record(stream)
            loss.backward()
            e2.record(stream)
            torch.cuda.synchronize()
            if rep > 0:
                fwd_ms.append(e0.elapsed_time(e1))
                bwd_ms.append(e1.elapsed_time(e2))
            loss_v = float(loss.detach())
        fw, bw = float(np.median(fwd_ms)), float(np.median(bwd_ms))
        modes[name] = {**kw, "fwd_ms": fw, "bwd_ms": bw, "ratio": bw / fw, "fwd_frames_per_s": F / (fw / 1e3),
                       "loss": loss_v, "grad_moving_norm": float(m.grad.norm()),
                       "plan_device_bytes": plan.device_bytes(), "reps": len(fwd_ms)}
        plan.close()
        del plan
        torch.cuda.empty_cache()
    head = modes.get("unrolled_store_sweeps") or modes.get("unrolled") or next(iter(modes.values()))
    return {"workload": f"{F} x 512x512x1 photon-count frames, registration loss (lambda 0.1)",
            "dtype": "f32", "pixel_order": "gauss_seidel",
            "headline": "unrolled_store_sweeps: the exact gradient (every half-sweep reversed, psi ticks "
                        "differentiated) with per-level checkpoints of the resized frames, input flow, every "
                        "half-sweep's moved pixels and each psi window's coefficients; the warp and J are "
                        "recomputed in the backward and each window's adjoint runs in one tiled launch.  "
                        "'unrolled' checkpoints only the state at each psi tick and recomputes the window's "
                        "sweeps and coefficients (less memory, more time); '_stepwise' runs the adjoint one "
                        "launch per half-sweep.  'implicit' holds psi at its last tick and differentiates the "
                        "level's fixed point with one SOR solve on the same operator: cheaper, but at "
                        "a_data = 0.45 it misses most of the exact derivative",
            "fwd_ms": head["fwd_ms"], "bwd_ms": head["bwd_ms"], "ratio": head["ratio"], "modes": modes}


def frame_model_bytes(levels, K_, iterations, update_lag):
    """Streaming-model bytes of one frame (float32 words): per level of N
    padded pixels, I iterations of 36 B (five folded coefficients read, du, dv
    read and written), floor(I / L) psi ticks of 24K + 28 B (J, du, dv read,
    coefficients written) and 4 (13K + 12) B of level setup (resize, warp, J,
    weight, flow upsample, median, accumulate)."""
    per_px = iterations * 36 + (iterations // update_lag) * (24 * K_ + 28) + 4 * (13 * K_ + 12)
    return float(sum((h + 2) * (w + 2) for (h, w, _, _) in levels) * per_px)


def run_config0(args, dev):
    """The plain method on one 256x256x1 pair with the default OFOptions (the
    reference's CPU configuration): get_displacement with host arrays in and
    out, then the compensation warp of the moving frame, per call."""
    import torch

    import pyflowreg_gb300 as G
    from pyflowreg_gb300.synthetic import pair_256

    fixed, moving, truth = pair_256(0)
    opts = dict(OPTIONS)
    res = {}
    for prec in ("fp64", "fp32"):
        flow = G.get_displacement(fixed, moving, precision=prec, **opts)  # warm-up: plan, tables
        G.imregister_wrapper(moving, flow[..., 0], flow[..., 1], fixed)
        torch.cuda.synchronize()
        times = []
        for _ in range(5):
            t0 = time.perf_counter()
            flow = G.get_displacement(fixed, moving, precision=prec, **opts)
            reg = G.imregister_wrapper(moving, flow[..., 0], flow[..., 1], fixed)
            times.append(time.perf_counter() - t0)
        d = flow - truth
        res[prec] = {"ms_per_pair": 1e3 * statistics.median(times),
                     "epe_vs_truth_px": float(np.sqrt((d ** 2).sum(-1)).mean()),
                     "compensated_shape": list(reg.shape)}
    return {"workload": "one 256x256x1 pair (40 blobs, sinusoid field of 4 px), default OFOptions, "
                        "get_displacement (numpy in and out) + compensation warp, wall clock, median of 5",
            **res}


def run_compensate_512(args, dev):
    """The 512x512x2 photon-count video as uint16 counts through the streamed
    compensate loop in float64, batches of 400 (OFOptions.buffer_size):
    preprocessing against the raw reference, the initial-field chain between
    batches, flows, compensation warp and statistics on the device."""
    import torch

    from pyflowreg_gb300.synthetic import TorchVideo

    N, B = args.compensate_frames, 400
    vid = TorchVideo(seed=1, h=H, w=W, K=K, device=dev)
    with torch.no_grad():
        ref_raw = vid.frames(0, 50).mean(0).double().cpu().numpy()
        raw = np.empty((N, H, W, K), np.uint16)
        for t0 in range(0, N, 100):
            n = min(100, N - t0)
            raw[t0:t0 + n] = vid.frames(50 + t0, n).clamp(0, 65535).to(torch.int32).cpu().numpy().astype(np.uint16)
    opts = dict(OPTIONS)
    opts.pop("min_level", None)
    out = run_compensate(raw, ref_raw, B, dict(opts, precision="fp64"))
    out["workload"] = (f"{N} x 512x512x2 uint16 frames through the streamed compensate loop in float64, batches of "
                       f"{B}: preprocess, initial-field chain, flows, compensation warp, statistics, registered "
                       "frames and flows to the host")
    return out


def run_uneven(args, dev, precision="fp32"):
    """Uneven-size batch: frames drawn uniformly from {256^2, 512^2, 796x512,
    1024^2} x {1, 2} channels, each size/channel pair a video of its own
    registered to the mean of its first 50 frames; one register() call for all
    frames (groups on 4 streams, launch sequences replayed as CUDA graphs)."""
    import torch

    from pyflowreg_gb300.batch import UnevenBatch
    from pyflowreg_gb300.synthetic import TorchVideo, preprocess_torch

    sizes = [(256, 256), (512, 512), (796, 512), (1024, 1024)]
    rng = np.random.default_rng(2)
    draws = [(sizes[rng.integers(4)], int(rng.integers(1, 3))) for _ in range(args.uneven_frames)]
    refs, frames = {}, []
    with torch.no_grad():
        for bi, ((h, w), k) in enumerate(sorted(set(draws))):
            vid = TorchVideo(seed=20 + bi, h=h, w=w, K=k, device=dev)
            ref_raw = vid.frames(0, 50).mean(0)
            refs[(h, w, k)] = (vid, ref_raw, preprocess_torch(ref_raw, ref_raw).contiguous())
        counters = {}
        for (hw, k) in draws:
            key = (hw[0], hw[1], k)
            vid, ref_raw, _ = refs[key]
            t = 50 + counters.get(key, 0)
            counters[key] = counters.get(key, 0) + 1
            frames.append(preprocess_torch(vid.frame(t), ref_raw).contiguous())
    opts = dict(OPTIONS)
    opts.pop("min_level", None)
    opts["precision"] = precision
    ub = UnevenBatch({k: v[2] for k, v in refs.items()}, graphs=True, **opts)
    ub.register(frames)  # plans, graph capture
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(args.steps, 1)
    e0.record(stream)
    for _ in range(reps):
        ub.register(frames)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    ub.close()
    counts = {f"{k[0]}x{k[1]}x{k[2]}": v for k, v in sorted(counters.items())}
    return {"workload": f"{len(frames)} frames of mixed size and channels, one register() call", "precision": precision,
            "frames_per_size": counts, "ms_per_batch": ms, "frames_per_s": len(frames) / (ms / 1e3),
            "graphs": True, "streams": 4}


def run_stream(args, dev):
    """Large-frame stream: 2048x2048x2 frames registered in batches of 32
    through StreamRegistrar (pinned host buffers, copies on a side stream
    overlapping compute).  The frames are the reference (3000 blobs per
    channel) warped by a rigid drift of up to 20 px plus a sinusoid field,
    with Poisson counts; they are rendered before the timed region into pinned
    host memory, which the source hands over without a copy."""
    import time

    import torch
    import torch.nn.functional as Fnn

    from pyflowreg_gb300.stream import StreamRegistrar
    from pyflowreg_gb300.synthetic import preprocess_torch

    Hs = Ws = 2048
    Ks, N, B = 2, args.stream_frames, 32
    g = torch.Generator(device=dev)
    g.manual_seed(4)
    yy, xx = torch.meshgrid(torch.arange(Hs, device=dev, dtype=torch.float32),
                            torch.arange(Ws, device=dev, dtype=torch.float32), indexing="ij")
    ref = torch.full((Ks, Hs, Ws), 0.05, device=dev)
    with torch.no_grad():
        for k in range(Ks):
            n = 3000
            cy, cx = torch.rand(n, generator=g, device=dev) * Hs, torch.rand(n, generator=g, device=dev) * Ws
            sg = 2 + 4 * torch.rand(n, generator=g, device=dev)
            am = 0.3 + 0.7 * torch.rand(n, generator=g, device=dev)
            for i0 in range(0, n, 100):
                sl = slice(i0, i0 + 100)
                # each blob on a 49 x 49 window around its centre
                oy = torch.arange(-24, 25, device=dev, dtype=torch.float32)
                py = (cy[sl, None].floor() + oy[None]).long()
                px = (cx[sl, None].floor() + oy[None]).long()
                gy = torch.exp(-(py.float() - cy[sl, None]) ** 2 / (2 * sg[sl, None] ** 2))
                gx = torch.exp(-(px.float() - cx[sl, None]) ** 2 / (2 * sg[sl, None] ** 2))
                vals = am[sl, None, None] * gy[:, :, None] * gx[:, None, :]
                ok = (py[:, :, None] >= 0) & (py[:, :, None] < Hs) & (px[:, None, :] >= 0) & (px[:, None, :] < Ws)
                idx = (py[:, :, None] * Ws + px[:, None, :])
                ref[k].view(-1).index_add_(0, idx[ok], vals[ok])
        host = torch.empty((N, Hs, Ws, Ks), dtype=torch.float32).pin_memory()
        raw_u16 = np.empty((N, Hs, Ws, Ks), np.uint16)  # photon counts as a camera would deliver them
        frames_raw = []
        for t in range(N):
            drift = 20.0 * min(1.0, t / max(N - 1, 1))
            ph = 2 * np.pi * t / 250.0
            u = drift * 0.8 + 2.0 * torch.sin(2 * np.pi * yy / 300.0 + ph)
            v = drift * 0.6 + 2.0 * torch.cos(2 * np.pi * xx / 260.0 + ph)
            grid = torch.stack([(xx - u) / (Ws - 1) * 2 - 1, (yy - v) / (Hs - 1) * 2 - 1], dim=-1)[None]
            mov = Fnn.grid_sample(ref[None], grid, mode="bicubic", padding_mode="border", align_corners=True)[0]
            lam = 50.0 + 1950.0 * float(torch.rand((), generator=g, device=dev))
            cnt = torch.poisson(lam * mov.clamp(min=0) / 2.0, generator=g)
            frames_raw.append(cnt.permute(1, 2, 0))
        ref_raw = torch.stack(frames_raw[:min(50, N)]).mean(0)
        for t in range(N):
            host[t].copy_(preprocess_torch(frames_raw[t], ref_raw))
            raw_u16[t] = frames_raw[t].clamp(0, 65535).to(torch.int32).cpu().numpy().astype(np.uint16)
        ref_raw_np = torch.stack([torch.from_numpy(raw_u16[t]).to(dev, torch.float64)
                                  for t in range(min(50, N))]).mean(0).cpu().numpy()
        refp = preprocess_torch(ref_raw, ref_raw).contiguous()
        del frames_raw
    opts = dict(OPTIONS)
    opts.pop("min_level", None)
    opts["precision"] = "fp32"
    sr = StreamRegistrar(refp, batch=B, **opts)
    sink_count = [0]
    # frames compared with the oracle: one per batch after the first, at its middle; each
    # batch after the first starts from the mean of the previous batch's last 20 flows
    n_epe = max(0, min(args.stream_epe_frames, N // B - 1))
    epe_t = [B * (i + 1) + B // 2 for i in range(n_epe)]
    kept, w_next = {}, {}

    def sink(t0, flows):
        sink_count[0] += len(flows)
        if n_epe:
            w_next[t0 + len(flows)] = flows[max(0, len(flows) - 20):].mean(0)
            for t in epe_t:
                if t0 <= t < t0 + len(flows):
                    kept[t] = (flows[t - t0].copy(), w_next.get(t0))

    sr.run(lambda t0, n: host[t0:t0 + n], min(N, 2 * B), sink)  # warm-up
    torch.cuda.synchronize()
    kept.clear()
    w_next.clear()
    t0 = time.perf_counter()
    info = sr.run(lambda t0, n: host[t0:t0 + n], N, sink)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    sr.close()
    stream = {"workload": f"{N} x 2048x2048x2 frames, batches of {B}, pinned host in/out, copies on a side stream",
              "precision": "fp32",
              "frames_per_s": N / dt, "seconds": dt, "h2d_bytes": info["h2d_bytes"], "d2h_bytes": info["d2h_bytes"],
              "timing": "wall clock around StreamRegistrar.run after a warm-up run"}
    if n_epe:
        stream["vs_oracle"] = stream_epe(refp, host, kept, OPTIONS)
    del host
    comp = run_compensate(raw_u16, ref_raw_np, B, opts)
    # the same loop in float64 (the reference's precision) on the first 64 frames
    comp["fp64"] = run_compensate(raw_u16[:min(N, 2 * B)], ref_raw_np, B, dict(opts, precision="fp64"))
    return stream, comp


def stream_epe(refp, host, kept, options):
    """fp32 flows of the 2048x2048x2 stream against the fp64 CPU oracle, one
    frame per host thread, each from its batch's initial field."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O

    fx = refp.cpu().numpy().astype(np.float64)
    ts = sorted(kept)

    def one(t):
        got, uv = kept[t]
        want = O.get_displacement_batch(fx, host[t:t + 1].numpy().astype(np.float64), n_threads=1,
                                        uv=None if uv is None else uv.astype(np.float64), **options)[0]
        d = got.astype(np.float64) - want
        return {"frame": t, "max_abs_px": float(np.abs(d).max()), "mean_epe_px": float(np.sqrt((d ** 2).sum(-1)).mean())}

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=len(ts)) as ex:
        per = list(ex.map(one, ts))
    return {"frames": per, "mean_epe_px": float(np.mean([p["mean_epe_px"] for p in per])),
            "oracle": "fp64 lexicographic C oracle, one frame per host thread", "seconds": time.perf_counter() - t0}


def run_compensate(raw_u16, ref_raw, B, opts):
    """The same video as raw uint16 counts through StreamCompensator: the
    compensate_recording batch loop on the device (preprocess against the raw
    reference, initial field, flows, compensation warp, statistics) with the
    registered frames and flows copied back to the host."""
    import time

    import torch

    from pyflowreg_gb300.pipeline import StreamCompensator

    N = raw_u16.shape[0]

    class CountingWriter:
        frames = 0

        def write_frames(self, frames):
            self.frames += frames.shape[0]

    sc = StreamCompensator(ref_raw, batch=B, **opts)
    sc.run(raw_u16[:min(N, 2 * B)], CountingWriter())  # warm-up
    torch.cuda.synchronize()
    writer = CountingWriter()
    t0 = time.perf_counter()
    info = sc.run(raw_u16, writer)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    sc.close()
    return {"precision": opts.get("precision", "fp64"),
            "workload": f"{N} x 2048x2048x2 uint16 frames through the streamed compensate loop, batches of {B}: "
                        "preprocess, initial field, flows, compensation warp, statistics, registered frames and "
                        "flows to the host",
            "frames_per_s": N / dt, "seconds": dt, "frames_written": writer.frames,
            "h2d_bytes": info["h2d_bytes"], "d2h_bytes": info["d2h_bytes"],
            "timing": "wall clock around StreamCompensator.run after a warm-up run"}


def weight_tensor(device):
    import torch

    w = torch.empty((H, W, K), dtype=torch.float32, device=device)
    for k in range(K):
        w[:, :, k] = WEIGHT[k] / sum(WEIGHT)
    return w


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def profiled_traffic(fp64=False):
    """DRAM bytes per algorithmic byte of the SOR kernel (float64 or float32)
    from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "dram_traffic.txt")
    key = "k_sor_chain64" if fp64 else "k_sor"
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 3 and parts[0] == key and parts[1] == "bytes_per_algorithmic_byte":
                return float(parts[2])
    except OSError:
        pass
    return None


# --------------------------------------------------------------------------
# GB300 arm
# --------------------------------------------------------------------------
def run_reference_gpu(args, dev, levels):
    """pyflowreg's own GPU path on this GPU: the flowreg_torch backend
    (core/__init__.py:140-197) runs get_displacement with its level solver
    level_solver_rbgs_torch (torch/core/level_solver.py:11-199) on the device
    in float64, each level's arrays copied to the device and du, dv back.
    That solver, loaded unmodified from the installed pyflowreg, is timed here
    on one 512x512x2 frame's levels with those copies; the numba pyramid,
    warp, tensor and median the backend runs around it on the CPU are not
    (numba is absent), so the figure bounds the backend's frame rate from
    above."""
    import importlib.util

    import torch

    path = os.path.join(REPO, "baseline", "_ref", "pyflowreg", "torch", "core", "level_solver.py")
    if not os.path.exists(path):
        return {"unavailable": "pyflowreg is not installed in baseline/_ref"}
    spec = importlib.util.spec_from_file_location("pyflowreg_reference_torch_level_solver", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    rng = np.random.default_rng(0)
    inputs = []
    for (h, w, ax, ay) in levels:
        m, n = h + 2, w + 2
        J = [np.abs(rng.standard_normal((m, n, K))) for _ in range(3)] + \
            [0.1 * rng.standard_normal((m, n, K)) for _ in range(3)]
        wgt = np.full((m, n, K), 0.5)
        u = 0.1 * rng.standard_normal((m, n))
        v = 0.1 * rng.standard_normal((m, n))
        inputs.append((J, wgt, u, v, (ax, ay), W / w, H / h))

    def frame():
        for J, wgt, u, v, alpha, hx, hy in inputs:
            t = [torch.as_tensor(a, dtype=torch.float64, device=dev) for a in (*J, wgt, u, v)]
            du, dv = mod.level_solver_rbgs_torch(*t, alpha, OPTIONS["iterations"], OPTIONS["update_lag"],
                                                 OPTIONS["a_data"], OPTIONS["a_smooth"], hx, hy)
            du.cpu().numpy()
            dv.cpu().numpy()

    frame()
    torch.cuda.synchronize()
    n_frames = max(1, args.reference_gpu_frames)
    t0 = time.perf_counter()
    for _ in range(n_frames):
        frame()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / n_frames
    return {"value": 1.0 / dt, "unit": "frames/s", "ms_per_frame": dt * 1e3, "frames": n_frames,
            "what": "level_solver_rbgs_torch (pyflowreg's flowreg_torch backend, float64, unmodified) on every "
                    "level of one 512x512x2 frame, with the backend's per-level host<->device copies; the "
                    "backend's CPU pyramid, warp, tensor and median are not included (upper bound of its "
                    "frame rate)"}


def fp64_peak(dev):
    """Float64 throughput of this GPU: cuBLAS DGEMM (n = 4096), best of 3, in
    TFLOP/s.  The float64 pipe is the roof of the float64 solver."""
    import torch

    n = 4096
    a = torch.randn((n, n), dtype=torch.float64, device=dev)
    b = torch.randn((n, n), dtype=torch.float64, device=dev)
    torch.mm(a, b)
    torch.cuda.synchronize()
    best = None
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.mm(a, b)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    return 2.0 * n ** 3 / (best / 1e3) / 1e12


def profiled_fp64_ops():
    """Float64 flops (FMA = 2) per pixel update of the float64 SOR kernel, fold
    included, from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "dram_traffic.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 3 and parts[0] == "k_sor_chain64" and parts[1] == "fp64_flops_per_pixel_update":
                return float(parts[2])
    except OSError:
        pass
    return None


def time_lanes(plan, frames, out, steps, warmup, stream, barrier=lambda: None):
    """Runs `steps` batched calls on the plan's lanes (each lane its frame range
    on its own stream, steps back to back without a join at step boundaries);
    returns the CUDA-event milliseconds of the timed steps."""
    import torch

    lane_plans = list(getattr(plan, "plans", [plan]))
    lane_streams = list(getattr(plan, "streams", [stream]))
    T = frames.shape[0]
    per_lane = -(-T // len(lane_plans))
    lanes = [(lane_plans[i], lane_streams[i], i * per_lane, min(T, (i + 1) * per_lane))
             for i in range(len(lane_plans)) if i * per_lane < T]

    def run_steps(n):
        start = torch.cuda.Event()
        start.record(stream)
        for lp, ls, t0, t1 in lanes:
            ls.wait_event(start)
        for _ in range(n):
            for lp, ls, t0, t1 in lanes:
                lp.displacement(frames[t0:t1], None, out[t0:t1], stream=ls)
        for lp, ls, t0, t1 in lanes:
            stream.wait_stream(ls)

    run_steps(max(warmup, 3))
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    run_steps(steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    return ev0.elapsed_time(ev1), len(lanes)


def sor_profile(G, params, plan, ref, wt, frames, out, stream):
    """CUDA-event time and model bytes of the SOR launches of one single-plan
    call of the batch, with the GPU to itself (lanes overlap their launches)."""
    import torch

    T = frames.shape[0]
    rplan = G.Plan(params, H, W, K, T)
    rplan.set_reference(ref, wt)
    for i in range(len(plan.level_tuning())):
        g, t_, gmax, _ = plan.level_tuning()[i]
        if rplan.fp64:
            rplan.set_level_tuning(i, 0, t_)
            continue
        v, nv = plan.level_variant(i)
        if nv > 0:
            rplan.set_level_variant(i, v)
        if gmax > 0:
            rplan.set_level_tuning(i, g, t_)
    rplan.displacement(frames, None, out)
    torch.cuda.synchronize()
    rplan.set_profiling(True)
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    rplan.displacement(frames, None, out)
    r1.record(stream)
    torch.cuda.synchronize()
    sor_n, sor_ms, sor_bytes = rplan.profile()
    rplan.close()
    return sor_n, sor_ms, sor_bytes, r0.elapsed_time(r1)


def run_gb300(args):
    import torch
    import torch.distributed as dist

    import pyflowreg_gb300 as G
    from pyflowreg_gb300 import _lib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if world > 1:
            dist.barrier()

    T = args.frames
    ref, frames = make_workload(T, dev, seed=1, frame0=50 + rank * T)
    wt = weight_tensor(dev)
    stream = torch.cuda.current_stream()
    precision = args.precision
    params = G.make_params(K=K, precision=precision, **OPTIONS)
    plan = G.get_plan(params, H, W, K, T)
    plan.set_reference(ref, wt)
    fp64 = plan.fp64
    out = torch.empty((T, H, W, 2), dtype=torch.float64 if fp64 else torch.float32, device=dev)

    tuning = None
    if not args.no_autotune:
        # launch-shape tuning on the workload itself (outside the timed region; flows unchanged)
        chosen = plan.autotune(frames, n_levels=args.autotune_levels, reps=1)
        if fp64:
            tuning = {f"level {i} ({plan.level_tuning()[i][3]} rows)":
                      {"kernel": "k_sor_chain64", "rows_per_cta": t or "by batch size"}
                      for i, (v, g, t, _) in chosen.items()}
        else:
            tuning = {f"level {i} ({plan.level_tuning()[i][3]} rows)":
                      {"kernel": {0: "diagonal_ring", 1: "rows_in_registers", 2: "rows_in_registers_chained"}[v],
                       "G": g, "threads": t or plan.level_tuning()[i][3]}
                      for i, (v, g, t, _) in chosen.items()}

    # ---- value: the batch resident in HBM, the plan's lanes on their own streams
    lib = _lib.load()
    sampler = ClockSampler(local)
    n0 = lib.frg_launch_count()
    sampler.start()
    ms, n_lanes = time_lanes(plan, frames, out, args.steps, args.warmup, stream, barrier)
    clocks = sampler.stop()
    launches = lib.frg_launch_count() - n0
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = world * T * args.steps / (ms / 1e3)
    out_kept = out.clone()

    # ---- the SOR kernel on its own: one single-plan call of the same batch
    sor_n, sor_ms, sor_bytes, rcall_ms = sor_profile(G, params, plan, ref, wt, frames, out, stream)

    # ---- e2e: the reference-facing batch call with host arrays (pageable numpy in, numpy out);
    # its host<->device copies (pinned staging, overlapped lane by lane) are inside the timed region
    fx_np = ref.cpu().numpy()
    mv_np = frames.cpu().numpy()
    w_np = wt.cpu().numpy()
    G.get_displacement_batch(fx_np, mv_np, weight=w_np, precision=precision, **OPTIONS)  # warm-up
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_out = G.get_displacement_batch(fx_np, mv_np, weight=w_np, precision=precision, **OPTIONS)
    torch.cuda.synchronize()
    e_s = time.perf_counter() - t0
    barrier()
    if world > 1:
        t = torch.tensor([e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e_s = float(t.item())
    e2e_value = world * T * args.steps / e_s
    e2e_equal = bool(np.array_equal(host_out, out_kept.cpu().numpy()))
    del host_out

    # ---- plain form: one frame per call (the same kernels, batch of one)
    plain = None
    if args.plain_frames > 0:
        pplan = G.Plan(params, H, W, K, 1)
        pplan.set_reference(ref, wt)
        pout = torch.empty((1, H, W, 2), dtype=out.dtype, device=dev)
        pplan.displacement(frames[:1], None, pout)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for i in range(args.plain_frames):
            pplan.displacement(frames[i:i + 1], None, pout)
        p1.record(stream)
        torch.cuda.synchronize()
        p_ms = p0.elapsed_time(p1)
        plain = {"value": args.plain_frames / (p_ms / 1e3), "unit": "frames/s", "frames": args.plain_frames,
                 "ms_per_frame": p_ms / args.plain_frames, "precision": precision}
        pplan.close()

    # ---- roofline of the SOR kernel
    peak, peak_src = measured_peak()
    achieved = (sor_bytes / (sor_ms / 1e3) / 1e9) if sor_ms > 0 else None
    per_launch_bytes = sor_bytes / max(sor_n, 1)
    ratio = profiled_traffic(fp64)
    bpp = 72 if fp64 else 36
    roofline = {
        "kernel": ("k_sor_chain64 (float64 exact-order chained wavefront SOR, one thread per row, state in "
                   "registers, coefficients folded once per pass, row strips of 64-256 rows as clusters)" if fp64
                   else "k_sor_chain (float32 exact-order chained wavefront SOR, one thread per row, state in "
                   "registers, fold in the loader)"),
        "bound": "hbm",
        "achieved": achieved,
        "peak": peak,
        "peak_source": peak_src,
        "unit": "GB/s",
        "frac": (achieved / peak) if achieved else None,
        "traffic": (per_launch_bytes * ratio) if ratio else None,
        "algorithmic_bytes_per_launch": per_launch_bytes,
        "launches": sor_n,
        "share_of_step": (sor_ms / rcall_ms) if rcall_ms > 0 else None,
        "measured_on": "one single-plan call of the same batch right after the timed region (CUDA events on the "
                       "launching stream around each SOR launch)",
        "note": f"achieved = {bpp} B per interior pixel per SOR iteration (streaming model: five coefficients "
                "and du, dv read, du, dv written) / CUDA-event time of the SOR launches; traffic = measured "
                "DRAM/model ratio of the committed ncu summary x model bytes per launch",
    }
    fp64_pipe = None
    if fp64:
        ops = profiled_fp64_ops()
        peak64 = fp64_peak(dev)
        its = sor_bytes / bpp  # pixel updates in the profiled call
        ach = (ops * its / (sor_ms / 1e3) / 1e12) if (ops and sor_ms > 0) else None
        fp64_pipe = {"bound": "fp64 pipe", "achieved_tflops": ach, "peak_tflops": peak64,
                     "peak_source": "cuBLAS DGEMM 4096^3 measured in this run", "frac": (ach / peak64) if ach else None,
                     "fp64_flops_per_pixel_update": ops,
                     "note": "the float64 SOR is bound by the float64 pipe (about 1/64 of the float32 rate on "
                             "GB300), not by HBM: achieved = float64 flops per pixel update (ncu count of the "
                             "kernel's DFMA x 2 + DADD + DMUL, fold included, profiles/dram_traffic.txt) x pixel "
                             "updates / SOR time, against cuBLAS DGEMM on the same GPU"}

    # the whole frame against the float32 streaming model of bytes per frame
    bpf = frame_model_bytes(plan.levels(), K, OPTIONS["iterations"], OPTIONS["update_lag"])
    frame_model = {"bytes_per_frame": bpf, "GBps_at_value": bpf * value / world / 1e9,
                   "frac_of_hbm": bpf * value / world / 1e9 / peak if peak else None,
                   "note": "float32 streaming-model bytes per frame (every level's padded pixels x (50 x 36 + "
                           "10 x (24K + 28) + 4 (13K + 12)) B) at the measured frames/s; the float64 path moves "
                           "twice the words and is bound by the float64 pipe, not by HBM"}

    cpu = parity = None
    reference_gpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, parity = cpu_baseline(args, ref, frames, out_kept, precision)
    if rank == 0 and world == 1 and args.reference_gpu_frames > 0:
        lv = plan.plans[0].levels() if hasattr(plan, "plans") else plan.levels()
        reference_gpu = run_reference_gpu(args, dev, lv)
    fp32 = None
    if rank == 0 and precision == "fp64" and args.fp32_secondary:
        fp32 = run_fp32_secondary(args, G, ref, wt, frames, stream, parity)
    if parity is not None:
        parity.pop("_oracle_flows", None)
    backward = run_diff(args, dev) if (rank == 0 and args.diff_frames > 0) else None
    config0 = run_config0(args, dev) if (rank == 0 and args.config0) else None
    compensate_512 = run_compensate_512(args, dev) if (rank == 0 and args.compensate_frames > 0) else None
    uneven = run_uneven(args, dev) if (rank == 0 and args.uneven_frames > 0) else None
    if uneven is not None:
        uneven["fp64"] = run_uneven(args, dev, "fp64")
    stream_2048, compensate_2048 = run_stream(args, dev) if (rank == 0 and args.stream_frames > 0) else (None, None)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "frames/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": max(args.warmup, 3),
            "ms_per_step": ms_per_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if fp64 else "f32",
            "data": "synthetic (seeded photon-count blob video, preprocessed on device)",
            "config": {"workload": "512x512x2 video, batched get_displacement against the mean of frames 0-49",
                       "precision": precision, "frames_per_step": T * world, "frames_per_rank": T, "height": H,
                       "width": W, "channels": K, "options": {**OPTIONS, "alpha": list(OPTIONS["alpha"]),
                                                              "weight": list(WEIGHT)},
                       "l2": "inputs larger than L2 (%.0f MB per step)" % (T * H * W * K * 4 / 1e6),
                       "parallelism": f"frames sharded over {world} GPU(s)",
                       "sor_launch_tuning": tuning,
                       "lanes": f"{n_lanes} plans over contiguous parts of the batch, each on its own stream, "
                                "running the steps without a join between lanes at step boundaries"
                                if n_lanes > 1 else "one plan"},
            "e2e": {"value": e2e_value, "unit": "frames/s",
                    "h2d_bytes_per_step": T * H * W * K * 4 + 2 * H * W * K * 4,
                    "d2h_bytes_per_step": T * H * W * 2 * (8 if fp64 else 4),
                    "api": "pyflowreg_gb300.get_displacement_batch(fixed, moving, weight=..., **options): numpy "
                           "arrays in, numpy flows out (the reference-facing batch call behind the gb300 executor)",
                    "copies": "pageable numpy -> pinned staging -> device per lane part (copies of one part "
                              "overlap the other parts' compute); each lane's last part read back by one copy "
                              "into the output array, page-locked while the lanes compute",
                    "timing": "wall clock around the calls after a warm-up call",
                    "flows_equal_device_resident_run": e2e_equal},
            "gpu_launches": int(launches),
            "roofline": roofline,
            "fp64_pipe": fp64_pipe,
            "plain": plain,
            "batched_over_plain": (value / world / plain["value"]) if plain else None,
            "fp32_fast_path": fp32,
            "bwd_fwd_ratio": backward["ratio"] if backward else None,
            "backward": backward,
            "frame_streaming_model": frame_model,
            "config0_pair": config0,
            "compensate_512": compensate_512,
            "uneven_batch": uneven,
            "stream_2048": stream_2048,
            "compensate_2048": compensate_2048,
            "clocks": clocks,
            "cpu_baseline": cpu,
            "reference_gpu": reference_gpu,
            "parity": parity,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_fp32_secondary(args, G, ref, wt, frames, stream, parity):
    """The float32 path on the same batch (secondary: outside the parity
    tolerance), with its own launch-shape tuning."""
    import torch

    T = frames.shape[0]
    params = G.make_params(K=K, precision="fp32", **OPTIONS)
    plan = G.get_plan(params, H, W, K, T)
    plan.set_reference(ref, wt)
    if not args.no_autotune:
        plan.autotune(frames, n_levels=4, reps=1)
    out = torch.empty((T, H, W, 2), dtype=torch.float32, device=frames.device)
    ms, _ = time_lanes(plan, frames, out, args.steps, args.warmup, stream)
    res = {"value": T * args.steps / (ms / 1e3), "unit": "frames/s", "dtype": "f32",
           "note": "float32 arithmetic: the algorithm amplifies its rounding to flows up to ~0.7 px from the "
                   "reference's (parity block)"}
    if parity is not None and "_oracle_flows" in parity:
        n = parity["frames"]
        res["parity"] = flow_diff(out[:n].cpu().numpy().astype(np.float64), parity["_oracle_flows"])
    return res


def flow_diff(a, b):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return {"max_abs_px": float(np.abs(d).max()), "mean_epe_px": float(np.sqrt((d ** 2).sum(-1)).mean())}


def cpu_baseline(args, ref, frames, gpu_out, precision):
    """The oracle, built -O3 for the host's CPU with the checker's float
    semantics, timed on the host cores on a bounded sample of the same frames
    (one frame per thread); the checker's flows on that sample give the
    parity of the timed GPU flows."""
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    n = args.cpu_sample or cores
    n = min(n, frames.shape[0])
    fx = ref.cpu().numpy().astype(np.float64)
    mv = frames[:n].cpu().numpy().astype(np.float64)
    wt = np.empty((H, W, K))
    for k in range(K):
        wt[:, :, k] = WEIGHT[k] / sum(WEIGHT)
    t0 = time.perf_counter()
    flows = O.get_displacement_batch(fx, mv, n_threads=cores, weight=wt, variant="o3", **OPTIONS)
    dt = time.perf_counter() - t0
    check = O.get_displacement_batch(fx, mv, n_threads=cores, weight=wt, **OPTIONS)
    assert np.array_equal(flows, check), "the timed oracle build must return the checker's flows"
    fast = None
    if args.cpu_fastmath:
        t0 = time.perf_counter()
        fm = O.get_displacement_batch(fx, mv, n_threads=cores, weight=wt, variant="fastmath", **OPTIONS)
        fdt = time.perf_counter() - t0
        fast = {"value": n / fdt, "unit": "frames/s", "flags": O.build_flags().get("fastmath"),
                "vs_checker": flow_diff(fm, flows),
                "note": "the analogue of numba's fastmath=True: faster, its flows move within the reference's "
                        "own rounding envelope"}
    # how far the reference's red-black GPU variants' order alone moves the flow (oracle, float64)
    rb = O.get_displacement_batch(fx, mv, n_threads=cores, weight=wt, variant="o3", order=O.ORDER_RED_BLACK,
                                  **OPTIONS)
    parity = {"frames": n, "precision": precision, "timed_path": flow_diff(gpu_out[:n].cpu().numpy(), flows),
              "tolerance": {"max_abs_px": 1e-3, "mean_epe_px": 1e-4},
              "red_black_order_vs_reference": flow_diff(rb, flows),
              "oracle": "fp64 lexicographic C restatement of pyflowreg's numba path, pinned to the reference's own "
                        "source by the golden fixtures",
              "_oracle_flows": flows}
    cpu = {"value": n / dt, "unit": "frames/s", "cores": cores, "kind": "port",
           "flags": O.build_flags().get("o3"),
           "sample": f"{n} frames of the same batch, one frame per thread (OpenMP), fp64 lexicographic oracle",
           "fastmath_build": fast}
    return cpu, parity


# --------------------------------------------------------------------------
# reference arm: the CPU restatement of pyflowreg's numba path
# --------------------------------------------------------------------------
def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch

    from oracle import oracle as O

    cores = os.cpu_count() or 1
    n = args.cpu_sample or cores
    ref, frames = make_workload(n, "cpu", seed=1, frame0=50)
    fx = ref.numpy().astype(np.float64)
    mv = frames.numpy().astype(np.float64)
    wt = np.empty((H, W, K))
    for k in range(K):
        wt[:, :, k] = WEIGHT[k] / sum(WEIGHT)
    for _ in range(args.warmup):
        O.get_displacement_batch(fx, mv[:1], n_threads=1, weight=wt, variant="o3", **OPTIONS)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.get_displacement_batch(fx, mv, n_threads=cores, weight=wt, variant="o3", **OPTIONS)
    dt = time.perf_counter() - t0
    value = n * args.steps / dt
    del torch
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded photon-count blob video, preprocessed)",
        "config": {"workload": "512x512x2 video, batched get_displacement against the mean of frames 0-49",
                   "frames_per_step": n, "height": H, "width": W, "channels": K},
        "cpu_baseline": {"value": value, "unit": "frames/s", "cores": cores, "kind": "port",
                         "flags": O.build_flags().get("o3"),
                         "sample": f"{n} frames per step, one frame per thread"},
        "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "pyflowreg's numba/OpenCV path cannot be installed here; the fp64 C restatement of it "
                "(oracle/) is timed instead",
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.only_diff:
        import torch

        torch.cuda.set_device(0)
        print(json.dumps(run_diff(args, torch.device("cuda", 0))))
        return
    if args.stream_only:
        import torch

        torch.cuda.set_device(0)
        stream, comp = run_stream(args, torch.device("cuda", 0))
        print(json.dumps({"stream_2048": stream, "compensate_2048": comp}))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
