"""Finite-difference check of the differentiable mode on full-size frames.

    python -m pyflowreg_gb300.diffcheck [--frames 2] [--size 512] [--directions 16]

Builds seeded photon-count frames (the video generator of the benchmark, one
channel), evaluates the registration loss
MSE(warp(moving, flow), unwarped truth) + 0.1 * mean |flow - true flow|^2 in
float64, and compares, on unit-norm random directions in (moving, fixed,
alpha), the directional derivative from the CUDA adjoint (unrolled exact,
unrolled with psi lagged, implicit) with central differences of the CUDA
forward at several steps.  Prints one JSON object.
"""

from __future__ import annotations

import argparse
import json

import numpy as np
import torch


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=2)
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--directions", type=int, default=16)
    ap.add_argument("--steps", default="1e-4,1e-6,1e-8")
    args = ap.parse_args(argv)

    from . import diff
    from .synthetic import TorchVideo, preprocess_torch

    dev = torch.device("cuda")
    F, S = args.frames, args.size
    vid = TorchVideo(seed=3, h=S, w=S, K=1, device=dev)
    with torch.no_grad():
        ref_raw = vid.frames(0, 50).mean(0)
        lo, hi = float(ref_raw.min()), float(ref_raw.max())
        moving = preprocess_torch(vid.frames(50, F), ref_raw).permute(0, 3, 1, 2).double().contiguous()
        fixed = preprocess_torch(ref_raw, ref_raw).permute(2, 0, 1).double().contiguous()
        tr = [vid.truth(50 + i) for i in range(F)]
        truth = torch.stack([(t[0] - lo) / (hi - lo) for t in tr]).permute(0, 3, 1, 2).double().contiguous()
        w_true = torch.stack([t[1] for t in tr]).permute(0, 3, 1, 2).double().contiguous()

    grads = {}
    plans = {}
    for name, kw in (("unrolled", {}), ("unrolled_lagged", {"psi_gradient": "lagged"}),
                     ("implicit", {"gradient": "implicit"})):
        plan = diff.DiffPlan(S, S, 1, F, dtype=torch.float64, **kw)
        plan.set_weight([1.0])
        m = moving.clone().requires_grad_(True)
        f = fixed.clone().requires_grad_(True)
        a = torch.tensor(1.5, dtype=torch.float64, device=dev, requires_grad=True)
        loss = diff.registration_loss(f, m, truth, w_true, a, plan)
        loss.backward()
        grads[name] = (m.grad.detach().clone(), f.grad.detach().clone(), float(a.grad))
        plans[name] = plan
    plan = plans["unrolled"]

    def loss_at(dm, df, da, s):
        with torch.no_grad():
            return float(diff.registration_loss(fixed + s * df, moving + s * dm, truth, w_true,
                                                torch.tensor(1.5 + s * da, dtype=torch.float64), plan))

    steps = [float(x) for x in args.steps.split(",")]
    gen = torch.Generator(device=dev)
    gen.manual_seed(123)
    rows = []
    for _ in range(args.directions):
        dm = torch.randn(moving.shape, generator=gen, device=dev, dtype=torch.float64)
        df = torch.randn(fixed.shape, generator=gen, device=dev, dtype=torch.float64)
        da = float(torch.randn((), generator=gen, device=dev, dtype=torch.float64))
        nrm = float(torch.sqrt((dm ** 2).sum() + (df ** 2).sum() + da * da))
        dm, df, da = dm / nrm, df / nrm, da / nrm
        row = {"fd": {}}
        for s in steps:
            row["fd"][f"{s:g}"] = (loss_at(dm, df, da, s) - loss_at(dm, df, da, -s)) / (2 * s)
        for name, (gm, gf, ga) in grads.items():
            row[name] = float((gm * dm).sum() + (gf * df).sum() + ga * da)
        rows.append(row)

    def rel(a, b):
        return abs(a - b) / max(abs(b), 1e-12)

    finest = f"{min(steps):g}"
    summary = {
        "workload": f"{F} x {S}x{S}x1 photon-count frames, float64, registration loss (lambda 0.1)",
        "directions": args.directions,
        "median_rel_err_unrolled_vs_fd": {k: float(np.median([rel(r["unrolled"], r["fd"][k]) for r in rows]))
                                          for k in rows[0]["fd"]},
        "max_rel_err_unrolled_vs_fd_finest": float(max(rel(r["unrolled"], r["fd"][finest]) for r in rows)),
        "cos_implicit_vs_unrolled_lagged_moving": float(
            (grads["implicit"][0] * grads["unrolled_lagged"][0]).sum()
            / (grads["implicit"][0].norm() * grads["unrolled_lagged"][0].norm())),
        "rows": rows,
    }
    print(json.dumps(summary))
    for p in plans.values():
        p.close()


if __name__ == "__main__":
    main()
