"""Generates tests/golden/rbgs_torch.npz from pyflowreg's own torch red-black
level solver (torch/core/level_solver.py:11-199), run with autograd enabled.

The reference's solve updates du/dv in place, which reverse-mode autograd
rejects, so the derivatives are taken in forward mode: every input is a dual
tensor (``torch.autograd.forward_ad``) with a seeded tangent, and the
reference's own ops, unmodified, carry the tangents through all iterations.
The module's global ``torch`` is replaced by a proxy whose ``no_grad()`` is a
null context (everything else forwards to torch).  The fixture stores the
inputs, the returned (du, dv) and, for each of a few seeded input directions,
the exact directional derivative (du_dot, dv_dot): the unrolled derivative of
the reference torch backend that the differentiable mode is checked against
(reverse-mode gradients dotted with a direction must reproduce it).

Run where the reference source is available (tests never import it):

    python tests/golden/make_golden_rbgs.py <path/to/pyflowreg/src>
"""

from __future__ import annotations

import contextlib
import importlib.util
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_golden_rbgs.py <path/to/pyflowreg/src>")
REF_SRC = sys.argv[1]


class _TorchWithGrad:
    def __getattr__(self, name):
        return getattr(torch, name)

    @staticmethod
    def no_grad():
        return contextlib.nullcontext()


def load_solver():
    path = os.path.join(REF_SRC, "pyflowreg", "torch", "core", "level_solver.py")
    spec = importlib.util.spec_from_file_location("ref_rbgs_level_solver", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.torch = _TorchWithGrad()
    return mod.level_solver_rbgs_torch


def case(rng, m, n, K, iterations, lag, a_data):
    J = {}
    # a positive definite 3x3 tensor per pixel and channel (rank one plus a small
    # isotropic part, so E stays away from 0 where psi's slope is ~1e9), zero ring
    g = rng.standard_normal((m, n, K, 3))
    g[..., 2] *= 0.3
    JJ = np.einsum("pqki,pqkj->pqkij", g, g) + 0.05 * np.eye(3)
    JJ[0, :] = JJ[-1, :] = 0
    JJ[:, 0] = JJ[:, -1] = 0
    for name, (a, b) in zip(("J11", "J22", "J33", "J12", "J13", "J23"),
                            ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))):
        J[name] = JJ[..., a, b].copy()
    W = np.zeros((m, n, K))
    W[1:-1, 1:-1, :] = rng.uniform(0.3, 1.0, K)
    u = np.pad(rng.standard_normal((m - 2, n - 2)) * 0.4, 1, mode="edge")
    v = np.pad(rng.standard_normal((m - 2, n - 2)) * 0.4, 1, mode="edge")
    hx, hy = 1.25, 0.8
    alpha = rng.uniform(1.0, 2.5, 2)

    solver = load_solver()
    import torch.autograd.forward_ad as fwAD

    names = ("J11", "J22", "J33", "J12", "J13", "J23", "u", "v", "alpha")
    base_vals = dict(J, u=u, v=v, alpha=alpha)
    out = dict(W=W, u=u, v=v, alpha=alpha, hx=hx, hy=hy, iterations=iterations, lag=lag,
               a_data=np.asarray(a_data, np.float64))
    for k, a in J.items():
        out[k] = a
    n_dir = 3
    for d in range(n_dir + 1):
        with fwAD.dual_level():
            duals = {}
            for nm in names:
                val = torch.tensor(base_vals[nm], dtype=torch.float64)
                if d == 0:
                    duals[nm] = val
                    continue
                tang = rng.standard_normal(val.shape)
                if nm.startswith("J"):
                    tang[0, :] = tang[-1, :] = 0
                    tang[:, 0] = tang[:, -1] = 0
                if nm in ("u", "v"):
                    tang = np.pad(tang[1:-1, 1:-1], 1, mode="edge")
                out[f"dir{d}_{nm}"] = tang
                duals[nm] = fwAD.make_dual(val, torch.tensor(tang, dtype=torch.float64))
            du, dv = solver(duals["J11"], duals["J22"], duals["J33"], duals["J12"], duals["J13"],
                            duals["J23"], torch.tensor(W), duals["u"], duals["v"],
                            [duals["alpha"][0], duals["alpha"][1]], iterations, lag,
                            torch.tensor(a_data, dtype=torch.float64), 1.0, hx, hy)
            if d == 0:
                out["du"], out["dv"] = du.numpy().copy(), dv.numpy().copy()
            else:
                out[f"dir{d}_du_dot"] = fwAD.unpack_dual(du).tangent.numpy().copy()
                out[f"dir{d}_dv_dot"] = fwAD.unpack_dual(dv).tangent.numpy().copy()
    out["n_dir"] = n_dir
    return out


def main():
    rng = np.random.default_rng(20240601)
    cases = {
        "a": case(rng, 12, 14, 1, 12, 5, [0.45]),
        "b": case(rng, 15, 11, 2, 17, 3, [0.45, 0.6]),
        "c": case(rng, 10, 10, 1, 6, 1, [1.0]),
    }
    flat = {f"{c}_{k}": np.asarray(v) for c, d in cases.items() for k, v in d.items()}
    np.savez_compressed(os.path.join(HERE, "rbgs_torch.npz"), **flat)
    print("wrote rbgs_torch.npz", {c: d["du"].shape for c, d in cases.items()})


if __name__ == "__main__":
    main()
