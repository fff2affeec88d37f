"""Uneven batches: frames of several sizes and channel counts registered in one call.

pyflowreg registers one frame at a time (the executors call get_displacement
per frame, motion_correction/parallelization/sequential.py:141-145), so a
recording of mixed sizes costs nothing extra there.  On the GPU a batch of
mixed sizes is grouped by (height, width, channels): each group runs through
its own cached plan as one batched launch sequence, the groups are spread
round-robin over a few CUDA streams so that small groups fill the SMs next to
large ones, and each group's launch sequence can be captured once as a CUDA
graph and replayed on later calls with the same group size.
"""

from __future__ import annotations

from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import api

Key = Tuple[int, int, int]


class UnevenBatch:
    """Registers lists of frames of mixed shapes against one reference per shape.

    references: {(H, W, K): reference (H, W, K) float32 CUDA tensor}
    weights: {(H, W, K): weight (H, W, K)} or None (1/K per channel)
    options: get_displacement options (alpha, levels, iterations, ...).
    """

    def __init__(self, references: Dict[Key, torch.Tensor], weights: Optional[Dict[Key, torch.Tensor]] = None,
                 n_streams: int = 4, graphs: bool = False, **options):
        self.refs = {tuple(k): v.contiguous() for k, v in references.items()}
        self.weights = {tuple(k): v.contiguous() for k, v in (weights or {}).items()}
        self.options = options
        self.streams = [torch.cuda.Stream() for _ in range(max(1, n_streams))]
        self.graphs = graphs
        self._graphs: Dict[Tuple[Key, int], tuple] = {}
        self._plans: Dict[Key, api.Plan] = {}

    def _plan(self, key: Key, n: int) -> api.Plan:
        H, W, K = key
        plan = self._plans.get(key)
        if plan is None or plan.max_frames < n:
            if plan is not None:
                plan.close()
            plan = api.Plan(api.make_params(K=K, **self.options), H, W, K, n)
            plan.set_reference(self.refs[key], self.weights.get(key))
            self._plans[key] = plan
        return plan

    def groups(self, frames: Sequence[torch.Tensor]) -> Dict[Key, List[int]]:
        out: Dict[Key, List[int]] = {}
        for i, f in enumerate(frames):
            key = tuple(int(s) for s in f.shape)
            if key not in self.refs:
                raise ValueError(f"no reference for frame shape {key}")
            out.setdefault(key, []).append(i)
        return out

    def register(self, frames: Sequence[torch.Tensor]) -> List[torch.Tensor]:
        """flows (H, W, 2) on the device (float64 with precision="fp64",
        float32 otherwise), in the order of `frames`."""
        groups = self.groups(frames)
        results: List[Optional[torch.Tensor]] = [None] * len(frames)
        main = torch.cuda.current_stream()
        # largest groups first, so they start before the small ones fill in
        order = sorted(groups.items(), key=lambda kv: -(kv[0][0] * kv[0][1] * kv[0][2] * len(kv[1])))
        for gi, (key, idx) in enumerate(order):
            st = self.streams[gi % len(self.streams)]
            st.wait_stream(main)
            with torch.cuda.stream(st):
                out = self._run_group(key, [frames[i] for i in idx], st)
            for j, i in enumerate(idx):
                results[i] = out[j]
        for st in self.streams:
            main.wait_stream(st)
        return results

    def _run_group(self, key: Key, group: List[torch.Tensor], st) -> torch.Tensor:
        n = len(group)
        plan = self._plan(key, n)
        if not self.graphs:
            batch = torch.stack(group)
            return plan.displacement(batch, None, None, stream=st)
        entry = self._graphs.get((key, n))
        if entry is None:
            H, W, K = key
            static_in = torch.empty((n, H, W, K), dtype=torch.float32, device=group[0].device)
            static_out = torch.empty((n, H, W, 2), dtype=torch.float64 if plan.fp64 else torch.float32,
                                     device=group[0].device)
            static_in.copy_(torch.stack(group))
            plan.displacement(static_in, None, static_out, stream=st)  # warm-up outside the capture
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=st):
                plan.displacement(static_in, None, static_out, stream=torch.cuda.current_stream())
            entry = (g, static_in, static_out)
            self._graphs[(key, n)] = entry
        g, static_in, static_out = entry
        torch.stack(group, out=static_in)
        g.replay()
        return static_out.clone()

    def close(self):
        self._graphs.clear()
        for p in self._plans.values():
            p.close()
        self._plans.clear()
