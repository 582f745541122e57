"""Launch-shape autotuner for the per-scene step kernel.

The kernel is built in several shapes (threads per scene block x the number of resident
blocks per SM its register budget targets; D2F_VARIANTS in csrc/pncg_kernel.cuh). Which
is fastest depends on the scene sizes and the precision: more blocks per SM hide more
memory latency but cap registers (and spill), wider blocks split a scene finer but pay more
per barrier. `tune` times every shape on a sample of the batch's own scenes — a few steps
each, from the same starting state — and returns the fastest, keyed by the batch's
scene-size bucket so a process reuses its choice.
"""
from __future__ import annotations

import numpy as np

VARIANTS = [(32, 16), (64, 8), (128, 4), (256, 2), (256, 3)]
_CACHE = {}


def size_bucket(prob):
    """Median triangles per scene, rounded to a power of two."""
    t = np.bincount(np.asarray(prob["tri2env"]), minlength=int(prob["B"]))
    return int(2 ** round(np.log2(max(float(np.median(t)), 1.0))))


def tune(prob, precision, steps=2, warmup=1, sample=1024, variants=VARIANTS, seed=0):
    """Returns ((threads, blocks_per_sm), table) with table = [(ms_per_step, threads, bps)]."""
    import torch
    from .device import DeviceSolver
    from .scene import subset_problem

    key = (precision, size_bucket(prob), torch.cuda.get_device_name())
    if key in _CACHE:
        return _CACHE[key]
    B = int(prob["B"])
    sub = prob
    if B > sample:
        envs = np.sort(np.random.default_rng(seed).choice(B, sample, replace=False))
        sub = subset_problem(prob, envs)
    table = []
    for nt, bps in variants:
        s = DeviceSolver(sub, precision=precision, threads=nt, blocks_per_sm=bps)
        for _ in range(warmup):
            s.step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        st = torch.cuda.current_stream()
        e0.record(st)
        for _ in range(steps):
            s.step()
        e1.record(st)
        torch.cuda.synchronize()
        table.append((e0.elapsed_time(e1) / steps, nt, bps))
        s.close()
        del s
    torch.cuda.empty_cache()
    best = min(table)
    out = ((best[1], best[2]), table)
    _CACHE[key] = out
    return out
