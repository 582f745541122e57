"""Flat .npz storage of a solver problem (a dict of arrays, scalars and sub-dicts) and of
the per-step commands and results recorded with it. TEST INFRASTRUCTURE."""
from __future__ import annotations

import numpy as np

SUBS = ("ipc", "tendon", "affine", "rigid", "springs", "pressure")


def pack(prob: dict, steps: list, meta: dict | None = None) -> dict:
    out = {}
    for k, v in prob.items():
        if v is None:
            continue
        if k in SUBS:
            for kk, vv in v.items():
                if vv is None:
                    continue
                out[f"prob.{k}.{kk}"] = np.asarray(vv)
        else:
            out[f"prob.{k}"] = np.asarray(v)
    for i, st in enumerate(steps):
        for k, v in st.items():
            if v is None:
                continue
            out[f"step{i}.{k}"] = np.asarray(v)
    out["n_steps"] = np.asarray(len(steps))
    for k, v in (meta or {}).items():
        out[f"meta.{k}"] = np.asarray(v)
    return out


def unpack(npz) -> tuple[dict, list, dict]:
    prob, meta = {}, {}
    n = int(npz["n_steps"])
    steps = [dict() for _ in range(n)]
    for key in npz.files:
        a = npz[key]
        parts = key.split(".")
        if parts[0] == "prob":
            val = a.item() if a.ndim == 0 else a
            if len(parts) == 3:
                prob.setdefault(parts[1], {})[parts[2]] = val
            else:
                prob[parts[1]] = val
        elif parts[0].startswith("step"):
            steps[int(parts[0][4:])][parts[1]] = a
        elif parts[0] == "meta":
            meta[parts[1]] = a.item() if a.ndim == 0 else a
    return prob, steps, meta


def load(path):
    with np.load(path, allow_pickle=False) as z:
        return unpack(z)
