"""Shared helpers of the test suite."""
from __future__ import annotations

import glob
import os
import types

import numpy as np

from conftest import GOLDEN

import fixture_io  # noqa: E402  (tests/golden)


def fixtures():
    """The forward-step fixtures (the adjoint ones, adjoint_*.npz, have their own tests)."""
    names = (os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    return sorted(n for n in names if not n.startswith("adjoint_"))


def load_fixture(name):
    return fixture_io.load(os.path.join(GOLDEN, f"{name}.npz"))


def package_ns(device="cuda"):
    import diff_2d_fem_gb300 as D
    return types.SimpleNamespace(Model=D.Model, ImplicitIntegrator=D.ImplicitIntegrator, device=device,
                                 mask_to_mesh=D.mask_to_mesh)


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def tile_problem(prob, n):
    """n independent copies of a one-environment problem as one batch (environments 0..n-1).
    Covers nodes, triangles, boundary nodes, kinematic nodes, external force and tendons."""
    if int(prob["B"]) != 1:
        raise ValueError("tile_problem takes a one-environment problem")
    for k in ("ipc", "affine", "rigid"):
        if prob.get(k) is not None:
            raise ValueError(f"tile_problem does not cover {k}")
    N = np.asarray(prob["x"]).shape[0]
    out = {k: v for k, v in prob.items() if np.ndim(v) == 0 and not isinstance(v, dict)}
    out["B"] = n
    for k in ("x", "v", "mass", "free", "rest", "fext"):
        if prob.get(k) is not None:
            out[k] = np.concatenate([np.asarray(prob[k])] * n)
    out["node2env"] = np.repeat(np.arange(n), N).astype(np.int32)
    tri = np.asarray(prob["tri"], np.int64)
    out["tri"] = np.concatenate([tri + e * N for e in range(n)]).astype(np.int32)
    for k in ("Bm", "area", "mu", "lam"):
        out[k] = np.concatenate([np.asarray(prob[k])] * n)
    out["tri2env"] = np.repeat(np.arange(n), len(tri)).astype(np.int32)
    bnd = np.asarray(prob["bnd"], np.int64)
    out["bnd"] = np.concatenate([bnd + e * N for e in range(n)]).astype(np.int32)
    out["b2e"] = np.repeat(np.arange(n), len(bnd)).astype(np.int32)
    bc = np.asarray(prob.get("bc_idx", np.zeros(0)), np.int64)
    out["bc_idx"] = np.concatenate([bc + e * N for e in range(n)]).astype(np.int32)
    out["colliders"] = np.asarray(prob["colliders"])
    td = prob.get("tendon")
    if td is not None:
        ne, nt = len(td["node"]), len(td["t2env"])
        sh = lambda a, e, m: np.where(np.asarray(a) >= 0, np.asarray(a) + e * m, -1)
        out["tendon"] = dict(
            node=np.concatenate([np.asarray(td["node"]) + e * N for e in range(n)]),
            prv=np.concatenate([sh(td["prv"], e, ne) for e in range(n)]),
            nxt=np.concatenate([sh(td["nxt"], e, ne) for e in range(n)]),
            tid=np.concatenate([np.asarray(td["tid"]) + e * nt for e in range(n)]),
            t2env=np.repeat(np.arange(n), nt),
            **{k: np.concatenate([np.asarray(td[k])] * n) for k in ("stiff", "L0", "Tcmd")})
    return out
