"""CUDA path vs the reference's golden vectors and the CPU oracle, through the C ABI.

Plain FP64: node positions within 1e-9 of the reference's (relative to the largest
coordinate), every step. The CUDA path sums in a different order than the reference's
serial atomics and forms the Jacobi diagonal in closed form (algebraically equal), so it
agrees to rounding, not bit for bit.
Mixed precision: within 1e-6 relative of the FP64 result.
"""
import numpy as np
import pytest

import oracle
import scenes
from helpers import fixtures, load_fixture, package_ns, rel_err

pytestmark = pytest.mark.gpu

# simplest scenes first, so that the first failure points at the least machinery
_ORDER = ["strip_small", "strip_cfg1", "tendon", "line_search", "batch_colliders", "grip", "rigid_region",
          "actuators", "body_mu", "kinematic_pose", "tilted_plane", "tendon_length", "mesh_cantilever", "mesh_bodies", "mesh_chamber"]
GPU_SCENES = [n for n in _ORDER if n in fixtures()] + [n for n in fixtures() if n not in _ORDER]
TOL_FP64 = 1e-9
TOL_MIXED = 1e-6


def _run_device(prob, steps, precision):
    from diff_2d_fem_gb300.device import DeviceSolver
    s = DeviceSolver(prob, precision=precision)
    out = []
    for st in steps:
        if "bc_target" in st:
            full = np.asarray(prob["x"], np.float64).copy()
            full[np.asarray(prob["bc_idx"])] = st["bc_target"]
            s.set_targets(full)
        if "Tcmd" in st:
            s.set_tendons(Tcmd=st["Tcmd"])
        s.step()
        it, ac, status = s.stats()
        assert (status == 0).all(), f"device status {status}"
        out.append((s.get_x(), it))
    s.close()
    return out


@pytest.mark.parametrize("name", GPU_SCENES)
def test_fp64_matches_reference(name):
    prob, steps, _ = load_fixture(name)
    res = _run_device(prob, steps, "fp64")
    for k, ((x, it), st) in enumerate(zip(res, steps)):
        e = rel_err(x, st["x"])
        assert e < TOL_FP64, f"{name} step {k}: rel err {e:.3e} (iters {it.tolist()} vs {st['iters'].tolist()})"


@pytest.mark.parametrize("name", ["strip_small", "strip_cfg1", "grip", "tendon"])
def test_mixed_close_to_fp64_when_converged(name):
    """Mixed precision against FP64 on CONVERGED steps: the iteration cap is lifted so both
    run to the reference's energy tolerance; a step cut off by the cap stops at an iterate
    that depends on the rounding of every earlier iteration, in either precision."""
    prob, steps, _ = load_fixture(name)
    prob = dict(prob)
    prob["iter_max"] = 3000
    prob["eps"] = 1e-13       # the default 1e-10 leaves ~sqrt(eps) of each step's motion
    r64 = _run_device(prob, steps, "fp64")
    rmx = _run_device(prob, steps, "mixed")
    for k, ((x64, _), (xmx, it)) in enumerate(zip(r64, rmx)):
        e = rel_err(xmx, x64)
        assert e < TOL_MIXED, f"{name} step {k}: rel err {e:.3e} (iters {it.tolist()})"


def test_config1_strip_200_steps_matches_oracle():
    """The single-scene headline configuration in full: 200 steps of the strip on the
    ground through the public API (Model / ImplicitIntegrator.simulate), against the
    oracle run on the same problem."""
    from diff_2d_fem_gb300 import scene as S
    sc = scenes.strip_cfg1(package_ns(), steps=200)
    m, integ, dt = sc["model"], sc["integ"], sc["dt"]
    prob = S.solver_problem(m, integ, dt)
    ref = oracle.OracleSolver(prob)
    for k in range(sc["steps"]):
        integ.simulate(m, dt)
        ref.step()
    x = m.get_x()
    e = rel_err(x, ref.x)
    assert e < TOL_FP64, f"rel err {e:.3e} after 200 steps"
    assert np.array_equal(integ.stats(m)["iters"], ref.state["iters"]) or e < TOL_FP64
