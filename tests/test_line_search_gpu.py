"""The backtracking energy line search on the device (PNCG2DSolver line_search,
implicit/solver.py:397-425), in both precisions and with affine bodies (AffineBodies.save /
trial, implicit/affine.py:383-389).

At its default tolerance the line search never halves a step of the reference's fixtures
(their runs with and without it are identical): these run the path (energies, the saved
state, the trial point) with no halving, FP64 against the oracle within 1e-9 every step.
With ls_tol = 0 every energy increase halves the step, which happens on the scenes with
affine bodies (grip, rigid_region, mesh_bodies: their runs with and without the line search
part on the oracle), and those are compared on converged steps (iteration cap lifted,
energy tolerance 1e-13), the device FP64 step against the oracle's within 1e-6 of the
coordinates: halvings taken on rounding-level energy differences near convergence differ
between the two sums' orders, so the unconverged iterates may part, but the steps end at the
same equilibrium. Mixed precision against FP64 on converged steps, within 1e-6, at the
default tolerance and on mesh_bodies at ls_tol = 1e-12, where the oracle halves as well.
"""
import numpy as np
import pytest

import oracle
from helpers import load_fixture, rel_err

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-9
TOL_CONVERGED = 1e-6
HALVING_SCENES = ["grip", "rigid_region", "mesh_bodies"]


def _device(prob, steps, precision):
    from diff_2d_fem_gb300.device import DeviceSolver
    s = DeviceSolver(prob, precision=precision)
    out = []
    for st in steps:
        if st.get("bc_target") is not None:
            full = np.asarray(prob["x"], np.float64).copy()
            full[np.asarray(prob["bc_idx"])] = st["bc_target"]
            s.set_targets(full)
        s.step()
        it, ac, status = s.stats()
        assert (status == 0).all(), f"device status {status}"
        out.append((s.get_x(), it))
    s.close()
    return out


def _oracle(prob, steps):
    r = oracle.OracleSolver(prob)
    out = []
    for st in steps:
        if st.get("bc_target") is not None:
            r.set_bc_target(st["bc_target"])
        r.step()
        out.append((r.x.copy(), r.state["iters"].copy()))
    return out


def _with(name, **kw):
    prob, steps, _ = load_fixture(name)
    prob = dict(prob, **kw)
    return prob, steps


@pytest.mark.parametrize("name", ["line_search", "grip", "rigid_region", "mesh_bodies"])
def test_fp64_line_search_without_halving_matches_oracle(name):
    prob, steps = _with(name, line_search=1)
    ref = _oracle(prob, steps)
    dev = _device(prob, steps, "fp64")
    for k, ((x, it), (xr, itr)) in enumerate(zip(dev, ref)):
        e = rel_err(x, xr)
        assert e < TOL_FP64, f"{name} step {k}: rel err {e:.3e} (iters {it.tolist()} vs {itr.tolist()})"


@pytest.mark.parametrize("name", HALVING_SCENES)
def test_zero_tolerance_halves_steps_on_the_oracle(name):
    """The scenes are tests of the halving: at their own budgets, the line search with
    ls_tol = 0 and no line search part by more than 1e-7 on the oracle."""
    p0, steps = _with(name, line_search=0)
    p1, _ = _with(name, line_search=1, ls_tol=0.0)
    a, b = _oracle(p0, steps)[-1][0], _oracle(p1, steps)[-1][0]
    assert rel_err(b, a) > 1e-7


@pytest.mark.parametrize("name", HALVING_SCENES)
def test_fp64_halving_line_search_converges_with_the_oracle(name):
    prob, steps = _with(name, line_search=1, ls_tol=0.0, iter_max=3000, eps=1e-13)
    ref = _oracle(prob, steps)
    dev = _device(prob, steps, "fp64")
    for k, ((x, it), (xr, itr)) in enumerate(zip(dev, ref)):
        e = rel_err(x, xr)
        assert e < TOL_CONVERGED, f"{name} step {k}: rel err {e:.3e} (iters {it.tolist()} vs {itr.tolist()})"


@pytest.mark.parametrize("name,ls_tol", [("line_search", 1e-7), ("grip", 1e-7), ("rigid_region", 1e-7),
                                         ("mesh_bodies", 1e-7), ("mesh_bodies", 1e-12)])
def test_mixed_line_search_matches_fp64_converged(name, ls_tol):
    """The mixed kernel's line search (energies in FP64 at x_b + r) against FP64 on converged
    steps; on mesh_bodies at ls_tol = 1e-12 the oracle halves steps too. (At ls_tol = 0 the
    mixed step halves on the FP32 rounding of its positions near convergence and stalls there:
    a tolerance below the mixed positions' energy resolution is not a setting for it.)"""
    prob, steps = _with(name, line_search=1, iter_max=3000, eps=1e-13, ls_tol=ls_tol)
    r64 = _device(prob, steps, "fp64")
    rmx = _device(prob, steps, "mixed")
    for k, ((x64, _), (xmx, it)) in enumerate(zip(r64, rmx)):
        e = rel_err(xmx, x64)
        assert e < TOL_CONVERGED, f"{name} step {k}: rel err {e:.3e} (iters {it.tolist()})"


def test_line_search_reaches_the_device_through_the_integrator():
    """ImplicitIntegrator(line_search=True) in both precisions builds solvers with the line
    search on (no refusal for mixed precision or affine bodies)."""
    import diff_2d_fem_gb300 as D
    for precision in ("fp64", "mixed"):
        m = D.Model()
        m.add_ground(0.0, mu=0.5)
        m.add_affine_body(np.ones((3, 3), np.uint8), physical_size=(0.0015, 0.0015), center=(0.0, 0.001),
                          density=1100.0)
        m.finalize()
        m.gravity = (0.0, -9.81)
        integ = D.ImplicitIntegrator(line_search=True, precision=precision)
        for _ in range(3):
            integ.simulate(m, 2e-3)
        st = integ.stats(m)
        assert (st["status"] == 0).all()
        assert np.isfinite(m.get_x()).all()
