"""The backtracking energy line search on the device (PNCG2DSolver line_search,
implicit/solver.py:397-425), in both precisions and with affine bodies (AffineBodies.save /
trial, implicit/affine.py:383-389).

The reference's own line_search fixture never halves a step (its runs with and without the
line search are identical), so a second scene forces halvings: a cantilever with a rigid
region (an affine piece) whose clamped column is moved by 1 mm in one step, far more than a
model step can follow. Its runs with and without the line search differ by tens of percent on
the oracle, so the halving and the affine trial state are exercised.

FP64: the device against the oracle on the same problem, 1e-9 of the coordinates, every step.
Mixed: against the FP64 device on converged steps (iteration cap lifted, energy tolerance
1e-13), 1e-6 of the coordinates: a step cut off by the cap stops at an iterate that depends
on the rounding of every earlier iteration, in either precision.
"""
import numpy as np
import pytest

import oracle
from helpers import load_fixture, rel_err

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-9
TOL_MIXED = 1e-6


def _jump_problem(line_search, max_iter=80, eps=None):
    """A 4 x 8-pixel cantilever (4 x 2 mm, E 0.5 MPa, nu 0.45) whose two right columns are a
    rigid region, clamped at its left column; the clamp's targets, per step k = 1, 2, 3, are
    its rest positions moved by (0.5, 1) mm x k."""
    import diff_2d_fem_gb300 as D
    from diff_2d_fem_gb300 import scene as S
    m = D.Model()
    h = m.add_soft_body(np.ones((4, 8), np.uint8), physical_size=(0.004, 0.002), center=(0.0, 0.003),
                        E=0.5e6, nu=0.45, density=1100.0)
    m.finalize()
    m.gravity = (0.0, -9.81)
    region = np.zeros((4, 8), bool)
    region[:, 6:] = True
    m.add_affine_region(h, region)
    X = m.rest_x(h)
    m.set_kinematic_constraint(h, np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0])
    integ = D.ImplicitIntegrator(line_search=line_search, rigid_modes=False, max_iter=max_iter, eps=eps,
                                 self_collision=False)
    prob = S.solver_problem(m, integ, 2e-3)
    t0 = np.asarray(prob["x"], np.float64)[np.asarray(prob["bc_idx"])]
    targets = [t0 + np.array([0.5e-3, 1.0e-3]) * (k + 1) for k in range(3)]
    return prob, targets


def _full(prob, t):
    full = np.asarray(prob["x"], np.float64).copy()
    full[np.asarray(prob["bc_idx"])] = t
    return full


def _device(prob, targets, precision):
    from diff_2d_fem_gb300.device import DeviceSolver
    s = DeviceSolver(prob, precision=precision)
    out = []
    for t in targets:
        if t is not None:
            s.set_targets(_full(prob, t))
        s.step()
        it, ac, st = s.stats()
        assert (st == 0).all(), f"device status {st}"
        out.append((s.get_x(), it))
    s.close()
    return out


def _oracle(prob, targets):
    r = oracle.OracleSolver(prob)
    out = []
    for t in targets:
        if t is not None:
            r.set_bc_target(t)
        r.step()
        out.append((r.x.copy(), r.state["iters"].copy()))
    return out


def test_the_jump_scene_halves_steps():
    """The scene is a test of the halving: on the oracle its line-search run and its plain run
    part by far more than any tolerance used here, at six iterations a step."""
    pl, tg = _jump_problem(False, max_iter=6)
    pls, _ = _jump_problem(True, max_iter=6)
    a, b = _oracle(pl, tg)[-1][0], _oracle(pls, tg)[-1][0]
    assert rel_err(b, a) > 1e-2


def test_fp64_line_search_with_affine_region_matches_oracle():
    """Six iterations a step: the halvings happen from the second step on, and the device and
    the oracle take the same ones (over a long unconverged run a decision taken at rounding
    distance from the threshold could part them)."""
    prob, tg = _jump_problem(True, max_iter=6)
    ref = _oracle(prob, tg)
    dev = _device(prob, tg, "fp64")
    for k, ((x, it), (xr, itr)) in enumerate(zip(dev, ref)):
        e = rel_err(x, xr)
        assert e < TOL_FP64, f"step {k}: rel err {e:.3e} (iters {it.tolist()} vs {itr.tolist()})"


def test_mixed_line_search_with_affine_region_matches_fp64_converged():
    prob, tg = _jump_problem(True, max_iter=4000, eps=1e-13)
    r64 = _device(prob, tg, "fp64")
    rmx = _device(prob, tg, "mixed")
    for k, ((x64, _), (xmx, it)) in enumerate(zip(r64, rmx)):
        e = rel_err(xmx, x64)
        assert e < TOL_MIXED, f"step {k}: rel err {e:.3e} (iters {it.tolist()})"


def _fixture_steps(steps):
    return [st.get("bc_target") for st in steps]


@pytest.mark.parametrize("name", ["line_search", "grip"])
def test_fp64_line_search_fixture_scenes_match_oracle(name):
    """The reference's line_search fixture (IPC contact on a disc), and the grip fixture (an
    affine block between two pads) run with the line search on: FP64 device against the
    oracle with the line search on."""
    prob, steps, _ = load_fixture(name)
    prob = dict(prob)
    prob["line_search"] = 1
    tg = _fixture_steps(steps)
    ref = _oracle(prob, tg)
    dev = _device(prob, tg, "fp64")
    for k, ((x, it), (xr, itr)) in enumerate(zip(dev, ref)):
        e = rel_err(x, xr)
        assert e < TOL_FP64, f"{name} step {k}: rel err {e:.3e} (iters {it.tolist()} vs {itr.tolist()})"


@pytest.mark.parametrize("name", ["line_search", "grip"])
def test_mixed_line_search_fixture_scenes_match_fp64_converged(name):
    prob, steps, _ = load_fixture(name)
    prob = dict(prob)
    prob["line_search"] = 1
    prob["iter_max"] = 3000
    prob["eps"] = 1e-13
    tg = _fixture_steps(steps)
    r64 = _device(prob, tg, "fp64")
    rmx = _device(prob, tg, "mixed")
    for k, ((x64, _), (xmx, it)) in enumerate(zip(r64, rmx)):
        e = rel_err(xmx, x64)
        assert e < TOL_MIXED, f"{name} step {k}: rel err {e:.3e} (iters {it.tolist()})"


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
