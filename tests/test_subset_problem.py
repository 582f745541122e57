"""The autotuner times launch shapes on a sample of a batch's scenes (scene.subset_problem).
A sampled scene must be exactly the scene it was sampled from: on the oracle, every scene of
a subset, in any order, steps bit for bit as it does inside the full batch. No GPU."""
import numpy as np
import pytest

import oracle
from diff_2d_fem_gb300 import scene, tune
from helpers import load_fixture


def _env_x(prob, x, e):
    return np.asarray(x)[np.asarray(prob["node2env"]) == e]


@pytest.mark.parametrize("name,envs", [("body_mu", [1]), ("body_mu", [1, 0]), ("strip_small", [0])])
def test_subset_scenes_step_as_in_the_batch(name, envs):
    prob, steps, _ = load_fixture(name)
    full = oracle.OracleSolver(prob)
    sub_prob = scene.subset_problem(prob, envs)
    sub = oracle.OracleSolver(sub_prob)
    bc_full = np.asarray(prob["bc_idx"], np.int64)
    for st in steps:
        if "bc_target" in st:
            full.set_bc_target(st["bc_target"])
            tgt = np.asarray(prob["x"], np.float64).copy()
            tgt[bc_full] = st["bc_target"]
            order = np.concatenate([np.flatnonzero(np.asarray(prob["node2env"]) == e) for e in envs])
            sub.set_bc_target(tgt[order][np.asarray(sub_prob["bc_idx"], np.int64)])
        full.step()
        sub.step()
        for k, e in enumerate(envs):
            assert np.array_equal(_env_x(sub_prob, sub.x, k), _env_x(prob, full.x, e)), (name, e)


def test_size_bucket():
    prob, _, _ = load_fixture("body_mu")
    b = tune.size_bucket(prob)
    assert b & (b - 1) == 0 and b > 0


@pytest.mark.parametrize("name", ["grip", "tendon", "actuators", "rigid_region"])
def test_a_one_scene_subset_is_the_scene(name):
    """Affine bodies, tendons, springs and pressure boundaries survive the slicing: the
    subset of the only scene steps bit for bit as the scene."""
    prob, steps, _ = load_fixture(name)
    full, sub = oracle.OracleSolver(prob), oracle.OracleSolver(scene.subset_problem(prob, [0]))
    for st in steps:
        for s in (full, sub):
            if "bc_target" in st:
                s.set_bc_target(st["bc_target"])
            if "Tcmd" in st:
                s.set_tendon(Tcmd=st["Tcmd"])
            s.step()
        assert np.array_equal(sub.x, full.x)


def test_a_sampled_scene_with_every_term_is_itself():
    """Three environments, each with a rigid block, a tendon-driven soft arm, a pressurised
    cavity, a pin and a spring (different sizes per environment): the subset [2, 0] steps
    each of its scenes bit for bit as inside the full batch."""
    import warnings
    from diff_2d_fem_gb300 import ImplicitIntegrator, Model
    px = 0.5e-3
    m = Model()
    m.add_ground(0.0, mu=0.6)
    for e in range(3):
        mk = np.ones((6, 8 + 2 * e), np.uint8)
        mk[2:4, 3:5] = 0
        arm = m.add_soft_body(mk, physical_size=((8 + 2 * e) * px, 6 * px), center=(0.0, 3 * px + 0.9 * px / 8),
                              E=1.0e6, nu=0.40, density=1100.0, env_id=e)
        m.add_affine_body(np.ones((3, 3), np.uint8), physical_size=(3 * px, 3 * px),
                          center=(0.0, 6 * px + 1.5 * px + 0.2 * px), density=900.0, env_id=e)
    m.finalize()
    m.gravity = (0.0, -9.81)
    for e in range(3):
        X = m.rest_x(2 * e)
        td = m.add_tendon(2 * e, through=[(x, 0.0015) for x in np.unique(np.round(X[:, 0], 9))[1:-1]])
        m.set_tendon_tension(td, 2.0 + e)
        ch = m.add_pressure_chambers(2 * e)
        m.set_pressure(ch[0], 1.0e4 * (e + 1))
        m.add_pin(2 * e, (X[:, 0].min(), X[:, 1].max()), stiffness=1.0e6)
        m.add_spring(2 * e, (X[:, 0].max(), X[:, 1].max()), point_b=(X[:, 0].max() + px, X[:, 1].max() + px),
                     stiffness=1.0e4, rest_length=0.5 * px)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob = scene.solver_problem(m, ImplicitIntegrator(max_iter=150), 1e-3)
    for key in ("affine", "tendon", "springs", "pressure"):
        assert prob.get(key) is not None, key
    envs = [2, 0]
    full = oracle.OracleSolver(prob)
    sub_prob = scene.subset_problem(prob, envs)
    sub = oracle.OracleSolver(sub_prob)
    for _ in range(4):
        full.step()
        sub.step()
    for k, e in enumerate(envs):
        assert np.array_equal(_env_x(sub_prob, sub.x, k), _env_x(prob, full.x, e)), e
