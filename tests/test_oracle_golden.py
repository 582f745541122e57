"""The CPU oracle against the golden vectors recorded from the reference's own kernels.

The fixtures in tests/golden/ were produced by running the reference's Model and
ImplicitIntegrator unchanged, kernel source included, through a serial Warp stand-in
(tests/golden/make_golden.py). The oracle restates the same arithmetic in C in the same
order, so the comparison is exact: node positions bit for bit, iteration counts equal.
"""
import numpy as np
import pytest

import oracle
from helpers import fixtures, load_fixture

NAMES = fixtures()


def test_fixtures_present():
    assert {"strip_small", "batch_colliders", "grip", "tendon", "line_search", "strip_cfg1",
            "rigid_region", "mesh_cantilever", "mesh_bodies", "actuators", "body_mu", "kinematic_pose", "mesh_chamber", "tilted_plane", "tendon_length"} <= set(NAMES)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_reference_bit_for_bit(name):
    prob, steps, meta = load_fixture(name)
    s = oracle.OracleSolver(prob)
    for k, st in enumerate(steps):
        if "bc_target" in st:
            s.set_bc_target(st["bc_target"])
        if "Tcmd" in st:
            s.set_tendon(Tcmd=st["Tcmd"])
        s.step()
        assert np.array_equal(s.state["iters"], st["iters"]), f"{name} step {k}: iterations differ"
        assert np.array_equal(s.x, st["x"]), \
            f"{name} step {k}: positions differ by {np.abs(s.x - st['x']).max():.3e}"
        assert np.array_equal(s.v, st["v"])
        if "q" in st:
            assert np.array_equal(s.state["a_q"], st["q"])


def test_fixtures_exercise_contact():
    """The scenes are not vacuous: contact, friction and sweeps actually happen."""
    prob, steps, _ = load_fixture("grip")
    x0 = np.asarray(prob["x"])
    assert np.abs(steps[-1]["x"] - x0).max() > 1e-5
    assert max(int(st["iters"].max()) for st in steps) > 40
    prob, steps, _ = load_fixture("strip_cfg1")
    y = steps[-1]["x"][:, 1]
    assert y.min() < float(prob["dhat"]), "the strip should have landed within the barrier's reach"
    prob, steps, _ = load_fixture("rigid_region")
    q = steps[-1]["q"][0]
    A = np.array([[q[1], q[2]], [q[4], q[5]]])
    assert abs(np.arctan2(A[1, 0] - A[0, 1], A[0, 0] + A[1, 1])) > 0.03, "the rigid piece should turn"
    assert np.abs(A.T @ A - np.eye(2)).max() < 1e-5, "and stay rigid"
