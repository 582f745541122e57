"""The host-side scene assembly against the reference's own: each golden fixture stores
the solver problem exactly as the reference builds it; building the same scene with this
package's Model / ImplicitIntegrator must give the same arrays."""
import numpy as np
import pytest

import scenes
from diff_2d_fem_gb300 import scene as S
from helpers import fixtures, load_fixture, package_ns

NAMES = [n for n in fixtures() if n in scenes.SCENES]


def _build(name):
    sc = scenes.SCENES[name](package_ns(device="cpu"))
    if sc["command"] is not None:
        sc["command"](0)
    return S.solver_problem(sc["model"], sc["integ"], sc["dt"]), sc


def _same(a, b, key):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, f"{key}: shape {a.shape} vs {b.shape}"
    if a.dtype.kind in "iub" or b.dtype.kind in "iub":
        assert np.array_equal(a.astype(np.int64), b.astype(np.int64)), f"{key} differs"
    else:
        assert np.array_equal(a.astype(np.float64), b.astype(np.float64)), \
            f"{key} differs by {np.abs(a.astype(np.float64) - b.astype(np.float64)).max():.3e}"


@pytest.mark.parametrize("name", NAMES)
def test_problem_matches_reference(name):
    ref, _, _ = load_fixture(name)
    mine, _ = _build(name)
    for key, val in ref.items():
        if key in ("ipc", "tendon", "affine", "rigid", "springs", "pressure"):
            assert mine.get(key) is not None, f"{key} missing"
            for kk, vv in val.items():
                if vv is None:
                    continue
                _same(mine[key][kk], vv, f"{key}.{kk}")
        elif np.ndim(val) == 0:
            assert float(mine[key]) == float(val), f"{key}: {mine[key]} vs {val}"
        else:
            _same(mine[key], val, key)
    for key in ("ipc", "tendon", "affine", "rigid", "fext", "springs", "pressure"):
        assert (key in ref) == (mine.get(key) is not None), f"{key} presence differs"


@pytest.mark.parametrize("name", [n for n in NAMES if scenes.SCENES[n](package_ns(device="cpu"))["command"]])
def test_commands_match_reference(name):
    """The per-step commands this package's Model produces for the scene (kinematic targets
    from set_kinematic_target / set_kinematic_pose, tendon tensions) are the reference's,
    step by step, bit for bit."""
    ref, steps, _ = load_fixture(name)
    sc = scenes.SCENES[name](package_ns(device="cpu"))
    m = sc["model"]
    bc = np.asarray(ref["bc_idx"], np.int64)
    for k, st in enumerate(steps):
        sc["command"](k)
        if "bc_target" in st:
            _same(np.asarray(m._targets, np.float64)[bc], st["bc_target"], f"step {k} bc_target")
        if "Tcmd" in st:
            _same(np.array([t.tension for t in m._tendons]), st["Tcmd"], f"step {k} Tcmd")


def test_min_distance_refuses_touching_bodies():
    """Touching bodies are refused before the first step (implicit/integrator.py:288-294)."""
    import diff_2d_fem_gb300 as D
    m = D.Model(device="cpu")
    m.add_soft_body(np.ones((2, 2)), physical_size=(0.002, 0.002), center=(0.0, 0.0))
    m.add_soft_body(np.ones((2, 2)), physical_size=(0.002, 0.002), center=(0.002, 0.0))
    m.finalize()
    prob = S.solver_problem(m, D.ImplicitIntegrator(), 1e-3)
    gap = S.min_distance(prob)
    assert gap.min() <= 0.0


def test_overlap_is_refused():
    import diff_2d_fem_gb300 as D
    m = D.Model(device="cpu")
    m.add_soft_body(np.ones((4, 4)), physical_size=(0.004, 0.004), center=(0.0, 0.0))
    m.add_soft_body(np.ones((4, 4)), physical_size=(0.004, 0.004), center=(0.001, 0.0))
    with pytest.raises(ValueError, match="overlap"):
        m.finalize()
