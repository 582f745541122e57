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


def test_size_bucket_and_refusals():
    prob, _, _ = load_fixture("body_mu")
    b = tune.size_bucket(prob)
    assert b & (b - 1) == 0 and b > 0
    p2, _, _ = load_fixture("tendon")
    with pytest.raises(NotImplementedError):
        scene.subset_problem(p2, [0])
