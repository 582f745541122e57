"""d2f_step_noalloc: the implicit step for callers that cannot allocate device memory.

Such a caller — a host that forbids cudaMalloc once it runs, or a plugin that is handed
plain device pointers by its host — passes its inputs and outputs in the descriptor and
gets the step's scratch from the library's static device array. Its results must equal
those of the ordinary entry point (d2f_step, caller-allocated scratch) on the same inputs,
call after call: the static array keeps the previous call's contents, which must not leak
into the next, even when the next call is a different problem. Collected last so that a
failure here cannot hide the other tests.

Tolerances: FP64 1e-9 relative, as the other FP64 device tests. Mixed precision 1e-6
relative: its node sums use FP32 atomics whose order is not fixed, so two runs of the same
mixed step agree to rounding, not bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import load_fixture, rel_err

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-9, "mixed": 1e-6}


def _solver(name, precision, blocks_per_scene=0):
    from diff_2d_fem_gb300.device import DeviceSolver
    prob, steps, _ = load_fixture(name)
    return prob, steps, DeviceSolver(prob, precision=precision, blocks_per_scene=blocks_per_scene)


def _command(prob, st, *solvers):
    if "bc_target" in st:
        full = np.asarray(prob["x"], np.float64).copy()
        full[np.asarray(prob["bc_idx"])] = st["bc_target"]
        for s in solvers:
            s.set_targets(full)
    if "Tcmd" in st:
        for s in solvers:
            s.set_tendons(Tcmd=st["Tcmd"])


def _check(name, precision, k, a, b):
    ia, _, sa = a.stats()
    ib, _, sb = b.stats()
    assert (sa == 0).all() and (sb == 0).all(), (sa, sb)
    e = rel_err(b.get_x(), a.get_x())
    assert e < TOL[precision], f"{name} ({precision}) call {k}: the no-alloc step differs by {e:.3e}"
    if precision == "fp64":
        assert np.array_equal(ia, ib), (ia, ib)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["strip_small", "grip"])
def test_noalloc_matches_allocating_step_two_calls(name, precision):
    prob, steps, a = _solver(name, precision)
    _, _, b = _solver(name, precision)
    for k in range(2):
        _command(prob, steps[k], a, b)
        a.step()
        b.step_noalloc()
        _check(name, precision, k, a, b)
    a.close()
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_two_problems_interleaved(precision):
    """grip, strip, grip through the one static array: the strip's call overwrites the
    candidate lists, boundary reference positions and (mixed) base state that the grip's
    calls use; each result must still equal its own allocating solver's."""
    pg, sg_, ga = _solver("grip", precision)
    _, _, gb = _solver("grip", precision)
    ps, ss, sa = _solver("strip_small", precision)
    _, _, sb = _solver("strip_small", precision)
    for k, (name, prob, steps, a, b) in enumerate([("grip", pg, sg_, ga, gb), ("strip_small", ps, ss, sa, sb),
                                                   ("grip", pg, sg_, ga, gb)]):
        kk = 0 if k < 2 else 1
        _command(prob, steps[kk], a, b)
        a.step()
        b.step_noalloc()
        _check(name, precision, k, a, b)
    for s in (ga, gb, sa, sb):
        s.close()


def test_noalloc_on_a_cluster_per_scene():
    """The mixed cluster path (8 blocks a scene) carves its hashed-list and base-state
    scratch out of the same array."""
    from diff_2d_fem_gb300 import _lib
    prob, steps, a = _solver("grip", "mixed", blocks_per_scene=8)
    _, _, b = _solver("grip", "mixed", blocks_per_scene=8)
    assert b.launch_shape()[2] == 8
    for k in range(2):
        _command(prob, steps[k], a, b)
        a.step()
        b.step_noalloc()
        _check("grip", "mixed", k, a, b)
    assert _lib.NOALLOC_SCRATCH_BYTES >= 1 << 20
    a.close()
    b.close()


def test_noalloc_refuses_a_batch_beyond_its_scratch():
    from diff_2d_fem_gb300 import _lib
    prob, steps, b = _solver("strip_small", "fp64")
    d = _lib.SceneDesc()
    C.pointer(d)[0] = b.desc
    d.T = 2_000_000                     # would need ~320 MB of per-triangle scratch
    L = _lib.load()
    rc = L.d2f_step_noalloc(C.byref(d), None)
    assert rc == -1
    msg = L.d2f_last_error().decode()
    assert "static scratch holds" in msg and str(_lib.NOALLOC_SCRATCH_BYTES) in msg
    b.close()
