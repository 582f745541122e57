"""d2f_step_noalloc: the implicit step for callers that cannot allocate device memory.

Such a caller — a host that forbids cudaMalloc once it runs, or a plugin that is handed
plain device pointers by its host — passes its inputs and outputs in the descriptor and
gets the step's scratch from the library's static device array. Its results must equal
those of the ordinary entry point (d2f_step, caller-allocated scratch) on the same inputs,
call after call: the static array keeps the previous call's contents, which must not leak
into the next. Collected last so that a failure here cannot hide the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import load_fixture, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _pair(name):
    from diff_2d_fem_gb300.device import DeviceSolver
    prob, steps, _ = load_fixture(name)
    return prob, steps, DeviceSolver(prob, precision="fp64"), DeviceSolver(prob, precision="fp64")


@pytest.mark.parametrize("name", ["strip_small", "grip"])
def test_noalloc_matches_allocating_step_two_calls(name):
    prob, steps, a, b = _pair(name)
    for k in range(2):
        st = steps[k]
        if "bc_target" in st:
            full = np.asarray(prob["x"], np.float64).copy()
            full[np.asarray(prob["bc_idx"])] = st["bc_target"]
            a.set_targets(full)
            b.set_targets(full)
        a.step()
        b.step_noalloc()
        ia, _, sa = a.stats()
        ib, _, sb = b.stats()
        assert (sa == 0).all() and (sb == 0).all()
        e = rel_err(b.get_x(), a.get_x())
        assert e < TOL, f"{name} call {k}: no-alloc step differs by {e:.3e}"
        assert np.array_equal(ia, ib)
    a.close()
    b.close()


def test_noalloc_refuses_a_batch_beyond_its_scratch():
    from diff_2d_fem_gb300 import _lib
    prob, steps, a, b = _pair("strip_small")
    d = _lib.SceneDesc()
    C.pointer(d)[0] = b.desc
    d.T = 2_000_000                     # would need ~320 MB of per-triangle scratch
    L = _lib.load()
    rc = L.d2f_step_noalloc(C.byref(d), None)
    assert rc == -1
    msg = L.d2f_last_error().decode()
    assert "static scratch holds" in msg and str(_lib.NOALLOC_SCRATCH_BYTES) in msg
    a.close()
    b.close()
