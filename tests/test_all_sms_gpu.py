"""The mixed step with every SM on one scene (blocks_per_scene = D2F_ALL_SMS): a cooperative
launch of one 512-thread block per SM, every phase split over all of them, phases ended by a
grid-wide barrier, reductions and the contact list's offsets and ACCD replay exchanged through
global memory in block order; scenes of a batch are taken in turn.

Checked like the cluster path: on converged steps against FP64 (1e-6 relative to the
coordinates on the reference fixtures and slabs; 1e-8 and the IPC energy to 5e-6 on the
contact-heavy state), and a batch of environments stepped in turn equal to FP64.
"""
import warnings

import numpy as np
import pytest

import oracle
from helpers import load_fixture, rel_err

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-6
ALL_SMS = -1


def _run(prob, steps, precision, cs=0):
    from diff_2d_fem_gb300.device import DeviceSolver
    import torch
    s = DeviceSolver(prob, precision=precision, blocks_per_scene=cs)
    if cs == ALL_SMS:
        nsm = torch.cuda.get_device_properties(0).multi_processor_count
        assert s.launch_shape() == (nsm, 512, nsm)
    out = []
    for st in steps:
        if "bc_target" in st:
            full = np.asarray(prob["x"], np.float64).copy()
            full[np.asarray(prob["bc_idx"])] = st["bc_target"]
            s.set_targets(full)
        if "Tcmd" in st:
            s.set_tendons(Tcmd=st["Tcmd"])
        s.step()
        _, _, status = s.stats()
        assert (status == 0).all(), f"device status {status}"
        out.append(s.get_x())
    s.close()
    return out


@pytest.mark.parametrize("name", ["strip_small", "grip", "tendon", "batch_colliders"])
def test_all_sms_matches_fp64_when_converged(name):
    """Ground contact and friction (strip), kinematic grip with IPC contact and an affine block
    (grip), tendons and rigid modes (tendon), three environments on colliders taken in turn
    (batch_colliders): every SM on the scene, run to convergence, against FP64."""
    prob, steps, _ = load_fixture(name)
    prob = dict(prob)
    prob["iter_max"] = 3000
    prob["eps"] = 1e-13
    r64 = _run(prob, steps, "fp64")
    rall = _run(prob, steps, "mixed", ALL_SMS)
    for k, (x64, xa) in enumerate(zip(r64, rall)):
        e = rel_err(xa, x64)
        assert e < TOL_MIXED, f"{name} step {k}: rel err {e:.3e}"


def test_all_sms_contact_converged_matches_fp64():
    """The contact-heavy state (a block gripped between two pads): one step run to
    convergence on every SM, within 1e-8 of FP64 and the IPC energy within 5e-6 relative
    (FP32 barrier forces between bodies, as test_contact_batch explains)."""
    from test_contact_batch import _contact_state
    from diff_2d_fem_gb300.device import DeviceSolver
    p2, tg, x0 = _contact_state()
    p2["iter_max"], p2["eps"] = 40000, 0.0
    xs = {}
    for prec, cs in (("fp64", 0), ("mixed", ALL_SMS)):
        s = DeviceSolver(p2, precision=prec, blocks_per_scene=cs)
        s.set_targets(tg)
        s.step()
        _, _, st = s.stats()
        assert (st == 0).all(), prec
        xs[prec] = s.get_x()
        s.close()
    assert rel_err(xs["mixed"], xs["fp64"]) < 1e-8
    o = oracle.OracleSolver(p2)
    e64 = o.ipc_energy(xs["fp64"], x0)[0]
    emx = o.ipc_energy(xs["mixed"], x0)[0]
    assert e64 > 0.0
    assert abs(emx - e64) / e64 < 5e-6


def test_all_sms_hashed_slab_matches_fp64():
    """A slab with 4792 boundary nodes (the contact list through the spatial hash, every
    block its own table) and six discs resting within the barrier distance on it: three
    converged steps on every SM agree with FP64."""
    from diff_2d_fem_gb300 import workloads, scene, ImplicitIntegrator
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        m, kw, dt = workloads.slab_with_holes(1, seed=2, H=48, W=640, n_holes=60, n_discs=6,
                                              drop=(20e-6, 40e-6))
        prob = scene.solver_problem(m, ImplicitIntegrator(**kw), dt)
    assert len(prob["bnd"]) >= 4096
    prob["iter_max"], prob["eps"] = 3000, 1e-13
    steps = [{}, {}, {}]
    x64 = _run(prob, steps, "fp64")[-1]
    xa = _run(prob, steps, "mixed", ALL_SMS)[-1]
    assert rel_err(xa, x64) < TOL_MIXED
