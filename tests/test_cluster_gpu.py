"""The mixed step with one thread-block cluster per scene (blocks_per_scene 8, 12 or 16): every
phase split over the cluster's blocks, reductions combined through distributed shared memory,
the contact list compacted across the blocks in pair order, affine bodies spread over the
cluster's warps and threads.

Checked like the block-per-scene mixed path: on converged steps against FP64 (1e-6 relative
to the coordinates on the reference fixtures; 1e-8 and the IPC energy to 5e-6 on the
contact-heavy state), and the library's default choice of clusters for a large scene.
"""
import warnings

import numpy as np
import pytest

import oracle
from helpers import load_fixture, rel_err

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-6


def _run(prob, steps, precision, cs=0):
    from diff_2d_fem_gb300.device import DeviceSolver
    s = DeviceSolver(prob, precision=precision, blocks_per_scene=cs)
    if cs:
        assert s.launch_shape()[2] == cs
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


@pytest.mark.parametrize("cs", [8, 12, 16])
@pytest.mark.parametrize("name", ["strip_small", "grip", "tendon"])
def test_cluster_matches_fp64_when_converged(name, cs):
    """Ground contact and friction (strip), kinematic grip with IPC contact (grip), tendons
    and rigid modes (tendon): a cluster per scene, run to convergence, against FP64."""
    prob, steps, _ = load_fixture(name)
    prob = dict(prob)
    prob["iter_max"] = 3000
    prob["eps"] = 1e-13
    r64 = _run(prob, steps, "fp64")
    rcl = _run(prob, steps, "mixed", cs)
    for k, (x64, xcl) in enumerate(zip(r64, rcl)):
        e = rel_err(xcl, x64)
        assert e < TOL_MIXED, f"{name} cs={cs} step {k}: rel err {e:.3e}"


def test_cluster_contact_converged_matches_fp64():
    """The contact-heavy state (a block gripped between two pads: IPC pairs between bodies
    with friction, an affine body): one step run to convergence with a 16-block cluster,
    within 1e-8 of FP64 and the IPC energy within 5e-6 relative (FP32 barrier forces between
    bodies, as test_contact_batch explains). 40000 iterations: the mixed
    path's FP32 atomic sums make its approach to the answer vary from run to run on this
    ill-conditioned step (1.4e-8 to 4.6e-7 from FP64 seen after 20000 iterations, 2e-11 to
    3e-10 after 40000)."""
    from test_contact_batch import _contact_state
    from diff_2d_fem_gb300.device import DeviceSolver
    p2, tg, x0 = _contact_state()
    p2["iter_max"], p2["eps"] = 40000, 0.0
    xs = {}
    for prec, cs in (("fp64", 0), ("mixed", 16)):
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


def test_large_scenes_default_to_clusters():
    """Two slabs with holes (18.8k nodes each, affine discs above them, lying on the ground):
    the library picks a 16-block cluster per scene by default, and three converged steps
    agree with FP64."""
    from diff_2d_fem_gb300 import workloads, scene, ImplicitIntegrator
    from diff_2d_fem_gb300.device import DeviceSolver
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        m, kw, dt = workloads.slab_with_holes(2, seed=1, H=48, W=384, n_holes=12, n_discs=3)
        prob = scene.solver_problem(m, ImplicitIntegrator(**kw), dt)
    prob["iter_max"], prob["eps"] = 3000, 1e-13
    xs = {}
    for prec in ("fp64", "mixed"):
        s = DeviceSolver(prob, precision=prec)
        assert s.launch_shape()[2] == (16 if prec == "mixed" else 1)
        for _ in range(3):
            s.step()
        _, _, st = s.stats()
        assert (st == 0).all(), prec
        xs[prec] = s.get_x()
        s.close()
    assert rel_err(xs["mixed"], xs["fp64"]) < TOL_MIXED


@pytest.mark.parametrize("cs", [1, 16])
def test_hashed_contact_list_matches_fp64(cs):
    """A slab with 4792 boundary nodes (the contact list built through the spatial hash on a
    cluster; by testing every edge-node pair on a block) and six discs resting within the
    barrier distance on it: three converged steps agree with FP64."""
    from diff_2d_fem_gb300 import workloads, scene, ImplicitIntegrator
    from diff_2d_fem_gb300.device import DeviceSolver
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        m, kw, dt = workloads.slab_with_holes(1, seed=2, H=48, W=640, n_holes=60, n_discs=6,
                                              drop=(20e-6, 40e-6))
        prob = scene.solver_problem(m, ImplicitIntegrator(**kw), dt)
    assert len(prob["bnd"]) >= 4096
    prob["iter_max"], prob["eps"] = 3000, 1e-13
    xs = {}
    for prec, c in (("fp64", 0), ("mixed", cs)):
        s = DeviceSolver(prob, precision=prec, blocks_per_scene=c)
        for _ in range(3):
            s.step()
        _, _, st = s.stats()
        assert (st == 0).all(), prec
        xs[prec] = s.get_x()
        s.close()
    assert rel_err(xs["mixed"], xs["fp64"]) < TOL_MIXED
