"""The device adjoint through contact between bodies (IPC barrier terms active at x_k, frozen,
frictionless, each distance's exact Hessian) and affine bodies (the reduced-coordinate system
S^T H S + h^2 K_A) — beyond the reference's adjoint, which refuses both
(implicit/adjoint.py:372-385) — against the CPU adjoint oracle (oracle/adjoint.py): its
sparse direct solves at the same states (1e-9), and its rollout gradients on the device
rollout's own forward states (1e-7). The oracle's tangents are themselves checked against
central differences of the forward oracle in tests/test_adjoint_oracle.py."""
import numpy as np
import pytest

from oracle import adjoint as OA
from helpers import load_fixture, rel_err

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def _solve_matches_direct(prob, xs, min_terms, min_aff=0):
    torch = _torch()
    from diff_2d_fem_gb300.device import DeviceSolver
    from diff_2d_fem_gb300.adjoint import AdjointPNCG2D
    s = DeviceSolver(prob, precision="fp64")
    adj = AdjointPNCG2D(s)
    free = np.asarray(prob["free"], np.float64)
    rng = np.random.default_rng(3)
    for k, x in enumerate(xs):
        assert len(OA.ipc_terms(x, prob)) >= min_terms, "no contact between the bodies at this state"
        rhs = rng.standard_normal(x.shape) * free
        for warm in (False, True):
            guess = torch.as_tensor(rng.standard_normal(x.shape)) if warm else None
            lam = adj.adjoint_solve(torch.as_tensor(x), torch.as_tensor(rhs), rtol=1e-14, maxiter=200000, guess=guess)
            torch.cuda.synchronize()
            assert int(adj.status.abs().max().item()) == 0, adj.status
            ref = OA.adjoint_solve(x, prob, rhs)
            e = rel_err(lam.cpu().numpy(), ref)
            assert e < 1e-9, (k, warm, e)
    s.close()


def test_adjoint_solve_with_an_affine_block_between_pads_matches_direct():
    """The grip fixture's states: two pads squeezing an affine block, IPC contact between the
    pads and the block active."""
    prob, steps, _ = load_fixture("grip")
    assert prob.get("affine") is not None
    _solve_matches_direct(prob, [np.asarray(st["x"]) for st in steps[1:]], min_terms=1)


def test_adjoint_solve_with_a_rigid_region_matches_direct():
    """The rigid_region fixture's states: a cantilever whose outer third is an affine region
    sharing its interface nodes with the soft root (no contact)."""
    prob, steps, _ = load_fixture("rigid_region")
    _solve_matches_direct(prob, [np.asarray(st["x"]) for st in steps], min_terms=0)


def _pressed_block():
    """A soft block pressed by its kinematic top onto a held slab, IPC contact between the
    bodies, friction off (the scene of the oracle's contact rollout test)."""
    from diff_2d_fem_gb300 import ImplicitIntegrator, Model, scene
    px = 0.5e-3
    m = Model()
    m.damping = 50.0
    slab = m.add_soft_body(np.ones((3, 16), np.uint8), physical_size=(16 * px, 3 * px), center=(0.0, -1.5 * px),
                           E=1.0e6, nu=0.40, density=1100.0)
    blk = m.add_soft_body(np.ones((6, 6), np.uint8), physical_size=(6 * px, 6 * px),
                          center=(0.3 * px, 3 * px + 0.6 * px / 8), E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    m.set_kinematic_constraint(slab, np.arange(m.body_nodes(slab).size))
    Xb = m.rest_x(blk)
    top = np.where(Xb[:, 1] > Xb[:, 1].max() - 1e-9)[0]
    m.set_kinematic_constraint(blk, top)
    prob = scene.solver_problem(m, ImplicitIntegrator(friction=False, max_iter=20000), 1e-3)
    prob = dict(prob, eps=1e-16, tol_x=0.0)
    T = 8
    targets = []
    for k in range(1, T + 1):
        tg = np.asarray(m.me.rest_pos, np.float64).copy()
        tg[m.body_nodes(blk)[top], 1] -= 0.08 * px * k
        targets.append(tg)
    return prob, np.stack(targets), T


def _rigid_cantilever():
    """A tip-loaded cantilever whose outer third is a rigid region (the scene of the oracle's
    affine rollout test)."""
    import warnings
    from diff_2d_fem_gb300 import ImplicitIntegrator, Model, scene
    m = Model()
    m.damping = 300.0
    h = m.add_soft_body(np.ones((3, 15), np.uint8), physical_size=(0.0075, 0.0015), center=(0.0, 0.0),
                        E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    region = np.zeros((3, 15), bool)
    region[:, 10:] = True
    m.add_affine_region(h, region)
    X = m.rest_x(h)
    m.set_kinematic_constraint(h, np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0])
    tip = np.where(X[:, 0] > X[:, 0].max() - 1e-9)[0]
    f = np.zeros_like(X)
    f[tip, 1] = -1.5 / len(tip)
    m.set_external_force(h, f)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob = scene.solver_problem(m, ImplicitIntegrator(self_collision=False, friction=False, max_iter=20000), 2e-3)
    return dict(prob, eps=1e-16, tol_x=0.0), None, 6


@pytest.mark.parametrize("scene_fn", [_pressed_block, _rigid_cantilever], ids=["ipc_pressed_block", "rigid_region"])
def test_rollout_gradient_matches_oracle(scene_fn):
    """The differentiable rollout (FP64 forward, checkpoints every 3 steps, the device adjoint
    backwards) against the oracle's rollout adjoint on the same forward states: dL/dE, dL/dx0
    and dL/dv0 of L = w . x_T."""
    torch = _torch()
    from diff_2d_fem_gb300.device import DeviceSolver
    from diff_2d_fem_gb300.adjoint import Rollout
    prob, targets, T = scene_fn()
    rng = np.random.default_rng(5)
    mu = np.asarray(prob["mu"])
    E = np.where(mu > 0, 0.8 + 0.4 * rng.random(len(mu)), 1.0)
    N = np.asarray(prob["x"]).shape[0]
    w = rng.standard_normal((N, 2))
    s = DeviceSolver(prob, precision="fp64")
    dev = s.dev
    ro = Rollout(s, steps=T, record=list(range(1, T + 1)), checkpoint_every=3, rtol=1e-14, max_iter=200000,
                 targets=targets)
    Et = torch.tensor(E, device=dev, requires_grad=True)
    x0 = torch.tensor(np.asarray(prob["x"]), device=dev, requires_grad=True)
    v0 = torch.tensor(np.asarray(prob["v"]), device=dev, requires_grad=True)
    out = ro(Et, None, x0, v0)
    (out[-1] * torch.as_tensor(w, device=dev)).sum().backward()
    assert int(np.abs(ro.info["adjoint_worst_status"]).max()) == 0
    xs = [np.asarray(prob["x"])] + [out[k].detach().cpu().numpy() for k in range(T)]
    if targets is not None:
        assert len(OA.ipc_terms(xs[-1], prob)) > 5, "no contact between the bodies"
    ref = OA.rollout_adjoint(prob, xs, {T: w}, E=E)
    assert rel_err(Et.grad.cpu().numpy(), ref["dE"]) < 1e-7
    assert rel_err(x0.grad.cpu().numpy(), ref["dx0"]) < 1e-7
    assert rel_err(v0.grad.cpu().numpy(), ref["dv0"]) < 1e-7
    s.close()
