"""The GPU adjoint (d2f_adjoint_solve / d2f_adjoint_vjp through diff_2d_fem_gb300.adjoint)
against the reference's adjoint fixture, the CPU adjoint oracle and central finite
differences of the GPU forward, batched."""
import numpy as np
import pytest

from oracle import adjoint as OA
from helpers import load_fixture, rel_err, tile_problem

pytestmark = pytest.mark.gpu

FD_TOL = 1e-4


def _torch():
    import torch
    return torch


def _device_solver(prob, precision="fp64"):
    from diff_2d_fem_gb300.device import DeviceSolver
    return DeviceSolver(prob, precision=precision)


def _press_disc():
    prob, steps, meta = load_fixture("adjoint_press_disc")
    xs = [np.asarray(meta["x0"])] + [np.asarray(s["x"]) for s in steps]
    E = meta["Emin"] + np.asarray(meta["rho"]) * (1.0 - meta["Emin"])
    targets = []
    for st in steps:
        full = np.asarray(prob["x"], np.float64).copy()
        full[np.asarray(prob["bc_idx"])] = st["bc_target"]
        targets.append(full)
    return prob, steps, meta, xs, E, np.stack(targets)


def test_adjoint_solve_matches_direct_solve():
    """Each step's system of the pressed block, solved by the device CG, against the oracle's
    sparse direct solve at the same (reference) states, random right-hand sides."""
    torch = _torch()
    from diff_2d_fem_gb300.adjoint import AdjointPNCG2D
    prob, steps, meta, xs, E, _ = _press_disc()
    s = _device_solver(prob)
    adj = AdjointPNCG2D(s, Emin=meta["Emin"])
    adj.set_modulus(E)
    rng = np.random.default_rng(3)
    for k in range(1, len(xs)):
        rhs = rng.standard_normal(xs[k].shape)
        lam = adj.adjoint_solve(torch.as_tensor(xs[k]), torch.as_tensor(rhs), rtol=1e-14)
        torch.cuda.synchronize()
        assert int(adj.status.max().item()) == 0 and int(adj.status.min().item()) == 0
        ref = OA.adjoint_solve(xs[k], prob, rhs, mu=E * prob["mu"], lam=E * prob["lam"])
        assert rel_err(lam.cpu().numpy(), ref) < 1e-10, k
    s.close()


def test_transient_adjoint_matches_reference():
    """AdjointPNCG2D.transient_adjoint on the reference's own forward states: dJ/drho of the
    reference (its MINRES at rtol 1e-13)."""
    from diff_2d_fem_gb300.adjoint import AdjointPNCG2D
    prob, steps, meta, xs, E, _ = _press_disc()
    s = _device_solver(prob)
    adj = AdjointPNCG2D(s, Emin=meta["Emin"])
    adj.set_density(meta["rho"])
    g = adj.transient_adjoint(xs, seed={len(steps): meta["seed_w"]}, rtol=1e-14).cpu().numpy()
    assert rel_err(g, meta["dJdrho"]) < 1e-9
    assert int(adj.worst_status.abs().max().item()) == 0
    s.close()


def test_rollout_forward_and_gradient_match_reference():
    """The differentiable rollout: forward states within 1e-9 of the reference's, dL/dE x
    (1 - Emin) within 1e-7 of the reference's dJ/drho; two-step checkpoints replay bit-exact."""
    torch = _torch()
    from diff_2d_fem_gb300.adjoint import Rollout
    prob, steps, meta, xs, E, targets = _press_disc()
    T = len(steps)
    s = _device_solver(prob)
    ro = Rollout(s, steps=T, record=list(range(1, T + 1)), checkpoint_every=2, rtol=1e-14, targets=targets,
                 Emin=meta["Emin"])
    dev = s.dev
    Et = torch.tensor(E, dtype=torch.float64, device=dev, requires_grad=True)
    x0 = torch.tensor(xs[0], dtype=torch.float64, device=dev, requires_grad=True)
    v0 = torch.zeros_like(x0, requires_grad=True)
    out = ro(Et, None, x0, v0)
    for k in range(T):
        assert rel_err(out[k].detach().cpu().numpy(), xs[k + 1]) < 1e-9, k
    w = torch.as_tensor(meta["seed_w"], device=dev)
    (out[-1] * w).sum().backward()
    assert ro.info["replay_mismatch"] == 0.0
    assert int(np.abs(ro.info["adjoint_worst_status"]).max()) == 0
    g = Et.grad.cpu().numpy() * (1.0 - meta["Emin"])
    assert rel_err(g, meta["dJdrho"]) < 1e-7
    s.close()


def _tendon():
    prob, _, _ = load_fixture("tendon")
    prob = dict(prob)
    prob["eps"], prob["iter_max"], prob["tol_x"] = 1e-16, 20000, 0.0
    return prob


def test_rollout_tendon_matches_oracle():
    """Cantilever bent by a tendon: every input's gradient (moduli, tension schedule, x0, v0)
    against the adjoint oracle run on the rollout's own forward states."""
    torch = _torch()
    from diff_2d_fem_gb300.adjoint import Rollout
    prob = _tendon()
    T = 4
    rng = np.random.default_rng(0)
    E = 0.8 + 0.4 * rng.random(len(prob["mu"]))
    tens = np.array([[5.0 + 5.0 * k] for k in range(T)])
    w = rng.standard_normal((np.asarray(prob["x"]).shape[0], 2))
    s = _device_solver(prob)
    dev = s.dev
    ro = Rollout(s, steps=T, record=list(range(1, T + 1)), checkpoint_every=3, rtol=1e-14)
    Et = torch.tensor(E, device=dev, requires_grad=True)
    Tt = torch.tensor(tens, device=dev, requires_grad=True)
    x0 = torch.tensor(np.asarray(prob["x"]), device=dev, requires_grad=True)
    v0 = torch.tensor(np.asarray(prob["v"]), device=dev, requires_grad=True)
    out = ro(Et, Tt, x0, v0)
    (out[-1] * torch.as_tensor(w, device=dev)).sum().backward()
    xs = [np.asarray(prob["x"])] + [out[k].detach().cpu().numpy() for k in range(T)]
    ref = OA.rollout_adjoint(prob, xs, {T: w}, E=E, tensions=tens)
    assert rel_err(Et.grad.cpu().numpy(), ref["dE"]) < 1e-8
    assert rel_err(Tt.grad.cpu().numpy(), ref["dT"]) < 1e-8
    assert rel_err(x0.grad.cpu().numpy(), ref["dx0"]) < 1e-8
    assert rel_err(v0.grad.cpu().numpy(), ref["dv0"]) < 1e-8
    s.close()


def test_rollout_matches_batched_central_differences():
    """Nine copies of the tendon cantilever in one batch: the base, and +/- perturbations of
    the moduli, the tension schedule, x0 and v0 along random directions. One forward of the
    batch gives every central difference; one backward gives the adjoint directional
    derivatives of each copy's loss. They agree to 1e-4."""
    torch = _torch()
    from diff_2d_fem_gb300.adjoint import Rollout
    base = _tendon()
    T, nb = 4, 9
    prob = tile_problem(base, nb)
    N1, T1 = np.asarray(base["x"]).shape[0], len(base["mu"])
    rng = np.random.default_rng(7)
    E1 = 0.8 + 0.4 * rng.random(T1)
    t1 = np.array([5.0 + 5.0 * k for k in range(T)])
    w1 = rng.standard_normal((N1, 2))
    free = np.asarray(base["free"], np.float64)
    dE, dT = rng.standard_normal(T1), rng.standard_normal(T)
    dx, dv = rng.standard_normal((N1, 2)) * free * 1e-5, rng.standard_normal((N1, 2)) * free * 1e-1
    eps = {"E": 1e-3, "T": 1e-1, "x0": 1.0, "v0": 1.0}
    E = np.tile(E1, (nb, 1))
    tens = np.tile(t1[:, None], (1, nb))                       # (steps, tendons = one per copy)
    x0 = np.tile(np.asarray(base["x"]), (nb, 1, 1))
    v0 = np.tile(np.asarray(base["v"]), (nb, 1, 1))
    E[1], E[2] = E1 * (1 + eps["E"] * dE), E1 * (1 - eps["E"] * dE)
    tens[:, 3], tens[:, 4] = t1 + eps["T"] * dT, t1 - eps["T"] * dT
    x0[5], x0[6] = x0[0] + eps["x0"] * dx, x0[0] - eps["x0"] * dx
    v0[7], v0[8] = v0[0] + eps["v0"] * dv, v0[0] - eps["v0"] * dv
    s = _device_solver(prob)
    dev = s.dev
    ro = Rollout(s, steps=T, checkpoint_every=2, rtol=1e-14)
    Et = torch.tensor(E.reshape(-1), device=dev, requires_grad=True)
    Tt = torch.tensor(tens, device=dev, requires_grad=True)
    xt = torch.tensor(x0.reshape(-1, 2), device=dev, requires_grad=True)
    vt = torch.tensor(v0.reshape(-1, 2), device=dev, requires_grad=True)
    out = ro(Et, Tt, xt, vt)[0].reshape(nb, N1, 2)
    L = (out * torch.as_tensor(w1, device=dev)[None]).sum(dim=(1, 2))
    L.sum().backward()
    Lh = L.detach().cpu().numpy()
    gE = Et.grad.reshape(nb, T1)[0].cpu().numpy()
    gT = Tt.grad[:, 0].cpu().numpy()
    gx = xt.grad.reshape(nb, N1, 2)[0].cpu().numpy()
    gv = vt.grad.reshape(nb, N1, 2)[0].cpu().numpy()
    checks = [("E", (Lh[1] - Lh[2]) / (2 * eps["E"]), float((gE * E1 * dE).sum())),
              ("T", (Lh[3] - Lh[4]) / (2 * eps["T"]), float((gT * dT).sum())),
              ("x0", (Lh[5] - Lh[6]) / (2 * eps["x0"]), float((gx * dx).sum())),
              ("v0", (Lh[7] - Lh[8]) / (2 * eps["v0"]), float((gv * dv).sum()))]
    for name, fd, adj in checks:
        assert abs(fd - adj) <= FD_TOL * abs(adj), (name, fd, adj)
    s.close()


def test_adjoint_refuses_a_mixed_precision_solver():
    from diff_2d_fem_gb300.adjoint import AdjointPNCG2D
    p2, _, _ = load_fixture("strip_small")
    m = _device_solver(p2, precision="mixed")
    with pytest.raises(ValueError):
        AdjointPNCG2D(m)
    m.close()


def test_tendon_arm_central_differences_32_entries():
    """The differentiation configuration on one arm: 100 steps at dt 2e-3, loss = squared
    distance of the tip to a target. 32 seeded entries — 24 pixel moduli, 8 step tensions —
    each perturbed by +/- h relative in copies of the arm inside one batch of 65 scenes;
    central differences against the adjoint gradient of the base copy to 1e-4, relative to
    the entry (or to 1 % of the largest checked entry, for the entries smaller than that).
    h = 1e-3: at h = 1e-6 the differences are dominated by the forward solve's convergence
    floor (positions to ~1e-12 relative), not by the gradient; the truncation error of
    central differences at 1e-3 is O(h^2) ~ 1e-6 relative."""
    torch = _torch()
    from diff_2d_fem_gb300 import workloads, scene, ImplicitIntegrator
    from diff_2d_fem_gb300.adjoint import Rollout
    T, h = 100, 1e-3
    m, kw, dt, ex = workloads.tendon_arms(1, seed=5, steps=T)
    base = scene.solver_problem(m, ImplicitIntegrator(**kw), dt)
    base["eps"], base["iter_max"], base["tol_x"] = 0.0, 1000, 0.0     # fully converged steps
    N1, T1 = np.asarray(base["x"]).shape[0], len(base["tri"])
    rng = np.random.default_rng(11)
    quad = np.asarray(m.me.tri_quad)                                   # triangle -> pixel
    pix = rng.choice(np.unique(quad), 24, replace=False)
    steps_k = np.sort(rng.choice(np.arange(T), 8, replace=False))
    ten1 = ex["tension"][:, 0]
    nb = 1 + 2 * 32
    prob = tile_problem(base, nb)
    E = np.ones((nb, T1))
    ten = np.tile(ten1[:, None], (1, nb))
    for j, p in enumerate(pix):
        E[1 + 2 * j, quad == p] = 1 + h
        E[2 + 2 * j, quad == p] = 1 - h
    for j, k in enumerate(steps_k):
        c = 1 + 2 * (24 + j)
        ten[k, c], ten[k, c + 1] = ten1[k] * (1 + h), ten1[k] * (1 - h)
    s = _device_solver(prob)
    dev = s.dev
    ro = Rollout(s, steps=T, checkpoint_every=10, rtol=1e-14, max_iter=50000)
    Et = torch.tensor(E.reshape(-1), device=dev, requires_grad=True)
    Tt = torch.tensor(ten, device=dev, requires_grad=True)
    x0 = torch.tensor(np.asarray(prob["x"]), device=dev)
    v0 = torch.zeros_like(x0)
    out = ro(Et, Tt, x0, v0)[0].reshape(nb, N1, 2)
    tip = int(ex["tip"][0])
    L = ((out[:, tip] - torch.as_tensor(ex["target"][0], device=dev)) ** 2).sum(dim=1)
    L.sum().backward()
    assert int(np.abs(ro.info["adjoint_worst_status"]).max()) == 0
    Lh = L.detach().cpu().numpy()
    gE = Et.grad.reshape(nb, T1)[0].cpu().numpy()
    gT = Tt.grad[:, 0].cpu().numpy()
    fd = np.array([(Lh[1 + 2 * j] - Lh[2 + 2 * j]) / (2 * h) for j in range(32)])
    adj = np.concatenate([[gE[quad == p].sum() for p in pix], gT[steps_k] * ten1[steps_k]])
    err = np.abs(fd - adj) / np.maximum(np.abs(adj), 1e-2 * np.abs(adj).max())
    assert err.max() < 1e-4, (err.max(), fd[err.argmax()], adj[err.argmax()], np.abs(adj).max())
    s.close()


def test_rollout_with_mixed_forward_matches_fp64_forward():
    """The same gradients with the forward and its replay in mixed precision (the FP64 adjoint
    linearised at the mixed states): within 1e-6 of the all-FP64 rollout's on the tendon
    cantilever, converged steps."""
    torch = _torch()
    from diff_2d_fem_gb300.adjoint import Rollout
    prob = _tendon()
    prob["iter_max"], prob["eps"] = 3000, 0.0
    T = 4
    rng = np.random.default_rng(2)
    E = 0.8 + 0.4 * rng.random(len(prob["mu"]))
    tens = np.array([[5.0 + 5.0 * k] for k in range(T)])
    w = rng.standard_normal((np.asarray(prob["x"]).shape[0], 2))
    grads = []
    for fp in ("fp64", "mixed"):
        s = _device_solver(prob)
        ro = Rollout(s, steps=T, checkpoint_every=2, rtol=1e-14, forward_precision=fp)
        Et = torch.tensor(E, device=s.dev, requires_grad=True)
        Tt = torch.tensor(tens, device=s.dev, requires_grad=True)
        x0 = torch.tensor(np.asarray(prob["x"]), device=s.dev)
        out = ro(Et, Tt, x0, torch.zeros_like(x0))
        (out[0] * torch.as_tensor(w, device=s.dev)).sum().backward()
        grads.append((Et.grad.cpu().numpy(), Tt.grad.cpu().numpy()))
        ro.close()
        s.close()
    assert rel_err(grads[1][0], grads[0][0]) < 1e-6
    assert rel_err(grads[1][1], grads[0][1]) < 1e-6
