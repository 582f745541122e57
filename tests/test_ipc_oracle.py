"""The oracle's IPC contact between bodies and its rigid-body mechanics on the CPU, after the
reference's tests/test_ipc.py (the potential itself: flat sliding costs nothing; gradient
and curvature are the derivatives of the energy; a prescribed body is swept, not placed)
and tests/test_rigid.py (a spinning free
body follows exact rigid backward Euler; the rigid-mode coarse space makes a free soft body
converge; a block on a slope slides or creeps at the closed-form speed)."""
import warnings

import numpy as np
import pytest

import oracle
from diff_2d_fem_gb300 import ImplicitIntegrator, Model, scene

E, NU, RHO, G0 = 1.0e6, 0.40, 1100.0, 9.81
PX = 0.5e-3


def _problem(m, integ, dt):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return scene.solver_problem(m, integ, dt)


def _soft(m, shape, center):
    return m.add_soft_body(np.ones(shape, np.uint8), physical_size=(shape[1] * PX, shape[0] * PX), center=center,
                           E=E, nu=NU, density=RHO)


def _slab_and_block(gap_in_dhat):
    m = Model()
    _soft(m, (4, 80), (0.0, -2 * PX))
    dhat = PX / 8
    block = _soft(m, (8, 24), (0.0, 4 * PX + gap_in_dhat * dhat))
    m.finalize()
    assert np.isclose(m.dhat, dhat) and np.isclose(m.body_kappa, 0.1 * E * PX / dhat)
    s = oracle.OracleSolver(_problem(m, ImplicitIntegrator(), 1e-3))
    return m, s, block


def _energy(s, x):
    return float(s.term("ipc", x, xn=x)[3][0])


def _gradient(s, x):
    return s.term("ipc", x, xn=x)[0]


@pytest.mark.parametrize("gap", [0.9, 0.5, 0.1])
def test_flat_sliding_costs_nothing(gap):
    """A block slid two edge lengths along a flat face at a fixed gap: about fifty pairs carry
    the contact and one slab node passes each end of the block per edge length, so the
    energy may change by one pair in fifty (3 %)."""
    m, s, block = _slab_and_block(gap)
    X = np.asarray(m.me.rest_pos, np.float64)
    nodes = m.body_nodes(block)
    Es = []
    for shift in np.linspace(0.0, 2 * PX, 81):
        x = X.copy()
        x[nodes, 0] += shift
        Es.append(_energy(s, x))
    Es = np.array(Es)
    assert Es.min() > 0.0
    assert (Es.max() - Es.min()) / Es.mean() < 0.03


def test_ipc_gradient_and_curvature_are_derivatives():
    """At a tilted, roughened contact state: the gradient is the derivative of the energy
    (central differences, 1e-6) and p^T H p the derivative of the gradient along p (1e-3)."""
    m, s, block = _slab_and_block(0.5)
    rng = np.random.default_rng(0)
    X = np.asarray(m.me.rest_pos, np.float64)
    nodes = m.body_nodes(block)
    x = X.copy()
    c = x[nodes].mean(0)
    th = 0.004
    R = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
    x[nodes] = (x[nodes] - c) @ R.T + c + np.array([0.13 * PX, 0.2 * m.dhat])
    x += 0.02 * m.dhat * rng.standard_normal(x.shape)
    g = _gradient(s, x)
    act = np.where(np.abs(g).sum(1) > 0)[0]
    assert len(act) > 30, "the probe state is not in contact"
    h = 1e-9
    num = np.zeros_like(g)
    for i in act:
        for k in range(2):
            xp, xm = x.copy(), x.copy()
            xp[i, k] += h
            xm[i, k] -= h
            num[i, k] = (_energy(s, xp) - _energy(s, xm)) / (2 * h)
    assert np.abs(g - num).max() / np.abs(g).max() < 1e-6
    p = np.zeros_like(x)
    p[act] = rng.standard_normal((len(act), 2))
    curv = float(s.term("ipc", x, p=p, xn=x)[2][0])
    hh = 1e-7 * m.dhat
    fd = float((((_gradient(s, x + hh * p) - _gradient(s, x - hh * p)) / (2 * hh)) * p).sum())
    assert abs(curv / fd - 1.0) < 1e-3, (curv, fd)


def _com(m, nodes, x):
    w = np.asarray(m.me.mass, np.float64)[nodes]
    return (w[:, None] * x[nodes]).sum(0) / w.sum()


def _rigid_backward_euler(X, mass, v0, omega, h, n):
    """Exact backward Euler of a free rigid body: each step projects the inertial predictor
    onto the rigid motions — the centroid moves with it, the rotation is the mass-weighted
    best fit (2-D Procrustes)."""
    c = (mass[:, None] * X).sum(0) / mass.sum()
    Xb = X - c
    x = X.copy()
    v = np.asarray(v0)[None] + omega * np.c_[-Xb[:, 1], Xb[:, 0]]
    for _ in range(n):
        xh = x + h * v
        ch = (mass[:, None] * xh).sum(0) / mass.sum()
        S = (mass[:, None, None] * (xh - ch)[:, :, None] * Xb[:, None, :]).sum(0)
        th = np.arctan2(S[1, 0] - S[0, 1], S[0, 0] + S[1, 1])
        Rm = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
        xn = Xb @ Rm.T + ch
        v = (xn - x) / h
        x = xn
    return x


def test_spinning_rigid_body_is_exact_backward_euler():
    """A free affine block launched at 0.1 m/s spinning at 20 rad/s: after 200 steps (~3.85 rad
    turned) within 1e-6 m of exact rigid backward Euler, and strained by less than 1e-6."""
    m = Model()
    m.damping = 0.0
    h = m.add_affine_body(np.ones((12, 16), np.uint8), physical_size=(0.008, 0.006), center=(0.0, 0.05),
                          density=RHO)
    m.finalize()
    m.set_body_velocity(h, velocity=(0.1, 0.0), omega=20.0)
    ref = _rigid_backward_euler(m.rest_x(h), np.asarray(m.me.mass, np.float64), (0.1, 0.0), 20.0, 1e-3, 200)
    integ = ImplicitIntegrator(eps=1e-12, self_collision=False, friction=False)
    s, xs, _ = oracle.run(_problem(m, integ, 1e-3), 200)
    q = s.state["a_q"].reshape(-1, 6)[0]
    A = np.array([[q[1], q[2]], [q[4], q[5]]])
    assert np.arctan2(A[1, 0] - A[0, 1], A[0, 0] + A[1, 1]) % (2 * np.pi) > 3.5
    assert np.abs(xs[-1][m.body_nodes(h)] - ref).max() < 1e-6
    assert np.abs(A.T @ A - np.eye(2)).max() < 1e-6


def test_rigid_modes_make_a_free_soft_body_converge():
    """A free soft block in free fall: with the rigid-mode coarse space, 5 iterations a step
    give the drop g h^2 n (n + 1) / 2 within 1e-4; Jacobi alone in 20 iterations a step
    leaves the block almost where it was."""
    def fall(its, rigid_modes):
        m = Model()
        m.damping = 0.0
        h = m.add_soft_body(np.ones((12, 16), np.uint8), physical_size=(0.008, 0.006), center=(0.0, 0.05),
                            E=E, nu=NU, density=RHO)
        m.finalize()
        m.gravity = (0.0, -G0)
        nodes = m.body_nodes(h)
        y0 = _com(m, nodes, np.asarray(m.me.rest_pos, np.float64))[1]
        integ = ImplicitIntegrator(max_iter=its, self_collision=False, friction=False, rigid_modes=rigid_modes)
        _, xs, _ = oracle.run(_problem(m, integ, 1e-3), 100)
        return (y0 - _com(m, nodes, xs[-1])[1]) / (G0 * 1e-6 * 100 * 101 / 2) - 1
    assert abs(fall(5, True)) < 1e-4
    assert fall(20, False) < -0.9


@pytest.mark.parametrize("kind", ["rigid", "soft"])
@pytest.mark.parametrize("th_deg,mu", [(30.0, 0.30), (15.0, 0.60)])
def test_block_on_a_slope(kind, th_deg, mu):
    """A block on the ground under tilted gravity, damping c: it slides at
    g (sin th - mu cos th) / c_e when tan th > mu, else creeps on the smoothed friction branch
    at g sin th / (mu g cos th / epsv + c_e), c_e = (1 - e^(-c dt)) / dt; within 1 %."""
    th = np.deg2rad(th_deg)
    c, dt = 20.0, 1e-3
    m = Model()
    m.add_ground(height=0.0, mu=mu)
    m.damping = c
    reach = 0.5e-3 / 8
    shape, size, center = np.ones((12, 16), np.uint8), (0.008, 0.006), (0.0, 0.003 + 0.9 * reach)
    if kind == "rigid":
        h = m.add_affine_body(shape, physical_size=size, center=center, density=RHO)
    else:
        h = m.add_soft_body(shape, physical_size=size, center=center, E=E, nu=NU, density=RHO)
    m.finalize()
    assert np.isclose(m.dhat, reach)
    integ = ImplicitIntegrator(self_collision=False)
    nodes = m.body_nodes(h)
    m.gravity = (0.0, -G0 * np.cos(th))
    s, _, _ = oracle.run(_problem(m, integ, dt), 300)
    s.set_fext(np.asarray(m.me.mass, np.float64)[:, None] * np.array([G0 * np.sin(th), -G0 * np.cos(th)]))
    xs = []
    for _ in range(400):
        s.step()
        xs.append(_com(m, nodes, s.x)[0])
    v = np.diff(np.array(xs)[-60:]).mean() / dt
    ce = (1.0 - np.exp(-dt * c)) / dt
    if np.tan(th) > mu:
        expect = G0 * (np.sin(th) - mu * np.cos(th)) / ce
    else:
        expect = G0 * np.sin(th) / (mu * G0 * np.cos(th) / m.epsv + ce)
    assert abs(v / expect - 1.0) < 0.01, (v, expect)


def _push(px_per_step, wall, steps=30):
    """A kinematic pusher driven 1.5 pixels a step into a free block, with or without a held
    wall beyond it: (model, pusher, block, final x, bc lag, smallest gap / dhat, smallest
    element area / rest area)."""
    m = Model()
    m.body_friction = 0.3
    m.damping = 20.0
    pusher = _soft(m, (12, 4), (0.0, 0.0))
    block = _soft(m, (8, 8), (8 * PX, 0.0))                 # two pixels ahead of the pusher
    if wall:
        stop = _soft(m, (12, 4), (17 * PX, 0.0))            # a held body, three pixels behind it
    m.finalize()
    m.set_kinematic_constraint(pusher, np.arange(m.body_nodes(pusher).size))
    if wall:
        m.set_kinematic_constraint(stop, np.arange(m.body_nodes(stop).size))
    prob = _problem(m, ImplicitIntegrator(), 1e-3)
    s = oracle.OracleSolver(prob)
    bc = np.asarray(prob["bc_idx"])
    gap = np.inf
    for k in range(1, steps + 1):
        m.set_kinematic_target(pusher, m.rigid_motion(pusher, (k * px_per_step * PX, 0.0)))
        s.set_bc_target(m._targets[bc])
        s.step()
        gap = min(gap, float(scene.min_distance(dict(prob, x=s.x)).min()) / m.dhat)
    x, X = s.x, np.asarray(m.me.rest_pos, np.float64)
    t = np.asarray(m.me.tri)
    area = lambda P: ((P[t[:, 1], 0] - P[t[:, 0], 0]) * (P[t[:, 2], 1] - P[t[:, 0], 1])
                      - (P[t[:, 1], 1] - P[t[:, 0], 1]) * (P[t[:, 2], 0] - P[t[:, 0], 0]))
    lag = float(np.linalg.norm(m._targets[bc] - x[bc], axis=1).max())
    assert np.isfinite(x).all() and gap > 0.0, gap
    return m, pusher, block, x, lag, float((area(x) / area(X)).min())


def test_a_prescribed_body_is_swept():
    """A kinematic body is swept to its target, not placed there: with nothing in its way it
    arrives (lag below 1e-9 pixel) and the block it pushes stays ahead of it unsquashed;
    against a held wall the target 45 pixels on cannot be reached, the pusher stops short
    (lag above 25 pixels) and the block is squeezed between the two, never through."""
    m, pusher, block, x, lag, squash = _push(1.5, wall=False)
    front = x[m.body_nodes(pusher), 0].max()
    assert lag < 1e-9 * PX, lag / PX
    assert x[m.body_nodes(block), 0].min() > front
    assert squash > 0.9
    m, pusher, block, x, lag, squash = _push(1.5, wall=True)
    xb = x[m.body_nodes(block)]
    assert lag > 25 * PX, lag / PX
    assert xb[:, 0].max() < 15 * PX and xb[:, 0].min() > x[m.body_nodes(pusher), 0].max()
    assert 0.05 < squash < 0.9, squash


def test_block_algebra():
    """The oracle's 6x6 affine algebra (reference tests/test_rigid.py:62-94): the Cholesky
    solve against numpy (1e-10); the reduced elastic Hessian symmetric and positive
    semi-definite at rotations and at strained, partly compressed states, where turning
    further costs nothing at a pure rotation (one null direction) and straining does."""
    rng = np.random.default_rng(0)
    n = 300
    M = rng.normal(size=(n, 6, 6))
    H = M @ M.transpose(0, 2, 1) + 0.1 * np.eye(6)
    b = rng.normal(size=(n, 6))
    x = np.stack([oracle.chol6_solve(H[k], b[k]) for k in range(n)])
    ref = np.linalg.solve(H, b[:, :, None])[:, :, 0]
    assert np.abs(x - ref).max() / np.abs(ref).max() < 1e-10
    th = rng.uniform(0, 2 * np.pi, n)
    c, s = np.cos(th), np.sin(th)
    R = np.stack([np.stack([c, -s], -1), np.stack([s, c], -1)], 1)
    S = np.eye(2) + 0.02 * rng.uniform(-1, 1, (n, 2, 2))
    S = 0.5 * (S + S.transpose(0, 2, 1))
    assert (np.linalg.det(R @ S) < 1).sum() > n // 4, "the sample should include compressed states"
    for name, A in (("rotation", R), ("strained", R @ S)):
        Hq = np.stack([oracle.affine_hessian(A[k], 1.0, 2.5) for k in range(n)])
        H4 = Hq[:, [1, 2, 4, 5]][:, :, [1, 2, 4, 5]]
        w = np.linalg.eigvalsh(H4)
        assert np.abs(H4 - H4.transpose(0, 2, 1)).max() < 1e-9 * w.max(), name
        assert (w[:, 0] > -1e-9 * w[:, -1]).all(), name
        if name == "rotation":
            assert (np.abs(w[:, 0]) < 1e-9 * w[:, -1]).all()
            assert (w[:, 1] > 0.1 * w[:, -1]).all()


def _pinch_and_lift(mu, lift=2.0e-3, n_close=50, n_lift=100, n_hold=25):
    """Two soft pads driven by their backs close on a rigid block on the ground, lift and
    hold: the block's rise as a fraction of the lift."""
    m = Model()
    m.body_friction = mu
    m.add_ground(0.0, mu=0.5)
    blk = m.add_affine_body(np.ones((8, 8), np.uint8), physical_size=(8 * PX, 8 * PX),
                            center=(0.0, 4 * PX + 0.9 * PX / 8), density=600.0)
    pads = [_soft(m, (8, 4), (sgn * 7 * PX, 4 * PX + 0.4e-3)) for sgn in (-1, +1)]
    m.finalize()
    m.gravity = (0.0, -G0)
    for sgn, h in zip((-1, +1), pads):
        X = m.rest_x(h)
        back = X[:, 0].min() if sgn < 0 else X[:, 0].max()
        m.set_kinematic_constraint(h, np.where(np.abs(X[:, 0] - back) < 1e-9)[0])
    prob = _problem(m, ImplicitIntegrator(), 1e-3)
    bc = np.asarray(prob["bc_idx"])
    s = oracle.OracleSolver(prob)
    nb = m.body_nodes(blk)
    y0 = s.x[nb, 1].mean()
    for k in range(1, n_close + n_lift + n_hold + 1):
        a, b = min(k / n_close, 1.0), min(max(k - n_close, 0) / n_lift, 1.0)
        for sgn, h in zip((-1, +1), pads):
            X = m.rest_x(h)
            X[:, 0] -= sgn * 1.125 * PX * a
            X[:, 1] += lift * b
            m.set_kinematic_target(h, X)
        s.set_bc_target(m._targets[bc])
        s.step()
    assert np.isfinite(s.x).all() and scene.min_distance(dict(prob, x=s.x)).min() > 0.0
    return (s.x[nb, 1].mean() - y0) / lift


def test_a_grip_needs_friction():
    """Pads pinching a rigid block lift it only through friction between the bodies: without
    friction it stays on the ground (below 5 % of the lift), with mu = 0.8 it comes up (above
    95 %) — after the reference's tests/test_ipc.py:185-212, at half its size."""
    assert abs(_pinch_and_lift(0.0)) < 0.05
    assert _pinch_and_lift(0.8) > 0.95
