"""The adjoint oracle (oracle/adjoint.py) against the reference's own adjoint and against
central finite differences of the CPU forward oracle. No GPU."""
import numpy as np

import oracle
from oracle import adjoint as OA
from helpers import load_fixture, rel_err

FD_TOL = 1e-4


def _press_disc():
    prob, steps, meta = load_fixture("adjoint_press_disc")
    xs = [np.asarray(meta["x0"])] + [np.asarray(s["x"]) for s in steps]
    E = meta["Emin"] + np.asarray(meta["rho"]) * (1.0 - meta["Emin"])
    return prob, steps, meta, xs, E


def test_forward_oracle_reproduces_reference_states():
    """The reference's forward states of the adjoint fixture, bit for bit (density applied)."""
    prob, steps, meta, xs, E = _press_disc()
    p = dict(prob)
    p["mu"], p["lam"] = E * prob["mu"], E * prob["lam"]
    _, oxs, _ = oracle.run(p, len(steps), lambda k: dict(bc_target=steps[k]["bc_target"]))
    for a, b in zip(oxs, xs[1:]):
        assert np.array_equal(a, b)


def test_adjoint_oracle_matches_reference_transient_adjoint():
    """dJ/drho of the reference's AdjointPNCG2D.transient_adjoint (MINRES, rtol 1e-13) on a
    block pressed onto a frictionless disc, barrier active at 3-4 nodes per step."""
    prob, steps, meta, xs, E = _press_disc()
    T = len(steps)
    res = OA.rollout_adjoint(prob, xs, {T: meta["seed_w"]}, E=E)
    assert rel_err(res["dE"] * (1.0 - meta["Emin"]), meta["dJdrho"]) < 1e-9


def test_element_tangent_is_the_derivative_of_the_force():
    prob, steps, meta, xs, E = _press_disc()
    x = xs[-1]
    K = OA.element_hessians(x, prob)
    tri = np.asarray(prob["tri"], np.int64)
    rng = np.random.default_rng(1)
    d = rng.standard_normal(x.shape) * 1e-6
    h = 1e-3
    fp = OA.element_forces(x + h * d, prob).reshape(len(tri), 6)
    fm = OA.element_forces(x - h * d, prob).reshape(len(tri), 6)
    fd = (fp - fm) / (2 * h)
    an = np.einsum("tij,tj->ti", K, d[tri].reshape(len(tri), 6))
    assert rel_err(an, fd) < 1e-6


def _tendon_setup():
    prob, _, _ = load_fixture("tendon")
    prob = dict(prob)
    prob["eps"], prob["iter_max"], prob["tol_x"] = 1e-16, 20000, 0.0
    T = 4
    tens = np.array([[5.0 + 5.0 * k] for k in range(T)])
    rng = np.random.default_rng(0)
    E = 0.8 + 0.4 * rng.random(len(prob["mu"]))
    w = rng.standard_normal((np.asarray(prob["x"]).shape[0], 2))
    return prob, T, tens, E, w, rng


def _loss(prob, T, E, tens, w, x0=None, v0=None):
    p = dict(prob)
    p["mu"], p["lam"] = E * prob["mu"], E * prob["lam"]
    if x0 is not None:
        p["x"] = x0
    if v0 is not None:
        p["v"] = v0
    _, xs, _ = oracle.run(p, T, lambda k: dict(Tcmd=tens[k]))
    return float((w * xs[-1]).sum()), [np.asarray(p["x"])] + xs


def test_adjoint_oracle_matches_central_differences():
    """A clamped cantilever bent by a tension-controlled tendon, 4 steps, damping on: the
    gradient of L = w . x_T with respect to per-element moduli, the tension schedule, x0 and
    v0, each along a random direction, against central differences of the forward oracle."""
    prob, T, tens, E, w, rng = _tendon_setup()
    _, xs = _loss(prob, T, E, tens, w)
    res = OA.rollout_adjoint(prob, xs, {T: w}, E=E, tensions=tens)
    free = np.asarray(prob["free"], np.float64)
    N = xs[0].shape[0]
    v0 = np.asarray(prob.get("v", np.zeros((N, 2))), np.float64)
    dE = rng.standard_normal(len(E))
    dT = rng.standard_normal(tens.shape)
    dx = rng.standard_normal((N, 2)) * free * 1e-5
    dv = rng.standard_normal((N, 2)) * free * 1e-1
    cases = [
        ("E", 1e-3, lambda e: _loss(prob, T, E * (1 + e * dE), tens, w)[0], float((res["dE"] * E * dE).sum())),
        ("T", 1e-1, lambda e: _loss(prob, T, E, tens + e * dT, w)[0], float((res["dT"] * dT).sum())),
        ("x0", 1.0, lambda e: _loss(prob, T, E, tens, w, x0=np.asarray(prob["x"]) + e * dx)[0],
         float((res["dx0"] * dx).sum())),
        ("v0", 1.0, lambda e: _loss(prob, T, E, tens, w, v0=v0 + e * dv)[0], float((res["dv0"] * dv).sum())),
    ]
    for name, eps, L, adj in cases:
        fd = (L(eps) - L(-eps)) / (2 * eps)
        assert abs(fd - adj) <= FD_TOL * abs(adj), (name, fd, adj)


def test_ipc_tangent_is_the_derivative_of_the_contact_force():
    """The adjoint oracle's frozen-set IPC tangent against central differences of the forward
    oracle's own IPC gradient, at a tilted, roughened contact state (1e-7)."""
    from diff_2d_fem_gb300 import ImplicitIntegrator, Model, scene
    px = 0.5e-3
    m = Model()
    m.add_soft_body(np.ones((4, 40), np.uint8), physical_size=(40 * px, 4 * px), center=(0.0, -2 * px),
                    E=1.0e6, nu=0.40, density=1100.0)
    blk = m.add_soft_body(np.ones((8, 12), np.uint8), physical_size=(12 * px, 8 * px),
                          center=(0.0, 4 * px + 0.5 * px / 8), E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    prob = scene.solver_problem(m, ImplicitIntegrator(friction=False), 1e-3)
    s = oracle.OracleSolver(prob)
    rng = np.random.default_rng(0)
    x = np.asarray(m.me.rest_pos, np.float64).copy()
    nodes = m.body_nodes(blk)
    c = x[nodes].mean(0)
    th = 0.004
    R = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
    x[nodes] = (x[nodes] - c) @ R.T + c + np.array([0.13 * px, 0.2 * m.dhat])
    x += 0.02 * m.dhat * rng.standard_normal(x.shape)
    N = x.shape[0]
    K = np.zeros((2 * N, 2 * N))
    terms = OA.ipc_terms(x, prob)
    assert len(terms) > 20
    for nd, b in terms:
        dof = np.array([2 * n + k for n in nd for k in range(2)])
        K[np.ix_(dof, dof)] += b
    assert np.abs(K - K.T).max() <= 1e-12 * np.abs(K).max()
    g0 = s.term("ipc", x, xn=x)[0]
    v = np.zeros_like(x)
    act = np.where(np.abs(g0).sum(1) > 0)[0]
    v[act] = rng.standard_normal((len(act), 2))
    hh = 1e-7 * m.dhat
    fd = (s.term("ipc", x + hh * v, xn=x + hh * v)[0] - s.term("ipc", x - hh * v, xn=x - hh * v)[0]) / (2 * hh)
    an = float(prob["dt"]) ** 2 * (K @ v.ravel()).reshape(-1, 2)
    assert rel_err(an, fd) < 1e-7


def test_adjoint_oracle_through_contact_between_bodies():
    """A soft block pressed by its kinematic top onto a held slab for 8 steps, IPC contact
    between the bodies active, friction off: the gradient of L = w . x_T with respect to the
    per-element moduli, x0 and v0, along random directions, against central differences of
    the forward oracle (1e-4) — an extension beyond the reference, which refuses IPC."""
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
    bc = np.asarray(prob["bc_idx"])
    T = 8
    targets = []
    for k in range(1, T + 1):
        tg = np.asarray(m.me.rest_pos, np.float64).copy()
        tg[m.body_nodes(blk)[top], 1] -= 0.08 * px * k
        targets.append(tg[bc])
    rng = np.random.default_rng(3)
    E = 0.8 + 0.4 * rng.random(len(prob["mu"]))
    N = np.asarray(prob["x"]).shape[0]
    w = rng.standard_normal((N, 2))

    def loss(E_, x0=None, v0=None):
        p = dict(prob)
        p["mu"], p["lam"] = E_ * prob["mu"], E_ * prob["lam"]
        if x0 is not None:
            p["x"] = x0
        if v0 is not None:
            p["v"] = v0
        _, xs, _ = oracle.run(p, T, lambda k: dict(bc_target=targets[k]))
        return float((w * xs[-1]).sum()), [np.asarray(p["x"], np.float64)] + xs

    _, xs = loss(E)
    assert len(OA.ipc_terms(xs[-1], prob)) > 5, "no contact between the bodies"
    res = OA.rollout_adjoint(prob, xs, {T: w}, E=E)
    free = np.asarray(prob["free"], np.float64)
    dE = rng.standard_normal(len(E))
    dx = rng.standard_normal((N, 2)) * free * 1e-5
    dv = rng.standard_normal((N, 2)) * free * 1e-2
    v0 = np.asarray(prob["v"], np.float64)
    # the block forgets x0 and v0 within the 8 damped steps: their effect on L is ~1e-12 of it,
    # where central differences are good to ~1e-4 only (the loss's own rounding)
    for name, eps, tol, L, adj in (
            ("E", 1e-3, FD_TOL, lambda e: loss(E * (1 + e * dE))[0], float((res["dE"] * E * dE).sum())),
            ("x0", 1.0, 1e-3, lambda e: loss(E, x0=np.asarray(prob["x"]) + e * dx)[0], float((res["dx0"] * dx).sum())),
            ("v0", 1.0, 1e-3, lambda e: loss(E, v0=v0 + e * dv)[0], float((res["dv0"] * dv).sum()))):
        fd = (L(eps) - L(-eps)) / (2 * eps)
        assert abs(fd - adj) <= tol * abs(adj), (name, fd, adj)


def test_adjoint_oracle_with_a_rigid_region():
    """A cantilever whose outer third is a rigid region (an affine body sharing its interface
    nodes), tip-loaded, 6 steps: the gradient of L = w . x_T with respect to the soft
    elements' moduli and to v0, along random directions, against central differences of the
    forward oracle (1e-4) — the reduced-coordinate adjoint, beyond the reference, which
    refuses affine bodies."""
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
    prob = dict(prob, eps=1e-16, tol_x=0.0)
    T = 6
    rng = np.random.default_rng(5)
    E = np.where(np.asarray(prob["mu"]) > 0, 0.8 + 0.4 * rng.random(len(prob["mu"])), 1.0)
    N = np.asarray(prob["x"]).shape[0]
    w = rng.standard_normal((N, 2))

    def loss(E_, v0=None):
        p = dict(prob)
        p["mu"], p["lam"] = E_ * prob["mu"], E_ * prob["lam"]
        if v0 is not None:
            p["v"] = v0
        _, xs, _ = oracle.run(p, T)
        return float((w * xs[-1]).sum()), [np.asarray(p["x"], np.float64)] + xs

    _, xs = loss(E)
    res = OA.rollout_adjoint(prob, xs, {T: w}, E=E)
    free = np.asarray(prob["free"], np.float64)
    dE = rng.standard_normal(len(E)) * (np.asarray(prob["mu"]) > 0)
    dv = rng.standard_normal((N, 2)) * free * 1e-2
    v0 = np.asarray(prob["v"], np.float64)
    for name, eps, L, adj in (
            ("E", 1e-3, lambda e: loss(E * (1 + e * dE))[0], float((res["dE"] * E * dE).sum())),
            ("v0", 1.0, lambda e: loss(E, v0=v0 + e * dv)[0], float((res["dv0"] * dv).sum()))):
        fd = (L(eps) - L(-eps)) / (2 * eps)
        assert abs(fd - adj) <= FD_TOL * abs(adj), (name, fd, adj)


def test_adjoint_oracle_through_a_level_set_collider():
    """A soft block pressed by its kinematic top onto a rounded box (and, in a second run, an
    ellipse) for 10 steps, frictionless: dL/dE along a random direction against central
    differences of the forward oracle (3e-4) — the collider tangent through the level set's
    gradient and Hessian (chvp_sdf_kernel, implicit/adjoint.py:101-114)."""
    import warnings
    from diff_2d_fem_gb300 import ImplicitIntegrator, Model, scene
    for shape, kw in (("box", dict(rx=0.004, ry=0.002, corner_radius=0.0015)), ("ellipse", dict(rx=0.005, ry=0.003))):
        m = Model()
        m.add_object(shape, center=(0.0, 0.0), mu=0.0, **kw)
        h = m.add_soft_body(np.ones((8, 6), np.uint8), physical_size=(0.003, 0.004),
                            center=(0.0005, kw.get("ry", 0.0) + 0.002 + 0.2e-3), E=1.0e6, nu=0.40, density=1100.0)
        m.finalize()
        X = m.rest_x(h)
        top = np.where(X[:, 1] > X[:, 1].max() - 1e-9)[0]
        m.set_kinematic_constraint(h, top)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            prob = scene.solver_problem(m, ImplicitIntegrator(friction=False, self_collision=False, max_iter=20000), 1e-3)
        prob = dict(prob, eps=1e-16, tol_x=0.0)
        bc = np.asarray(prob["bc_idx"])
        T = 10
        targets = []
        for k in range(1, T + 1):
            tg = np.asarray(m.me.rest_pos, np.float64).copy()
            tg[top, 1] -= 0.03e-3 * k
            targets.append(tg[bc])
        rng = np.random.default_rng(11)
        E = 0.8 + 0.4 * rng.random(len(prob["mu"]))
        N = np.asarray(prob["x"]).shape[0]
        w = rng.standard_normal((N, 2))

        def loss(E_):
            p = dict(prob)
            p["mu"], p["lam"] = E_ * prob["mu"], E_ * prob["lam"]
            _, xs, _ = oracle.run(p, T, lambda k: dict(bc_target=targets[k]))
            return float((w * xs[-1]).sum()), [np.asarray(p["x"], np.float64)] + xs

        _, xs = loss(E)
        d, _, _ = oracle.sdf_full(prob["colliders"][0], xs[-1][np.asarray(prob["bnd"])])
        assert (d < m.dhat).sum() >= 2, f"{shape}: no contact"
        res = OA.rollout_adjoint(prob, xs, {T: w}, E=E)
        dE = rng.standard_normal(len(E))
        # the forward steps stop at a floor of ~1e-12 of the loss (the level set's contact
        # slows the last iterations): central differences at 3e-3 sit between that noise and
        # their own O(h^2) error, good to ~1e-4 (the reference bounds this case at 3 %)
        fd = (loss(E * (1 + 3e-3 * dE))[0] - loss(E * (1 - 3e-3 * dE))[0]) / 6e-3
        adj = float((res["dE"] * E * dE).sum())
        assert abs(fd - adj) <= 3e-4 * abs(adj), (shape, fd, adj)
