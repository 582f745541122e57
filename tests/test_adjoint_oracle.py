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
