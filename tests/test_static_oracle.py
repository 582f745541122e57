"""The oracle's implicit step against static equilibria found by Newton's method
(oracle/static.py), on the CPU: where beam theory and the discretisation differ by several
per cent, only a solution of the same discrete problem says how well the PNCG solve did.
After the reference's tests/test_rigid.py (a rigid region in a soft cantilever) and
tests/test_actuation.py (a tendon and an active bilayer bending a cantilever)."""
import warnings

import numpy as np

import oracle
from oracle import static as ST
from diff_2d_fem_gb300 import ImplicitIntegrator, Model, scene

E, NU, RHO = 1.0e6, 0.40, 1100.0
EP = E / (1 - NU * NU)                      # plane-strain modulus
FAR = (0.0, -5.0)                           # a collider parked out of reach


def _problem(m, integ, dt):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return scene.solver_problem(m, integ, dt)


def _cantilever(ny, aspect, hb=0.004, damping=2000.0):
    m = Model()
    m.add_disc(center=FAR, radius=0.01)
    m.damping = damping
    h = m.add_soft_body(np.ones((ny, ny * aspect), np.uint8), physical_size=(hb * aspect, hb), center=(0.0, 0.0),
                        E=E, nu=NU, density=RHO)
    m.finalize()
    X = np.asarray(m.me.rest_pos, np.float64)
    left = np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0]
    m.set_kinematic_constraint(h, left)
    return m, h, X, left


def _curvature(X, x, L):
    """Curvature of the mid-line between 20 % and 80 % of the span: a least-squares circle."""
    mid = np.where(np.abs(X[:, 1]) < 1e-9)[0]
    mid = mid[np.argsort(X[mid, 0])]
    s = (X[mid, 0] - X[mid, 0].min()) / L
    p = x[mid[(s > 0.2) & (s < 0.8)]]
    p = p - p.mean(0)
    a, b, c = np.linalg.lstsq(np.c_[2 * p, np.ones(len(p))], (p ** 2).sum(1), rcond=None)[0]
    return 1.0 / np.sqrt(c + a * a + b * b)


def _newton(m, fixed, Bm=None, area=None, **kw):
    me = m.me
    return ST.solve_static(me.rest_pos, me.tri, me.D_m_inv if Bm is None else Bm,
                           me.rest_area if area is None else area, me.mu, me.lam, fixed, **kw)


def _settle(m, steps, dt=5e-2):
    integ = ImplicitIntegrator(max_iter=2000, eps=1e-14, tol_x=0.0, alpha_max=1e9, self_collision=False,
                               friction=False)
    _, xs, _ = oracle.run(_problem(m, integ, dt), steps)
    return xs[-1]


def test_newton_tangent_and_force_are_derivatives():
    """The static solver's own pin: its force is the derivative of its energy and its tangent
    the derivative of its force (central differences), elastic and tendon terms alike."""
    m, h, X, _ = _cantilever(3, 4, 0.003)
    rng = np.random.default_rng(5)
    x = X + 2e-5 * rng.standard_normal(X.shape)
    me = m.me
    nodes = np.arange(0, X.shape[0], 3)
    for fn in (lambda y, t=True: ST.elastic(y, me.tri, me.D_m_inv, me.rest_area, me.mu, me.lam, t),
               lambda y, t=True: ST.tendon(y, nodes, 7.0)):
        E0, g, K = fn(x)
        v = rng.standard_normal(X.shape)
        eps = 1e-7
        Ep, gp, _ = fn(x + eps * v, False)
        Em, gm, _ = fn(x - eps * v, False)
        assert abs((Ep - Em) / (2 * eps) - (g * v).sum()) < 1e-6 * np.abs(g).sum() * np.abs(v).max()
        Kv = (K @ v.ravel()).reshape(-1, 2)
        assert np.abs((gp - gm) / (2 * eps) - Kv).max() < 1e-5 * np.abs(Kv).max()


def test_rigid_region_bends_like_newton():
    """A cantilever whose outer 40 % is a rigid region, tip-loaded: the oracle, run to rest,
    deflects the tip as the Newton equilibrium of the same mesh in which that part is simply
    1000 times stiffer (within 1 %), and the region turns without straining."""
    m = Model()
    m.damping = 300.0
    h = m.add_soft_body(np.ones((6, 30), np.uint8), physical_size=(0.020, 0.004), center=(0.0, 0.0),
                        E=E, nu=NU, density=RHO)
    m.finalize()
    region = np.zeros((6, 30), bool)
    region[:, 18:] = True
    m.add_affine_region(h, region)
    X = np.asarray(m.me.rest_pos, np.float64)
    left = np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0]
    tip = np.where(X[:, 0] > X[:, 0].max() - 1e-9)[0]
    m.set_kinematic_constraint(h, left)
    f = np.zeros_like(X)
    f[tip, 1] = -6.0 / len(tip)                                  # 6 N/m down, at the tip
    xr, res = _newton(m, left, fext=f, ramps=10)
    assert res < 1e-8
    m.set_external_force(h, f)
    integ = ImplicitIntegrator(self_collision=False, friction=False)
    prob = _problem(m, integ, 2e-3)
    s, xs, _ = oracle.run(prob, 300)
    x = xs[-1]
    d, dr = (x[tip, 1] - X[tip, 1]).mean(), (xr[tip, 1] - X[tip, 1]).mean()
    assert dr < -1e-3, "the load should bend the beam by more than a millimetre"
    assert abs(d / dr - 1.0) < 0.01, (d, dr)
    q = s.state["a_q"].reshape(-1, 6)[0]
    A = np.array([[q[1], q[2]], [q[4], q[5]]])
    assert np.abs(A.T @ A - np.eye(2)).max() < 1e-3
    assert abs(np.arctan2(A[1, 0] - A[0, 1], A[0, 0] + A[1, 1])) > 0.05


def test_tendon_bends_a_cantilever_like_newton():
    """A tendon at e = h/4 above the mid-line through every column loads the beam with the
    pure moment T e: the Newton equilibrium approaches beam theory's T e / (E' I) as the mesh
    refines (within 15 % at 8 elements through the thickness, closer at 16), and the oracle's
    step, run to rest, reaches the Newton curvature of its mesh within 1.5 %."""
    hb, aspect, T = 0.004, 5, 60.0
    e = hb / 4.0
    beam = T * e / (EP * hb ** 3 / 12)

    def setup(ny):
        m, h, X, left = _cantilever(ny, aspect, hb)
        td = m.add_tendon(h, through=[(xx, e) for xx in np.unique(np.round(X[:, 0], 9))])
        m.set_tendon_tension(td, T)
        return m, X, left, m._tendons[td].nodes

    kr = {}
    for ny in (8, 16):
        m, X, left, nodes = setup(ny)
        xr, res = _newton(m, left, tendon_nodes=nodes, T=T)
        assert res < 1e-8
        kr[ny] = _curvature(X, xr, hb * aspect)
    assert abs(kr[16] / beam - 1) < abs(kr[8] / beam - 1) < 0.15, (kr, beam)
    m, X, _, _ = setup(8)
    k = _curvature(X, _settle(m, 12), hb * aspect)
    assert abs(k / kr[8] - 1) < 0.015, (k, kr[8])


def test_active_bilayer_bends_like_newton():
    """The lower half of a cantilever contracts by 1 % (an active region): a bimetal strip.
    The Newton equilibrium of the changed rest shape is within 15 % of Timoshenko's
    1.5 eps / h, and the oracle's step reaches it within 1.5 %."""
    hb, aspect, ny, eps_a = 0.004, 5, 8, 0.01
    m, h, X, left = _cantilever(ny, aspect, hb)
    region = np.zeros((ny, ny * aspect), bool)
    region[: ny // 2] = True
    r = m.add_active_region(h, region)
    m.set_activation(r, 1.0 - eps_a)
    Bm, area, _ = scene.rest_shape(m)
    xr, res = _newton(m, left, Bm=Bm, area=area)
    assert res < 1e-8
    kr = _curvature(X, xr, hb * aspect)
    assert abs(kr / (1.5 * eps_a / hb) - 1) < 0.15, kr
    k = _curvature(X, _settle(m, 12), hb * aspect)
    assert abs(k / kr - 1) < 0.015, (k, kr)
