"""The numpy restatement of the reference's strain and stress read-outs (oracle/fields.py,
the checker of the device's d2f_element_fields) against closed forms, on the CPU — after the
reference's tests/test_fields.py: uniform scaling, rigid motion, signed principal values in
any orientation, the hydrostatic state of a pressurised body, and a sagging cantilever
(Newton equilibrium) in tension on top and compression below."""
import warnings

import numpy as np

import oracle
from oracle import fields as FLD
from oracle import static as ST
from diff_2d_fem_gb300 import ImplicitIntegrator, Model, scene

E, NU, RHO = 1.0e6, 0.40, 1100.0
MU = E / (2 * (1 + NU))
LAM = E * NU / ((1 + NU) * (1 - 2 * NU))


def _block():
    m = Model()
    h = m.add_soft_body(np.ones((6, 8), np.uint8), physical_size=(0.008, 0.006), center=(0.0, 0.0),
                        E=E, nu=NU, density=RHO)
    m.finalize()
    return m, h


def _field(m, x, field, signed=False):
    me = m.me
    return FLD.element_field(me.tri, me.D_m_inv, me.mu, me.lam, x, field, signed)


def test_closed_forms():
    m, _ = _block()
    X = np.asarray(m.me.rest_pos, np.float64)
    assert _field(m, X, "strain").max() < 1e-12 and _field(m, X, "stress").max() < 1e-6
    for s in (0.9, 1.05, 1.3):
        x = s * (X - X.mean(0)) + X.mean(0)
        e = 0.5 * (s * s - 1.0)
        assert np.allclose(_field(m, x, "strain"), 2.0 * abs(e) / 3.0, rtol=1e-12, atol=0)
        assert np.allclose(_field(m, x, "stress"), MU * abs(s * s - 1.0) / (s * s), rtol=1e-9, atol=0)
    th = 0.7
    R = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
    x = X @ R.T + [0.004, -0.01]
    assert _field(m, x, "strain").max() < 1e-12
    assert _field(m, x, "stress").max() < 1e-6 * E


def test_signed_fields():
    m, _ = _block()
    X = np.asarray(m.me.rest_pos, np.float64)
    c = X.mean(0)
    for (s1, s2), e_expect in (((1.10, 0.95), 0.5 * (1.10 ** 2 - 1)), ((1.02, 0.90), 0.5 * (0.90 ** 2 - 1))):
        J = s1 * s2
        sig = [(MU * si * si + LAM * np.log(J) - MU) / J for si in (s1, s2)]
        s_expect = sig[int(np.argmax(np.abs(sig)))]
        for th in (0.0, 0.6, -1.3):
            R = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
            x = (X - c) @ (R @ np.diag([s1, s2]) @ R.T).T + c
            assert np.allclose(_field(m, x, "strain", True), e_expect, rtol=1e-10, atol=0)
            assert np.allclose(_field(m, x, "stress", True), s_expect, rtol=1e-9, atol=0)
            assert np.allclose(_field(m, x @ R.T, "strain", True), e_expect, rtol=1e-10, atol=0)


def test_stress_of_a_hydrostatic_state():
    """The same pressure in both cavities and outside: every element at the in-plane stress
    -p (1e-3), no shear; the von Mises stress is |-p - sigma_zz| (2e-3)."""
    p = 6.0e4
    mk = np.ones((20, 14), np.uint8)
    mk[5:15, 4:10] = 0
    mk[2:4, 8:12] = 0
    m = Model()
    m.damping = 2000.0
    m.add_disc(center=(0.0, -5.0), radius=0.01)
    m.add_soft_body(mk, physical_size=(0.014, 0.020), center=(0.03, 0.05), E=E, nu=NU, density=RHO)
    m.finalize()
    h = 0
    for ch in m.add_pressure_chambers(h) + [m.add_ambient_pressure(h)]:
        m.set_pressure(ch, p)
    integ = ImplicitIntegrator(max_iter=2000, eps=1e-14, tol_x=0.0, self_collision=False, friction=False)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob = scene.solver_problem(m, integ, 5e-3)
    _, xs, _ = oracle.run(prob, 30)
    F = FLD.deformation_gradient(m.me.tri, m.me.D_m_inv, xs[-1])
    J = np.linalg.det(F)
    S = (MU * (F @ F.transpose(0, 2, 1)) + (LAM * np.log(J) - MU)[:, None, None] * np.eye(2)) / J[:, None, None]
    for i in (0, 1):
        assert np.abs(S[:, i, i] / -p - 1.0).max() < 1e-3
    assert np.abs(S[:, 0, 1]).max() < 1e-3 * p
    szz = LAM * np.log(J) / J
    assert np.allclose(_field(m, xs[-1], "stress"), np.abs(-p - szz), rtol=2e-3)


def test_a_sagging_cantilever_is_pulled_on_top():
    """A cantilever clamped at x = 0 sagging under its own weight (the Newton equilibrium):
    near the clamp the top face is in tension and the bottom in compression, in strain and
    stress alike."""
    m = Model()
    h = m.add_soft_body(np.ones((8, 40), np.uint8), physical_size=(0.040, 0.008), center=(0.020, 0.0),
                        E=E, nu=NU, density=RHO)
    m.finalize()
    me = m.me
    X = m.rest_x(h)
    left = np.where(X[:, 0] < 1e-9)[0]
    x, res = ST.solve_static(me.rest_pos, me.tri, me.D_m_inv, me.rest_area, me.mu, me.lam, left,
                             fext=np.asarray(me.mass)[:, None] * [0.0, -200.0])
    assert res < 1e-8 and x[:, 1].min() < -1e-4
    cen = X[np.asarray(me.tri)].mean(1)
    near = cen[:, 0] < 0.010
    top, bottom = near & (cen[:, 1] > 0.003), near & (cen[:, 1] < -0.003)
    for field in ("strain", "stress"):
        v = _field(m, x, field, True)
        assert (v[top] > 0).all() and (v[bottom] < 0).all(), field
