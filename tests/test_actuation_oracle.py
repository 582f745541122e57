"""Actuators on the CPU: the Model's chamber / spring / active-region geometry, the oracle's
spring and pressure terms against finite differences of their own energy, and closed-form
states solved by the oracle (the reference's tests/test_actuation.py cases 1 and 2).

Besides the golden fixture tests/golden/actuators.npz (recorded from the reference's own
kernels through the serial Warp stand-in, reproduced bit for bit in test_oracle_golden.py),
the oracle is pinned here by the derivative identities (gradient = d energy, curvature =
d gradient, diagonal = the true second derivative) and by states with exact answers: a
hydrostatic pressure compresses any body uniformly, a fully active body takes the
prescribed shape stress-free.
"""
import warnings

import numpy as np
import pytest

import oracle
from diff_2d_fem_gb300 import ImplicitIntegrator, Model, scene
from diff_2d_fem_gb300 import actuators as act

E, NU, RHO = 1.0e6, 0.40, 1100.0
FAR = (0.0, -5.0)


def _model(mask, size, center=(0.0, 0.0), damping=2000.0, second=None):
    m = Model()
    m.add_disc(center=FAR, radius=0.01)
    m.damping = damping
    h = m.add_soft_body(mask, physical_size=size, center=center, E=E, nu=NU, density=RHO)
    h2 = None
    if second is not None:
        h2 = m.add_soft_body(np.ones((4, 4), np.uint8), physical_size=(0.004, 0.004), center=second,
                             E=E, nu=NU, density=RHO)
    m.finalize()
    return m, h, h2


def _cavity_block(second=None):
    mk = np.ones((20, 14), np.uint8)
    mk[5:15, 4:10] = 0
    return _model(mk, (0.014, 0.020), center=(0.03, 0.05), second=second)


def _integ(max_iter=3000, **kw):
    return ImplicitIntegrator(max_iter=max_iter, eps=1e-14, tol_x=2e-9, conv_check=8,
                              self_collision=False, friction=False, **kw)


def _prob(m, integ, dt):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return scene.solver_problem(m, integ, dt)


# ---------------------------------------------------------------------- geometry
def test_chamber_geometry():
    m, h, _ = _cavity_block()
    ch = m.add_pressure_chambers(h)
    assert len(ch) == 1
    pw, ph = m.pixel_size(h)
    assert abs(m.chamber_area(ch[0]) - 60 * pw * ph) < 1e-12
    amb = m.add_ambient_pressure(h)
    assert abs(m.chamber_area(amb) - 280 * pw * ph) < 1e-12        # outline encloses solid + cavity
    c = m._chambers[ch[0]]
    assert len(c.ea) == 2 * (10 + 6)                              # the cavity's perimeter in pixels
    with pytest.raises(ValueError):
        m.add_pressure_chamber(h, at=(0.0, 0.0))                      # off the body
    mk = np.ones((20, 14), np.uint8)
    mk[5:15, 4:10] = 0
    mk[2:4, 8:12] = 0
    m2, h2, _ = _model(mk, (0.014, 0.020), center=(0.03, 0.05))
    assert len(m2.add_pressure_chambers(h2)) == 2
    mk[10, 0:5] = 0                                                   # a channel to the outside
    m3, h3, _ = _model(mk, (0.014, 0.020), center=(0.03, 0.05))
    assert len(m3.add_pressure_chambers(h3)) == 1
    with pytest.raises(ValueError):
        m3.add_pressure_chamber(h3, at=(0.03 - 0.007 + 6.5 * 0.001, 0.05 - 0.010 + 10.5 * 0.001))


def test_activation_matrix_and_region():
    A = act.activation_matrix(0.85, 1.10, np.deg2rad(30.0))
    f = np.array([np.cos(np.deg2rad(30.0)), np.sin(np.deg2rad(30.0))])
    assert np.allclose(A @ f, 0.85 * f)
    assert np.allclose(np.linalg.svd(A)[1], [1.10, 0.85])
    assert np.allclose(act.activation_matrix(1.08), 1.08 * np.eye(2))
    mk = np.ones((16, 10), np.uint8)
    mk[5:9, 3:7] = 0
    m, h, _ = _model(mk, (0.010, 0.016))
    r = m.add_active_region(h, np.ones_like(mk))
    assert len(m._regions[r].elems) == 2 * int(mk.sum())
    with pytest.raises(ValueError):
        m.add_active_region(h, np.ones_like(mk))                      # overlaps
    m.set_activation(r, 1.08)
    Bm, area, Dm = scene.rest_shape(m)
    e1 = Dm[:, :2]
    Bm0 = np.asarray(m.me.D_m_inv, np.float64).reshape(-1, 2, 2)
    assert np.allclose(area, 1.08 ** 2 * np.asarray(m.me.rest_area))
    assert np.allclose(Bm.reshape(-1, 2, 2), Bm0 / 1.08)
    rest, tri = m.me.rest_pos, np.asarray(m.me.tri)
    assert np.allclose(e1, 1.08 * (rest[tri[:, 1]] - rest[tri[:, 0]]))


def test_spring_api():
    m, h, h2 = _cavity_block(second=(0.03, 0.065))
    s1 = m.add_spring(h, (0.024, 0.059), h2, (0.029, 0.064), stiffness=2.0e4)
    pin = m.add_pin(h, (0.036, 0.041))
    assert m._springs[pin].b == -1 and m._springs[pin].length == 0.0
    assert m._springs[s1].length > 0.0
    t, ln = m.spring_force(s1)
    assert abs(t) < 1e-9 and ln > 0
    with pytest.raises(NotImplementedError):
        m.add_pin(h, (0.03, 0.05), handle_b=h2)
    with pytest.raises(ValueError):
        m.set_spring_anchor(s1, (0.0, 0.0))


# ---------------------------------------------------------------------- derivatives
def _harness(prob, rng_seed=1):
    o = oracle.OracleSolver(prob)
    rng = np.random.default_rng(rng_seed)
    rest = np.asarray(prob["x"], np.float64)
    X = rest - rest.mean(0)
    x0 = rest + 0.045 * X[:, ::-1] * [1, -1] + 2e-4 * np.sin(300 * X) + 1.5e-4 * rng.standard_normal(rest.shape)
    xn = x0 - 2e-4 * rng.standard_normal(rest.shape)
    return o, x0, xn, rng


def _check_derivatives(prob, which):
    """The reference's derivative check (tests/test_actuation.py:_check_derivatives)."""
    o, x0, xn, rng = _harness(prob)
    g, dH, _, _ = o.term(which, x0, xn=xn)
    assert np.abs(g).max() > 0
    assert dH.min() >= 0.0
    d = rng.standard_normal(x0.shape)
    d /= np.abs(d).max()
    energy = lambda x: o.term(which, x, xn=xn)[3].sum()
    grad = lambda x: o.term(which, x, xn=xn)[0]
    fd = lambda f, e: (f(x0 + e * d) - f(x0 - e * d)) / (2 * e)
    err = min(abs(fd(energy, e) - (g * d).sum()) / abs(fd(energy, e)) for e in (4e-5, 2e-5, 1e-5))
    assert err < 1e-3, f"{which}: gradient vs d energy {err:.1e}"
    ph = o.term(which, x0, p=d, xn=xn)[2].sum()
    err = min(abs((fd(grad, e) * d).sum() - ph) / abs(ph) for e in (4e-5, 2e-5, 1e-5))
    assert err < 1e-3, f"{which}: pHp vs d gradient {err:.1e}"
    if dH.max() > 0:
        idx = np.argwhere(dH > 1e-3 * dH.max())
        for i, c in idx[:: max(1, len(idx) // 12)]:
            e = np.zeros_like(x0)
            e[i, c] = 1.0
            true = (grad(x0 + 2e-5 * e)[i, c] - grad(x0 - 2e-5 * e)[i, c]) / 4e-5
            assert abs(true - dH[i, c]) < 2e-3 * abs(true), f"{which}: diagonal {dH[i, c]:.4e} vs {true:.4e}"


def test_pressure_derivatives():
    m, h, _ = _cavity_block()
    m.set_pressure(m.add_pressure_chambers(h)[0], 3.0e4)
    m.set_pressure(m.add_ambient_pressure(h), 1.1e4)
    _check_derivatives(_prob(m, _integ(max_iter=1), 1e-3), "pressure")


def test_spring_derivatives():
    m, h, h2 = _cavity_block(second=(0.03, 0.065))
    s1 = m.add_spring(h, (0.024, 0.059), h2, (0.029, 0.064), stiffness=2.0e4)
    s2 = m.add_spring(h, (0.036, 0.041), None, (0.040, 0.035), stiffness=3.0e4, rest_length=0.004)
    m.add_pin(h, (0.024, 0.041), stiffness=1.0e4)
    m.set_spring_length(s2, 0.003)
    # stretched springs only: a compressed one's tangential stiffness is clamped at zero in
    # the diagonal and in p^T H p (actuation.py:391-393), which no derivative reproduces
    m.set_spring_length(s1, 0.5 * m._springs[s1].length)
    prob = _prob(m, _integ(max_iter=1), 1e-3)
    sp = prob["springs"]
    assert list(sp["b"][1:]) == [-1, -1] and sp["L0"][1] == 0.003
    _check_derivatives(prob, "springs")


# ---------------------------------------------------------------------- closed forms (oracle)
def _hydrostatic_stretch(p):
    mu, lam = E / (2 * (1 + NU)), E * NU / ((1 + NU) * (1 - 2 * NU))
    sig = lambda s: (mu * (s - 1 / s) + 2 * lam * np.log(s) / s) / s     # Neo-Hookean, F = s I
    lo, hi = 0.5, 1.0
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        lo, hi = (mid, hi) if sig(mid) < -p else (lo, mid)
    return 0.5 * (lo + hi)


def test_hydrostatic_state_is_exact_oracle():
    """The same pressure in both cavities and outside: a uniform stretch s with sigma(s) = -p,
    for any geometry (reference tests/test_actuation.py:148-180)."""
    p = 6.0e4
    s_exact = _hydrostatic_stretch(p)
    mk = np.ones((20, 14), np.uint8)
    mk[5:15, 4:10] = 0
    mk[2:4, 8:12] = 0
    m, h, _ = _model(mk, (0.014, 0.020), center=(0.03, 0.05))
    for c in m.add_pressure_chambers(h) + [m.add_ambient_pressure(h)]:
        m.set_pressure(c, p)
    _, xs, _ = oracle.run(_prob(m, _integ(max_iter=2000), 5e-3), 30)
    X = np.asarray(m.me.rest_pos, np.float64)
    Xc = X - X.mean(0)
    x = xs[-1]
    s_fem = float(((x - x.mean(0)) * Xc).sum() / (Xc ** 2).sum())
    assert abs(s_fem - s_exact) < 5e-3 * (1 - s_exact), (s_fem, s_exact)
    dev = np.abs((x - x.mean(0)) - s_exact * Xc).max()
    assert dev < 1e-4 * np.ptp(X[:, 1])
    # the cavities' sign flipped: nowhere near hydrostatic, so the test can fail
    for i, c in enumerate(m._chambers):
        m.set_pressure(i, -p if c.sign > 0 else p)
    _, xs, _ = oracle.run(_prob(m, _integ(max_iter=2000), 5e-3), 30)
    x = xs[-1]
    assert np.abs((x - x.mean(0)) - s_exact * Xc).max() > 100 * dev


def test_active_material_free_growth_oracle():
    """An unconstrained body whose every element changes rest shape by A takes the shape A
    (reference tests/test_actuation.py:217-237): isotropic 1.08, then 0.85 along a fiber at
    30 degrees with 1.10 across."""
    mk = np.ones((16, 10), np.uint8)
    mk[5:9, 3:7] = 0
    m, h, _ = _model(mk, (0.010, 0.016))
    m.set_activation(m.add_active_region(h, np.ones_like(mk)), 1.08)
    _, xs, _ = oracle.run(_prob(m, _integ(alpha_max=1e9), 2e-2), 10)
    X = np.asarray(m.me.rest_pos, np.float64)
    x = xs[-1]
    assert np.abs((x - x.mean(0)) - 1.08 * (X - X.mean(0))).max() < 1e-4 * 0.016
    m, h, _ = _model(mk, (0.010, 0.016))
    th = np.deg2rad(30.0)
    m.set_activation(m.add_active_region(h, np.ones_like(mk), fiber=th), 0.85, transverse=1.10)
    _, xs, _ = oracle.run(_prob(m, _integ(alpha_max=1e9), 2e-2), 10)
    x = xs[-1]
    F = np.linalg.lstsq(X - X.mean(0), x - x.mean(0), rcond=None)[0].T
    assert np.allclose(np.linalg.svd(F)[1], [1.10, 0.85], atol=2e-4)
    f = np.array([np.cos(th), np.sin(th)])
    assert abs(np.linalg.norm(F @ f) - 0.85) < 2e-4


def test_chambers_of_random_masks_are_closed_and_oriented():
    """Random masks with cavities, corner-touching voids and channels to the outside: every
    sealed cavity becomes a chamber whose walls form closed loops (each node entered as often
    as left) enclosing exactly its pixels, the outline encloses solid plus cavities, and the
    void regions that reach the border are no chambers."""
    rng = np.random.default_rng(11)
    for trial in range(12):
        mk = (rng.random((18, 26)) > 0.22).astype(np.uint8)
        mk[0], mk[-1], mk[:, 0], mk[:, -1] = 1, 1, 1, 1
        if trial % 3 == 0:
            mk[9, :6] = 0                                     # a channel to the outside
        m, h, _ = _model(mk, (0.026, 0.018), center=(0.0, 0.05))
        lab, sealed = act.enclosed_voids(mk)
        chambers = m.add_pressure_chambers(h)                 # raises if a loop is open or mis-oriented
        assert len(chambers) == len(sealed)
        pw, ph = m.pixel_size(h)
        for c in chambers:
            ea, eb = m._chambers[c].ea, m._chambers[c].eb
            assert np.array_equal(np.sort(ea), np.sort(eb))     # closed: in-degree = out-degree
        total = sum(m._chambers[c].area0 for c in chambers)
        assert abs(total - sum((lab == k).sum() for k in sealed) * pw * ph) < 1e-15
        amb = m.add_ambient_pressure(h)
        assert abs(m.chamber_area(amb) - (mk.sum() + sum((lab == k).sum() for k in sealed)) * pw * ph) < 1e-12
