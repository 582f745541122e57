"""Device read-outs: per-element strain and stress (Model.element_strain / element_stress,
d2f_element_fields) against the numpy restatement of core/fields.py, and a closed form."""
import numpy as np
import pytest

from oracle import fields as OF

pytestmark = pytest.mark.gpu


def _model():
    from diff_2d_fem_gb300 import Model
    m = Model()
    mk = np.ones((12, 20), np.uint8)
    mk[4:8, 6:12] = 0
    E = np.exp(np.random.default_rng(0).uniform(np.log(2e5), np.log(2e6), mk.shape))
    h = m.add_soft_body(mk, physical_size=(0.020, 0.012), center=(0.0, 0.0), E=E, nu=0.45, density=1000.0)
    m.finalize()
    return m, h


@pytest.mark.parametrize("field", ["strain", "stress"])
@pytest.mark.parametrize("signed", [False, True])
def test_element_fields_match_numpy(field, signed):
    m, h = _model()
    rng = np.random.default_rng(1)
    X = np.asarray(m.me.rest_pos, np.float64)
    x = X + 0.08 * (X - X.mean(0))[:, ::-1] * [1, -1] + 3e-4 * np.sin(400 * X) + 1e-5 * rng.standard_normal(X.shape)
    got = (m.element_strain if field == "strain" else m.element_stress)(x, signed=signed)
    ref = OF.element_field(m.me.tri, m.me.D_m_inv, m.me.mu, m.me.lam, x, field, signed)
    assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()
    sub = (m.element_strain if field == "strain" else m.element_stress)(x, handle=h, signed=signed)
    assert np.array_equal(sub, got[m.body_elements(h)])


def test_uniform_stretch_closed_form():
    """F = s I: Green-Lagrange e = (s^2 - 1)/2 in-plane, E_zz = 0: von Mises 2|e|/3, signed e."""
    m, _ = _model()
    X = np.asarray(m.me.rest_pos, np.float64)
    s = 1.03
    e = 0.5 * (s * s - 1.0)
    x = s * X
    assert np.allclose(m.element_strain(x), 2.0 * e / 3.0, rtol=1e-12)
    assert np.allclose(m.element_strain(x, signed=True), e, rtol=1e-12)


def _settle(m, steps=300, dt=5e-3):
    from diff_2d_fem_gb300 import ImplicitIntegrator
    integ = ImplicitIntegrator(precision="fp64", max_iter=2000, eps=1e-14)
    for _ in range(steps):
        integ.simulate(m, dt)
    return m._solver


def test_resting_block_contact_force_balances_weight():
    """A block settled on the ground: the ground's contact force on its nodes carries its
    weight, the ground's reaction is its weight downward, and with the block at rest the
    friction in the reaction vanishes (PNCG2DSolver.contact_force / collider_force)."""
    from diff_2d_fem_gb300 import Model
    m = Model()
    m.add_ground(0.0, mu=0.5)
    m.damping = 20.0
    h = m.add_soft_body(np.ones((8, 8), np.uint8), physical_size=(0.008, 0.008), center=(0.0, 0.0041),
                        E=2.0e5, nu=0.4, density=1000.0)
    m.finalize()
    m.gravity = (0.0, -9.81)
    s = _settle(m)
    W = float(np.asarray(m.me.mass).sum()) * 9.81
    F = s.contact_force(bodies=False)
    assert abs(F[:, 1].sum() - W) < 1e-3 * W
    assert abs(F[:, 0].sum()) < 1e-3 * W
    R = s.collider_force(0)
    assert np.allclose(R[0], [0.0, -W], atol=1e-3 * W)
    Rf = s.collider_force(0, include_friction=True)
    assert np.allclose(Rf, R, atol=1e-3 * W)
    assert np.abs(s.contact_force(colliders=False)).max() < 1e-9 * W


def test_stacked_blocks_contact_between_bodies():
    """A block settled on another: the contact between bodies pushes the upper block up by
    its weight, and its forces sum to zero over both (action and reaction)."""
    from diff_2d_fem_gb300 import Model
    m = Model()
    m.add_ground(0.0, mu=0.5)
    m.damping = 20.0
    lo = m.add_soft_body(np.ones((6, 10), np.uint8), physical_size=(0.010, 0.006), center=(0.0, 0.0031),
                         E=3.0e5, nu=0.4, density=1000.0)
    up = m.add_soft_body(np.ones((6, 6), np.uint8), physical_size=(0.006, 0.006), center=(0.0, 0.0095),
                         E=3.0e5, nu=0.4, density=1000.0)
    m.finalize()
    m.gravity = (0.0, -9.81)
    s = _settle(m)
    Wup = float(np.asarray(m.me.mass)[m.body_nodes(up)].sum()) * 9.81
    Fb = s.contact_force(colliders=False)
    assert np.abs(Fb.sum(0)).max() < 1e-9 * Wup
    assert abs(Fb[m.body_nodes(up), 1].sum() - Wup) < 1e-2 * Wup
    F = s.contact_force()
    Wall = float(np.asarray(m.me.mass).sum()) * 9.81
    assert abs(F[:, 1].sum() - Wall) < 1e-2 * Wall


def test_energy_readout_matches_oracle():
    """PNCG2DSolver.energy: every term of every scene at the state three steps left, against
    the oracle's energy at its own (1e-9-equal) state; reading it moves nothing."""
    import oracle
    from diff_2d_fem_gb300 import ImplicitIntegrator
    from test_actuation_gpu import _actuated, _simulate
    from test_actuation_oracle import _prob
    m, _, _ = _actuated()
    integ = ImplicitIntegrator(precision="fp64")
    prob = _prob(m, integ, 1e-3)
    o, _, _ = oracle.run(prob, 3)
    _simulate(m, integ, 3)
    s = m._solver
    x0 = s.get_x()
    e = s.energy()
    eo = o.energy()
    assert np.abs(e - eo).max() <= 1e-7 * np.abs(eo).max()
    assert np.array_equal(s.get_x(), x0)
    _simulate(m, integ, 1)
    o.step()
    from helpers import rel_err
    assert rel_err(s.get_x(), o.x) < 1e-9
