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
