"""Physical checks of the oracle on the CPU, the counterparts of the device tests in
test_physics_gpu.py on smaller or shorter cases: environments do not interact, a free rigid
body falls exactly as backward Euler, a pinned bar swings with the period of a physical
pendulum, a block slides down a held slab at the Coulomb speed, a thrown block neither
touches nor enters another body and keeps the momentum through the impact — after the
reference's tests/test_rigid.py, test_scene.py and test_ipc.py.

These pin the oracle's physics by closed forms, independent of the golden fixtures, so the
checker the device path is compared against is itself checked against mechanics."""
import warnings

import numpy as np
import pytest

import oracle
from diff_2d_fem_gb300 import ImplicitIntegrator, Model, scene

G0 = 9.81
PX = 0.5e-3


def _problem(m, integ, dt):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return scene.solver_problem(m, integ, dt)


def _com(m, nodes, x):
    w = np.asarray(m.me.mass, np.float64)[nodes]
    return (w[:, None] * x[nodes]).sum(0) / w.sum()


def test_environments_do_not_interact_oracle():
    """A design alone and the same design in a batch of three (the middle one different),
    pressed by gravity onto a disc: positions identical bit for bit (every reduction of the
    oracle runs per environment, over that environment's nodes in order)."""
    rng = np.random.default_rng(3)
    d1 = np.ones((12, 6), np.uint8)
    d1[3:9, 2:4] = 0
    d2 = (rng.random((12, 6)) > 0.15).astype(np.uint8)
    d2[-1] = 1
    d2[:, 0] = 1

    def run(designs):
        m = Model()
        m.add_disc(center=(0.05, 0.030), radius=0.006, mu=0.6)
        hs = [m.add_soft_body(d, physical_size=(0.006, 0.012), center=(0.05, 0.0435), E=1.0e6, nu=0.40,
                              density=1100.0, env_id=i) for i, d in enumerate(designs)]
        m.finalize()
        m.gravity = (0.0, -G0)
        integ = ImplicitIntegrator(precision="fp64")
        s, xs, _ = oracle.run(_problem(m, integ, 2e-3), 40)
        return m, hs, s, xs[-1]

    ma, (ha,), sa, xa = run([d1])
    mb, hb, sb, xb = run([d1, d2, d1])
    na = ma.body_nodes(ha)
    assert xa[na, 1].min() < 0.0435 - 0.006 - 1e-4, "the body never reached the disc"
    assert np.isfinite(xb).all()
    for env, h in ((0, hb[0]), (2, hb[2])):
        assert np.array_equal(xb[mb.body_nodes(h)], xa[na]), env
    assert np.abs(xb[mb.body_nodes(hb[1])].mean(0) - xa[na].mean(0)).max() > 1e-6


def test_free_rigid_body_is_exact_backward_euler_oracle():
    """Free fall of an affine block: after n steps of h the drop is g h^2 n (n + 1) / 2, within
    1e-9; a free rigid body converges in a few iterations."""
    m = Model()
    m.damping = 0.0
    h = m.add_affine_body(np.ones((6, 6), np.uint8), physical_size=(0.006, 0.006), center=(0.0, 0.05),
                          density=1000.0)
    m.finalize()
    m.gravity = (0.0, -G0)
    nodes = m.body_nodes(h)
    y0 = _com(m, nodes, m.get_x())[1]
    integ = ImplicitIntegrator(self_collision=False, friction=False, precision="fp64")
    _, xs, its = oracle.run(_problem(m, integ, 1e-3), 100)
    err = (y0 - _com(m, nodes, xs[-1])[1]) / (G0 * 1e-6 * 100 * 101 / 2) - 1
    assert abs(err) < 1e-9, err
    assert max(int(i[0]) for i in its) <= 4
    # the block neither turns nor deforms in free fall
    d = xs[-1][nodes] - m.get_x()[nodes]
    assert np.ptp(d[:, 0]) < 1e-12 and np.ptp(d[:, 1]) < 1e-12


def test_pin_makes_a_pendulum_oracle():
    """A rigid bar pinned at one end under gravity 10 degrees off its axis swings with the
    period of a physical pendulum (within 1 %), and the pin holds (within 1 um)."""
    m = Model()
    m.damping = 0.0
    h = m.add_affine_body(np.ones((4, 24), np.uint8), physical_size=(0.012, 0.002), center=(0.006, 0.0),
                          density=1100.0)
    m.finalize()
    pin = m.add_pin(h, (0.0, 0.0))
    nodes = m.body_nodes(h)
    X = m.rest_x(h)
    mass = np.asarray(m.me.mass, np.float64)[nodes]
    pivot = X[np.linalg.norm(X, axis=1).argmin()]
    d = np.linalg.norm((mass[:, None] * X).sum(0) / mass.sum() - pivot)
    Ip = (mass * ((X - pivot) ** 2).sum(1)).sum()
    th0 = np.deg2rad(10.0)
    period = 2 * np.pi * np.sqrt(Ip / (mass.sum() * G0 * d)) * (1 + th0 ** 2 / 16)
    m.gravity = (G0 * np.cos(th0), -G0 * np.sin(th0))
    dt = 5e-4
    integ = ImplicitIntegrator(self_collision=False, friction=False, precision="fp64")
    _, xs, _ = oracle.run(_problem(m, integ, dt), int(1.1 * period / dt))
    sp = m._springs[pin]
    far = nodes[np.linalg.norm(X - pivot, axis=1).argmax()]
    r0 = m.get_x()[far] - m.get_x()[sp.a]
    ang, gap = [], 0.0
    for x in xs:
        r = x[far] - x[sp.a]
        ang.append(np.arctan2(r0[0] * r[1] - r0[1] * r[0], r0 @ r) + th0)
        gap = max(gap, float(np.linalg.norm(x[sp.a] - sp.anchor)))
    ang = np.array(ang)
    t = dt * np.arange(1, len(ang) + 1)
    k = np.where(np.sign(ang[1:]) != np.sign(ang[:-1]))[0]
    assert len(k) >= 2
    cross = [t[i] - ang[i] * dt / (ang[i + 1] - ang[i]) for i in k[:2]]
    got = 2.0 * (cross[1] - cross[0])
    assert abs(got / period - 1.0) < 0.01, (got, period)
    assert gap < 1e-6, gap


def test_slides_at_the_coulomb_speed_oracle():
    """A rigid block on a held slab under tilted gravity, friction 0.3 between the bodies: it
    rests within the barrier's reach, then slides at the steady speed
    g (sin th - mu cos th) / c_e of the damped backward-Euler step (c_e = (1 - e^(-c dt)) / dt),
    within 1 %."""
    c, dt, mu = 200.0, 1e-3, 0.3
    ce = (1.0 - np.exp(-dt * c)) / dt
    th = np.deg2rad(30.0)
    m = Model()
    m.damping = c
    m.body_friction = mu
    slab = m.add_soft_body(np.ones((4, 40), np.uint8), physical_size=(40 * PX, 4 * PX), center=(0.0, 0.0),
                           E=1.0e6, nu=0.40, density=1100.0)
    block = m.add_affine_body(np.ones((6, 6), np.uint8), physical_size=(6 * PX, 6 * PX),
                              center=(-0.006, 0.001 + 0.0015 + 0.9 * PX / 8), density=1100.0)
    m.finalize()
    m.set_kinematic_constraint(slab, np.arange(m.body_nodes(slab).size))
    integ = ImplicitIntegrator(precision="fp64")
    nb, ns = m.body_nodes(block), m.body_nodes(slab)
    m.gravity = (0.0, -G0 * np.cos(th))
    s, xs, _ = oracle.run(_problem(m, integ, dt), 100)
    x = xs[-1]
    gap = x[nb, 1].min() - x[ns, 1].max()
    assert 0.5 * m.dhat < gap < m.dhat, gap / m.dhat
    s.set_fext(np.asarray(m.me.mass, np.float64)[:, None] * np.array([G0 * np.sin(th), -G0 * np.cos(th)]))
    xb = []
    for _ in range(250):
        s.step()
        xb.append(s.x[nb, 0].mean())
    v = np.diff(np.array(xb)[-150:]).mean() / dt
    expect = G0 * (np.sin(th) - mu * np.cos(th)) / ce
    assert abs(v / expect - 1.0) < 0.01, (v, expect)


def _throw(other, px_per_step, diagonal=False, steps=100):
    """A rigid block thrown at another body, stepped by the oracle: (smallest gap over the run
    in units of dhat, whether a node of the thrown block entered a held block's box, relative
    momentum change)."""
    dt = 2.5e-4
    v0 = px_per_step * PX / dt
    m = Model()
    rigid = lambda c: m.add_affine_body(np.ones((6, 6), np.uint8), physical_size=(6 * PX, 6 * PX), center=c,
                                        density=1100.0)
    if diagonal:
        a, at = rigid((-5 * PX, 5 * PX)), (3 * PX, -3 * PX)
    else:
        a, at = rigid((0.0, 0.0)), (10 * PX, 0.8 * PX)
    b = rigid(at) if other == "rigid" else m.add_soft_body(np.ones((6, 6), np.uint8), physical_size=(6 * PX, 6 * PX),
                                                           center=at, E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    if other == "held":
        m.set_kinematic_constraint(b, np.arange(m.body_nodes(b).size))
    m.set_body_velocity(a, velocity=(v0 / np.sqrt(2.0), -v0 / np.sqrt(2.0)) if diagonal else (v0, 0.0))
    integ = ImplicitIntegrator(friction=False, precision="fp64")
    prob = _problem(m, integ, dt)
    s = oracle.OracleSolver(prob)
    mass = np.asarray(m.me.mass, np.float64)
    na, nb = m.body_nodes(a), m.body_nodes(b)
    both = np.concatenate([na, nb])
    mom = lambda v: (mass[both, None] * v[both]).sum(0)
    p0 = mom(prob["v"])
    xb = m.rest_x(b)
    lo, hi = xb.min(0) + 1e-9, xb.max(0) - 1e-9
    gap, inside = np.inf, False
    for _ in range(steps):
        s.step()
        gap = min(gap, float(scene.min_distance(dict(prob, x=s.x)).min()) / m.dhat)
        if other == "held":
            inside |= bool(((s.x[na] > lo) & (s.x[na] < hi)).all(1).any())
    assert np.isfinite(s.x).all()
    return gap, inside, float(np.linalg.norm(mom(s.v) - p0) / np.linalg.norm(p0))


@pytest.mark.parametrize("other,diagonal", [("soft", False), ("rigid", False), ("held", True), ("held", False)])
def test_nothing_passes_through_oracle(other, diagonal):
    """A rigid block thrown at 4 pixels a step at a soft, a rigid or a held block, head on and
    corner to corner: the surfaces never touch and nothing enters the held block."""
    gap, inside, _ = _throw(other, 4.0, diagonal)
    assert 0.0 < gap < 1.0 and not inside, (gap, inside)                   # contact, never touching


def test_momentum_goes_through_an_impact_oracle():
    """At half a pixel a step into a free soft block, momentum is kept through the impact
    (within 2e-3)."""
    gap, _, dp = _throw("soft", 0.5, steps=80)
    assert gap < 1.0, "the blocks never came within the barrier's reach"
    assert dp < 2e-3, dp


def _lift_scene():
    """A soft block resting on a disc, under gravity."""
    m = Model()
    m.add_disc(center=(0.0, 0.0), radius=0.004, mu=0.5)
    h = m.add_soft_body(np.ones((6, 6), np.uint8), physical_size=(0.003, 0.003),
                        center=(0.0, 0.004 + 0.0015 + 0.9 * 0.0005 / 8), E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    m.gravity = (0.0, -G0)
    return m, h


def test_a_moved_collider_carries_the_body_oracle():
    """set_collider_center between steps: the Model's colliders follow, and a disc raised by
    0.05 dhat a step under a block resting on it carries the block up by as much (within
    0.1 %) against the same run with the disc left in place (the oracle moves the same disc)."""
    m, h = _lift_scene()
    assert m.object.kind == 0 and np.allclose(m.object.c, (0.0, 0.0))
    integ = ImplicitIntegrator(precision="fp64")
    prob = _problem(m, integ, 1e-3)
    s, still = oracle.OracleSolver(prob), oracle.OracleSolver(prob)
    nodes = m.body_nodes(h)
    for _ in range(60):
        s.step()
        still.step()
    dy = 0.05 * m.dhat
    for k in range(1, 41):
        m.set_collider_center(0, (0.0, k * dy))
        s.set_collider_centers([[c.cx, c.cy] for c in m.colliders])
        s.step()
        still.step()
    assert np.allclose(m.colliders[0].c, (0.0, 40 * dy))
    rise = s.x[nodes, 1].mean() - still.x[nodes, 1].mean()
    assert abs(rise / (40 * dy) - 1.0) < 1e-3, rise / (40 * dy)


def test_import_surface():
    """The names a user of the reference imports (its objects, viz and Renderer modules are
    plotting and windowing, not part of this package)."""
    import diff_2d_fem_gb300 as D
    for name in ("Model", "SimConfig", "Mesh", "build_scene", "check_mesh", "mask_to_mesh",
                 "ImplicitIntegrator", "AdjointPNCG2D"):
        assert hasattr(D, name), name


def _cantilever(m, E_, center, size=(0.020, 0.004), shape=(6, 30), env_id=0, density=1100.0):
    return m.add_soft_body(np.ones(shape, np.uint8), physical_size=size, center=center, E=E_, nu=0.40,
                           density=density, env_id=env_id)


def _clamp_droop(m, hs, steps=60):
    for h in hs:
        X = m.rest_x(h)
        m.set_kinematic_constraint(h, np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0])
    m.gravity = (0.0, -G0)
    m.damping = 100.0
    _, xs, _ = oracle.run(_problem(m, ImplicitIntegrator(max_iter=120, self_collision=False, friction=False), 1e-3),
                          steps)
    return xs[-1]


def test_bodies_keep_their_own_geometry_and_material():
    """A cantilever alone and beside a softer, heavier one on another grid in the same scene:
    each body's mass is its own density times its area (1e-9), the shared body droops as it
    does alone (1e-3 of the sag: the two share one environment's step length until both have
    converged), and the softer, heavier one sags more — after the reference's
    tests/test_scene.py:40-78."""
    one = Model()
    h1 = _cantilever(one, 4.0e6, (0.0, 0.0))
    one.finalize()
    xa = _clamp_droop(one, [h1])[one.body_nodes(h1)]
    two = Model()
    hs = _cantilever(two, 1.0e6, (0.0, 0.03), size=(0.016, 0.004), shape=(8, 32), density=2000.0)
    hb = _cantilever(two, 4.0e6, (0.0, 0.0))
    with pytest.warns(UserWarning, match="mixes pixel sizes"):
        two.finalize()
    mass = np.asarray(two.me.mass)
    assert np.isclose(mass[two.body_nodes(hs)].sum(), 2000.0 * 0.016 * 0.004, rtol=1e-9)
    assert np.isclose(mass[two.body_nodes(hb)].sum(), 1100.0 * 0.020 * 0.004, rtol=1e-9)
    x2 = _clamp_droop(two, [hs, hb])
    sag = np.abs(xa - one.rest_x(h1)).max()
    assert sag > 1e-5
    assert np.abs(xa - x2[two.body_nodes(hb)]).max() / sag < 1e-3
    assert np.abs(x2[two.body_nodes(hs)] - two.rest_x(hs)).max() > 2.0 * sag


def test_contact_scales_and_overlap():
    """Contact parameters left unset are scaled to the scene (reach 1/8 pixel, kappa and the
    body stiffness from the softest modulus), and two bodies in one place are refused unless
    they live in different environments — after the reference's tests/test_scene.py:111-151."""
    m = Model()
    m.add_ground(height=0.0, mu=0.6)
    block = np.ones((12, 16), np.uint8)
    reach = 0.5e-3 / 8
    m.add_soft_body(block, physical_size=(0.008, 0.006), E=1.0e6, nu=0.40, density=1100.0,
                    center=(0.0, 0.003 + 0.9 * reach))
    m.add_soft_body(block, physical_size=(0.008, 0.006), E=1.0e6, nu=0.40, density=1100.0,
                    center=(0.0, 0.003 + 0.9 * reach + 0.0068))
    m.finalize()
    assert np.isclose(m.dhat, reach) and np.isclose(m.kappa, 3.2e4) and np.isclose(m.self_stiffness, 2.0e5)
    bad = Model()
    for _ in range(2):
        bad.add_soft_body(np.ones((8, 8), np.uint8), physical_size=(0.008, 0.008), center=(0.0, 0.0))
    with pytest.raises(ValueError, match="env_id"):
        bad.finalize()
    ok = Model()
    for i in range(2):
        ok.add_soft_body(np.ones((8, 8), np.uint8), physical_size=(0.008, 0.008), center=(0.0, 0.0), env_id=i)
    assert ok.finalize().n_envs == 2


def test_collider_centres_reach_the_solver_buffer():
    """DeviceSolver.set_collider_centers writes the centres into columns 1-2 of the collider
    rows the step kernels read, leaving every other parameter as it was (host logic, on a CPU
    tensor standing in for the device buffer)."""
    import types
    import torch
    from diff_2d_fem_gb300.device import DeviceSolver
    rows = torch.arange(24, dtype=torch.float64).reshape(3, 8)
    fake = types.SimpleNamespace(_t={"colliders": rows.clone()})
    DeviceSolver.set_collider_centers(fake, [[0.5, -0.25], [1.5, 2.5], [7.0, 8.0]])
    got = fake._t["colliders"]
    assert torch.equal(got[:, 1:3], torch.tensor([[0.5, -0.25], [1.5, 2.5], [7.0, 8.0]], dtype=torch.float64))
    keep = [0, 3, 4, 5, 6, 7]
    assert torch.equal(got[:, keep], rows[:, keep])
    m = Model()
    m.add_disc((0.0, 0.0), 0.01)
    m.add_object("box", (0.1, 0.2), 0.02, 0.01, corner_radius=0.003)
    m.add_ground(0.0)
    assert [c.kind for c in m.colliders] == [0, 2, 4] and Model().object.kind == -1
    m.set_collider_center(1, (0.3, 0.4))
    assert np.allclose(m.colliders[1].c, (0.3, 0.4)) and m.colliders[1].rref == 0.003
