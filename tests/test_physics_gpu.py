"""Physical checks of the device step through the public API, after the reference's
tests/test_rigid.py, test_scene.py, test_objects.py and test_ipc.py: environments do not
interact (bit for bit in FP64), a free rigid body falls exactly as backward Euler, a pinned
bar swings with the period of a physical pendulum, every collider shape develops contact
without a node inside it, a block slides down a held slab at the Coulomb speed, nothing
passes through anything, momentum goes through an impact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G0 = 9.81


def _com(model, h):
    m = np.asarray(model.me.mass, np.float64)[model.body_nodes(h)]
    return (m[:, None] * model.get_body_x(h)).sum(0) / m.sum()


def test_environments_do_not_interact():
    """A design alone and the same design in a batch of three (the middle one different),
    pressed by gravity onto a disc: FP64 positions and the disc's reaction identical bit for
    bit (each scene runs alone in its block, in a fixed order of operations)."""
    from diff_2d_fem_gb300 import Model, ImplicitIntegrator
    rng = np.random.default_rng(3)
    d1 = np.ones((24, 12), np.uint8)
    d1[6:18, 4:8] = 0
    d2 = (rng.random((24, 12)) > 0.15).astype(np.uint8)
    d2[-1] = 1
    d2[:, 0] = 1

    def run(designs):
        m = Model()
        m.add_disc(center=(0.05, 0.030), radius=0.006, mu=0.6)
        hs = [m.add_soft_body(d, physical_size=(0.012, 0.024), center=(0.05, 0.0495), E=1.0e6, nu=0.40,
                              density=1100.0, env_id=i) for i, d in enumerate(designs)]
        m.finalize()
        m.gravity = (0.0, -G0)
        integ = ImplicitIntegrator(precision="fp64", threads=128)
        for _ in range(60):
            integ.simulate(m, 2e-3)
        return m, hs, integ

    alone, (ha,), ia = run([d1])
    batch, hb, ib = run([d1, d2, d1])
    xa = alone.get_body_x(ha)
    Fa, Fb = ia.collider_force(alone)[0], ib.collider_force(batch)
    assert np.linalg.norm(Fa) > 0.1, "no contact developed"
    for env, h in ((0, hb[0]), (2, hb[2])):
        assert np.array_equal(batch.get_body_x(h), xa), env
        assert np.array_equal(Fb[env], Fa), env
    assert np.abs(batch.get_body_x(hb[1]).mean(0) - xa.mean(0)).max() > 1e-6


def test_free_rigid_body_is_exact_backward_euler():
    """Free fall of an affine block: after n steps of h the drop is g h^2 n (n + 1) / 2 (backward
    Euler), within 1e-9; a free rigid body converges at once."""
    from diff_2d_fem_gb300 import Model, ImplicitIntegrator
    m = Model()
    m.damping = 0.0
    h = m.add_affine_body(np.ones((6, 6), np.uint8), physical_size=(0.006, 0.006), center=(0.0, 0.05),
                          density=1000.0)
    m.finalize()
    m.gravity = (0.0, -G0)
    y0 = _com(m, h)[1]
    integ = ImplicitIntegrator(self_collision=False, friction=False, precision="fp64")
    for _ in range(100):
        integ.simulate(m, 1e-3)
    err = (y0 - _com(m, h)[1]) / (G0 * 1e-6 * 100 * 101 / 2) - 1
    assert abs(err) < 1e-9, err
    assert integ.stats(m)["iters"][0] <= 4


def test_pin_makes_a_pendulum():
    """A rigid bar pinned at one end under gravity 10 degrees off its axis swings with the
    period of a physical pendulum (within 1 %), and the pin holds (within 1 um)."""
    from diff_2d_fem_gb300 import Model, ImplicitIntegrator
    m = Model()
    m.damping = 0.0
    h = m.add_affine_body(np.ones((4, 24), np.uint8), physical_size=(0.012, 0.002), center=(0.006, 0.0),
                          density=1100.0)
    m.finalize()
    pin = m.add_pin(h, (0.0, 0.0))
    X = m.rest_x(h)
    mass = np.asarray(m.me.mass, np.float64)[m.body_nodes(h)]
    pivot = X[np.linalg.norm(X, axis=1).argmin()]
    d = np.linalg.norm((mass[:, None] * X).sum(0) / mass.sum() - pivot)
    Ip = (mass * ((X - pivot) ** 2).sum(1)).sum()
    th0 = np.deg2rad(10.0)
    period = 2 * np.pi * np.sqrt(Ip / (mass.sum() * G0 * d)) * (1 + th0 ** 2 / 16)
    m.gravity = (G0 * np.cos(th0), -G0 * np.sin(th0))
    dt = 5e-4
    integ = ImplicitIntegrator(self_collision=False, friction=False, precision="fp64")
    ang, gap = [], 0.0
    for _ in range(int(1.1 * period / dt)):
        integ.simulate(m, dt)
        ang.append(m.affine_state(0)["angle"] + th0)
        gap = max(gap, abs(m.spring_force(pin)[1]))
    ang = np.array(ang)
    t = dt * np.arange(1, len(ang) + 1)
    k = np.where(np.sign(ang[1:]) != np.sign(ang[:-1]))[0]
    assert len(k) >= 2
    cross = [t[i] - ang[i] * dt / (ang[i + 1] - ang[i]) for i in k[:2]]
    got = 2.0 * (cross[1] - cross[0])
    assert abs(got / period - 1.0) < 0.01, (got, period)
    assert gap < 1e-6, gap


SHAPES = {"disc": dict(rx=0.006), "ellipse": dict(rx=0.008, ry=0.005),
          "box": dict(rx=0.007, ry=0.005, corner_radius=0.002),
          "triangle": dict(rx=0.007, corner_radius=0.002)}


@pytest.mark.parametrize("shape", list(SHAPES))
def test_every_shape_develops_contact(shape):
    """A soft column pressed onto each collider shape by its kinematic top (12 mm in 60
    steps): a contact reaction develops and no node ends up inside the object (its level set,
    evaluated by the oracle's restatement of sdf_eval, stays positive) — after the
    reference's tests/test_objects.py."""
    import oracle
    from diff_2d_fem_gb300 import Model, ImplicitIntegrator
    m = Model()
    m.add_object(shape, center=(0.05, 0.030), mu=0.5, **SHAPES[shape])
    h = m.add_soft_body(np.ones((40, 16), np.uint8), physical_size=(0.016, 0.040), center=(0.05, 0.060),
                        E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    x0 = m.get_body_x(h)
    top = np.where(x0[:, 1] > x0[:, 1].max() - 1e-4)[0]
    m.set_kinematic_constraint(h, top)
    integ = ImplicitIntegrator(max_iter=100, precision="fp64")
    fmax = 0.0
    for t in range(1, 61):
        x = m.get_body_x(h)
        x[top, 1] = x0[top, 1] - 0.012 * t / 60
        m.set_kinematic_target(h, x)
        integ.simulate(m, 1e-3)
        fmax = max(fmax, float(np.linalg.norm(integ.collider_force(m)[0])))
    x = m.get_body_x(h)
    assert np.all(np.isfinite(x))
    assert fmax > 1.0, fmax
    row = m._colliders[0].row()
    assert oracle.sdf(row, x).min() > 0.0


PX = 0.5e-3


@pytest.mark.parametrize("kind,mu,th_deg", [("rigid", 0.0, 40.0), ("rigid", 0.3, 30.0), ("soft", 0.3, 30.0)])
def test_slides_at_the_coulomb_speed(kind, mu, th_deg):
    """A block on a held slab under tilted gravity (contact between bodies with friction mu):
    it rests within the barrier's reach, then slides at the steady speed
    g (sin th - mu cos th) / c_e of the damped backward-Euler step (c_e = (1 - e^(-c dt)) / dt),
    within 1 % (rigid) or 2 % (soft) — after the reference's tests/test_ipc.py."""
    from diff_2d_fem_gb300 import Model, ImplicitIntegrator
    c, dt = 200.0, 1e-3
    ce = (1.0 - np.exp(-dt * c)) / dt
    th = np.deg2rad(th_deg)
    m = Model()
    m.damping = c
    m.body_friction = mu
    slab = m.add_soft_body(np.ones((6, 60), np.uint8), physical_size=(60 * PX, 6 * PX), center=(0.0, 0.0),
                           E=1.0e6, nu=0.40, density=1100.0)
    at = (-0.010, 0.0015 + 0.002 + 0.9 * PX / 8)
    if kind == "rigid":
        block = m.add_affine_body(np.ones((8, 8), np.uint8), physical_size=(8 * PX, 8 * PX), center=at,
                                  density=1100.0)
    else:
        block = m.add_soft_body(np.ones((8, 8), np.uint8), physical_size=(8 * PX, 8 * PX), center=at,
                                E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    m.set_kinematic_constraint(slab, np.arange(m.body_nodes(slab).size))
    integ = ImplicitIntegrator(precision="fp64")
    m.gravity = (0.0, -G0 * np.cos(th))
    for _ in range(100):
        integ.simulate(m, dt)
    gap = m.get_body_x(block)[:, 1].min() - m.get_body_x(slab)[:, 1].max()
    assert 0.5 * m.dhat < gap < m.dhat, gap / m.dhat
    m.gravity = (G0 * np.sin(th), -G0 * np.cos(th))
    xs = []
    for _ in range(300):
        integ.simulate(m, dt)
        xs.append(m.get_body_x(block)[:, 0].mean())
    v = np.diff(np.array(xs)[-200:]).mean() / dt
    expect = G0 * (np.sin(th) - mu * np.cos(th)) / ce
    assert abs(v / expect - 1.0) < (0.01 if kind == "rigid" else 0.02), (v, expect)


def _throw(other, px_per_step, diagonal=False, steps=120):
    """A rigid block thrown at another body: (smallest gap over the run in units of dhat,
    whether a node of the thrown block entered a held block's box, relative momentum change)."""
    from diff_2d_fem_gb300 import Model, ImplicitIntegrator, scene
    dt = 2.5e-4
    v0 = px_per_step * PX / dt
    m = Model()
    rigid = lambda c: m.add_affine_body(np.ones((8, 8), np.uint8), physical_size=(8 * PX, 8 * PX), center=c,
                                        density=1100.0)
    if diagonal:
        a, at = rigid((-6 * PX, 6 * PX)), (4 * PX, -4 * PX)
    else:
        a, at = rigid((0.0, 0.0)), (13 * PX, 0.8 * PX)
    b = rigid(at) if other == "rigid" else m.add_soft_body(np.ones((8, 8), np.uint8), physical_size=(8 * PX, 8 * PX),
                                                           center=at, E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    if other == "held":
        m.set_kinematic_constraint(b, np.arange(m.body_nodes(b).size))
    m.set_body_velocity(a, velocity=(v0 / np.sqrt(2.0), -v0 / np.sqrt(2.0)) if diagonal else (v0, 0.0))
    integ = ImplicitIntegrator(friction=False, precision="fp64")
    mass = np.asarray(m.me.mass, np.float64)
    mom = lambda: (mass[:, None] * np.concatenate([m.get_body_v(a), m.get_body_v(b)])).sum(0)
    p0 = mom()
    gap, inside = np.inf, False
    for _ in range(steps):
        integ.simulate(m, dt)
        prob = dict(m._solver.prob, x=m.get_x())
        gap = min(gap, float(scene.min_distance(prob).min()) / m.dhat)
        if other == "held":
            xa, xb = m.get_body_x(a), m.rest_x(b)
            lo, hi = xb.min(0) + 1e-9, xb.max(0) - 1e-9
            inside |= bool(((xa > lo) & (xa < hi)).all(1).any())
    assert np.isfinite(m.get_x()).all()
    return gap, inside, float(np.linalg.norm(mom() - p0) / np.linalg.norm(p0))


@pytest.mark.parametrize("other,diagonal", [("soft", False), ("rigid", False), ("held", True), ("held", False)])
def test_nothing_passes_through(other, diagonal):
    """A rigid block thrown at 5 pixels a step at a soft, a rigid or a held block, head on and
    corner to corner: the surfaces never touch and nothing enters the held block — after the
    reference's tests/test_ipc.py."""
    gap, inside, _ = _throw(other, 5.0, diagonal)
    assert gap > 0.0 and not inside, (gap, inside)


def test_momentum_goes_through_an_impact():
    """At half a pixel a step into a free soft block, momentum is kept through the impact
    (within 2e-3)."""
    _, _, dp = _throw("soft", 0.5)
    assert dp < 2e-3, dp


def test_a_moved_collider_carries_the_body():
    """Model.set_collider_center between steps, through the public API: a soft block resting
    on a disc that is then raised by 0.05 dhat a step. The device step follows the moved disc
    as the oracle does (FP64; 1e-7 of the coordinates: friction makes this contact run
    sensitive at 1e-10, while a move that was not applied would differ by 2e-2), and the block
    has risen with the disc."""
    import oracle
    from diff_2d_fem_gb300 import Model, ImplicitIntegrator, scene
    m = Model()
    m.add_disc(center=(0.0, 0.0), radius=0.004, mu=0.5)
    h = m.add_soft_body(np.ones((6, 6), np.uint8), physical_size=(0.003, 0.003),
                        center=(0.0, 0.004 + 0.0015 + 0.9 * 0.0005 / 8), E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    m.gravity = (0.0, -G0)
    integ = ImplicitIntegrator(precision="fp64")
    s = oracle.OracleSolver(scene.solver_problem(m, integ, 1e-3))
    dy = 0.05 * m.dhat
    nodes = m.body_nodes(h)
    y60 = None
    for k in range(100):
        if k == 60:
            y60 = s.x[nodes, 1].mean()
        if k >= 60:
            m.set_collider_center(0, (0.0, (k - 59) * dy))
            s.set_collider_centers([[0.0, (k - 59) * dy]])
        integ.simulate(m, 1e-3)
        s.step()
    x = m.get_x()
    assert np.abs(x - s.x).max() < 1e-7 * np.abs(s.x).max(), np.abs(x - s.x).max()
    assert x[nodes, 1].mean() - y60 > 20 * dy
