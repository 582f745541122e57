"""The golden scenes, written against the reference's public API (Model /
ImplicitIntegrator), so that the same definition builds the scene in the reference (to
record golden vectors, make_golden.py) and in diff_2d_fem_gb300 (to check parity).

Each builder takes a namespace with `Model` and `ImplicitIntegrator` and returns
dict(model, integ, dt, steps, command) where command(k) sets the commands of step k.
"""
from __future__ import annotations

import numpy as np


def strip_small(ns):
    m = ns.Model(device=ns.device)
    m.add_ground(0.0, mu=0.8)
    m.add_soft_body(np.ones((3, 12), np.uint8), physical_size=(0.009, 0.00225), center=(0.0, 0.0013),
                    E=0.5e6, nu=0.40, density=1100.0)
    m.finalize(); m.gravity = (0.0, -9.81)
    return dict(model=m, integ=ns.ImplicitIntegrator(), dt=2e-3, steps=4, command=None)


def strip_cfg1(ns, steps=12):
    """The strip on the ground of the single-scene configuration (6x72 pixels, 511 nodes)."""
    m = ns.Model(device=ns.device)
    m.add_ground(0.0, mu=0.8)
    m.add_soft_body(np.ones((6, 72), np.uint8), physical_size=(0.054, 0.0045), center=(0.0, 0.0030),
                    E=0.5e6, nu=0.40, density=1100.0)
    m.finalize(); m.gravity = (0.0, -9.81)
    return dict(model=m, integ=ns.ImplicitIntegrator(), dt=2e-3, steps=steps, command=None)


def batch_colliders(ns):
    """Three environments with different designs pressed by kinematic top rows onto a disc,
    an ellipse, a rounded box and a rounded triangle; friction on; IPC self-contact sweeps
    the kinematic nodes."""
    rng = np.random.default_rng(3)
    d1 = np.ones((6, 4), np.uint8); d1[2:4, 1:3] = 0
    d2 = (rng.random((6, 4)) > 0.15).astype(np.uint8); d2[-1] = 1; d2[:, 0] = 1
    m = ns.Model(device=ns.device)
    m.add_disc(center=(0.0, 0.0), radius=0.004, mu=0.6)
    m.add_object("ellipse", (0.006, 0.001), 0.002, 0.001, mu=0.3)
    m.add_object("box", (-0.006, 0.001), 0.0015, 0.001, corner_radius=0.0004, mu=0.5)
    m.add_object("triangle", (0.0, -0.008), 0.002, corner_radius=0.0003, mu=0.4)
    hs = [m.add_soft_body(d, physical_size=(0.004, 0.006), center=(0.0, 0.0072), E=1.0e6, nu=0.40,
                          density=1100.0, env_id=i) for i, d in enumerate([d1, d2, d1])]
    m.finalize()
    x0 = [m.rest_x(h) for h in hs]
    tops = [np.where(x[:, 1] > x[:, 1].max() - 1e-9)[0] for x in x0]
    for h, t in zip(hs, tops):
        m.set_kinematic_constraint(h, t)

    def command(k):
        for h, x, t in zip(hs, x0, tops):
            tgt = x.copy(); tgt[t, 1] -= 0.0012 * (k + 1) / 4
            m.set_kinematic_target(h, tgt)
    return dict(model=m, integ=ns.ImplicitIntegrator(max_iter=60), dt=1e-3, steps=4, command=command)


def grip(ns):
    """Two soft pads with kinematic backs close on a free rigid block above the ground:
    IPC contact between bodies with friction, an affine body, kinematic sweeps."""
    PX = 0.5e-3
    m = ns.Model(device=ns.device)
    m.body_friction = 0.8
    m.add_ground(0.0, mu=0.5)
    m.add_affine_body(np.ones((4, 4), np.uint8), physical_size=(4 * PX, 4 * PX),
                      center=(0.0, 2 * PX + 0.9 * PX / 8), density=600.0)
    pads = [m.add_soft_body(np.ones((4, 2), np.uint8), physical_size=(2 * PX, 4 * PX),
                            center=(s * 3.25 * PX, 2 * PX + 0.4e-3), E=1.0e6, nu=0.40, density=1100.0)
            for s in (-1, +1)]
    m.finalize(); m.gravity = (0.0, -9.81)
    rest = [m.rest_x(p) for p in pads]
    for s, p, X in zip((-1, +1), pads, rest):
        back = X[:, 0].min() if s < 0 else X[:, 0].max()
        m.set_kinematic_constraint(p, np.where(np.abs(X[:, 0] - back) < 1e-9)[0])

    def command(k):
        a = min((k + 1) / 4.0, 1.0)
        for s, p, X in zip((-1, +1), pads, rest):
            Y = X.copy(); Y[:, 0] -= s * 0.35 * PX * a
            m.set_kinematic_target(p, Y)
    return dict(model=m, integ=ns.ImplicitIntegrator(max_iter=120), dt=1e-3, steps=5, command=command)


def tendon(ns):
    """A cantilever clamped at its left end and bent by a tension-controlled tendon."""
    m = ns.Model(device=ns.device); m.damping = 50.0
    h = m.add_soft_body(np.ones((3, 16), np.uint8), physical_size=(0.008, 0.0015), center=(0.0, 0.0),
                        E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    X = m.rest_x(h)
    m.set_kinematic_constraint(h, np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0])
    cable = m.add_tendon(h, through=[(x, 0.0005) for x in np.unique(np.round(X[:, 0], 9))])

    def command(k):
        m.set_tendon_tension(cable, 5.0 + 5.0 * k)
    return dict(model=m, integ=ns.ImplicitIntegrator(self_collision=False, friction=False, max_iter=80),
                dt=1e-3, steps=4, command=command)


def line_search(ns):
    """The energy line search, on a soft block dropped on a disc collider, no rigid modes."""
    m = ns.Model(device=ns.device)
    m.add_disc(center=(0.0, -0.004), radius=0.004, mu=0.5)
    m.add_soft_body(np.ones((3, 4), np.uint8), physical_size=(0.002, 0.0015), center=(0.0002, 0.0008),
                    E=0.5e6, nu=0.40, density=1100.0)
    m.finalize(); m.gravity = (0.0, -9.81)
    return dict(model=m, integ=ns.ImplicitIntegrator(line_search=True, rigid_modes=False, max_iter=50),
                dt=2e-3, steps=4, command=None)


def rigid_region(ns):
    """A cantilever whose outer third is a rigid region (an affine piece sharing its interface
    nodes with the soft root), clamped at its left end and bent by a tip load."""
    m = ns.Model(device=ns.device); m.damping = 300.0
    h = m.add_soft_body(np.ones((3, 15), np.uint8), physical_size=(0.0075, 0.0015), center=(0.0, 0.0),
                        E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    region = np.zeros((3, 15), bool); region[:, 10:] = True
    m.add_affine_region(h, region)
    X = m.rest_x(h)
    m.set_kinematic_constraint(h, np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0])
    tip = np.where(X[:, 0] > X[:, 0].max() - 1e-9)[0]
    f = np.zeros_like(X); f[tip, 1] = -1.5 / len(tip)
    m.set_external_force(h, f)
    return dict(model=m, integ=ns.ImplicitIntegrator(self_collision=False, friction=False, max_iter=300),
                dt=2e-3, steps=4, command=None)


def jittered_grid(nx, ny, size, center, jitter=0.0, seed=0):
    """A triangle mesh of an (nx, ny)-cell rectangle: interior vertices moved by up to
    `jitter` cells in each direction, each cell cut along alternating diagonals."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(-0.5, 0.5, nx + 1) * size[0] + center[0]
    ys = np.linspace(-0.5, 0.5, ny + 1) * size[1] + center[1]
    V = np.stack(np.meshgrid(xs, ys, indexing="ij"), -1).reshape(-1, 2)
    ix, iy = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="ij")
    inner = ((ix > 0) & (ix < nx) & (iy > 0) & (iy < ny)).reshape(-1)
    V[inner] += jitter * rng.uniform(-1.0, 1.0, (inner.sum(), 2)) * np.array([size[0] / nx, size[1] / ny])
    T = []
    for i in range(nx):
        for j in range(ny):
            a, b, c, d = i * (ny + 1) + j, (i + 1) * (ny + 1) + j, (i + 1) * (ny + 1) + j + 1, i * (ny + 1) + j + 1
            T += [[a, b, c], [a, c, d]] if (i + j) % 2 == 0 else [[a, b, d], [b, c, d]]
    return V, np.asarray(T, np.int64)


def mesh_cantilever(ns):
    """A cantilever given as a jittered triangle mesh, clamped at its left end and sagging
    under gravity; self-contact on (its exclusion includes pairs close through the material)."""
    m = ns.Model(device=ns.device)
    V, T = jittered_grid(12, 3, (0.012, 0.003), (0.0, 0.0), jitter=0.25, seed=1)
    h = m.add_soft_mesh(V, T, E=0.5e6, nu=0.40, density=1100.0)
    m.finalize(); m.gravity = (0.0, -9.81)
    X = m.rest_x(h)
    m.set_kinematic_constraint(h, np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0])
    return dict(model=m, integ=ns.ImplicitIntegrator(max_iter=400), dt=2e-3, steps=4, command=None)


def mesh_bodies(ns):
    """Mesh bodies in contact: a jittered soft mesh block (per-triangle stiffness) dropped on a
    rigid mesh plate lying on the ground, and a kinematic mesh pusher closing in from the
    side; friction between bodies."""
    PX = 0.5e-3
    m = ns.Model(device=ns.device)
    m.body_friction = 0.5
    m.add_ground(0.0, mu=0.6)
    Vp, Tp = jittered_grid(8, 2, (8 * PX, 2 * PX), (0.0, PX + 0.9 * PX / 8))
    plate = m.add_affine_mesh(Vp, Tp, density=900.0)
    Vs, Ts = jittered_grid(4, 4, (4 * PX, 4 * PX), (0.0, 2 * PX + 2 * PX + 0.5 * PX / 8 + 0.9 * PX / 8),
                           jitter=0.2, seed=4)
    E = np.where(np.arange(len(Ts)) % 3 == 0, 2.0e6, 1.0e6)
    soft = m.add_soft_mesh(Vs, Ts, E=E, nu=0.40, density=1100.0)
    Vk, Tk = jittered_grid(2, 3, (2 * PX, 3 * PX), (3.5 * PX, 2 * PX + 2 * PX + 0.9 * PX / 8))
    pusher = m.add_kinematic_mesh(Vk, Tk)
    m.finalize(); m.gravity = (0.0, -9.81)
    X = m.rest_x(pusher)

    def command(k):
        m.set_kinematic_target(pusher, X - np.array([0.15 * PX * (k + 1), 0.0]))
    return dict(model=m, integ=ns.ImplicitIntegrator(max_iter=120), dt=1e-3, steps=4, command=command)


def actuators(ns):
    """A soft block with a sealed cavity on the ground: the cavity pressurised and the
    outline under an ambient pressure, the lower half actively contracting, a corner pinned
    to the world and another corner on a world spring, under gravity."""
    PX = 0.5e-3
    m = ns.Model(device=ns.device)
    m.add_ground(0.0, mu=0.6)
    mk = np.ones((8, 8), np.uint8); mk[3:6, 2:6] = 0
    h = m.add_soft_body(mk, physical_size=(8 * PX, 8 * PX), center=(0.0, 4 * PX + 0.9 * PX / 8),
                        E=0.5e6, nu=0.40, density=1100.0)
    m.finalize(); m.gravity = (0.0, -9.81)
    ch = m.add_pressure_chambers(h)
    m.set_pressure(ch[0], 3.0e4)
    m.set_pressure(m.add_ambient_pressure(h), 5.0e3)
    region = np.zeros((8, 8), bool); region[:4] = True
    m.set_activation(m.add_active_region(h, region), 0.97)
    m.add_pin(h, (-4 * PX, 8 * PX + 0.9 * PX / 8), stiffness=1.0e6)
    m.add_spring(h, (4 * PX, 8 * PX + 0.9 * PX / 8), point_b=(6 * PX, 10 * PX), stiffness=2.0e4, rest_length=PX)
    return dict(model=m, integ=ns.ImplicitIntegrator(max_iter=200), dt=2e-3, steps=4, command=None)


def body_mu(ns):
    """Friction per body (the harmonic mean of the two bodies' mu at every pair) and a
    stiffness map: in each of two environments a block slides down a slab held at its base
    under tilted gravity; the slab's lower rows are four times stiffer."""
    PX = 0.5e-3
    m = ns.Model(device=ns.device)
    Emap = np.full((3, 16), 0.5e6); Emap[0] = 2.0e6
    for env, mu_b in enumerate((0.2, 0.6)):
        m.add_soft_body(np.ones((3, 16), np.uint8), physical_size=(16 * PX, 3 * PX), center=(0.0, -1.5 * PX),
                        E=Emap, nu=0.40, density=1100.0, env_id=env, mu=0.8)
        m.add_soft_body(np.ones((4, 4), np.uint8), physical_size=(4 * PX, 4 * PX),
                        center=(-2 * PX, 2 * PX + 0.9 * PX / 8), E=1.0e6, nu=0.40, density=1100.0,
                        env_id=env, mu=mu_b)
    m.finalize()
    for h in (0, 2):
        X = m.rest_x(h)
        m.set_kinematic_constraint(h, np.where(X[:, 1] < X[:, 1].min() + 1e-9)[0])
    th = np.deg2rad(25.0)
    m.gravity = (9.81 * np.sin(th), -9.81 * np.cos(th))
    return dict(model=m, integ=ns.ImplicitIntegrator(max_iter=150), dt=1e-3, steps=5, command=None)


def kinematic_pose(ns):
    """A kinematic body (add_kinematic_body) turned and moved by set_kinematic_pose presses a
    soft block against a disc; a tendon in the block is tightened step by step."""
    PX = 0.5e-3
    m = ns.Model(device=ns.device)
    m.add_disc(center=(0.0, -0.004), radius=0.004, mu=0.4)
    blk = m.add_soft_body(np.ones((4, 6), np.uint8), physical_size=(6 * PX, 4 * PX),
                          center=(0.0, 2 * PX + 0.9 * PX / 8), E=1.0e6, nu=0.40, density=1100.0)
    jaw = m.add_kinematic_body(np.ones((2, 8), np.uint8), physical_size=(8 * PX, 2 * PX),
                               center=(0.0, 4 * PX + 1 * PX + 0.5e-3))
    m.finalize()
    X = m.rest_x(blk)
    cable = m.add_tendon(blk, through=[(x, X[:, 1].max() - PX) for x in np.unique(np.round(X[:, 0], 9))])

    def command(k):
        m.set_kinematic_pose(jaw, translation=(0.1 * PX * (k + 1), -0.3 * PX * (k + 1)), angle=0.02 * (k + 1))
        m.set_tendon_tension(cable, 0.5 * (k + 1))
    return dict(model=m, integ=ns.ImplicitIntegrator(max_iter=1000), dt=1e-3, steps=3, command=command)


def mesh_chamber(ns):
    """A ring meshed in polar coordinates with its hole pressurised and an ambient pressure on
    its outline, resting on the ground under gravity."""
    ri, ro, n_t, n_r = 0.002, 0.004, 16, 2
    r = np.linspace(ri, ro, n_r + 1)
    th = 2.0 * np.pi * np.arange(n_t) / n_t
    V = np.array([(rk * np.cos(t), rk * np.sin(t) + ro + 0.5e-3 / 8) for rk in r for t in th])
    T = []
    for k in range(n_r):
        for j in range(n_t):
            a, b = k * n_t + j, k * n_t + (j + 1) % n_t
            c, d = a + n_t, b + n_t
            T += [(a, b, d), (a, d, c)] if (j + k) % 2 else [(a, b, c), (b, d, c)]
    m = ns.Model(device=ns.device)
    m.add_ground(0.0, mu=0.6)
    h = m.add_soft_mesh(V, np.array(T), E=0.5e6, nu=0.40, density=1100.0)
    m.finalize(); m.gravity = (0.0, -9.81)
    ch = m.add_pressure_chamber(h, at=(0.0, ro + 0.5e-3 / 8))
    m.set_pressure(ch, 2.0e4)
    m.set_pressure(m.add_ambient_pressure(h), 5.0e3)
    return dict(model=m, integ=ns.ImplicitIntegrator(max_iter=400), dt=2e-3, steps=3, command=None)


def tilted_plane(ns):
    """A soft block on a plane tilted by 30 degrees (add_plane with a turned normal), placed
    there as a turned mesh (mask_to_mesh), friction 0.3, under gravity: it slides."""
    th = np.deg2rad(30.0)
    n = np.array([-np.sin(th), np.cos(th)])
    PX = 0.5e-3
    V, T, _ = ns.mask_to_mesh(np.ones((4, 4), np.uint8), (4 * PX, 4 * PX), (0.0, 0.0))
    R = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
    m = ns.Model(device=ns.device)
    m.add_plane(normal=n, origin=(0.0, 0.0), mu=0.3)
    m.add_soft_mesh(V @ R.T + (2 * PX + 0.9 * PX / 8) * n, T, E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    m.gravity = (0.0, -9.81)
    return dict(model=m, integ=ns.ImplicitIntegrator(max_iter=200), dt=2e-3, steps=4, command=None)


def tendon_length(ns):
    """A clamped cantilever bent by a length-controlled tendon (a stiff cable shortened to 97 %
    of its built length), together with a tension-controlled one below the mid-line."""
    m = ns.Model(device=ns.device); m.damping = 50.0
    h = m.add_soft_body(np.ones((3, 16), np.uint8), physical_size=(0.008, 0.0015), center=(0.0, 0.0),
                        E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    X = m.rest_x(h)
    m.set_kinematic_constraint(h, np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0])
    cols = np.unique(np.round(X[:, 0], 9))
    top = m.add_tendon(h, through=[(x, 0.0005) for x in cols], stiffness=2.0e4)
    m.set_tendon_length(top, 0.97 * m.tendon_length(top))
    low = m.add_tendon(h, through=[(x, -0.0005) for x in cols])
    m.set_tendon_tension(low, 3.0)
    return dict(model=m, integ=ns.ImplicitIntegrator(self_collision=False, friction=False, max_iter=400),
                dt=1e-3, steps=2, command=None)


SCENES = {"strip_small": strip_small, "batch_colliders": batch_colliders, "grip": grip,
          "tendon": tendon, "line_search": line_search, "strip_cfg1": strip_cfg1,
          "rigid_region": rigid_region, "mesh_cantilever": mesh_cantilever, "mesh_bodies": mesh_bodies,
          "actuators": actuators, "body_mu": body_mu, "kinematic_pose": kinematic_pose,
          "mesh_chamber": mesh_chamber, "tilted_plane": tilted_plane,
          "tendon_length": tendon_length}
