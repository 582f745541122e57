"""Bodies given as triangle meshes (add_soft_mesh / add_affine_mesh / add_kinematic_mesh),
stepped by the oracle on the CPU — after the reference's tests/test_mesh.py:

  1. a mesh body given the pixel body's own triangles (mask_to_mesh) IS that body: the same
     arrays, contact scales, pressure boundaries and trajectory, bit for bit;
  2. nothing depends on orientation: a turned hanging bar hangs as the upright one;
  3. an unstructured (jittered) cantilever reaches the Newton equilibrium of its mesh;
  4. a graded mesh keeps its own nodes apart: the exclusion through the material covers
     the boundary pairs a hop count misses;
  5. a mesh design in a batch is itself, bit for bit;
  6. regions by triangle (active growth, a rigid part) and a hole as a pressure chamber;
  7. what is refused: malformed meshes, overlapping bodies, pixel-only calls, a pinched
     pressure boundary.
The device path consumes the same arrays; tests/golden/mesh_*.npz pin the scene build and
the oracle against the reference's own code, and the device against those fixtures."""
import warnings

import numpy as np
import pytest

import oracle
from oracle import static as ST
import diff_2d_fem_gb300 as D
from diff_2d_fem_gb300 import ImplicitIntegrator, Model, scene

E, NU, RHO, G0 = 1.0e6, 0.40, 1100.0, 9.81
EP = E / (1 - NU * NU)
PX = 2.0 ** -10                     # dyadic: pixel and mesh lengths are exact
FAR = (0.0, -5.0)


def _problem(m, integ, dt):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return scene.solver_problem(m, integ, dt)


def _integ(**kw):
    return ImplicitIntegrator(**{**dict(max_iter=3000, eps=1e-14, tol_x=2e-9, conv_check=8,
                                        self_collision=False, friction=False), **kw})


def _rot(V, th):
    c, s = np.cos(th), np.sin(th)
    return np.asarray(V, np.float64) @ np.array([[c, -s], [s, c]]).T


def _jittered(nx, ny, size, origin=(0.0, 0.0), jitter=0.25, seed=0):
    """A criss-cross mesh of an (nx, ny)-cell rectangle, interior nodes moved at random."""
    rng = np.random.default_rng(seed)
    xs, ys = np.linspace(0, size[0], nx + 1), np.linspace(0, size[1], ny + 1)
    V = np.stack(np.meshgrid(xs, ys, indexing="ij"), -1).reshape(-1, 2)
    inner = (V[:, 0] > 0) & (V[:, 0] < size[0]) & (V[:, 1] > 0) & (V[:, 1] < size[1])
    V[inner] += jitter * np.array([size[0] / nx, size[1] / ny]) * rng.uniform(-1, 1, (inner.sum(), 2))
    n = lambda i, j: i * (ny + 1) + j
    T = []
    for i in range(nx):
        for j in range(ny):
            a, b, c, d = n(i, j), n(i + 1, j), n(i + 1, j + 1), n(i, j + 1)
            T += [(a, b, c), (a, c, d)] if (i + j) % 2 else [(a, b, d), (b, c, d)]
    return V + np.asarray(origin, np.float64), np.array(T)


def _polar_ring(ri, ro, n_t, n_r=None):
    """A ring meshed in polar coordinates; n_r None: radii in geometric progression, so the
    element size grows from the inner to the outer edge."""
    if n_r is None:
        q = 1.0 + 2.0 * np.pi / n_t
        n_r = int(np.ceil(np.log(ro / ri) / np.log(q)))
        r = ri * (ro / ri) ** np.linspace(0.0, 1.0, n_r + 1)
    else:
        r = np.linspace(ri, ro, n_r + 1)
    th = 2.0 * np.pi * np.arange(n_t) / n_t
    V = np.array([(rk * np.cos(t), rk * np.sin(t)) for rk in r for t in th])
    T = []
    for k in range(n_r):
        for j in range(n_t):
            a, b = k * n_t + j, k * n_t + (j + 1) % n_t
            c, d = a + n_t, b + n_t
            T += [(a, b, d), (a, d, c)] if (j + k) % 2 else [(a, b, c), (b, d, c)]
    return V, np.array(T)


# ---------------------------------------------------------------- 1. a mesh body is a pixel body
def _slab_and_block(as_mesh):
    mk = np.ones((6, 20), np.uint8)
    mk[4:, 8:12] = 0
    Emap = np.full(mk.shape, 0.8e6)
    Emap[:2] = 2.0e6
    size, center = (20 * PX, 6 * PX), (0.0, 3 * PX + PX / 4)
    blk, bsize, bcenter = np.ones((4, 4), np.uint8), (4 * PX, 4 * PX), (-5 * PX, 10 * PX + PX / 4)
    m = Model()
    m.body_friction = 0.3
    m.add_ground(height=0.0, mu=0.6)
    if as_mesh:
        V, T, pix = D.mask_to_mesh(mk, size, center)
        a = m.add_soft_mesh(V, T, E=Emap[pix[:, 0], pix[:, 1]], nu=NU, density=RHO)
        Vb, Tb, _ = D.mask_to_mesh(blk, bsize, bcenter)
        b = m.add_affine_mesh(Vb, Tb, density=600.0)
    else:
        a = m.add_soft_body(mk, physical_size=size, center=center, E=Emap, nu=NU, density=RHO)
        b = m.add_affine_body(blk, physical_size=bsize, center=bcenter, density=600.0)
    m.finalize()
    m.gravity = (0.0, -G0)
    return m, a, b


def test_mesh_body_reproduces_the_pixel_body():
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        (mp, _, _), (mm, _, _) = _slab_and_block(False), _slab_and_block(True)
    for k in ("rest_pos", "tri", "D_m_inv", "rest_area", "mu", "lam", "mass", "boundary_nodes",
              "boundary_edges", "excl_ptr", "excl_idx", "node_starts", "tri_starts", "boundary_starts"):
        assert np.array_equal(getattr(mp.me, k), getattr(mm.me, k)), f"mesh array {k} differs"
    for attr in ("dx", "dhat", "kappa", "body_kappa", "self_stiffness"):
        assert getattr(mp, attr) == getattr(mm, attr), attr
    ip, im = ImplicitIntegrator(), ImplicitIntegrator()
    assert ip.cfl_number(mp, 1e-3) == im.cfl_number(mm, 1e-3)
    _, xp, _ = oracle.run(_problem(mp, ip, 1e-3), 40)
    _, xm, _ = oracle.run(_problem(mm, im, 1e-3), 40)
    assert np.abs(xp[-1] - mp.me.rest_pos).max() > 1e-5
    assert np.array_equal(xp[-1], xm[-1]), "the trajectories differ"


def _cavity_body(as_mesh):
    mk = np.ones((20, 14), np.uint8)
    mk[5:15, 4:10] = 0
    mk[2:4, 8:12] = 0
    size, center = (14 * PX, 20 * PX), (0.03, 0.05)
    m = Model()
    m.add_disc(center=FAR, radius=0.01)
    m.damping = 2000.0
    if as_mesh:
        V, T, _ = D.mask_to_mesh(mk, size, center)
        h = m.add_soft_mesh(V, T, E=E, nu=NU, density=RHO)
    else:
        h = m.add_soft_body(mk, physical_size=size, center=center, E=E, nu=NU, density=RHO)
    m.finalize()
    return m, h


def test_mesh_pressure_boundaries_are_the_pixel_ones():
    models = []
    for as_mesh in (False, True):
        m, h = _cavity_body(as_mesh)
        ch = m.add_pressure_chambers(h) + [m.add_ambient_pressure(h)]
        assert len(ch) == 3
        for c, p in zip(ch, (4e4, 2e4, 1e4)):
            m.set_pressure(c, p)
        models.append((m, ch))
    (mp, cp), (mm, cm) = models
    for i, j in zip(cp, cm):
        ep = set(zip(mp._chambers[i].ea.tolist(), mp._chambers[i].eb.tolist()))
        em = set(zip(mm._chambers[j].ea.tolist(), mm._chambers[j].eb.tolist()))
        assert ep == em, f"chamber {i}: the mesh's boundary is not the pixel one"
        assert abs(mp.chamber_area(i) - mm.chamber_area(j)) <= 1e-12 * mp.chamber_area(i)
    xs = [oracle.run(_problem(m, _integ(max_iter=300), 5e-3), 8)[1][-1] for m, _ in models]
    assert np.abs(xs[0] - xs[1]).max() < 1e-12
    assert np.abs(xs[1] - mm.me.rest_pos).max() > 1e-5, "the pressure did nothing"


# ---------------------------------------------------------------- 2. orientation
def test_a_turned_bar_hangs_as_an_upright_one():
    """A bar hanging under its own weight, upright and turned by 30 degrees with gravity
    turned with it: the same extension, close to rho g L^2 / (2 E')."""
    L, w, g, th = 0.060, 0.006, 200.0, np.deg2rad(30.0)
    V, T, _ = D.mask_to_mesh(np.ones((30, 3), np.uint8), (w, L), (0.0, 0.0))
    top = np.where(V[:, 1] > V[:, 1].max() - 1e-9)[0]
    bottom = np.where(V[:, 1] < V[:, 1].min() + 1e-9)[0]
    out = []
    for a in (0.0, th):
        m = Model()
        m.damping = 2000.0
        m.add_disc(center=FAR, radius=0.01)
        h = m.add_soft_mesh(_rot(V, a), T, E=E, nu=NU, density=RHO)
        m.finalize()
        m.set_kinematic_constraint(h, top)
        m.gravity = tuple(_rot([[0.0, -g]], a)[0])
        _, xs, _ = oracle.run(_problem(m, _integ(tol_x=0.0), 2e-2), 12)
        out.append(_rot(xs[-1], -a))
    ext = -(out[0][bottom, 1] - V[bottom, 1]).mean()
    exact = RHO * g * L * L / (2 * EP)
    assert abs(ext - exact) < 0.03 * exact, (ext, exact)
    assert np.abs(out[1] - out[0]).max() < 1e-6 * ext


# ---------------------------------------------------------------- 3. unstructured meshes
def test_jittered_cantilever_against_newton():
    """A 5:1 cantilever of jittered triangles bent by its own weight: the oracle's step, run
    to rest, reaches the Newton equilibrium of the same mesh within 1e-6."""
    V, T = _jittered(30, 6, (0.020, 0.004), origin=(0.0, -0.002), seed=1)
    m = Model()
    m.damping = 2000.0
    m.add_disc(center=FAR, radius=0.01)
    h = m.add_soft_mesh(V, T, E=E, nu=NU, density=RHO)
    m.finalize()
    left, tip = np.where(V[:, 0] < 1e-12)[0], np.where(V[:, 0] > 0.020 - 1e-12)[0]
    m.set_kinematic_constraint(h, left)
    g = 40.0
    fext = np.asarray(m.me.mass, np.float64)[:, None] * np.array([0.0, -g])
    me = m.me
    xr, res = ST.solve_static(me.rest_pos, me.tri, me.D_m_inv, me.rest_area, me.mu, me.lam, left, fext=fext)
    assert res < 1e-8
    m.gravity = (0.0, -g)
    _, xs, _ = oracle.run(_problem(m, _integ(max_iter=2000, tol_x=0.0, alpha_max=1e9), 5e-2), 12)
    d, dr = (xs[-1][tip, 1] - V[tip, 1]).mean(), (xr[tip, 1] - V[tip, 1]).mean()
    assert dr < -2e-4
    assert abs(d / dr - 1.0) < 1e-6, (d, dr)


# ---------------------------------------------------------------- 4. graded meshes
def _active_gap(me):
    """Smallest distance at rest between a boundary node and a boundary edge that contact
    would let act on each other (the node excluded from neither end of the edge)."""
    bn = np.asarray(me.boundary_nodes)
    slot = {int(n): k for k, n in enumerate(bn)}
    X = np.asarray(me.rest_pos, np.float64)
    ptr, idx = me.excl_ptr, me.excl_idx
    best = np.inf
    for a, b in np.asarray(me.boundary_edges):
        ex = set(idx[ptr[slot[int(a)]]:ptr[slot[int(a)] + 1]].tolist()) | \
            set(idx[ptr[slot[int(b)]]:ptr[slot[int(b)] + 1]].tolist())
        ok = np.array([k not in ex for k in range(len(bn))])
        P, t = X[bn[ok]], X[b] - X[a]
        if len(P):
            s = np.clip(((P - X[a]) @ t) / (t @ t), 0.0, 1.0)
            best = min(best, float(np.linalg.norm(P - (X[a] + s[:, None] * t), axis=1).min()))
    return best


def test_a_graded_mesh_keeps_its_own_nodes_apart():
    V, T = _polar_ring(0.0001, 0.010, n_t=32)                  # elements from 0.02 to 2 mm
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")                        # the 100:1 element-size warning
        m = Model()
        h = m.add_soft_mesh(V, T, E=E, nu=NU, density=RHO)
    m.finalize()
    hop_only = D.build_scene([dict(vertices=V, triangles=T, young=E, nu=NU, rho=RHO, env=0)])
    assert _active_gap(hop_only) < m.dhat, "this mesh should defeat a hop-count exclusion"
    assert _active_gap(m.me) > m.dhat
    prob = _problem(m, ImplicitIntegrator(), 1e-3)
    assert scene.min_distance(prob).min() > m.dhat
    _, xs, _ = oracle.run(prob, 1)
    assert np.abs(xs[-1] - m.me.rest_pos).max() < 1e-12, "the body pushes on itself at rest"


# ---------------------------------------------------------------- 5. batches
def test_a_mesh_design_in_a_batch_is_itself():
    V1, T1 = _jittered(4, 8, (0.008, 0.016), origin=(0.046, 0.0375), seed=4)
    V2, T2 = _jittered(4, 8, (0.008, 0.016), origin=(0.046, 0.0375), seed=5)

    def run(designs):
        m = Model()
        m.add_disc(center=(0.05, 0.030), radius=0.006, mu=0.6)
        hs = [m.add_soft_mesh(V, T, E=E, nu=NU, density=RHO, env_id=i) for i, (V, T) in enumerate(designs)]
        m.finalize()
        tops = []
        for hh in hs:
            X = m.rest_x(hh)
            top = np.where(X[:, 1] > X[:, 1].max() - 1e-9)[0]
            m.set_kinematic_constraint(hh, top)
            tops.append((hh, X, top))
        prob = _problem(m, ImplicitIntegrator(), 1e-3)
        bc = np.asarray(prob["bc_idx"])

        def cmd(t):
            for hh, X, top in tops:
                tg = X.copy()
                tg[top, 1] = X[top, 1] - 0.004 * (t + 1) / 25
                m.set_kinematic_target(hh, tg)
            return dict(bc_target=m._targets[bc])
        _, xs, _ = oracle.run(prob, 25, cmd)
        return m, hs, xs[-1]

    alone, (ha,), xa = run([(V1, T1)])
    batch, hb, xb = run([(V1, T1), (V2, T2), (V1, T1)])
    na = alone.body_nodes(ha)
    assert xa[na, 1].min() < 0.030 + 0.006 + 1e-4, "no contact developed"
    for env in (0, 2):
        assert np.array_equal(xb[batch.body_nodes(hb[env])], xa[na]), env
    assert np.abs(xb[batch.body_nodes(hb[1])] - xa[na]).max() > 1e-6


# ---------------------------------------------------------------- 6. regions and pressure
def test_regions_by_triangle():
    V, T = _jittered(5, 8, (0.010, 0.016), origin=(-0.005, -0.008), seed=6)
    m = Model()
    m.damping = 2000.0
    m.add_disc(center=FAR, radius=0.01)
    h = m.add_soft_mesh(V, T, E=E, nu=NU, density=RHO)
    m.finalize()
    m.set_activation(m.add_active_region(h, np.ones(len(T), bool)), 1.08)
    _, xs, _ = oracle.run(_problem(m, _integ(alpha_max=1e9), 2e-2), 10)
    X, x = np.asarray(m.me.rest_pos, np.float64), xs[-1]
    assert np.abs((x - x.mean(0)) - 1.08 * (X - X.mean(0))).max() < 1e-4 * 0.016

    m = Model()
    m.damping = 300.0
    V, T = _jittered(30, 6, (0.020, 0.004), origin=(0.0, -0.002), seed=7)
    h = m.add_soft_mesh(V, T, E=E, nu=NU, density=RHO)
    m.finalize()
    right = np.flatnonzero(V[T].mean(1)[:, 0] > 0.012)                   # triangle indices
    m.add_affine_region(h, right)
    m.set_kinematic_constraint(h, np.where(V[:, 0] < 1e-12)[0])
    m.gravity = (0.0, -200.0)
    s, _, _ = oracle.run(_problem(m, ImplicitIntegrator(self_collision=False, friction=False), 2e-3), 100)
    q = s.state["a_q"].reshape(-1, 6)[0]
    A = np.array([[q[1], q[2]], [q[4], q[5]]])
    assert np.abs(A.T @ A - np.eye(2)).max() < 1e-5, "the rigid part strained"
    assert abs(np.arctan2(A[1, 0] - A[0, 1], A[0, 0] + A[1, 1])) > 1e-3, "the rigid part should have turned"


def test_a_ring_under_internal_pressure():
    """Lame's thick-walled ring in plane strain at small strain, on a ring meshed in polar
    coordinates (its outline is the circle's own polygon): the cavity's area change within
    1 % of 2 pi a u(a)."""
    ri, ro, p = 0.012, 0.023, 1.0e-3 * E
    V, T = _polar_ring(ri, ro, n_t=64, n_r=6)
    m = Model()
    m.damping = 2000.0
    m.add_disc(center=FAR, radius=0.01)
    h = m.add_soft_mesh(V, T, E=E, nu=NU, density=RHO)
    m.finalize()
    ch = m.add_pressure_chamber(h, at=(0.0, 0.0))
    assert m.add_pressure_chambers(h) == [len(m._chambers) - 1]        # the one hole, again
    A0 = m.chamber_area(ch)
    m.set_pressure(ch, p)
    _, xs, _ = oracle.run(_problem(m, _integ(max_iter=4000, tol_x=0.0), 5e-3), 25)
    c = m._chambers[ch]
    from diff_2d_fem_gb300 import actuators as act
    A1 = c.sign * act.loop_area(xs[-1], c.ea, c.eb, c.ref)
    a = np.sqrt(A0 / np.pi)
    b = np.sqrt((m.element_areas(h).sum() + A0) / np.pi)
    ua = (1 + NU) / E * p * a * a / (b * b - a * a) * ((1 - 2 * NU) * a + b * b / a)
    dA, exact = A1 - A0, 2 * np.pi * a * ua
    assert abs(dA - exact) < 0.01 * exact, (dA, exact)


# ---------------------------------------------------------------- 7. mass and refusals
def test_mass_and_what_is_refused():
    V, T = _jittered(4, 3, (0.004, 0.003), seed=8)
    m = Model()
    h = m.add_soft_mesh(V, T, E=E, nu=NU, density=RHO)
    V2, T2 = _jittered(2, 2, (0.002, 0.002), origin=(0.001, 0.001))     # inside the first
    m.add_soft_mesh(V2, T2, E=E, nu=NU, density=RHO)
    with pytest.raises(ValueError, match="overlap"):
        m.finalize()
    m = Model()
    h = m.add_soft_mesh(V, T, E=E, nu=NU, density=RHO)
    m.finalize()
    assert abs(np.asarray(m.me.mass).sum() - RHO * 0.004 * 0.003) < 1e-12 * RHO * 0.004 * 0.003
    with pytest.raises(ValueError, match="mesh body"):
        m.pixel_size(h)
    with pytest.raises(ValueError, match="mesh body"):
        m.to_pixels(h, np.zeros(len(T)))
    with pytest.raises(ValueError, match="triangles"):
        m.to_elements(h, np.zeros(len(T) + 1))
    with pytest.raises(ValueError, match="distinct"):
        m.add_active_region(h, np.array([0, 0]))
    with pytest.raises(ValueError, match="stiffness per triangle"):
        Model().add_soft_mesh(V, T, E=np.ones(3))
    # two squares touching at one corner: the pressure boundary is pinched there
    Vp = np.array([[0, 0], [1, 0], [1, 1], [0, 1], [2, 1], [2, 2], [1, 2]], float) * 1e-3
    Tp = np.array([[0, 1, 2], [0, 2, 3], [2, 4, 5], [2, 5, 6]])
    m = Model()
    h = m.add_soft_mesh(Vp, Tp, E=E, nu=NU, density=RHO)
    m.finalize()
    with pytest.raises(ValueError, match="two boundary loops meet"):
        m.add_ambient_pressure(h)


BAD = {
    "shape": (np.zeros((2, 2)), np.array([[0, 1, 2]]), "vertices must be"),
    "finite": (np.array([[0, 0], [1, 0], [np.nan, 1]]), np.array([[0, 1, 2]]), "not finite"),
    "range": (np.array([[0, 0], [1, 0], [0, 1]]), np.array([[0, 1, 3]]), "0-based"),
    "repeat": (np.array([[0, 0], [1, 0], [0, 1]]), np.array([[0, 1, 1]]), "repeat a vertex"),
    "duplicate": (np.array([[0, 0], [1, 0], [0, 1]]), np.array([[0, 1, 2], [2, 0, 1]]), "duplicate"),
    "unused": (np.array([[0, 0], [1, 0], [0, 1], [5, 5]]), np.array([[0, 1, 2]]), "belong to no triangle"),
    "degenerate": (np.array([[0, 0], [1, 0], [2, 0]]), np.array([[0, 1, 2]]), "zero area"),
    "fold": (np.array([[0, 0], [1, 0], [0.5, 1], [0.5, 0.5]]), np.array([[0, 1, 2], [0, 1, 3]]), "folds"),
    "three": (np.array([[0, 0], [1, 0], [0.5, 1], [0.5, -1], [0.2, 0.9]]),
              np.array([[0, 1, 2], [0, 1, 3], [0, 1, 4]]), "shared by 3"),
    "coincident": (np.array([[0, 0], [1, 0], [0, 1], [3, 0], [4, 0], [3, 1], [0, 1]]),
                   np.array([[0, 1, 2], [3, 4, 5], [3, 5, 6]]), "same place"),
    "crack": (np.array([[0, 0], [2, 0], [1, 1], [1, 0], [1, -1]]), np.array([[0, 1, 2], [0, 4, 3]]),
              "lies on boundary edge"),
    "cross": (np.array([[0, 0], [2, 0], [1, 2], [1, 1], [3, 1], [2, 3]]),
              np.array([[0, 1, 2], [3, 4, 5]]), "cross"),
}


@pytest.mark.parametrize("case", list(BAD))
def test_check_mesh_names_each_defect(case):
    V, T, msg = BAD[case]
    with pytest.raises(ValueError, match=msg):
        D.check_mesh(np.asarray(V, np.float64) * 1e-3, T)


@pytest.mark.parametrize("mode", ["elastic", "disc"])
def test_adjoint_on_a_jittered_mesh(mode):
    """The adjoint oracle on a body of jittered triangles, its top driven down and sideways
    for 12 steps, without and with a frictionless disc in contact: dJ/d(density) against
    central differences of the forward oracle along the gradient and along a random
    direction (reference tests/test_mesh.py:242-288 bounds these at 2 % and 1 %)."""
    from oracle import adjoint as OA
    T_, DT, Emin = 12, 2.0e-4, 1e-3
    m = Model()
    m.add_disc(center=(0.05, -1.0 if mode == "elastic" else 0.0335), radius=0.006, mu=0.0)
    V, Tr = _jittered(6, 10, (0.012, 0.024), origin=(0.044, 0.040), seed=2)
    h = m.add_soft_mesh(V, Tr, E=E, nu=NU, density=RHO)
    m.finalize()
    x0 = m.rest_x(h)
    top = np.where(x0[:, 1] > x0[:, 1].max() - 1e-9)[0]
    m.set_kinematic_constraint(h, top)
    prob = _problem(m, ImplicitIntegrator(max_iter=3000, eps=1e-14, tol_x=1e-8, conv_check=8,
                                          self_collision=False, friction=False), DT)
    prob["eps"], prob["iter_max"], prob["tol_x"] = 1e-16, 20000, 0.0
    bc = np.asarray(prob["bc_idx"])
    targets = []
    for t in range(1, T_ + 1):
        tg = np.asarray(m.me.rest_pos, np.float64).copy()
        tg[top, 1] -= 0.003 * t / T_
        tg[top, 0] += 0.002 * t / T_
        targets.append(tg[bc])
    rng = np.random.default_rng(0)
    rho0 = 0.45 + 0.5 * rng.random(len(Tr))
    low = np.where(x0[:, 1] < np.median(x0[:, 1]))[0]
    c = np.zeros((m.n_nodes, 2))
    c[low, 0] = 1.0 / len(low)

    def rollout(rho):
        p = dict(prob)
        Em = Emin + rho * (1.0 - Emin)
        p["mu"], p["lam"] = Em * prob["mu"], Em * prob["lam"]
        _, xs, _ = oracle.run(p, T_, lambda k: dict(bc_target=targets[k]))
        return [np.asarray(prob["x"], np.float64)] + xs

    xs = rollout(rho0)
    if mode == "disc":
        assert xs[-1][:, 1].min() < 0.0335 + 0.006 + m.dhat, "no contact with the disc"
    res = OA.rollout_adjoint(prob, xs, {T_: c}, E=Emin + rho0 * (1.0 - Emin))
    g = res["dE"] * (1.0 - Emin)
    assert np.isfinite(g).all() and np.linalg.norm(g) > 0
    J = lambda rho: float((c * rollout(rho)[-1]).sum())
    for d in (g / np.abs(g).max(), rng.standard_normal(len(Tr))):
        d = d / np.abs(d).max()
        fd = (J(rho0 + 0.05 * d) - J(rho0 - 0.05 * d)) / 0.1
        assert abs(g @ d - fd) < 1e-3 * np.linalg.norm(g) * np.linalg.norm(d), (g @ d, fd)
        assert abs(g @ d - fd) < 1e-2 * abs(fd), (g @ d, fd)


def test_mesh_warnings():
    """Slivers and a wide spread of element sizes are accepted with a warning, and a mesh
    body near another one at rest is warned about before the first step."""
    V = np.array([[0, 0], [1, 0], [0.5, 0.01], [0.5, -1]], float) * 1e-3
    with pytest.warns(UserWarning, match="slivers"):
        D.check_mesh(V, np.array([[0, 1, 2], [0, 3, 1]]))
    Vr, Tr = _polar_ring(0.0001, 0.010, n_t=32)
    with pytest.warns(UserWarning, match="the smallest element"):
        Model().add_soft_mesh(Vr, Tr, E=E, nu=NU, density=RHO)
    m = Model()
    Va, Ta = _jittered(2, 2, (0.002, 0.002))
    m.add_soft_mesh(Va, Ta, E=E, nu=NU, density=RHO)
    m.add_soft_mesh(Va + np.array([0.002 + 0.3 * 0.25e-3 / 8, 0.0]), Ta, E=E, nu=NU, density=RHO)
    m.finalize()
    integ = ImplicitIntegrator()
    with pytest.warns(UserWarning, match="inside the barrier's reach"):
        try:
            integ._build(m, 1e-3)
        except RuntimeError:                 # no CUDA device here: the warning comes first
            pass


def test_a_mesh_block_rests_on_a_pixel_slab():
    """A jittered mesh block dropped on a pixel slab lying on the ground (contact between a
    mesh body and a pixel body): it comes to rest within the barrier's reach of the slab —
    after the reference's tests/test_mesh.py:322-340."""
    m = Model()
    m.damping = 60.0
    m.add_ground(height=0.0, mu=0.6)
    slab = m.add_soft_body(np.ones((4, 16), np.uint8), physical_size=(16 * PX, 4 * PX),
                           center=(0.0, 2 * PX + 0.9 * PX / 8), E=E, nu=NU, density=RHO)
    V, T = _jittered(6, 6, (6 * PX, 6 * PX), origin=(-3 * PX, 4 * PX + 0.6 * PX), seed=3)
    block = m.add_soft_mesh(V, T, E=E, nu=NU, density=RHO)
    m.finalize()
    m.gravity = (0.0, -G0)
    prob = _problem(m, ImplicitIntegrator(), 2e-3)
    s, xs, _ = oracle.run(prob, 200)
    gap = float(scene.min_distance(dict(prob, x=xs[-1])).min())
    assert 0.0 < gap < m.dhat, gap / m.dhat
    assert np.abs(s.v[m.body_nodes(block)]).max() < 2e-3
    assert xs[-1][m.body_nodes(block), 1].min() > xs[-1][m.body_nodes(slab), 1].max()
