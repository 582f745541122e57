"""Seeded synthetic scenes with the shapes of the benchmark configurations.

  strip_on_ground()      one 6 x 72-pixel strip (511 nodes, 864 triangles) lying on the
                         ground: the single-scene configuration
  rectangles_on_ground() a batch of uneven soft rectangles on the ground (H ~ U{4..16},
                         W ~ U{32..128} pixels of 0.75 mm, per-pixel E log-uniform in
                         [0.1, 2] MPa, ground mu ~ U[0.3, 0.9] per scene, top-edge pressure
                         ~ U[0, 5] kPa): the batching configuration
  pads_and_block()       a contact-heavy batch: a soft pad pushed by a kinematic jaw squeezes
                         an affine rigid block against a second, static pad (IPC contact
                         between bodies with per-scene friction)
  slab_with_holes()      the large-scene configuration: a 256 x 1024-pixel soft slab with 200
                         circular holes resting on the ground, 32 affine discs dropped on it
  tendon_arms()          a batch of soft arms (16 x 64 pixels of 0.5 mm) pinned at one end
                         and bent by a tension-controlled tendon, per-pixel E log-uniform
                         in [0.2, 1.5] MPa, a piecewise-linear tension schedule and a target
                         point per arm: the differentiation configuration

Each returns (model, integrator kwargs, dt). No dataset is involved: the scenes are drawn
from numpy.random.default_rng(seed) with the stated distributions.
"""
from __future__ import annotations

import numpy as np

from .model import Model


def strip_on_ground():
    m = Model()
    m.add_ground(0.0, mu=0.8)
    m.add_soft_body(np.ones((6, 72), np.uint8), physical_size=(0.054, 0.0045), center=(0.0, 0.0030),
                    E=0.5e6, nu=0.40, density=1100.0)
    m.finalize()
    m.gravity = (0.0, -9.81)
    return m, {}, 2e-3


def rectangles_on_ground(n_scenes=4096, seed=0, px=0.75e-3, gtol=1e-6):
    """The batching configuration: n_scenes independent soft rectangles on the ground."""
    rng = np.random.default_rng(seed)
    H = rng.integers(4, 17, n_scenes)
    W = rng.integers(32, 129, n_scenes)
    mu_g = rng.uniform(0.3, 0.9, n_scenes)
    pres = rng.uniform(0.0, 5.0e3, n_scenes)
    m = Model()
    m.add_ground(0.0, mu=0.6)
    dhat = px / 8.0
    hs = []
    for i in range(n_scenes):
        h_, w_ = int(H[i]), int(W[i])
        E = np.exp(rng.uniform(np.log(1.0e5), np.log(2.0e6), (h_, w_)))
        hs.append(m.add_soft_body(np.ones((h_, w_), np.uint8), physical_size=(w_ * px, h_ * px),
                                  center=(0.0, 0.5 * h_ * px + 0.9 * dhat), E=E, nu=0.40,
                                  density=1100.0, env_id=i))
    m.finalize()
    m.set_collider_mu(0, mu_g)
    m.gravity = (0.0, -9.81)
    # top-edge pressure as nodal loads: p x tributary edge length, downward
    f = np.zeros((m.n_nodes, 2))
    for i, h in enumerate(hs):
        nodes = m.body_nodes(h)
        X = m.me.rest_pos[nodes]
        top = np.abs(X[:, 1] - X[:, 1].max()) < 1e-12
        trib = np.full(top.sum(), px)
        xs = X[top, 0]
        trib[(xs == xs.min()) | (xs == xs.max())] = 0.5 * px
        f[nodes[top], 1] = -pres[i] * trib
    m._fext = f
    m._ctrl_version += 1
    return m, dict(gtol=gtol), 2e-3


def tension_schedule(rng, n_scenes, steps=100, knots=6, lo=0.0, hi=50.0):
    """(steps, n_scenes) piecewise-linear tension schedules: `knots` values U[lo, hi] per
    scene at evenly spaced steps, linear in between."""
    kk = np.linspace(0.0, steps - 1, knots)
    vals = rng.uniform(lo, hi, (n_scenes, knots))
    t = np.arange(steps, dtype=np.float64)
    return np.stack([np.interp(t, kk, vals[i]) for i in range(n_scenes)], 1)


def tendon_arms(n_scenes=256, seed=0, px=0.5e-3, steps=100):
    """The differentiation configuration: n_scenes soft arms, each a 16 x 64-pixel mask
    (8 mm x 32 mm) pinned at its first node column, per-pixel E log-uniform in [0.2, 1.5] MPa
    (nu 0.40, density 1100), a tension-controlled tendon through the nodes of node row 2
    (counted from the bottom), a `steps`-step piecewise-linear tension schedule in [0, 50] N/m
    and a target point for the tip node (the tendon's last eyelet) within 4 mm of its rest
    position. No gravity, no contact.

    Returns (model, integrator kwargs, dt, extras), extras = dict(handles, E_pixels
    (n, 16, 64), tension (steps, n), tip (n,) node indices, target (n, 2), tendons (n,))."""
    rng = np.random.default_rng(seed)
    H, W = 16, 64
    m = Model()
    hs, Es = [], []
    for i in range(n_scenes):
        E = np.exp(rng.uniform(np.log(2.0e5), np.log(1.5e6), (H, W)))
        Es.append(E)
        hs.append(m.add_soft_body(np.ones((H, W), np.uint8), physical_size=(W * px, H * px),
                                  center=(0.5 * W * px, 0.5 * H * px), E=E, nu=0.40, density=1100.0,
                                  env_id=i))
    m.finalize()
    tips, tendons, targets = [], [], []
    for i, h in enumerate(hs):
        X = m.rest_x(h)
        m.set_kinematic_constraint(h, np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0])
        row = np.where(np.abs(X[:, 1] - (X[:, 1].min() + 2 * px)) < 1e-9)[0]
        row = row[np.argsort(X[row, 0])]
        tendons.append(m.add_tendon(h, nodes=row))
        tip = int(m.body_nodes(h)[row[-1]])
        tips.append(tip)
        targets.append(m.me.rest_pos[tip] + rng.uniform(-4e-3, 4e-3, 2))
    tension = tension_schedule(rng, n_scenes, steps)
    kw = dict(self_collision=False, friction=False, precision="fp64")
    return m, kw, 2e-3, dict(handles=hs, E_pixels=np.stack(Es), tension=tension, tip=np.asarray(tips),
                            target=np.asarray(targets), tendons=np.asarray(tendons))


def pads_and_block(n_scenes=512, seed=0, steps=150, jaw_speed=0.01):
    """The contact-heavy configuration: per scene, a 40 x 40-pixel soft pad (0.5 mm pixels,
    20 mm, E 0.3 MPa, nu 0.45) whose outer column is a kinematic jaw translating at 10 mm/s,
    a 16 x 16-pixel affine block (1 mm pixels, 16 mm, density 600, the model's 1 GPa rigid
    modulus) 0.3 mm from it, and a second pad held still 0.3 mm beyond the block; the block's
    height offset is U[-2, 2] mm, the body friction per scene U[0.4, 0.8], d-hat 0.1 mm,
    gravity on. Returns (model, integrator kwargs, dt, extras) with extras = dict(command)
    where command(k) sets the jaw targets of step k (0-based)."""
    rng = np.random.default_rng(seed)
    m = Model()
    m.dhat = 1.0e-4
    gap, half_b, pad = 0.3e-3, 8.0e-3, 20.0e-3
    off = rng.uniform(-2.0e-3, 2.0e-3, n_scenes)
    mu = rng.uniform(0.4, 0.8, n_scenes)
    left, right = [], []
    for i in range(n_scenes):
        cy = 0.5 * pad
        left.append(m.add_soft_body(np.ones((40, 40), np.uint8), physical_size=(pad, pad),
                                    center=(-(half_b + gap + 0.5 * pad), cy), E=0.3e6, nu=0.45,
                                    density=1100.0, env_id=i, mu=float(mu[i])))
        m.add_affine_body(np.ones((16, 16), np.uint8), physical_size=(2 * half_b, 2 * half_b),
                          center=(0.0, cy + off[i]), density=600.0, env_id=i, mu=float(mu[i]))
        right.append(m.add_soft_body(np.ones((40, 40), np.uint8), physical_size=(pad, pad),
                                     center=(half_b + gap + 0.5 * pad, cy), E=0.3e6, nu=0.45,
                                     density=1100.0, env_id=i, mu=float(mu[i])))
    m.finalize()
    m.gravity = (0.0, -9.81)
    jaws = []
    for hl, hr in zip(left, right):
        X = m.rest_x(hl)
        jl = np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0]
        m.set_kinematic_constraint(hl, jl)
        Y = m.rest_x(hr)
        m.set_kinematic_constraint(hr, np.where(Y[:, 0] > Y[:, 0].max() - 1e-9)[0])
        jaws.append((hl, X, jl))
    dt = 1.0e-3

    def command(k):
        for hl, X, jl in jaws:
            tgt = X.copy()
            tgt[jl, 0] += jaw_speed * dt * (k + 1)
            m.set_kinematic_target(hl, tgt)
    return m, {}, dt, dict(command=command, steps=steps, offset=off, mu=mu)


def _disc_mask(r):
    """A (2r, 2r) pixel mask of a disc of radius r pixels (pixel centres inside)."""
    c = np.arange(2 * r) + 0.5 - r
    return ((c[None, :] ** 2 + c[:, None] ** 2) <= r * r).astype(np.uint8)


def slab_with_holes(n_scenes=1, seed=0, H=256, W=1024, px=0.5e-3, n_holes=200, n_discs=32,
                    hole_r=(3, 12), disc_r=(8, 20), drop=(5e-3, 50e-3)):
    """The large-scene configuration: per scene, an H x W-pixel soft slab (E 1 MPa, nu 0.40,
    density 1100) lying on the ground with n_holes circular holes of radius U{hole_r} pixels
    at seeded, non-overlapping centres, and n_discs affine discs of radius U{disc_r} pixels
    (density U[500, 2000]) placed U[drop] above the slab (default 5-50 mm) at seeded,
    non-overlapping x; gravity on, IPC contact between bodies and with the ground. Defaults:
    256 x 1024 pixels of 0.5 mm (0.128 m x 0.512 m), 200 holes, 32 discs."""
    rng = np.random.default_rng(seed)
    m = Model()
    m.add_ground(0.0)
    dhat = px / 8.0
    for e in range(n_scenes):
        mask = np.ones((H, W), np.uint8)
        yy, xx = np.mgrid[0:H, 0:W]
        placed = []
        tries = 0
        while len(placed) < n_holes and tries < 200 * n_holes:
            tries += 1
            r = int(rng.integers(hole_r[0], hole_r[1] + 1))
            cy, cx = rng.uniform(r + 2, H - r - 2), rng.uniform(r + 2, W - r - 2)
            if any((cy - a) ** 2 + (cx - b) ** 2 < (r + q + 2) ** 2 for a, b, q in placed):
                continue
            placed.append((cy, cx, r))
            mask[(yy + 0.5 - cy) ** 2 + (xx + 0.5 - cx) ** 2 < r * r] = 0
        m.add_soft_body(mask, physical_size=(W * px, H * px), center=(0.0, 0.5 * H * px + 0.9 * dhat),
                        E=1.0e6, nu=0.40, density=1100.0, env_id=e)
        xs = []
        tries = 0
        while len(xs) < n_discs and tries < 200 * n_discs:
            tries += 1
            r = int(rng.integers(disc_r[0], disc_r[1] + 1))
            x = rng.uniform(-0.5 * W * px + r * px, 0.5 * W * px - r * px)
            if any(abs(x - a) < (r + q) * px + 2 * px for a, q in xs):
                continue
            xs.append((x, r))
            y = H * px + rng.uniform(drop[0], drop[1]) + r * px
            m.add_affine_body(_disc_mask(r), physical_size=(2 * r * px, 2 * r * px), center=(x, y),
                              density=float(rng.uniform(500.0, 2000.0)), env_id=e)
    m.finalize()
    m.gravity = (0.0, -9.81)
    return m, {}, 1e-3
