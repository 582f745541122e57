"""Seeded synthetic scenes with the shapes of the benchmark configurations.

  strip_on_ground()      one 6 x 72-pixel strip (511 nodes, 864 triangles) lying on the
                         ground: the single-scene configuration
  rectangles_on_ground() a batch of uneven soft rectangles on the ground (H ~ U{4..16},
                         W ~ U{32..128} pixels of 0.75 mm, per-pixel E log-uniform in
                         [0.1, 2] MPa, ground mu ~ U[0.3, 0.9] per scene, top-edge pressure
                         ~ U[0, 5] kPa): the batching configuration

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
