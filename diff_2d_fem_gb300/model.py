"""Model — the scene container, with the reference's API (sim_model.py).

    model = Model()
    model.add_ground(0.0, mu=0.8)
    h = model.add_soft_body(mask, physical_size=(0.054, 0.0045), center=(0.0, 0.003),
                            E=0.5e6, nu=0.40, density=1100.0)
    model.finalize()
    model.gravity = (0.0, -9.81)
    integ = ImplicitIntegrator()
    for t in range(T):
        integ.simulate(model, 2e-3)

Bodies are pixel masks (row 0 at the bottom) rasterised into P1 triangles; every body
lives in an environment (`env_id`), environments never interact and are solved together.
The host side here only assembles arrays; the step itself runs on the GPU (integrator.py).
New, keyword-only, beyond the reference: a per-environment collider friction
(`set_collider_mu`), which the reference cannot express (its colliders carry one mu for
every environment, implicit/solver.py:235-242).
"""
from __future__ import annotations

import warnings
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import actuators as _act
from . import mesh as _mesh

NONE, DISC, ELLIPSE, BOX, TRIANGLE, HALFSPACE = -1, 0, 1, 2, 3, 4
NAMES = {"disc": DISC, "ellipse": ELLIPSE, "box": BOX, "square": BOX, "triangle": TRIANGLE}


@dataclass
class SimConfig:
    """Material defaults, damping and contact parameters (reference core/config.py:13-29)."""
    young: float = 1.0e6
    nu: float = 0.40
    rho_mass: float = 1000.0
    damping: float = 0.0
    ipc_d_hat: Optional[float] = None
    obstacle_stiffness: Optional[float] = None
    contact_stiffness: Optional[float] = None
    obstacle_friction: float = 0.5
    obstacle_friction_epsv: float = 1.0e-3


@dataclass
class Collider:
    """A collider's parameters as the solver reads them: kind (DISC, ELLIPSE, BOX,
    TRIANGLE, HALFSPACE; NONE for no collider), centre (cx, cy) — a plane's origin — and
    rx, ry (disc: radius; ellipse / box: half-extents; plane: the unit normal), rref (box,
    triangle: corner radius; ellipse: level-set scale)."""
    kind: int = DISC
    cx: float = 0.0
    cy: float = 0.0
    rx: float = 0.0
    ry: float = 0.0
    rref: float = 0.0

    @property
    def c(self):
        return np.array([self.cx, self.cy])


class Model:
    def __init__(self, device="cuda", config=None):
        self.cfg = SimConfig() if config is None else config
        self.device = device
        self._colliders = []
        self._col_mu_env = {}
        self._bodies = []
        self._constrained = {}
        self.me = None
        self._solver = None
        self._targets = None
        self._node_range, self._tri_range = [], []
        self._v0 = None
        self._x_host = None
        self._epoch = 0
        self.time = 0.0
        self._gravity = (0.0, 0.0)
        self._fext = None
        self._tendons = []
        self._chambers = []
        self._springs = []
        self._regions = []
        self._regions_of = {}
        self._affine = []
        self._affine_of = {}
        self._extra_excl = []
        self._mesh_info = {}
        self.body_contact = "ipc"
        self.body_friction = 0.0
        self.body_kappa = None
        self.rigid_young = 1.0e9
        self.rigid_nu = 0.30
        self._act_version = 0
        self._ctrl_version = 0

    # ---- contact / material attributes over the config (sim_model.py:118-127)
    def _p(name):
        return property(lambda s: getattr(s.cfg, name), lambda s, v: setattr(s.cfg, name, v))
    dhat = _p("ipc_d_hat")
    kappa = _p("obstacle_stiffness")
    self_stiffness = _p("contact_stiffness")
    mu = _p("obstacle_friction")
    epsv = _p("obstacle_friction_epsv")
    damping = _p("damping")
    del _p

    # ---- colliders (sim_model.py:133-184)
    def add_disc(self, center, radius, mu=None):
        return self.add_object("disc", center, radius, mu=mu)

    def add_plane(self, normal, origin, mu=None):
        n = np.asarray(normal, np.float64)
        if not np.linalg.norm(n) > 0:
            raise ValueError("the plane normal must be non-zero")
        n = n / np.linalg.norm(n)
        return self._set_collider(HALFSPACE, origin, float(n[0]), float(n[1]), 0.0, mu)

    def add_ground(self, height=0.0, mu=None):
        return self.add_plane((0.0, 1.0), (0.0, height), mu=mu)

    def add_object(self, kind, center, rx, ry=None, corner_radius=3.0e-3, mu=None):
        k = NAMES[kind] if isinstance(kind, str) else int(kind)
        rx = float(rx)
        ry = rx if ry is None else float(ry)
        rref = float(corner_radius) if k in (BOX, TRIANGLE) else rx
        return self._set_collider(k, center, rx, ry, rref, mu)

    def _set_collider(self, kind, center, rx, ry, rref, mu):
        if self._solver is not None:
            raise RuntimeError("add colliders before the first simulate()")
        mu = float(self.cfg.obstacle_friction if mu is None else mu)
        self._colliders.append(dict(kind=int(kind), cx=float(center[0]), cy=float(center[1]),
                                    rx=rx, ry=ry, rref=rref, r=rx, mu=mu))
        return len(self._colliders) - 1

    def set_collider_center(self, index, center):
        """Move a collider (sim_model.py:176-184). Before the first step this places it;
        during a rollout it TELEPORTS the shape between steps — the move is not swept, so keep
        each step's displacement well under the current clearance, and friction treats the
        collider as stationary."""
        c = self._colliders[index]
        c["cx"], c["cy"] = float(center[0]), float(center[1])
        if self._solver is not None:
            self._solver.set_collider_centers([[k["cx"], k["cy"]] for k in self._colliders])

    @property
    def colliders(self):
        """Every collider as a host-side Collider record (kind, cx, cy, rx, ry, rref)."""
        return [Collider(kind=c["kind"], cx=c["cx"], cy=c["cy"], rx=c["rx"], ry=c["ry"], rref=c["rref"])
                for c in self._colliders]

    @property
    def object(self):
        """The first collider (kind NONE when the scene has none)."""
        cs = self.colliders
        return cs[0] if cs else Collider(kind=NONE)

    def set_collider_mu(self, index, mu_per_env):
        """Per-environment Coulomb coefficient of collider `index` ((n_envs,) array). New
        in this implementation: the reference has one mu per collider for every
        environment."""
        if self._solver is not None:
            raise RuntimeError("set per-environment friction before the first simulate()")
        self._col_mu_env[int(index)] = np.asarray(mu_per_env, np.float64).copy()

    # ---- bodies (sim_model.py:199-264)
    def add_soft_body(self, mask, physical_size, center, E=None, nu=None, density=None, env_id=0, mu=None):
        if self.me is not None:
            raise RuntimeError("add bodies before finalize()")
        mask = (np.asarray(mask) > 0.5).astype(np.uint8)
        if mask.ndim != 2 or not mask.any():
            raise ValueError("the mask must be a 2-D array with at least one solid pixel")
        if E is not None and not np.isscalar(E):
            E = np.asarray(E, np.float64)
            if E.shape != mask.shape:
                raise ValueError(f"stiffness map is {E.shape}, the mask is {mask.shape}")
            if (E[mask > 0] <= 0).any():
                raise ValueError("stiffness map must be positive wherever the mask is solid")
        if int(env_id) < 0:
            raise ValueError("env_id must be >= 0")
        if mu is not None:
            mu = float(mu)
            if not (np.isfinite(mu) and mu >= 0.0):
                raise ValueError(f"mu must be a finite number >= 0, not {mu}")
        c = self.cfg
        self._bodies.append(dict(mask=mask, size=tuple(float(v) for v in physical_size),
                                 center=tuple(float(v) for v in center),
                                 E=(c.young if E is None else (float(E) if np.isscalar(E) else E)),
                                 nu=float(c.nu if nu is None else nu),
                                 rho=float(c.rho_mass if density is None else density),
                                 env=int(env_id), mu=mu))
        return len(self._bodies) - 1

    def add_affine_body(self, mask, physical_size, center, density=None, env_id=0, E=None, nu=None, mu=None):
        h = self.add_soft_body(mask, physical_size, center, E=(self.rigid_young if E is None else E),
                               nu=(self.rigid_nu if nu is None else nu), density=density,
                               env_id=env_id, mu=mu)
        if not np.isscalar(self._bodies[h]["E"]):
            raise ValueError("a rigid body takes a scalar stiffness")
        self._bodies[h]["affine"] = True
        return h

    def add_kinematic_body(self, mask, physical_size, center, env_id=0, mu=None):
        h = self.add_soft_body(mask, physical_size, center, env_id=env_id, mu=mu)
        self._bodies[h]["kinematic"] = True
        return h

    # ---- bodies given as triangle meshes (sim_model.py:280-338)
    def add_soft_mesh(self, vertices, triangles, E=None, nu=None, density=None, env_id=0, mu=None):
        """A soft body given as a triangle mesh: vertices (n, 2) at rest [m], triangles (m, 3)
        0-based, either winding. Vertex i is node i of the body and triangle j its element j,
        so node- and element-addressed calls use the mesh's own numbering; per-pixel inputs
        become per-triangle arrays (E of shape (m,), regions as (m,) booleans or triangle
        indices) and a hole in the mesh is a pressure chamber. The mesh is validated first
        (mesh.check_mesh). Returns a handle."""
        if self.me is not None:
            raise RuntimeError("add bodies before finalize()")
        info = self._check_mesh(vertices, triangles)
        m = len(info["triangles"])
        if E is not None and not np.isscalar(E):
            E = np.asarray(E, np.float64)
            if E.shape != (m,):
                raise ValueError(f"stiffness per triangle is {E.shape}; the mesh has {m} triangles")
            if not (np.isfinite(E).all() and (E > 0).all()):
                raise ValueError("stiffness must be positive and finite on every triangle")
        if int(env_id) < 0:
            raise ValueError("env_id must be >= 0")
        if mu is not None:
            mu = float(mu)
            if not (np.isfinite(mu) and mu >= 0.0):
                raise ValueError(f"mu must be a finite number >= 0, not {mu}")
        c = self.cfg
        V = info["vertices"]
        self._bodies.append(dict(mesh=True, vertices=V, triangles=info["triangles"], h=info["h"],
                                 h_cfl=info["h_cfl"], L_max=info["L_max"],
                                 center=tuple(float(v) for v in 0.5 * (V.min(0) + V.max(0))),
                                 E=(c.young if E is None else (float(E) if np.isscalar(E) else E)),
                                 nu=float(c.nu if nu is None else nu),
                                 rho=float(c.rho_mass if density is None else density),
                                 env=int(env_id), mu=mu))
        return len(self._bodies) - 1

    def add_affine_mesh(self, vertices, triangles, density=None, env_id=0, E=None, nu=None, mu=None):
        """A rigid (affine) body given as a triangle mesh. Returns a handle."""
        h = self.add_soft_mesh(vertices, triangles, E=(self.rigid_young if E is None else E),
                               nu=(self.rigid_nu if nu is None else nu), density=density,
                               env_id=env_id, mu=mu)
        if not np.isscalar(self._bodies[h]["E"]):
            raise ValueError("a rigid body takes a scalar stiffness")
        self._bodies[h]["affine"] = True
        return h

    def add_kinematic_mesh(self, vertices, triangles, env_id=0, mu=None):
        """A body of prescribed motion given as a triangle mesh. Returns a handle."""
        h = self.add_soft_mesh(vertices, triangles, env_id=env_id, mu=mu)
        self._bodies[h]["kinematic"] = True
        return h

    def _check_mesh(self, vertices, triangles):
        """check_mesh once per distinct mesh (a batch repeats the same one), warning when the
        element sizes spread over more than a decade."""
        import hashlib
        V = np.ascontiguousarray(vertices, np.float64)
        T = np.ascontiguousarray(triangles)
        key = (V.shape, T.shape, str(T.dtype), hashlib.sha1(V.tobytes() + T.tobytes()).hexdigest())
        cache = self._mesh_info
        if key not in cache:
            info = _mesh.check_mesh(V, T)
            size = np.sqrt(2.0 * info["area"])
            if size.max() > 10.0 * size.min():
                warnings.warn(f"this mesh's elements range from {size.min() * 1e3:.3g} to "
                              f"{size.max() * 1e3:.3g} mm; the iterations a step needs follow the "
                              f"smallest element, so a few small ones make every step dearer.",
                              stacklevel=4)
            cache[key] = info
        return cache[key]

    def _is_mesh(self, handle):
        return bool(self._bodies[handle].get("mesh"))

    def _need_pixels(self, handle, what):
        if self._is_mesh(handle):
            raise ValueError(f"body {handle} is a mesh body: {what} needs a pixel body. A mesh body "
                             f"takes per-triangle arrays instead.")

    # ---- build (sim_model.py:391-429)
    def finalize(self):
        if not self._bodies:
            raise ValueError("add at least one soft body before finalize()")
        B = self._bodies
        # a mesh body's boundary pairs closer than this through the material are excluded
        # from its self-contact (sim_model.py:396-399)
        dx = self.dx
        r_excl = max(2.0 * dx, 16.0 * (self.cfg.ipc_d_hat if self.cfg.ipc_d_hat is not None else dx / 8.0))
        geom = lambda b: (dict(vertices=b["vertices"], triangles=b["triangles"], excl_radius=r_excl, checked=True)
                          if b.get("mesh") else dict(mask_xy=b["mask"].T.copy(), size=b["size"], center=b["center"]))
        self.me = _mesh.build_scene([dict(**geom(b), young=(b["E"] if np.isscalar(b["E"]) else 1.0), nu=b["nu"],
                                          rho=b["rho"], env=b["env"]) for b in B])
        me = self.me
        self._node_range = [np.arange(*me.body_node_range[h]) for h in range(len(B))]
        self._tri_range = [np.arange(*me.body_tri_range[h]) for h in range(len(B))]
        for h, b in enumerate(B):
            if np.isscalar(b["E"]):
                continue
            tris = self._tri_range[h]
            scale = b["E"] if b.get("mesh") else self._pixel_field(h, b["E"])
            me.mu[tris] = me.mu[tris] * scale
            me.lam[tris] = me.lam[tris] * scale
        self._check_layout()
        self._scale_contact()
        self._targets = me.rest_pos.astype(np.float64).copy()
        self._x_host = me.rest_pos.astype(np.float64).copy()
        self._v0 = np.zeros_like(self._x_host)
        for h, b in enumerate(B):
            if b.get("affine"):
                self._add_affine(h, self._tri_range[h])
            if b.get("kinematic"):
                self._constrained[h] = self._node_range[h].copy()
        return self

    def _pixel_field(self, h, field):
        q = np.asarray(self.me.tri_quad)[self._tri_range[h]]
        ny = self._bodies[h]["mask"].shape[0]
        return np.asarray(field, np.float64)[q % ny, q // ny]

    def add_affine_region(self, handle, region, E=None, nu=None):
        """Make part of a soft body rigid (sim_model.py:432-453): the solid pixels of the
        (H, W) boolean map `region`, laid out like the mask, become one affine piece that
        shares its interface nodes with the soft material around it. E, nu: the stiffness
        the piece resists strain with (default model.rigid_young / rigid_nu). Call after
        finalize() and before the first step; two pieces need at least one soft element
        between them. Returns the piece's index (as affine_state takes it)."""
        self._need_mesh()
        if self._solver is not None:
            raise RuntimeError("add rigid regions before the first simulate()")
        elems = self._region_elements(handle, region)
        mu, lam = _mesh.lame(self.rigid_young if E is None else float(E),
                             self.rigid_nu if nu is None else float(nu))
        self.me.mu[elems] = mu
        self.me.lam[elems] = lam
        return self._add_affine(handle, elems)

    def _region_elements(self, handle, region):
        """Global element ids of part of a body (sim_model.py:1103-1132): the solid pixels of
        an (H, W) map laid out like a pixel body's mask; for a mesh body (m,) booleans or
        distinct triangle indices."""
        b = self._bodies[handle]
        if b.get("mesh"):
            tris = self._tri_range[handle]
            m = len(tris)
            r = np.asarray(region)
            if r.dtype == bool:
                if r.shape != (m,):
                    raise ValueError(f"region is a boolean array of shape {r.shape}; mesh body {handle} "
                                     f"has {m} triangles: give ({m},) booleans or triangle indices")
                loc = np.flatnonzero(r)
            else:
                if r.ndim != 1 or not np.issubdtype(r.dtype, np.integer):
                    raise ValueError(f"region of a mesh body: ({m},) booleans or a 1-D array of triangle "
                                     f"indices; got {r.dtype} of shape {r.shape}")
                loc = np.unique(r)
                if len(loc) != len(r) or (len(loc) and (loc[0] < 0 or loc[-1] >= m)):
                    raise ValueError(f"triangle indices must be distinct and in 0..{m - 1}")
            if len(loc) == 0:
                raise ValueError("the region contains no triangle of this body")
            return tris[loc]
        region = np.asarray(region) > 0
        if region.shape != b["mask"].shape:
            raise ValueError(f"region is {region.shape}, the mask is {b['mask'].shape}")
        H = b["mask"].shape[0]
        tris = self._tri_range[handle]
        q = np.asarray(self.me.tri_quad)[tris]
        elems = tris[region[q % H, q // H]]
        if len(elems) == 0:
            raise ValueError("the region contains no solid pixel of this body")
        return elems

    def _add_affine(self, handle, elems):
        me = self.me
        mine = self._affine_of.setdefault(handle, [])
        if mine and np.intersect1d(elems, np.concatenate(mine)).size:
            raise ValueError("rigid regions must not overlap")
        mine.append(np.asarray(elems, np.int64))
        nodes = np.unique(np.asarray(me.tri)[elems].reshape(-1))
        # the boundary nodes of one rigid piece never move relative to each other: exclude
        # every pair of them from contact (sim_model.py:466-476)
        env = self._bodies[handle]["env"]
        lo, hi = int(me.boundary_starts[env]), int(me.boundary_starts[env + 1])
        loc = np.nonzero(np.isin(me.boundary_nodes[lo:hi], nodes))[0]
        self._extra_excl.append((lo, loc))
        self._affine.append(dict(body=handle, elems=np.asarray(elems, np.int64), nodes=nodes))
        return len(self._affine) - 1

    def exclusion_csr(self):
        """The scene's self-contact exclusion (mesh hops + rigid pieces) as a CSR over the
        boundary slots, columns environment-local and sorted."""
        me = self.me
        ptr, idx = me.excl_ptr, me.excl_idx
        if not self._extra_excl:
            return ptr, idx
        rows = [set(idx[ptr[s]:ptr[s + 1]].tolist()) for s in range(len(ptr) - 1)]
        for lo, loc in self._extra_excl:
            for a in loc:
                rows[lo + a].update(int(v) for v in loc)
        new_ptr = np.zeros(len(rows) + 1, np.int64)
        new_ptr[1:] = np.cumsum([len(r) for r in rows])
        new_idx = np.concatenate([np.sort(np.fromiter(r, np.int64)) for r in rows]) if rows else np.zeros(0, np.int64)
        return new_ptr, new_idx

    def _scale_contact(self):
        """Contact parameters left unset, from the scene's own scales (sim_model.py:487-497)."""
        c = self.cfg
        soft = [b for b in self._bodies if not b.get("affine") and not b.get("kinematic")]
        E = min((float(b["E"]) if np.isscalar(b["E"]) else
                 float(b["E"].min()) if b.get("mesh") else float(b["E"][b["mask"] > 0].min())
                 for b in soft), default=1.0e6)
        if c.ipc_d_hat is None:
            c.ipc_d_hat = self.dx / 8.0
        if c.obstacle_stiffness is None:
            c.obstacle_stiffness = 4.0e-3 * E * self.dx / c.ipc_d_hat
        if c.contact_stiffness is None:
            c.contact_stiffness = 0.2 * E
        if self.body_kappa is None:
            self.body_kappa = 0.1 * E * self.dx / c.ipc_d_hat

    def _check_layout(self):
        """Bodies of one environment must not start inside one another (sim_model.py:499-535)."""
        envs = {}
        for h, b in enumerate(self._bodies):
            envs.setdefault(b["env"], []).append(h)
        memo = {}
        for env, hs in envs.items():
            for i, a in enumerate(hs):
                for c in hs[i + 1:]:
                    if self._is_mesh(a) or self._is_mesh(c):
                        key = (self._geom_key(a), self._geom_key(c))
                        if key not in memo:
                            memo[key] = _mesh.meshes_overlap(*self._body_geometry(a), *self._body_geometry(c))
                        hit = memo[key]
                    else:
                        hit = self._overlap(a, c) or self._overlap(c, a)
                    if hit:
                        raise ValueError(
                            f"bodies {a} and {c} overlap in environment {env}. Bodies of one "
                            f"environment collide with each other and must start apart; give "
                            f"the members of a batch their own environment with env_id=i.")
            if any(self._is_mesh(h) for h in hs):
                sz = [self.element_size(h) for h in hs]
                if max(sz) > 1.25 * min(sz):
                    warnings.warn(f"environment {env} mixes element sizes (pixel width, or a mesh body's "
                                  f"median boundary edge) from {min(sz) * 1e3:.3g} to {max(sz) * 1e3:.3g} "
                                  f"mm. Contact between bodies has ONE thickness, set by the largest.",
                                  stacklevel=3)
                continue
            px = [self.pixel_size(h)[0] for h in hs]
            if max(px) > 1.25 * min(px):
                warnings.warn(f"environment {env} mixes pixel sizes from {min(px) * 1e3:.3g} to "
                              f"{max(px) * 1e3:.3g} mm. Contact between bodies has ONE thickness, "
                              f"set by the largest. Prefer one pixel size per scene.", stacklevel=3)

    def _geom_key(self, h):
        b = self._bodies[h]
        if b.get("mesh"):
            return ("mesh", id(b["vertices"]), id(b["triangles"]))
        return ("mask", b["mask"].shape, b["mask"].tobytes(), b["size"], b["center"])

    def _body_geometry(self, h):
        """A body's rest mesh in its own numbering: (nodes (n, 2), triangles (m, 3))."""
        nodes = self._node_range[h]
        s0, s1 = int(nodes[0]), int(nodes[-1]) + 1
        return np.asarray(self.me.rest_pos[s0:s1], np.float64), np.asarray(self.me.tri)[self._tri_range[h]] - s0

    def _overlap(self, a, c):
        A, C = self._bodies[a], self._bodies[c]
        (aw, ah), (ax, ay) = A["size"], A["center"]
        (cw, ch), (cx, cy) = C["size"], C["center"]
        if abs(ax - cx) >= 0.5 * (aw + cw) or abs(ay - cy) >= 0.5 * (ah + ch):
            return False
        H, W = A["mask"].shape
        row, col = np.nonzero(A["mask"])
        px = ax - 0.5 * aw + (col + 0.5) * aw / W
        py = ay - 0.5 * ah + (row + 0.5) * ah / H
        Hc, Wc = C["mask"].shape
        jc = np.floor((px - (cx - 0.5 * cw)) / (cw / Wc)).astype(int)
        jr = np.floor((py - (cy - 0.5 * ch)) / (ch / Hc)).astype(int)
        ok = (jc >= 0) & (jc < Wc) & (jr >= 0) & (jr < Hc)
        return bool(C["mask"][jr[ok], jc[ok]].any())

    # ---- layout queries (sim_model.py:572-700)
    @property
    def n_bodies(self):
        return len(self._bodies)

    @property
    def n_envs(self):
        return int(self.me.n_envs) if self.me is not None else \
            (max(b["env"] for b in self._bodies) + 1 if self._bodies else 0)

    @property
    def n_nodes(self):
        return int(self.me.rest_pos.shape[0])

    @property
    def n_elements(self):
        return int(self.me.tri.shape[0])

    def body_env(self, handle):
        return self._bodies[handle]["env"]

    def body_nodes(self, handle):
        return self._node_range[handle].copy()

    def body_elements(self, handle):
        return self._tri_range[handle].copy()

    def pixel_size(self, handle):
        """(width, height) of one pixel of a body [m]; a mesh body has none."""
        if self._is_mesh(handle):
            raise ValueError(f"body {handle} is a mesh body: it has no pixels. Its length scale is "
                             f"element_size({handle}).")
        b = self._bodies[handle]
        H, W = b["mask"].shape
        return b["size"][0] / W, b["size"][1] / H

    def element_size(self, handle):
        """A body's contact length scale [m]: its pixel width, or a mesh body's median
        boundary-edge length."""
        b = self._bodies[handle]
        return float(b["h"]) if b.get("mesh") else self.pixel_size(handle)[0]

    def _cfl_length(self, handle):
        """The element size a wave crosses per element: the smaller pixel side, or a mesh
        body's smallest sqrt(2 x triangle area)."""
        b = self._bodies[handle]
        return float(b["h_cfl"]) if b.get("mesh") else min(self.pixel_size(handle))

    @property
    def dx(self):
        """Element size [m]: the largest over the bodies (it sets the thickness of contact
        between bodies)."""
        return max(self.element_size(h) for h in range(len(self._bodies)))

    def element_areas(self, handle):
        return np.asarray(self.me.rest_area, np.float64)[self._tri_range[handle]].copy()

    def rest_x(self, handle):
        return self.me.rest_pos[self._node_range[handle]].copy()

    def to_elements(self, handle, field):
        """An (H, W) pixel field on each of a body's elements (body_elements order); a mesh
        body's (m,) field is checked and returned as it is."""
        b = self._bodies[handle]
        field = np.asarray(field, np.float64)
        if b.get("mesh"):
            m = len(self._tri_range[handle])
            if field.shape != (m,):
                raise ValueError(f"field is {field.shape}; mesh body {handle} has {m} triangles")
            return field.copy()
        if field.shape != b["mask"].shape:
            raise ValueError(f"field is {field.shape}, the mask is {b['mask'].shape}")
        return self._pixel_field(handle, field)

    def to_pixels(self, handle, values):
        self._need_pixels(handle, "to_pixels")
        H, W = self._bodies[handle]["mask"].shape
        q = np.asarray(self.me.tri_quad)[self._tri_range[handle]]
        out = np.zeros((H, W))
        np.add.at(out, (q % H, q // H), np.asarray(values, np.float64))
        return out

    # ---- read-outs (sim_model.py:625-642, core/fields.py), computed on the GPU
    def element_strain(self, x=None, handle=None, signed=False):
        """Strain of every element at positions x (default: now), or of one body's elements
        in body_elements order: the von Mises equivalent of the Green-Lagrange strain (>= 0);
        signed=True: the in-plane principal strain of larger magnitude (+ tension)."""
        return self._field("strain", x, handle, signed)

    def element_stress(self, x=None, handle=None, signed=False):
        """Cauchy stress [Pa] of every element at positions x (default: now) with the bodies'
        own moduli, or of one body's elements: von Mises (>= 0), or with signed=True the
        in-plane principal stress of larger magnitude (+ tension)."""
        return self._field("stress", x, handle, signed)

    def _field(self, field, x, handle, signed=False):
        import torch
        from . import _lib
        if not torch.cuda.is_available():
            raise RuntimeError("element read-outs run on the GPU: no CUDA device")
        L = _lib.load()
        dev = torch.device(self.device if str(self.device).startswith("cuda") else "cuda")
        me = self.me
        c = getattr(self, "_field_bufs", None)
        if c is None:
            f64 = torch.float64
            c = self._field_bufs = dict(
                tri=torch.as_tensor(np.asarray(me.tri), dtype=torch.int32, device=dev).contiguous(),
                Bm=torch.as_tensor(np.asarray(me.D_m_inv, np.float64).reshape(-1, 4), dtype=f64, device=dev).contiguous(),
                mu=torch.as_tensor(np.asarray(me.mu, np.float64), dtype=f64, device=dev),
                lam=torch.as_tensor(np.asarray(me.lam, np.float64), dtype=f64, device=dev))
        T = int(c["tri"].shape[0])
        xx = torch.as_tensor(np.asarray(self.get_x() if x is None else x, np.float64), device=dev).contiguous()
        out = torch.empty(T, dtype=torch.float64, device=dev)
        slot = {("strain", False): 6, ("strain", True): 7, ("stress", False): 8, ("stress", True): 9}[(field, bool(signed))]
        args = [None] * 4
        args[slot - 6] = out.data_ptr()
        rc = L.d2f_element_fields(T, c["tri"].data_ptr(), c["Bm"].data_ptr(), c["mu"].data_ptr(), c["lam"].data_ptr(),
                                  xx.data_ptr(), *args, torch.cuda.current_stream(dev).cuda_stream)
        _lib.check(rc, "d2f_element_fields")
        v = out.cpu().numpy()
        return v if handle is None else v[self._tri_range[handle]]

    def rigid_motion(self, handle, translation=(0.0, 0.0), angle=0.0, about=None):
        x = self.rest_x(handle)
        c = np.asarray(self._bodies[handle]["center"] if about is None else about, np.float64)
        ca, sa = np.cos(angle), np.sin(angle)
        R = np.array([[ca, -sa], [sa, ca]])
        return (x - c) @ R.T + c + np.asarray(translation, np.float64)

    # ---- kinematic boundary conditions (sim_model.py:384-388, 686-692)
    def set_kinematic_constraint(self, handle, node_indices):
        self._constrained[handle] = self._node_range[handle][np.asarray(node_indices, int)]

    def set_kinematic_target(self, handle, targets):
        self._targets[self._node_range[handle]] = np.asarray(targets, np.float64)

    def set_kinematic_pose(self, handle, translation=(0.0, 0.0), angle=0.0, about=None):
        self.set_kinematic_target(handle, self.rigid_motion(handle, translation, angle, about))

    def all_constrained(self):
        if not self._constrained:
            return np.zeros(0, np.int64)
        return np.unique(np.concatenate([np.asarray(v, np.int64) for v in self._constrained.values()]))

    # ---- state I/O (sim_model.py:694-796)
    def get_x(self):
        if self._solver is not None:
            self._x_host = self._solver.get_x()
        return self._x_host.copy()

    def get_body_x(self, handle):
        return self.get_x()[self._node_range[handle]]

    def get_body_v(self, handle):
        v = self._v0 if self._solver is None else self._solver.get_v()
        return np.asarray(v)[self._node_range[handle]].copy()

    def set_body_velocity(self, handle, velocity=(0.0, 0.0), omega=0.0, about=None):
        nodes = self._node_range[handle]
        x = self.get_x()[nodes].astype(np.float64)
        c = np.asarray(about, np.float64) if about is not None else x.mean(0)
        r = x - c
        v = np.asarray(velocity, np.float64)[None, :] + omega * np.stack([-r[:, 1], r[:, 0]], 1)
        self._v0[nodes] = v
        if self._solver is not None:
            self._solver.set_nodes(nodes, v=v)

    def set_body_x(self, handle, x, v=None):
        nodes = self._node_range[handle]
        x = np.asarray(x, np.float64).reshape(len(nodes), 2)
        self._x_host[nodes] = x
        self._targets[nodes] = x
        if v is not None:
            self._v0[nodes] = np.asarray(v, np.float64).reshape(len(nodes), 2)
        if self._solver is not None:
            self._solver.set_nodes(nodes, x=x, v=None if v is None else self._v0[nodes], xn=True)
            self._solver.sync_affine([i for i, a in enumerate(self._affine) if a["body"] == handle])

    def set_body_pose(self, handle, translation=(0.0, 0.0), angle=0.0, about=None, velocity=(0.0, 0.0), omega=0.0):
        self.set_body_x(handle, self.rigid_motion(handle, translation, angle, about))
        self.set_body_velocity(handle, velocity, omega)

    def reset(self, env_ids=None):
        """Back to rest at zero velocity, kinematic targets included (sim_model.py:761-796)."""
        rest = self.me.rest_pos.astype(np.float64)
        s = self._solver
        if env_ids is None:
            self._targets = rest.copy()
            self._x_host = rest.copy()
            self._v0 = np.zeros_like(rest)
            self._epoch += 1
            self.time = 0.0
            if s is not None:
                s.reset_envs(None)
            return
        pick = np.zeros(self.n_envs, np.int32)
        pick[np.atleast_1d(env_ids)] = 1
        nodes = pick[np.asarray(self.me.node2env)] != 0
        self._targets[nodes] = rest[nodes]
        self._x_host[nodes] = rest[nodes]
        self._v0[nodes] = 0.0
        self._epoch += 1
        if s is not None:
            s.reset_envs(pick)

    # ---- actuation (sim_model.py:806-967)
    def _need_mesh(self):
        if self.me is None:
            raise RuntimeError("call finalize() before adding actuators")

    @property
    def gravity(self):
        return self._gravity

    @gravity.setter
    def gravity(self, g):
        self._gravity = (float(g[0]), float(g[1]))
        self._ctrl_version += 1

    def set_external_force(self, handle, force):
        """Nodal forces on a body, (n_body_nodes, 2) [N/m], held until changed."""
        self._need_mesh()
        if self._fext is None:
            self._fext = np.zeros((self.me.rest_pos.shape[0], 2), np.float64)
        self._fext[self._node_range[handle]] = np.asarray(force, np.float64)
        self._ctrl_version += 1

    def add_tendon(self, handle, through=None, nodes=None, stiffness=None):
        """Thread a cable through a body (sim_model.py:931-958). Returns a handle."""
        self._need_mesh()
        ids = self._node_range[handle]
        if (through is None) == (nodes is None):
            raise ValueError("give exactly one of `through` (points) or `nodes` (indices)")
        if nodes is not None:
            path = ids[np.asarray(nodes, int)]
        else:
            pts = np.atleast_2d(np.asarray(through, np.float64))
            pos = self.me.rest_pos[ids]
            dd = np.linalg.norm(pos[None, :, :] - pts[:, None, :], axis=2)
            path = np.asarray(ids)[dd.argmin(1)]
            keep = np.concatenate([[True], path[1:] != path[:-1]])
            path = path[keep]
        if len(path) < 2:
            raise ValueError("a tendon needs at least two distinct eyelets")
        if stiffness is not None and stiffness <= 0:
            raise ValueError("stiffness must be positive (or None for a tension-controlled cable)")
        xs = self.me.rest_pos[np.asarray(path)]
        length = float(np.linalg.norm(np.diff(xs, axis=0), axis=1).sum())
        self._tendons.append(dict(body=handle, nodes=np.asarray(path, np.int64),
                                  stiffness=0.0 if stiffness is None else float(stiffness),
                                  tension=0.0, length=length))
        self._act_version += 1
        return len(self._tendons) - 1

    def set_tendon_tension(self, tendon, tension):
        t = self._tendons[tendon]
        if t["stiffness"] > 0:
            raise ValueError("this tendon is length-controlled; use set_tendon_length")
        t["tension"] = float(tension)
        self._ctrl_version += 1

    def set_tendon_length(self, tendon, length):
        t = self._tendons[tendon]
        if t["stiffness"] <= 0:
            raise ValueError("this tendon is tension-controlled; use set_tendon_tension")
        t["length"] = float(length)
        self._ctrl_version += 1

    def tendon_length(self, tendon):
        """Current path length of a cable through its eyelets [m]."""
        x = self.get_x()[self._tendons[tendon]["nodes"]]
        return float(np.linalg.norm(np.diff(x, axis=0), axis=1).sum())

    def tendon_tension(self, tendon):
        """Current tension of a cable [N/m] (zero when a length-controlled cable is slack)."""
        t = self._tendons[tendon]
        if t["stiffness"] > 0:
            return t["stiffness"] * max(self.tendon_length(tendon) - t["length"], 0.0)
        return max(t["tension"], 0.0)

    # ---- pneumatic / hydraulic: pressure in sealed cavities (sim_model.py:825-929)
    def _node_of(self, handle):
        """Vectorised (ix, iy) grid corner -> global node id (or -1) of a pixel body."""
        me = self.me
        base, ny = int(me.body_node_range[handle][0]), int(me.body_grid[handle][1])
        live = np.asarray(me.grid_to_live_node_per_body[handle])

        def node_of(ix, iy):
            loc = live[(ny + 1) * np.asarray(ix, np.int64) + np.asarray(iy, np.int64)]
            return np.where(loc < 0, -1, base + loc)
        return node_of

    def add_pressure_chambers(self, handle, min_pixels=1):
        """Make every sealed cavity of a body (a void region enclosed by solid, not reaching the
        edge of the pixel grid) a pressure chamber. Returns their handles, ordered by the
        cavity's first pixel, bottom row first then left to right. On a mesh body every hole
        of the mesh is a chamber (min_pixels does not apply), ordered by its lowest node,
        then left to right."""
        self._need_mesh()
        if self._is_mesh(handle):
            holes = [lp for lp in self._mesh_loops(handle) if lp[2] > 0]
            rest = self.me.rest_pos
            lowest = lambda lp: tuple(rest[lp[0][np.argmin(rest[lp[0], 1])]][::-1])
            return [self._register_chamber(handle, ea, eb, A, sign=1.0) for ea, eb, A in sorted(holes, key=lowest)]
        mask = self._bodies[handle]["mask"]
        lab, ids = _act.enclosed_voids(mask)
        ids = [k for k in ids if (lab == k).sum() >= min_pixels]
        ids.sort(key=lambda k: tuple(np.argwhere(lab == k)[0]))
        return [self._add_chamber(handle, lab, k) for k in ids]

    def add_pressure_chamber(self, handle, at):
        """Make the sealed cavity holding the world point `at` a pressure chamber (on a mesh
        body: the hole of the mesh that holds it)."""
        self._need_mesh()
        if self._is_mesh(handle):
            rest = np.asarray(self.me.rest_pos, np.float64)
            for ea, eb, A in self._mesh_loops(handle):
                if A > 0 and _act.point_in_loop(at, rest, ea, eb):
                    return self._register_chamber(handle, ea, eb, A, sign=1.0)
            raise ValueError(f"point {tuple(at)} is not inside a hole of this mesh body")
        b = self._bodies[handle]
        mask = b["mask"]
        px = _act.pixel_of(at, b["size"], b["center"], mask.shape)
        if px is None or mask[px] > 0:
            raise ValueError(f"point {tuple(at)} is not inside a void of this body")
        lab, ids = _act.enclosed_voids(mask)
        if lab[px] not in ids:
            raise ValueError(f"the void at {tuple(at)} is open to the outside, not a sealed cavity")
        return self._add_chamber(handle, lab, int(lab[px]))

    def add_ambient_pressure(self, handle):
        """A pressure on a body's outer surface (its outline, including channels open to the
        outside); positive squeezes the body. Returns a handle used with set_pressure. On a
        mesh body: every boundary loop of the mesh that is not a hole."""
        self._need_mesh()
        if self._is_mesh(handle):
            out = [lp for lp in self._mesh_loops(handle) if lp[2] < 0]
            return self._register_chamber(handle, np.concatenate([lp[0] for lp in out]),
                                          np.concatenate([lp[1] for lp in out]), -sum(lp[2] for lp in out),
                                          sign=-1.0)
        mask = self._bodies[handle]["mask"]
        lab, ids = _act.enclosed_voids(mask)
        ea, eb = _act.exterior_edges(mask, lab, ids, self._node_of(handle))
        n_px = int((mask > 0).sum() + sum((lab == k).sum() for k in ids))
        pw, ph = self.pixel_size(handle)
        return self._register_chamber(handle, ea, eb, n_px * pw * ph, sign=-1.0)

    def _add_chamber(self, handle, lab, label):
        ea, eb = _act.chamber_edges(self._bodies[handle]["mask"], lab, label, self._node_of(handle))
        pw, ph = self.pixel_size(handle)
        return self._register_chamber(handle, ea, eb, int((lab == label).sum()) * pw * ph, sign=1.0)

    def _mesh_loops(self, handle):
        """A mesh body's boundary loops in global node ids, fluid on the left:
        [(ea, eb, signed area)], holes > 0, outline < 0 (sim_model.py:881-894). Checked: the
        outline encloses exactly the material and the holes."""
        nodes = self._node_range[handle]
        s0 = int(nodes[0])
        tri = np.asarray(self.me.tri)[self._tri_range[handle]] - s0
        rest = np.asarray(self.me.rest_pos, np.float64)[nodes]
        loops = [(ea + s0, eb + s0, A) for ea, eb, A in _act.mesh_boundary_loops(tri, rest)]
        outline = -sum(A for _, _, A in loops if A < 0)
        inside = self.element_areas(handle).sum() + sum(A for _, _, A in loops if A > 0)
        if abs(outline - inside) > 1e-9 * outline:
            raise RuntimeError(f"mesh body {handle}: its outline encloses {outline:.9e} m^2, its "
                               f"material and holes {inside:.9e}")
        return loops

    def _register_chamber(self, handle, ea, eb, expect, sign):
        """sign +1: edges counter-clockwise round a cavity; -1: clockwise round the body. The
        edges must enclose `expect` m^2 (the closure and orientation check)."""
        rest = self.me.rest_pos
        ref = rest[np.concatenate([ea, eb])].mean(0)
        got = sign * _act.loop_area(rest, ea, eb, ref)
        if not expect > 0 or abs(got - expect) > 1e-6 * expect:
            raise RuntimeError(f"pressure boundary encloses {got:.6e} m^2, expected {expect:.6e}")
        self._chambers.append(dict(body=handle, ea=np.asarray(ea, np.int64), eb=np.asarray(eb, np.int64),
                                   ref=np.asarray(ref, np.float64), area0=float(expect), sign=sign,
                                   pressure=0.0))
        self._act_version += 1
        return len(self._chambers) - 1

    def set_pressure(self, chamber, pressure):
        """Gauge pressure of the fluid in a chamber [Pa]. Positive inflates a cavity (and
        squeezes a body through an ambient-pressure handle)."""
        self._chambers[chamber]["pressure"] = float(pressure)
        self._ctrl_version += 1

    def chamber_area(self, chamber):
        """Current area inside a pressure boundary [m^2]: a cavity's volume per unit depth; for
        an ambient-pressure handle, the area inside the body's outline."""
        c = self._chambers[chamber]
        return c["sign"] * _act.loop_area(self.get_x(), c["ea"], c["eb"], c["ref"])

    # ---- springs, pins and joints (sim_model.py:988-1066)
    def _nearest(self, handle, point):
        ids = self._node_range[handle]
        d = np.linalg.norm(self.me.rest_pos[ids] - np.asarray(point, np.float64)[None, :], axis=1)
        return int(ids[d.argmin()])

    def add_spring(self, handle_a, point_a, handle_b=None, point_b=None, stiffness=None, rest_length=None):
        """A linear spring from a point of one body to a point of another, or with
        handle_b=None to a point fixed in the world (point_b, default where point_a snapped
        to). Ends snap to the nearest node of their body. stiffness k [Pa] (default
        model.rigid_young); rest_length None keeps the built length. Returns a handle."""
        self._need_mesh()
        ia = self._nearest(handle_a, point_a)
        if handle_b is None:
            ib = -1
            anchor = np.asarray(self.me.rest_pos[ia] if point_b is None else point_b, np.float64)
        else:
            ib = self._nearest(handle_b, point_a if point_b is None else point_b)
            if self.body_env(handle_a) != self.body_env(handle_b):
                raise ValueError("a spring cannot join bodies of different environments")
            if ib == ia:
                raise ValueError("both ends of the spring snapped to the same node")
            anchor = np.asarray(self.me.rest_pos[ib], np.float64)
        L = float(np.linalg.norm(self.me.rest_pos[ia] - anchor)) if rest_length is None else float(rest_length)
        if handle_b is not None and L <= 0.0:
            raise ValueError("a spring between two bodies needs a rest length: at zero it would "
                             "pull two nodes to one place while contact holds the bodies apart")
        k = float(self.rigid_young if stiffness is None else stiffness)
        if k <= 0 or L < 0:
            raise ValueError("spring stiffness must be positive and its rest length non-negative")
        self._springs.append(dict(a=int(ia), b=int(ib), stiffness=k, length=L, anchor=anchor,
                                  env=self.body_env(handle_a)))
        self._act_version += 1
        return len(self._springs) - 1

    def add_pin(self, handle, point, handle_b=None, stiffness=None):
        """Pin a point of a body to the world where it is (a zero-length stiff spring): the
        body can still turn about it."""
        if handle_b is not None:
            raise NotImplementedError(
                "a pin between two bodies is not supported: it would hold two nodes at one "
                "place while contact holds the bodies apart. Pin to the world (leave handle_b "
                "out), or use add_spring with a rest length.")
        return self.add_spring(handle, point, None, point, stiffness, rest_length=0.0)

    def set_spring_length(self, spring, length):
        """Rest length of a spring [m] (drive it for a linear actuator)."""
        self._springs[spring]["length"] = float(length)
        self._ctrl_version += 1

    def set_spring_anchor(self, spring, point):
        """Move the world end of a world spring or pin."""
        if self._springs[spring]["b"] >= 0:
            raise ValueError("this spring joins two bodies and has no world anchor")
        self._springs[spring]["anchor"] = np.asarray(point, np.float64)
        self._ctrl_version += 1

    def spring_force(self, spring):
        """(tension [N/m], negative in compression; current length [m]) of a spring."""
        sp = self._springs[spring]
        x = self.get_x()
        ln = float(np.linalg.norm(x[sp["a"]] - (x[sp["b"]] if sp["b"] >= 0 else sp["anchor"])))
        return sp["stiffness"] * (ln - sp["length"]), ln

    # ---- active material (sim_model.py:1068-1096)
    def add_active_region(self, handle, region, fiber=None):
        """Mark part of a body ((H, W) boolean map laid out like its mask) as actively
        deforming material; fiber None for isotropic change, else an angle [rad] or a
        2-vector along which `stretch` acts. Returns a handle."""
        self._need_mesh()
        elems = self._region_elements(handle, region)
        mine = self._regions_of.setdefault(handle, [])
        if mine and np.intersect1d(elems, np.concatenate(mine)).size:
            raise ValueError("active regions must not overlap")
        mine.append(np.asarray(elems, np.int64))
        self._regions.append(dict(body=handle, elems=np.asarray(elems, np.int64), fiber=fiber, A=np.eye(2)))
        self._act_version += 1
        return len(self._regions) - 1

    def set_activation(self, region, stretch, transverse=1.0):
        """Rest-length ratio of an active region: 1 passive, 0.9 a 10 % contraction; along
        the fiber with `transverse` across it, or isotropic without a fiber."""
        if stretch <= 0 or transverse <= 0:
            raise ValueError("stretch ratios must be positive")
        r = self._regions[region]
        r["A"] = _act.activation_matrix(stretch, transverse, r["fiber"])
        self._ctrl_version += 1

    def affine_state(self, index):
        s = self._solver
        if s is None:
            a = self._affine[index]
            m = np.asarray(self.me.mass)[a["nodes"]]
            c = (m[:, None] * self.me.rest_pos[a["nodes"]]).sum(0) / m.sum()
            return dict(position=c, angle=0.0, A=np.eye(2))
        q = s.get_affine_q()[index]
        A = np.array([[q[1], q[2]], [q[4], q[5]]])
        return dict(position=np.array([q[0], q[3]]), angle=float(np.arctan2(A[1, 0] - A[0, 1], A[0, 0] + A[1, 1])), A=A)
