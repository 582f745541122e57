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

Bodies are pixel masks (row 0 at the bottom) rasterised into P1 triangles, or triangle
meshes; every body lives in an environment (`env_id`), environments never interact and are
solved together. This class only records what the user declares (typed records of
parts.py) and assembles host arrays; the step itself runs on the GPU (integrator.py).

Beyond the reference, keyword-only: a per-environment collider friction
(`set_collider_mu`), which the reference cannot express (its colliders carry one mu for
every environment, implicit/solver.py:235-242).
"""
from __future__ import annotations

import hashlib
import warnings
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import actuators as _act
from . import mesh as _mesh
from . import parts as _parts
from .parts import (NONE, DISC, ELLIPSE, BOX, TRIANGLE, HALFSPACE, Collider, ColliderSpec, Body, Chamber,
                    Tendon, ActiveRegion, RigidPiece, Spring)

NAMES = _parts.SHAPE_CODES


@dataclass
class SimConfig:
    """Material defaults, damping and contact parameters (reference core/config.py:13-29).
    A parameter left at None is scaled to the scene at finalize()."""
    young: float = 1.0e6
    nu: float = 0.40
    rho_mass: float = 1000.0
    damping: float = 0.0
    ipc_d_hat: Optional[float] = None
    obstacle_stiffness: Optional[float] = None
    contact_stiffness: Optional[float] = None
    obstacle_friction: float = 0.5
    obstacle_friction_epsv: float = 1.0e-3


def _config_property(attr):
    return property(lambda self: getattr(self.cfg, attr), lambda self, v: setattr(self.cfg, attr, v))


class Model:
    # contact and material parameters, stored on the config (sim_model.py:118-127)
    dhat = _config_property("ipc_d_hat")
    kappa = _config_property("obstacle_stiffness")
    self_stiffness = _config_property("contact_stiffness")
    mu = _config_property("obstacle_friction")
    epsv = _config_property("obstacle_friction_epsv")
    damping = _config_property("damping")

    def __init__(self, device="cuda", config=None):
        self.cfg = config if config is not None else SimConfig()
        self.device = device
        self.me = None                 # the assembled scene (mesh.Mesh), from finalize()
        self.time = 0.0
        # contact between bodies: the IPC barrier; Coulomb coefficient and stiffness
        self.body_contact = "ipc"
        self.body_friction = 0.0
        self.body_kappa = None
        # stiffness a rigid (affine) piece resists strain with
        self.rigid_young = 1.0e9
        self.rigid_nu = 0.30
        # declarations
        self._bodies: list[Body] = []
        self._colliders: list[ColliderSpec] = []
        self._col_mu_env: dict = {}
        self._chambers: list[Chamber] = []
        self._tendons: list[Tendon] = []
        self._regions: list[ActiveRegion] = []
        self._affine: list[RigidPiece] = []
        self._springs: list[Spring] = []
        self._mesh_info: dict = {}
        # per-body element sets already claimed by rigid pieces / active regions
        self._claimed = {"rigid": {}, "active": {}}
        self._extra_excl: list = []    # (first boundary slot of the env, env-local slots) of rigid pieces
        # layout and state, from finalize()
        self._node_range: list = []
        self._tri_range: list = []
        self._constrained: dict = {}   # body -> global node ids under kinematic control
        self._targets = None           # (N, 2) kinematic targets
        self._x_host = None            # (N, 2) positions while no solver holds them
        self._v0 = None                # (N, 2) velocities while no solver holds them
        self._gravity = (0.0, 0.0)
        self._fext = None              # (N, 2) nodal force besides gravity
        self._solver = None            # bound by the integrator at the first step
        self._epoch = 0
        self._act_version = 0          # bumped when an actuator is added: the solver is rebuilt
        self._ctrl_version = 0         # bumped when a command changes: values are pushed

    # =========================================================================== colliders
    # (sim_model.py:133-184)
    def add_ground(self, height=0.0, mu=None):
        return self.add_plane((0.0, 1.0), (0.0, height), mu=mu)

    def add_plane(self, normal, origin, mu=None):
        n = np.asarray(normal, np.float64)
        length = np.linalg.norm(n)
        if not length > 0:
            raise ValueError("the plane normal must be non-zero")
        unit = n / length
        return self._new_collider(HALFSPACE, origin, float(unit[0]), float(unit[1]), 0.0, mu)

    def add_disc(self, center, radius, mu=None):
        return self.add_object("disc", center, radius, mu=mu)

    def add_object(self, kind, center, rx, ry=None, corner_radius=3.0e-3, mu=None):
        code = NAMES[kind] if isinstance(kind, str) else int(kind)
        rx = float(rx)
        ry = float(rx if ry is None else ry)
        rref = float(corner_radius) if code in (BOX, TRIANGLE) else rx
        return self._new_collider(code, center, rx, ry, rref, mu)

    def _new_collider(self, kind, center, rx, ry, rref, mu):
        if self._solver is not None:
            raise RuntimeError("add colliders before the first simulate()")
        self._colliders.append(ColliderSpec(kind=int(kind), cx=float(center[0]), cy=float(center[1]), rx=rx, ry=ry,
                                            rref=rref, mu=float(self.cfg.obstacle_friction if mu is None else mu)))
        return len(self._colliders) - 1

    def set_collider_center(self, index, center):
        """Move a collider (sim_model.py:176-184). Before the first step this places it;
        during a rollout it TELEPORTS the shape between steps — the move is not swept, so keep
        each step's displacement well under the current clearance, and friction treats the
        collider as stationary."""
        c = self._colliders[index]
        c.cx, c.cy = float(center[0]), float(center[1])
        if self._solver is not None:
            self._solver.set_collider_centers([[k.cx, k.cy] for k in self._colliders])

    @property
    def colliders(self):
        """Every collider as a host-side Collider record (kind, cx, cy, rx, ry, rref)."""
        return [c.public() for c in self._colliders]

    @property
    def object(self):
        """The first collider (kind NONE when the scene has none)."""
        return self._colliders[0].public() if self._colliders else Collider(kind=NONE)

    def set_collider_mu(self, index, mu_per_env):
        """Per-environment Coulomb coefficient of collider `index` ((n_envs,) array). New
        in this implementation: the reference has one mu per collider for every
        environment."""
        if self._solver is not None:
            raise RuntimeError("set per-environment friction before the first simulate()")
        self._col_mu_env[int(index)] = np.array(mu_per_env, np.float64)

    # =========================================================================== bodies
    # (sim_model.py:199-338)
    def _declare(self, body: Body) -> int:
        if self.me is not None:
            raise RuntimeError("add bodies before finalize()")
        self._bodies.append(body)
        return len(self._bodies) - 1

    def _defaults(self, E, nu, density):
        c = self.cfg
        return (c.young if E is None else E, float(c.nu if nu is None else nu),
                float(c.rho_mass if density is None else density))

    def add_soft_body(self, mask, physical_size, center, E=None, nu=None, density=None, env_id=0, mu=None):
        return self._pixel_body(mask, physical_size, center, E, nu, density, env_id, mu, "soft")

    def add_affine_body(self, mask, physical_size, center, density=None, env_id=0, E=None, nu=None, mu=None):
        E = self.rigid_young if E is None else E
        nu = self.rigid_nu if nu is None else nu
        return self._pixel_body(mask, physical_size, center, E, nu, density, env_id, mu, "affine")

    def add_kinematic_body(self, mask, physical_size, center, env_id=0, mu=None):
        return self._pixel_body(mask, physical_size, center, None, None, None, env_id, mu, "kinematic")

    def _pixel_body(self, mask, physical_size, center, E, nu, density, env_id, mu, role):
        if self.me is not None:
            raise RuntimeError("add bodies before finalize()")
        m = _parts.solid_mask(mask)
        field = _parts.stiffness_field(E, m.shape, per_triangle=False, solid=m)
        env = _parts.env_index(env_id)
        mu = _parts.friction_coefficient(mu)
        if role == "affine" and field is not None and not np.isscalar(field):
            raise ValueError("a rigid body takes a scalar stiffness")
        E, nu, rho = self._defaults(field, nu, density)
        return self._declare(Body(env=env, E=E if not np.isscalar(E) else float(E), nu=nu, rho=rho, mu=mu,
                                  center=(float(center[0]), float(center[1])), role=role, mask=m,
                                  size=(float(physical_size[0]), float(physical_size[1]))))

    def add_soft_mesh(self, vertices, triangles, E=None, nu=None, density=None, env_id=0, mu=None):
        """A soft body given as a triangle mesh: vertices (n, 2) at rest [m], triangles (m, 3)
        0-based, either winding. Vertex i is node i of the body and triangle j its element j,
        so node- and element-addressed calls use the mesh's own numbering; per-pixel inputs
        become per-triangle arrays (E of shape (m,), regions as (m,) booleans or triangle
        indices) and a hole in the mesh is a pressure chamber. The mesh is validated first
        (mesh.check_mesh). Returns a handle."""
        return self._mesh_body(vertices, triangles, E, nu, density, env_id, mu, "soft")

    def add_affine_mesh(self, vertices, triangles, density=None, env_id=0, E=None, nu=None, mu=None):
        """A rigid (affine) body given as a triangle mesh. Returns a handle."""
        E = self.rigid_young if E is None else E
        nu = self.rigid_nu if nu is None else nu
        return self._mesh_body(vertices, triangles, E, nu, density, env_id, mu, "affine")

    def add_kinematic_mesh(self, vertices, triangles, env_id=0, mu=None):
        """A body of prescribed motion given as a triangle mesh. Returns a handle."""
        return self._mesh_body(vertices, triangles, None, None, None, env_id, mu, "kinematic")

    def _mesh_body(self, vertices, triangles, E, nu, density, env_id, mu, role):
        if self.me is not None:
            raise RuntimeError("add bodies before finalize()")
        info = self._measured_mesh(vertices, triangles)
        V, T = info["vertices"], info["triangles"]
        field = _parts.stiffness_field(E, (len(T),), per_triangle=True)
        env = _parts.env_index(env_id)
        mu = _parts.friction_coefficient(mu)
        if role == "affine" and field is not None and not np.isscalar(field):
            raise ValueError("a rigid body takes a scalar stiffness")
        E, nu, rho = self._defaults(field, nu, density)
        mid = 0.5 * (V.min(0) + V.max(0))
        return self._declare(Body(env=env, E=E if not np.isscalar(E) else float(E), nu=nu, rho=rho, mu=mu,
                                  center=(float(mid[0]), float(mid[1])), role=role, vertices=V, triangles=T,
                                  h=info["h"], h_cfl=info["h_cfl"], L_max=info["L_max"]))

    def _measured_mesh(self, vertices, triangles):
        """mesh.check_mesh of a mesh, once per distinct mesh (a batch repeats one), with a
        warning when its element sizes spread over more than a decade."""
        V = np.ascontiguousarray(vertices, np.float64)
        T = np.ascontiguousarray(triangles)
        digest = hashlib.sha1(V.tobytes() + T.tobytes()).hexdigest()
        key = (V.shape, T.shape, str(T.dtype), digest)
        info = self._mesh_info.get(key)
        if info is None:
            info = _mesh.check_mesh(V, T)
            side = np.sqrt(2.0 * info["area"])
            if side.max() > 10.0 * side.min():
                warnings.warn(f"this mesh's elements range from {side.min() * 1e3:.3g} to "
                              f"{side.max() * 1e3:.3g} mm; the iterations a step needs follow the "
                              f"smallest element, so a few small ones make every step dearer.",
                              stacklevel=4)
            self._mesh_info[key] = info
        return info

    def _is_mesh(self, handle):
        return self._bodies[handle].is_mesh

    def _need_pixels(self, handle, what):
        if self._is_mesh(handle):
            raise ValueError(f"body {handle} is a mesh body: {what} needs a pixel body. A mesh body "
                             f"takes per-triangle arrays instead.")

    # =========================================================================== finalize
    # (sim_model.py:391-429)
    def finalize(self):
        if not self._bodies:
            raise ValueError("add at least one soft body before finalize()")
        # a mesh body's boundary pairs closer than this THROUGH THE MATERIAL are left out of
        # its self-contact (sim_model.py:396-399)
        dx = self.dx
        dhat0 = self.cfg.ipc_d_hat if self.cfg.ipc_d_hat is not None else dx / 8.0
        r_excl = max(2.0 * dx, 16.0 * dhat0)
        specs = []
        for b in self._bodies:
            spec = dict(young=float(b.E) if b.uniform else 1.0, nu=b.nu, rho=b.rho, env=b.env)
            if b.is_mesh:
                spec.update(vertices=b.vertices, triangles=b.triangles, excl_radius=r_excl, checked=True)
            else:
                spec.update(mask_xy=b.mask.T.copy(), size=b.size, center=b.center)
            specs.append(spec)
        me = self.me = _mesh.build_scene(specs)
        self._node_range = [np.arange(lo, hi) for lo, hi in me.body_node_range]
        self._tri_range = [np.arange(lo, hi) for lo, hi in me.body_tri_range]
        for h, b in enumerate(self._bodies):      # stiffness fields scale the moduli per element
            if not b.uniform:
                scale = b.E if b.is_mesh else self._pixel_field(h, b.E)
                el = self._tri_range[h]
                me.mu[el] *= scale
                me.lam[el] *= scale
        self._check_layout()
        self._scale_contact()
        rest = np.asarray(me.rest_pos, np.float64)
        self._targets, self._x_host, self._v0 = rest.copy(), rest.copy(), np.zeros_like(rest)
        for h, b in enumerate(self._bodies):
            if b.role == "affine":
                self._add_affine(h, self._tri_range[h])
            elif b.role == "kinematic":
                self._constrained[h] = self._node_range[h].copy()
        return self

    def _pixel_field(self, h, field):
        """A body's (H, W) pixel field on its elements (body_elements order)."""
        quad = np.asarray(self.me.tri_quad)[self._tri_range[h]]
        H = self._bodies[h].mask.shape[0]
        return np.asarray(field, np.float64)[quad % H, quad // H]

    def _scale_contact(self):
        """The contact parameters left unset, from the scene's scales (sim_model.py:487-497):
        E of the softest soft body and the element size dx."""
        c = self.cfg
        E = min((b.min_E() for b in self._bodies if b.is_soft), default=1.0e6)
        dx = self.dx
        if c.ipc_d_hat is None:
            c.ipc_d_hat = dx / 8.0
        if c.obstacle_stiffness is None:
            c.obstacle_stiffness = 4.0e-3 * E * dx / c.ipc_d_hat
        if c.contact_stiffness is None:
            c.contact_stiffness = 0.2 * E
        if self.body_kappa is None:
            self.body_kappa = 0.1 * E * dx / c.ipc_d_hat

    def _check_layout(self):
        """Bodies of one environment must start apart (sim_model.py:499-535); warns when an
        environment mixes element sizes (contact between bodies has one thickness)."""
        by_env: dict = {}
        for h, b in enumerate(self._bodies):
            by_env.setdefault(b.env, []).append(h)
        seen: dict = {}
        for env, hs in by_env.items():
            for i in range(len(hs)):
                for j in range(i + 1, len(hs)):
                    if self._bodies_overlap(hs[i], hs[j], seen):
                        raise ValueError(
                            f"bodies {hs[i]} and {hs[j]} overlap in environment {env}. Bodies of one "
                            f"environment collide with each other and must start apart; give "
                            f"the members of a batch their own environment with env_id=i.")
            meshes = any(self._bodies[h].is_mesh for h in hs)
            sizes = [self.element_size(h) if meshes else self.pixel_size(h)[0] for h in hs]
            if max(sizes) > 1.25 * min(sizes):
                lo, hi = min(sizes) * 1e3, max(sizes) * 1e3
                if meshes:
                    warnings.warn(f"environment {env} mixes element sizes (pixel width, or a mesh body's "
                                  f"median boundary edge) from {lo:.3g} to {hi:.3g} "
                                  f"mm. Contact between bodies has ONE thickness, set by the largest.",
                                  stacklevel=3)
                else:
                    warnings.warn(f"environment {env} mixes pixel sizes from {lo:.3g} to "
                                  f"{hi:.3g} mm. Contact between bodies has ONE thickness, "
                                  f"set by the largest. Prefer one pixel size per scene.", stacklevel=3)

    def _bodies_overlap(self, a, c, memo):
        A, C = self._bodies[a], self._bodies[c]
        if not (A.is_mesh or C.is_mesh):
            return _parts.cells_covered(A, C) or _parts.cells_covered(C, A)
        key = (A.geometry_key(), C.geometry_key())
        if key not in memo:
            memo[key] = _mesh.meshes_overlap(*self._body_geometry(a), *self._body_geometry(c))
        return memo[key]

    def _body_geometry(self, h):
        """A body's rest mesh in its own numbering: (nodes (n, 2), triangles (m, 3))."""
        lo, hi = self.me.body_node_range[h]
        tri = np.asarray(self.me.tri)[self._tri_range[h]] - lo
        return np.asarray(self.me.rest_pos[lo:hi], np.float64), tri

    # =========================================================================== rigid pieces
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
        mu, lam = _mesh.lame(self.rigid_young if E is None else float(E), self.rigid_nu if nu is None else float(nu))
        self.me.mu[elems] = mu
        self.me.lam[elems] = lam
        return self._add_affine(handle, elems)

    def _region_elements(self, handle, region):
        """Global element ids of part of a body (sim_model.py:1103-1132): the solid pixels of
        an (H, W) map laid out like a pixel body's mask; for a mesh body (m,) booleans or
        distinct triangle indices."""
        b = self._bodies[handle]
        tris = self._tri_range[handle]
        if not b.is_mesh:
            sel = np.asarray(region) > 0
            if sel.shape != b.mask.shape:
                raise ValueError(f"region is {sel.shape}, the mask is {b.mask.shape}")
            picked = tris[self._pixel_field(handle, sel) > 0]
            if not len(picked):
                raise ValueError("the region contains no solid pixel of this body")
            return picked
        m = len(tris)
        r = np.asarray(region)
        if r.dtype == bool:
            if r.shape != (m,):
                raise ValueError(f"region is a boolean array of shape {r.shape}; mesh body {handle} "
                                 f"has {m} triangles: give ({m},) booleans or triangle indices")
            local = np.flatnonzero(r)
        elif r.ndim == 1 and np.issubdtype(r.dtype, np.integer):
            local = np.unique(r)
            if len(local) != len(r) or (len(local) and not (0 <= local[0] and local[-1] < m)):
                raise ValueError(f"triangle indices must be distinct and in 0..{m - 1}")
        else:
            raise ValueError(f"region of a mesh body: ({m},) booleans or a 1-D array of triangle "
                             f"indices; got {r.dtype} of shape {r.shape}")
        if not len(local):
            raise ValueError("the region contains no triangle of this body")
        return tris[local]

    def _claim(self, kind, handle, elems, what):
        """Elements taken by a rigid piece or an active region; pieces of one kind may not
        share an element."""
        taken = self._claimed[kind].setdefault(handle, np.zeros(0, np.int64))
        if np.intersect1d(elems, taken).size:
            raise ValueError(f"{what} must not overlap")
        self._claimed[kind][handle] = np.union1d(taken, elems)

    def _add_affine(self, handle, elems):
        elems = np.asarray(elems, np.int64)
        self._claim("rigid", handle, elems, "rigid regions")
        me = self.me
        nodes = np.unique(np.asarray(me.tri)[elems])
        # the boundary nodes of one rigid piece never move relative to each other: no
        # contact between any two of them (sim_model.py:466-476)
        env = self._bodies[handle].env
        first, last = int(me.boundary_starts[env]), int(me.boundary_starts[env + 1])
        slots = np.flatnonzero(np.isin(me.boundary_nodes[first:last], nodes))
        self._extra_excl.append((first, slots))
        self._affine.append(RigidPiece(body=handle, elems=elems, nodes=nodes))
        return len(self._affine) - 1

    def exclusion_csr(self):
        """The scene's self-contact exclusion (mesh hops + rigid pieces) as a CSR over the
        boundary slots, columns environment-local and sorted."""
        ptr, idx = self.me.excl_ptr, self.me.excl_idx
        if not self._extra_excl:
            return ptr, idx
        n = len(ptr) - 1
        rows = [np.repeat(np.arange(n), np.diff(ptr))]
        cols = [np.asarray(idx, np.int64)]
        for first, slots in self._extra_excl:
            rows.append(np.repeat(first + slots, len(slots)))
            cols.append(np.tile(slots, len(slots)))
        r, c = np.concatenate(rows), np.concatenate(cols)
        key = np.unique(r * (int(c.max(initial=0)) + 1) + c)
        width = int(c.max(initial=0)) + 1
        r, c = key // width, key % width
        new_ptr = np.zeros(n + 1, np.int64)
        np.add.at(new_ptr, r + 1, 1)
        return np.cumsum(new_ptr), c.astype(np.int64)

    # =========================================================================== layout queries
    # (sim_model.py:572-700)
    @property
    def n_bodies(self):
        return len(self._bodies)

    @property
    def n_envs(self):
        if self.me is not None:
            return int(self.me.n_envs)
        return 1 + max((b.env for b in self._bodies), default=-1)

    @property
    def n_nodes(self):
        return int(self.me.rest_pos.shape[0])

    @property
    def n_elements(self):
        return int(self.me.tri.shape[0])

    def body_env(self, handle):
        return self._bodies[handle].env

    def body_nodes(self, handle):
        return self._node_range[handle].copy()

    def body_elements(self, handle):
        return self._tri_range[handle].copy()

    def pixel_size(self, handle):
        """(width, height) of one pixel of a body [m]; a mesh body has none."""
        b = self._bodies[handle]
        if b.is_mesh:
            raise ValueError(f"body {handle} is a mesh body: it has no pixels. Its length scale is "
                             f"element_size({handle}).")
        rows, cols = b.mask.shape
        return b.size[0] / cols, b.size[1] / rows

    def element_size(self, handle):
        """A body's contact length scale [m]: its pixel width, or a mesh body's median
        boundary-edge length."""
        b = self._bodies[handle]
        return float(b.h) if b.is_mesh else self.pixel_size(handle)[0]

    def _cfl_length(self, handle):
        """The element size a wave crosses per element: the smaller pixel side, or a mesh
        body's smallest sqrt(2 x triangle area)."""
        b = self._bodies[handle]
        return float(b.h_cfl) if b.is_mesh else min(self.pixel_size(handle))

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
        want = (len(self._tri_range[handle]),) if b.is_mesh else b.mask.shape
        if field.shape != want:
            if b.is_mesh:
                raise ValueError(f"field is {field.shape}; mesh body {handle} has {want[0]} triangles")
            raise ValueError(f"field is {field.shape}, the mask is {want}")
        return field.copy() if b.is_mesh else self._pixel_field(handle, field)

    def to_pixels(self, handle, values):
        self._need_pixels(handle, "to_pixels")
        H, W = self._bodies[handle].mask.shape
        quad = np.asarray(self.me.tri_quad)[self._tri_range[handle]]
        return np.bincount(quad, weights=np.asarray(values, np.float64), minlength=H * W).reshape(W, H).T.copy()

    # =========================================================================== read-outs
    # (sim_model.py:625-642, core/fields.py), computed on the GPU
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
        bufs = getattr(self, "_field_bufs", None)
        if bufs is None:
            me = self.me
            put = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
            bufs = self._field_bufs = dict(
                tri=put(me.tri, torch.int32), Bm=put(np.asarray(me.D_m_inv, np.float64).reshape(-1, 4), torch.float64),
                mu=put(me.mu, torch.float64), lam=put(me.lam, torch.float64))
        n = int(bufs["tri"].shape[0])
        xx = torch.as_tensor(np.asarray(self.get_x() if x is None else x, np.float64), device=dev).contiguous()
        out = torch.empty(n, dtype=torch.float64, device=dev)
        which = ["strain", "stress"].index(field) * 2 + int(bool(signed))   # output slot of d2f_element_fields
        slots = [None] * 4
        slots[which] = out.data_ptr()
        _lib.check(L.d2f_element_fields(n, bufs["tri"].data_ptr(), bufs["Bm"].data_ptr(), bufs["mu"].data_ptr(),
                                        bufs["lam"].data_ptr(), xx.data_ptr(), *slots,
                                        torch.cuda.current_stream(dev).cuda_stream), "d2f_element_fields")
        v = out.cpu().numpy()
        return v if handle is None else v[self._tri_range[handle]]

    def rigid_motion(self, handle, translation=(0.0, 0.0), angle=0.0, about=None):
        """A body's rest nodes turned by `angle` about `about` (default its centre) and moved
        by `translation`."""
        pivot = np.asarray(self._bodies[handle].center if about is None else about, np.float64)
        c, s = np.cos(angle), np.sin(angle)
        rot = np.array([[c, -s], [s, c]])
        return (self.rest_x(handle) - pivot) @ rot.T + pivot + np.asarray(translation, np.float64)

    # =========================================================================== kinematic bodies
    # (sim_model.py:384-388, 686-692)
    def set_kinematic_constraint(self, handle, node_indices):
        self._constrained[handle] = self._node_range[handle][np.asarray(node_indices, int)]

    def set_kinematic_target(self, handle, targets):
        self._targets[self._node_range[handle]] = np.asarray(targets, np.float64)

    def set_kinematic_pose(self, handle, translation=(0.0, 0.0), angle=0.0, about=None):
        self.set_kinematic_target(handle, self.rigid_motion(handle, translation, angle, about))

    def all_constrained(self):
        held = [np.asarray(v, np.int64) for v in self._constrained.values()]
        return np.unique(np.concatenate(held)) if held else np.zeros(0, np.int64)

    # =========================================================================== state I/O
    # (sim_model.py:694-796)
    def get_x(self):
        if self._solver is not None:
            self._x_host = self._solver.get_x()
        return self._x_host.copy()

    def get_body_x(self, handle):
        return self.get_x()[self._node_range[handle]]

    def get_body_v(self, handle):
        v = self._v0 if self._solver is None else self._solver.get_v()
        return np.array(v)[self._node_range[handle]]

    def set_body_velocity(self, handle, velocity=(0.0, 0.0), omega=0.0, about=None):
        ids = self._node_range[handle]
        pos = self.get_x()[ids]
        pivot = pos.mean(0) if about is None else np.asarray(about, np.float64)
        arm = pos - pivot
        v = np.asarray(velocity, np.float64) + omega * np.c_[-arm[:, 1], arm[:, 0]]
        self._v0[ids] = v
        if self._solver is not None:
            self._solver.set_nodes(ids, v=v)

    def set_body_x(self, handle, x, v=None):
        ids = self._node_range[handle]
        x = np.asarray(x, np.float64).reshape(len(ids), 2)
        self._x_host[ids] = x
        self._targets[ids] = x
        if v is not None:
            self._v0[ids] = np.asarray(v, np.float64).reshape(len(ids), 2)
        s = self._solver
        if s is not None:
            s.set_nodes(ids, x=x, v=None if v is None else self._v0[ids], xn=True)
            s.sync_affine([k for k, piece in enumerate(self._affine) if piece.body == handle])

    def set_body_pose(self, handle, translation=(0.0, 0.0), angle=0.0, about=None, velocity=(0.0, 0.0), omega=0.0):
        self.set_body_x(handle, self.rigid_motion(handle, translation, angle, about))
        self.set_body_velocity(handle, velocity, omega)

    def reset(self, env_ids=None):
        """Back to rest at zero velocity, kinematic targets included (sim_model.py:761-796)."""
        rest = self.me.rest_pos.astype(np.float64)
        self._epoch += 1
        if env_ids is None:
            self._targets, self._x_host, self._v0 = rest.copy(), rest.copy(), np.zeros_like(rest)
            self.time = 0.0
            if self._solver is not None:
                self._solver.reset_envs(None)
            return
        pick = np.zeros(self.n_envs, np.int32)
        pick[np.atleast_1d(env_ids)] = 1
        back = pick[np.asarray(self.me.node2env)] > 0
        self._targets[back] = rest[back]
        self._x_host[back] = rest[back]
        self._v0[back] = 0.0
        if self._solver is not None:
            self._solver.reset_envs(pick)

    # =========================================================================== actuation
    # (sim_model.py:806-1096)
    def _need_mesh(self):
        if self.me is None:
            raise RuntimeError("call finalize() before adding actuators")

    def _added(self, records, item):
        records.append(item)
        self._act_version += 1
        return len(records) - 1

    def _commanded(self):
        self._ctrl_version += 1

    @property
    def gravity(self):
        return self._gravity

    @gravity.setter
    def gravity(self, g):
        self._gravity = (float(g[0]), float(g[1]))
        self._commanded()

    def set_external_force(self, handle, force):
        """Nodal forces on a body, (n_body_nodes, 2) [N/m], held until changed."""
        self._need_mesh()
        if self._fext is None:
            self._fext = np.zeros((self.n_nodes, 2), np.float64)
        self._fext[self._node_range[handle]] = np.asarray(force, np.float64)
        self._commanded()

    # ---- tendons
    def add_tendon(self, handle, through=None, nodes=None, stiffness=None):
        """Thread a cable through a body (sim_model.py:931-958): through world points (each
        snaps to the body's nearest node; repeats collapse) or through node indices of the
        body. stiffness None: tension-controlled; > 0: length-controlled. Returns a handle."""
        self._need_mesh()
        if (through is None) == (nodes is None):
            raise ValueError("give exactly one of `through` (points) or `nodes` (indices)")
        ids = self._node_range[handle]
        if nodes is not None:
            path = ids[np.asarray(nodes, int)]
        else:
            snapped = [self._nearest(handle, p) for p in np.atleast_2d(np.asarray(through, np.float64))]
            path = np.array([n for k, n in enumerate(snapped) if k == 0 or n != snapped[k - 1]], np.int64)
        if len(path) < 2:
            raise ValueError("a tendon needs at least two distinct eyelets")
        if stiffness is not None and stiffness <= 0:
            raise ValueError("stiffness must be positive (or None for a tension-controlled cable)")
        rest_len = _path_length(self.me.rest_pos, path)
        return self._added(self._tendons, Tendon(body=handle, nodes=np.asarray(path, np.int64),
                                                 stiffness=float(stiffness or 0.0), length=rest_len))

    def set_tendon_tension(self, tendon, tension):
        t = self._tendons[tendon]
        if t.stiffness > 0:
            raise ValueError("this tendon is length-controlled; use set_tendon_length")
        t.tension = float(tension)
        self._commanded()

    def set_tendon_length(self, tendon, length):
        t = self._tendons[tendon]
        if t.stiffness <= 0:
            raise ValueError("this tendon is tension-controlled; use set_tendon_tension")
        t.length = float(length)
        self._commanded()

    def tendon_length(self, tendon):
        """Current path length of a cable through its eyelets [m]."""
        return _path_length(self.get_x(), self._tendons[tendon].nodes)

    def tendon_tension(self, tendon):
        """Current tension of a cable [N/m] (zero when a length-controlled cable is slack)."""
        t = self._tendons[tendon]
        if t.stiffness <= 0:
            return max(t.tension, 0.0)
        return t.stiffness * max(self.tendon_length(tendon) - t.length, 0.0)

    # ---- pressure in sealed cavities and on the outside (sim_model.py:825-929)
    def _grid_nodes(self, handle):
        """(ix, iy) grid corner -> global node id (-1 where no node) of a pixel body."""
        me = self.me
        first = int(me.body_node_range[handle][0])
        rows_p1 = int(me.body_grid[handle][1]) + 1
        live = np.asarray(me.grid_to_live_node_per_body[handle])

        def lookup(ix, iy):
            loc = live[np.asarray(ix, np.int64) * rows_p1 + np.asarray(iy, np.int64)]
            return np.where(loc >= 0, loc + first, -1)
        return lookup

    def add_pressure_chambers(self, handle, min_pixels=1):
        """Make every sealed cavity of a body (a void region enclosed by solid, not reaching the
        edge of the pixel grid) a pressure chamber. Returns their handles, ordered by the
        cavity's first pixel, bottom row first then left to right. On a mesh body every hole
        of the mesh is a chamber (min_pixels does not apply), ordered by its lowest node,
        then left to right."""
        self._need_mesh()
        if self._is_mesh(handle):
            rest = self.me.rest_pos
            holes = [lp for lp in self._mesh_loops(handle) if lp[2] > 0]

            def lowest(lp):
                n = lp[0][np.argmin(rest[lp[0], 1])]
                return (rest[n, 1], rest[n, 0])
            return [self._new_chamber(handle, ea, eb, A, +1.0) for ea, eb, A in sorted(holes, key=lowest)]
        labels, sealed = _act.enclosed_voids(self._bodies[handle].mask)
        big = [k for k in sealed if np.count_nonzero(labels == k) >= min_pixels]
        first_px = {k: tuple(np.argwhere(labels == k)[0]) for k in big}
        return [self._cavity(handle, labels, k) for k in sorted(big, key=first_px.get)]

    def add_pressure_chamber(self, handle, at):
        """Make the sealed cavity holding the world point `at` a pressure chamber (on a mesh
        body: the hole of the mesh that holds it)."""
        self._need_mesh()
        if self._is_mesh(handle):
            rest = np.asarray(self.me.rest_pos, np.float64)
            for ea, eb, A in self._mesh_loops(handle):
                if A > 0 and _act.point_in_loop(at, rest, ea, eb):
                    return self._new_chamber(handle, ea, eb, A, +1.0)
            raise ValueError(f"point {tuple(at)} is not inside a hole of this mesh body")
        b = self._bodies[handle]
        px = _act.pixel_of(at, b.size, b.center, b.mask.shape)
        if px is None or b.mask[px] > 0:
            raise ValueError(f"point {tuple(at)} is not inside a void of this body")
        labels, sealed = _act.enclosed_voids(b.mask)
        if labels[px] not in sealed:
            raise ValueError(f"the void at {tuple(at)} is open to the outside, not a sealed cavity")
        return self._cavity(handle, labels, int(labels[px]))

    def add_ambient_pressure(self, handle):
        """A pressure on a body's outer surface (its outline, including channels open to the
        outside); positive squeezes the body. Returns a handle used with set_pressure. On a
        mesh body: every boundary loop of the mesh that is not a hole."""
        self._need_mesh()
        if self._is_mesh(handle):
            outer = [lp for lp in self._mesh_loops(handle) if lp[2] < 0]
            ea = np.concatenate([lp[0] for lp in outer])
            eb = np.concatenate([lp[1] for lp in outer])
            return self._new_chamber(handle, ea, eb, -sum(lp[2] for lp in outer), -1.0)
        mask = self._bodies[handle].mask
        labels, sealed = _act.enclosed_voids(mask)
        ea, eb = _act.exterior_edges(mask, labels, sealed, self._grid_nodes(handle))
        inside_px = np.count_nonzero(mask) + int(np.isin(labels, sealed).sum())
        pw, ph = self.pixel_size(handle)
        return self._new_chamber(handle, ea, eb, inside_px * pw * ph, -1.0)

    def _cavity(self, handle, labels, label):
        mask = self._bodies[handle].mask
        ea, eb = _act.chamber_edges(mask, labels, label, self._grid_nodes(handle))
        pw, ph = self.pixel_size(handle)
        return self._new_chamber(handle, ea, eb, np.count_nonzero(labels == label) * pw * ph, +1.0)

    def _mesh_loops(self, handle):
        """A mesh body's boundary loops in global node ids, fluid on the left:
        [(ea, eb, signed area)], holes > 0, outline < 0 (sim_model.py:881-894). Checked: the
        outline encloses exactly the material and the holes."""
        lo, hi = self.me.body_node_range[handle]
        tri = np.asarray(self.me.tri)[self._tri_range[handle]] - lo
        loops = [(ea + lo, eb + lo, A) for ea, eb, A in
                 _act.mesh_boundary_loops(tri, np.asarray(self.me.rest_pos, np.float64)[lo:hi])]
        holes = sum(A for *_, A in loops if A > 0)
        outline = -sum(A for *_, A in loops if A < 0)
        material = float(self.element_areas(handle).sum())
        if abs(outline - (material + holes)) > 1e-9 * outline:
            raise RuntimeError(f"mesh body {handle}: its outline encloses {outline:.9e} m^2, its "
                               f"material and holes {material + holes:.9e}")
        return loops

    def _new_chamber(self, handle, ea, eb, expect, sign):
        """sign +1: edges counter-clockwise round a cavity; -1: clockwise round the body. The
        edges must enclose `expect` m^2 (the closure and orientation check)."""
        rest = self.me.rest_pos
        ref = rest[np.concatenate([ea, eb])].mean(0)
        got = sign * _act.loop_area(rest, ea, eb, ref)
        if not expect > 0 or abs(got - expect) > 1e-6 * expect:
            raise RuntimeError(f"pressure boundary encloses {got:.6e} m^2, expected {expect:.6e}")
        return self._added(self._chambers, Chamber(body=handle, ea=np.asarray(ea, np.int64),
                                                   eb=np.asarray(eb, np.int64), ref=np.asarray(ref, np.float64),
                                                   area0=float(expect), sign=sign))

    def set_pressure(self, chamber, pressure):
        """Gauge pressure of the fluid in a chamber [Pa]. Positive inflates a cavity (and
        squeezes a body through an ambient-pressure handle)."""
        self._chambers[chamber].pressure = float(pressure)
        self._commanded()

    def chamber_area(self, chamber):
        """Current area inside a pressure boundary [m^2]: a cavity's volume per unit depth; for
        an ambient-pressure handle, the area inside the body's outline."""
        c = self._chambers[chamber]
        return c.sign * _act.loop_area(self.get_x(), c.ea, c.eb, c.ref)

    # ---- springs, pins and joints (sim_model.py:988-1066)
    def _nearest(self, handle, point):
        ids = self._node_range[handle]
        gap = self.me.rest_pos[ids] - np.asarray(point, np.float64)
        return int(ids[np.argmin(np.linalg.norm(gap, axis=1))])

    def add_spring(self, handle_a, point_a, handle_b=None, point_b=None, stiffness=None, rest_length=None):
        """A linear spring from a point of one body to a point of another, or with
        handle_b=None to a point fixed in the world (point_b, default where point_a snapped
        to). Ends snap to the nearest node of their body. stiffness k [Pa] (default
        model.rigid_young); rest_length None keeps the built length. Returns a handle."""
        self._need_mesh()
        rest = self.me.rest_pos
        ia = self._nearest(handle_a, point_a)
        to_world = handle_b is None
        if to_world:
            ib = -1
            anchor = np.array(rest[ia] if point_b is None else point_b, np.float64)
        else:
            if self.body_env(handle_a) != self.body_env(handle_b):
                raise ValueError("a spring cannot join bodies of different environments")
            ib = self._nearest(handle_b, point_a if point_b is None else point_b)
            if ib == ia:
                raise ValueError("both ends of the spring snapped to the same node")
            anchor = np.array(rest[ib], np.float64)
        L = float(np.linalg.norm(rest[ia] - anchor)) if rest_length is None else float(rest_length)
        if not to_world and L <= 0.0:
            raise ValueError("a spring between two bodies needs a rest length: at zero it would "
                             "pull two nodes to one place while contact holds the bodies apart")
        k = float(self.rigid_young if stiffness is None else stiffness)
        if k <= 0 or L < 0:
            raise ValueError("spring stiffness must be positive and its rest length non-negative")
        return self._added(self._springs, Spring(a=ia, b=ib, stiffness=k, length=L, anchor=anchor,
                                                 env=self.body_env(handle_a)))

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
        self._springs[spring].length = float(length)
        self._commanded()

    def set_spring_anchor(self, spring, point):
        """Move the world end of a world spring or pin."""
        sp = self._springs[spring]
        if sp.b >= 0:
            raise ValueError("this spring joins two bodies and has no world anchor")
        sp.anchor = np.array(point, np.float64)
        self._commanded()

    def spring_force(self, spring):
        """(tension [N/m], negative in compression; current length [m]) of a spring."""
        sp = self._springs[spring]
        x = self.get_x()
        other = x[sp.b] if sp.b >= 0 else sp.anchor
        ln = float(np.linalg.norm(x[sp.a] - other))
        return sp.stiffness * (ln - sp.length), ln

    # ---- active material (sim_model.py:1068-1096)
    def add_active_region(self, handle, region, fiber=None):
        """Mark part of a body ((H, W) boolean map laid out like its mask) as actively
        deforming material; fiber None for isotropic change, else an angle [rad] or a
        2-vector along which `stretch` acts. Returns a handle."""
        self._need_mesh()
        elems = np.asarray(self._region_elements(handle, region), np.int64)
        self._claim("active", handle, elems, "active regions")
        return self._added(self._regions, ActiveRegion(body=handle, elems=elems, fiber=fiber))

    def set_activation(self, region, stretch, transverse=1.0):
        """Rest-length ratio of an active region: 1 passive, 0.9 a 10 % contraction; along
        the fiber with `transverse` across it, or isotropic without a fiber."""
        if stretch <= 0 or transverse <= 0:
            raise ValueError("stretch ratios must be positive")
        r = self._regions[region]
        r.A = _act.activation_matrix(stretch, transverse, r.fiber)
        self._commanded()

    def affine_state(self, index):
        """Position (the piece's centre of mass), angle and 2x2 map A of a rigid piece."""
        s = self._solver
        if s is None:
            nodes = self._affine[index].nodes
            m = np.asarray(self.me.mass)[nodes]
            com = m @ self.me.rest_pos[nodes] / m.sum()
            return dict(position=com, angle=0.0, A=np.eye(2))
        q = s.get_affine_q()[index]
        A = np.array([[q[1], q[2]], [q[4], q[5]]])
        return dict(position=np.array([q[0], q[3]]), angle=float(np.arctan2(A[1, 0] - A[0, 1], A[0, 0] + A[1, 1])), A=A)


def _path_length(x, nodes):
    """Length of the polyline through the nodes' positions."""
    return float(np.linalg.norm(np.diff(np.asarray(x, np.float64)[np.asarray(nodes)], axis=0), axis=1).sum())
