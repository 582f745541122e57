"""The records a Model keeps: bodies, colliders and actuators, as typed dataclasses, with
the argument checks the add_* calls share.

The Model (model.py) owns lists of these; the problem builder (scene.py) and the
integrator read them to lay the scene out on the device. Handles returned to the user are
indices into those lists.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional, Union

import numpy as np

NONE, DISC, ELLIPSE, BOX, TRIANGLE, HALFSPACE = -1, 0, 1, 2, 3, 4
SHAPE_CODES = {"disc": DISC, "ellipse": ELLIPSE, "box": BOX, "square": BOX, "triangle": TRIANGLE}

Stiffness = Union[float, np.ndarray]


# ----------------------------------------------------------------------------- bodies
@dataclass
class Body:
    """One body. `pixels`: a mask (H, W), row 0 at the bottom, of physical `size` centred at
    `center`; otherwise a triangle mesh (`vertices`, `triangles`) with its measured sizes
    (`h` median boundary edge, `h_cfl` smallest sqrt(2 area), `L_max` longest boundary
    edge). `E` is a scalar or a field (per pixel, or per triangle of a mesh)."""
    env: int
    E: Stiffness
    nu: float
    rho: float
    mu: Optional[float]
    center: tuple
    role: str = "soft"                       # "soft" | "affine" | "kinematic"
    mask: Optional[np.ndarray] = None
    size: Optional[tuple] = None
    vertices: Optional[np.ndarray] = None
    triangles: Optional[np.ndarray] = None
    h: float = 0.0
    h_cfl: float = 0.0
    L_max: float = 0.0

    @property
    def is_mesh(self) -> bool:
        return self.mask is None

    @property
    def is_soft(self) -> bool:
        return self.role == "soft"

    @property
    def uniform(self) -> bool:
        return np.isscalar(self.E)

    def min_E(self) -> float:
        if self.uniform:
            return float(self.E)
        if self.is_mesh:
            return float(np.min(self.E))
        return float(np.min(self.E[self.mask > 0]))

    def geometry_key(self):
        """Identifies the body's rest geometry (bodies of a batch repeat it)."""
        if self.is_mesh:
            return ("mesh", id(self.vertices), id(self.triangles))
        return ("mask", self.mask.shape, self.mask.tobytes(), self.size, self.center)


# ----------------------------------------------------------------------------- colliders
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


@dataclass
class ColliderSpec(Collider):
    """A collider of a model: its shape and its Coulomb coefficient."""
    mu: float = 0.5

    def row(self):
        """The 8 numbers of a collider row the kernels read: kind, cx, cy, rx, ry, rref, r, mu."""
        return [float(self.kind), self.cx, self.cy, self.rx, self.ry, self.rref, self.rx, self.mu]

    def public(self) -> Collider:
        return Collider(self.kind, self.cx, self.cy, self.rx, self.ry, self.rref)


# ----------------------------------------------------------------------------- actuators
@dataclass
class Chamber:
    """A closed loop of boundary edges (ea -> eb, fluid on the left) with its gauge pressure.
    sign +1: a cavity; -1: the outline of a body under ambient pressure. area0: the rest area
    the loop encloses; ref: a point the shoelace sum is taken about."""
    body: int
    ea: np.ndarray
    eb: np.ndarray
    ref: np.ndarray
    area0: float
    sign: float
    pressure: float = 0.0


@dataclass
class Tendon:
    """A cable through the eyelets `nodes` (global ids). stiffness 0: tension-controlled
    (`tension`); > 0: length-controlled (`length` is the commanded rest length)."""
    body: int
    nodes: np.ndarray
    stiffness: float
    length: float
    tension: float = 0.0


@dataclass
class ActiveRegion:
    """Elements of a body whose rest shape is scaled by the 2x2 activation A."""
    body: int
    elems: np.ndarray
    fiber: object = None
    A: np.ndarray = field(default_factory=lambda: np.eye(2))


@dataclass
class RigidPiece:
    """An affine (rigid) piece: its elements and the nodes they touch."""
    body: int
    elems: np.ndarray
    nodes: np.ndarray


@dataclass
class Spring:
    """A linear spring from node a to node b, or to the world point `anchor` when b < 0."""
    a: int
    b: int
    stiffness: float
    length: float
    anchor: np.ndarray
    env: int


# ----------------------------------------------------------------------------- argument checks
def solid_mask(mask) -> np.ndarray:
    """A pixel mask as uint8 0/1; refuses anything but a 2-D mask with a solid pixel."""
    m = (np.asarray(mask) > 0.5).astype(np.uint8)
    if m.ndim != 2 or not m.any():
        raise ValueError("the mask must be a 2-D array with at least one solid pixel")
    return m


def stiffness_field(E, shape, per_triangle: bool, solid=None):
    """None, a scalar, or a field of `shape` (checked). Per pixel: positive wherever the
    mask is solid; per triangle: positive and finite everywhere."""
    if E is None or np.isscalar(E):
        return None if E is None else float(E)
    E = np.asarray(E, np.float64)
    if per_triangle:
        if E.shape != shape:
            raise ValueError(f"stiffness per triangle is {E.shape}; the mesh has {shape[0]} triangles")
        if not (np.isfinite(E).all() and (E > 0).all()):
            raise ValueError("stiffness must be positive and finite on every triangle")
    else:
        if E.shape != shape:
            raise ValueError(f"stiffness map is {E.shape}, the mask is {shape}")
        if (E[solid > 0] <= 0).any():
            raise ValueError("stiffness map must be positive wherever the mask is solid")
    return E


def env_index(env_id) -> int:
    e = int(env_id)
    if e < 0:
        raise ValueError("env_id must be >= 0")
    return e


def friction_coefficient(mu):
    if mu is None:
        return None
    mu = float(mu)
    if not (np.isfinite(mu) and mu >= 0.0):
        raise ValueError(f"mu must be a finite number >= 0, not {mu}")
    return mu


def cells_covered(a: Body, b: Body) -> bool:
    """Does a solid pixel centre of pixel body `a` fall on a solid pixel of body `b`? (Pixel
    bodies that only touch along pixel edges share no centre.)"""
    (aw, ah), (ax, ay) = a.size, a.center
    (bw, bh), (bx, by) = b.size, b.center
    if abs(ax - bx) >= 0.5 * (aw + bw) or abs(ay - by) >= 0.5 * (ah + bh):
        return False
    rows, cols = np.nonzero(a.mask)
    Ha, Wa = a.mask.shape
    Hb, Wb = b.mask.shape
    cx = (ax - 0.5 * aw) + (cols + 0.5) * (aw / Wa)
    cy = (ay - 0.5 * ah) + (rows + 0.5) * (ah / Ha)
    jb = np.floor((cx - (bx - 0.5 * bw)) / (bw / Wb)).astype(np.int64)
    ib = np.floor((cy - (by - 0.5 * bh)) / (bh / Hb)).astype(np.int64)
    inside = (jb >= 0) & (jb < Wb) & (ib >= 0) & (ib < Hb)
    return bool(b.mask[ib[inside], jb[inside]].any())
