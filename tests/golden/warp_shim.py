"""A minimal, serial stand-in for the NVIDIA Warp runtime — TEST INFRASTRUCTURE ONLY.

The reference implementation (Diff_2D_FEM) writes every kernel in Warp's Python DSL and
needs the third-party `warp-lang` package (unpinned, `warp-lang>=1.0`, tested on 1.11) to
run them. That package is not installed here. This module implements the small part of
Warp's public Python API the reference uses — typed vectors and matrices, arrays, atomics,
`wp.launch`, a hash-grid broadphase — with Warp's documented CPU semantics: a launch runs
its thread ids 0..dim-1 one after another, so every atomic is applied in thread order.
The reference's own kernel source then executes unchanged, in pure Python.

It exists for one purpose: to generate golden vectors from the reference's own code
(`make_golden.py`) that pin the C oracle. It is slow (pure Python), so only small scenes
and a few steps are run through it. Nothing in the product imports it.

Arithmetic conventions that fix the rounding of each operation (Warp's native headers
use the same ones as far as the public documentation describes them):
  * all float64 arithmetic is IEEE double without fused multiply-add;
  * dot(a, b) = a0*b0 + a1*b1 + ... left to right; matrix products sum over k left to
    right; ddot(A, B) sums A_ij*B_ij in row-major order;
  * determinant(2x2) = m00*m11 - m10*m01; inverse(2x2) = adj(m) * (1/det);
    inverse(3x3) = cofactor transpose * (1/det);
  * length(v) = sqrt(dot(v, v)).
The hash-grid query returns every point of the querying environment's z-slab in
ascending index order: a superset of Warp's cell query (the kernels filter by distance
themselves), in a fixed order so that accumulations are reproducible.
"""
from __future__ import annotations

import math
import sys
import types as _pytypes

import numpy as np

_TID = [0]


# ----------------------------------------------------------------------------- scalars
float64 = float


def float32(x):
    return np.float32(x)


def float16(x):
    return np.float16(x)


int32 = int
int64 = int
uint8 = int
uint32 = int
uint64 = int
int8 = int


def _isvec(o):
    return isinstance(o, Vec)


def _ismat(o):
    return isinstance(o, Mat)


# ----------------------------------------------------------------------------- vectors
class Vec:
    __slots__ = ("v",)
    N = 0
    S = float

    def __init__(self, *args):
        n = type(self).N
        S = type(self).S
        if len(args) == 0:
            self.v = [S(0)] * n
        elif len(args) == 1 and isinstance(args[0], (list, tuple, np.ndarray, Vec)):
            src = args[0].v if isinstance(args[0], Vec) else list(args[0])
            self.v = [S(a) for a in src]
        elif len(args) == 1:
            self.v = [S(args[0])] * n
        else:
            assert len(args) == n, (len(args), n)
            self.v = [S(a) for a in args]

    @classmethod
    def _new(cls, lst):
        o = object.__new__(cls)
        o.v = lst
        return o

    def __getitem__(self, i):
        return self.v[i]

    def __setitem__(self, i, val):
        self.v[i] = val

    def __len__(self):
        return len(self.v)

    def __iter__(self):
        return iter(self.v)

    def __add__(self, o):
        return self._new([a + b for a, b in zip(self.v, o.v)])

    def __sub__(self, o):
        return self._new([a - b for a, b in zip(self.v, o.v)])

    def __neg__(self):
        return self._new([-a for a in self.v])

    def __mul__(self, s):
        if isinstance(s, (Vec, Mat)):
            raise TypeError("vector * vector/matrix is not a Warp operation")
        return self._new([a * s for a in self.v])

    def __rmul__(self, s):
        return self._new([s * a for a in self.v])

    def __truediv__(self, s):
        return self._new([a / s for a in self.v])

    def __repr__(self):
        return f"{type(self).__name__}({self.v})"


_VEC_CACHE = {}


def _vec_type(n, S):
    key = (n, S)
    if key not in _VEC_CACHE:
        _VEC_CACHE[key] = type(f"vec{n}", (Vec,), {"N": n, "S": S, "__slots__": ()})
    return _VEC_CACHE[key]


# ----------------------------------------------------------------------------- matrices
class Mat:
    __slots__ = ("m",)
    R = 0
    C = 0
    S = float

    def __init__(self, *args):
        R, C, S = type(self).R, type(self).C, type(self).S
        if len(args) == 0:
            self.m = [[S(0)] * C for _ in range(R)]
        elif len(args) == R * C:
            self.m = [[S(args[i * C + j]) for j in range(C)] for i in range(R)]
        elif len(args) == 1 and isinstance(args[0], (list, tuple, np.ndarray)):
            a = np.asarray(args[0], np.float64).reshape(R, C)
            self.m = [[S(a[i, j]) for j in range(C)] for i in range(R)]
        elif len(args) == R and all(isinstance(a, Vec) for a in args):
            self.m = [[S(x) for x in a.v] for a in args]
        else:
            raise TypeError(f"cannot build {R}x{C} matrix from {len(args)} args")

    @classmethod
    def _new(cls, rows):
        o = object.__new__(cls)
        o.m = rows
        return o

    def __getitem__(self, ij):
        if isinstance(ij, tuple):
            return self.m[ij[0]][ij[1]]
        return _vec_type(type(self).C, type(self).S)._new(list(self.m[ij]))

    def __setitem__(self, ij, val):
        if isinstance(ij, tuple):
            self.m[ij[0]][ij[1]] = val
        else:
            self.m[ij] = list(val.v)

    def __add__(self, o):
        return self._new([[a + b for a, b in zip(r, s)] for r, s in zip(self.m, o.m)])

    def __sub__(self, o):
        return self._new([[a - b for a, b in zip(r, s)] for r, s in zip(self.m, o.m)])

    def __neg__(self):
        return self._new([[-a for a in r] for r in self.m])

    def _matmul(self, o):
        if isinstance(o, Mat):
            K = type(self).C
            rows = []
            for i in range(type(self).R):
                ri = self.m[i]
                row = []
                for j in range(type(o).C):
                    s = ri[0] * o.m[0][j]
                    for k in range(1, K):
                        s = s + ri[k] * o.m[k][j]
                    row.append(s)
                rows.append(row)
            return _mat_type(type(self).R, type(o).C, type(self).S)._new(rows)
        if isinstance(o, Vec):
            out = []
            for i in range(type(self).R):
                ri = self.m[i]
                s = ri[0] * o.v[0]
                for k in range(1, type(self).C):
                    s = s + ri[k] * o.v[k]
                out.append(s)
            return _vec_type(type(self).R, type(self).S)._new(out)
        raise TypeError

    def __mul__(self, o):
        if isinstance(o, (Mat, Vec)):
            return self._matmul(o)
        return self._new([[a * o for a in r] for r in self.m])

    def __rmul__(self, s):
        return self._new([[s * a for a in r] for r in self.m])

    def __matmul__(self, o):
        return self._matmul(o)

    def __truediv__(self, s):
        return self._new([[a / s for a in r] for r in self.m])

    def __repr__(self):
        return f"{type(self).__name__}({self.m})"


_MAT_CACHE = {}


def _mat_type(r, c, S):
    key = (r, c, S)
    if key not in _MAT_CACHE:
        _MAT_CACHE[key] = type(f"mat{r}{c}", (Mat,), {"R": r, "C": c, "S": S, "__slots__": ()})
    return _MAT_CACHE[key]


vec2d = _vec_type(2, float)
vec3d = _vec_type(3, float)
vec4d = _vec_type(4, float)
vec2f = _vec_type(2, float32)
vec3f = _vec_type(3, float32)
vec2 = vec2f
vec3 = vec3f
vec2i = _vec_type(2, int)
vec3i = _vec_type(3, int)
vec4i = _vec_type(4, int)
mat22d = _mat_type(2, 2, float)
mat33d = _mat_type(3, 3, float)
mat22f = _mat_type(2, 2, float32)
mat33f = _mat_type(3, 3, float32)
mat22 = mat22f
mat33 = mat33f


class _Types:
    @staticmethod
    def vector(length, dtype):
        return _vec_type(int(length), dtype)

    @staticmethod
    def matrix(shape, dtype):
        return _mat_type(int(shape[0]), int(shape[1]), dtype)


types_ns = _Types()


# ----------------------------------------------------------------------------- builtins
def tid():
    return _TID[0]


def constant(x):
    return x


def func(f):
    return f


def struct(cls):
    return cls


def max(a, b):  # noqa: A001
    if isinstance(a, Vec):
        return a._new([x if x > y else y for x, y in zip(a.v, b.v)])
    return a if a > b else b


def min(a, b):  # noqa: A001
    if isinstance(a, Vec):
        return a._new([x if x < y else y for x, y in zip(a.v, b.v)])
    return a if a < b else b


def clamp(x, lo, hi):
    return min(max(x, lo), hi)


def abs(x):  # noqa: A001
    return x if x >= 0 else -x


def sqrt(x):
    return math.sqrt(x)


def log(x):
    return math.log(x)


def exp(x):
    return math.exp(x)


def sin(x):
    return math.sin(x)


def cos(x):
    return math.cos(x)


def atan2(y, x):
    return math.atan2(y, x)


def floor(x):
    return math.floor(x)


def dot(a, b):
    av, bv = a.v, b.v
    s = av[0] * bv[0]
    for k in range(1, len(av)):
        s = s + av[k] * bv[k]
    return s


def length(a):
    return math.sqrt(dot(a, a))


def length_sq(a):
    return dot(a, a)


def normalize(a):
    ln = length(a)
    return a / ln if ln > 0 else a * 0.0


def cross(a, b):
    if len(a.v) == 2:
        return a.v[0] * b.v[1] - a.v[1] * b.v[0]
    x = a.v[1] * b.v[2] - a.v[2] * b.v[1]
    y = a.v[2] * b.v[0] - a.v[0] * b.v[2]
    z = a.v[0] * b.v[1] - a.v[1] * b.v[0]
    return a._new([x, y, z])


def cw_mul(a, b):
    if isinstance(a, Mat):
        return a._new([[x * y for x, y in zip(r, s)] for r, s in zip(a.m, b.m)])
    return a._new([x * y for x, y in zip(a.v, b.v)])


def cw_div(a, b):
    return a._new([x / y for x, y in zip(a.v, b.v)])


def outer(a, b):
    return _mat_type(len(a.v), len(b.v), type(a).S)._new([[x * y for y in b.v] for x in a.v])


def transpose(m):
    R, C = type(m).R, type(m).C
    return _mat_type(C, R, type(m).S)._new([[m.m[i][j] for i in range(R)] for j in range(C)])


def ddot(a, b):
    s = None
    for r, q in zip(a.m, b.m):
        for x, y in zip(r, q):
            s = x * y if s is None else s + x * y
    return s


def determinant(m):
    a = m.m
    if len(a) == 2:
        return a[0][0] * a[1][1] - a[1][0] * a[0][1]
    if len(a) == 3:
        return (a[0][0] * (a[1][1] * a[2][2] - a[2][1] * a[1][2])
                - a[0][1] * (a[1][0] * a[2][2] - a[2][0] * a[1][2])
                + a[0][2] * (a[1][0] * a[2][1] - a[2][0] * a[1][1]))
    raise NotImplementedError


def inverse(m):
    a = m.m
    det = determinant(m)
    if len(a) == 2:
        if det == 0.0:
            return m._new([[0.0, 0.0], [0.0, 0.0]])
        r = 1.0 / det
        return m._new([[a[1][1] * r, -a[0][1] * r], [-a[1][0] * r, a[0][0] * r]])
    if len(a) == 3:
        if det == 0.0:
            return m._new([[0.0] * 3 for _ in range(3)])
        b = [[0.0] * 3 for _ in range(3)]
        b[0][0] = a[1][1] * a[2][2] - a[1][2] * a[2][1]
        b[1][0] = a[1][2] * a[2][0] - a[1][0] * a[2][2]
        b[2][0] = a[1][0] * a[2][1] - a[1][1] * a[2][0]
        b[0][1] = a[0][2] * a[2][1] - a[0][1] * a[2][2]
        b[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0]
        b[2][1] = a[0][1] * a[2][0] - a[0][0] * a[2][1]
        b[0][2] = a[0][1] * a[1][2] - a[0][2] * a[1][1]
        b[1][2] = a[0][2] * a[1][0] - a[0][0] * a[1][2]
        b[2][2] = a[0][0] * a[1][1] - a[0][1] * a[1][0]
        r = 1.0 / det
        return m._new([[x * r for x in row] for row in b])
    raise NotImplementedError


# ----------------------------------------------------------------------------- arrays
def _conv(dtype):
    """Element <-> storage conversion for a dtype."""
    if isinstance(dtype, type) and issubclass(dtype, Vec):
        return "vec"
    if isinstance(dtype, type) and issubclass(dtype, Mat):
        return "mat"
    return "scalar"


class array:  # noqa: N801
    def __init__(self, data=None, dtype=float, device=None, shape=None, copy=True, **kw):
        self.dtype = dtype
        self.kind = _conv(dtype)
        self.device = device
        if data is None:
            n = shape if isinstance(shape, int) else (shape[0] if shape else 0)
            self._alloc(n)
        else:
            self._from_np(np.asarray(data))

    def _alloc(self, n):
        if self.kind == "vec":
            self.d = [self.dtype() for _ in range(n)]
        elif self.kind == "mat":
            self.d = [self.dtype() for _ in range(n)]
        else:
            z = self.dtype(0) if self.dtype not in (float32,) else np.float32(0)
            self.d = [z] * n

    def _from_np(self, a):
        if self.kind == "vec":
            N = self.dtype.N
            a = a.reshape(-1, N)
            self.d = [self.dtype(row.tolist()) for row in a]
        elif self.kind == "mat":
            R, C = self.dtype.R, self.dtype.C
            a = a.reshape(-1, R, C)
            self.d = [self.dtype(*row.reshape(-1).tolist()) for row in a]
        else:
            S = self.dtype
            if S is float:
                self.d = [float(v) for v in a.reshape(-1).tolist()]
            elif S is int:
                self.d = [int(v) for v in a.reshape(-1).tolist()]
            else:
                self.d = [S(v) for v in a.reshape(-1)]

    # element access: values are COPIED out, as Warp's value types are
    def __getitem__(self, i):
        v = self.d[i]
        if self.kind == "vec":
            return v._new(list(v.v))
        if self.kind == "mat":
            return v._new([list(r) for r in v.m])
        return v

    def __setitem__(self, i, val):
        if self.kind == "vec":
            self.d[i] = self.dtype._new(list(val.v))
        elif self.kind == "mat":
            self.d[i] = self.dtype._new([list(r) for r in val.m])
        else:
            self.d[i] = val

    def __len__(self):
        return len(self.d)

    @property
    def shape(self):
        return (len(self.d),)

    @property
    def size(self):
        return len(self.d)

    def numpy(self):
        if self.kind == "vec":
            return np.array([v.v for v in self.d], dtype=np.float64 if self.dtype.S is not int else np.int32).reshape(-1, self.dtype.N)
        if self.kind == "mat":
            return np.array([v.m for v in self.d], dtype=np.float64).reshape(-1, self.dtype.R, self.dtype.C)
        if self.dtype is int:
            return np.array(self.d, dtype=np.int64)
        return np.array(self.d, dtype=np.float64)

    def assign(self, src):
        if isinstance(src, array):
            src = src.numpy()
        n = len(self.d)
        self._from_np(np.asarray(src))
        assert len(self.d) == n

    def zero_(self):
        self._alloc(len(self.d))

    def fill_(self, val):
        if self.kind == "scalar":
            self.d = [self.dtype(val)] * len(self.d)
        else:
            self.d = [self.dtype(val) for _ in range(len(self.d))]

    @property
    def ptr(self):
        return id(self)

    @property
    def id(self):
        return self


def zeros(shape, dtype=float, device=None, **kw):
    n = shape if isinstance(shape, int) else shape[0]
    return array(None, dtype=dtype, device=device, shape=int(n))


def empty(shape, dtype=float, device=None, **kw):
    return zeros(shape, dtype=dtype, device=device)


def full(shape, value, dtype=float, device=None, **kw):
    a = zeros(shape, dtype=dtype, device=device)
    a.fill_(value)
    return a


def clone(a, device=None):
    b = array(None, dtype=a.dtype, device=a.device, shape=len(a.d))
    b.assign(a.numpy())
    return b


def copy(dest, src, dest_offset=0, src_offset=0, count=None):
    n = len(src.d) - src_offset if count is None else count
    for k in range(n):
        dest[dest_offset + k] = src[src_offset + k]


def atomic_add(arr, i, val):
    old = arr.d[i]
    if arr.kind == "vec":
        arr.d[i] = old._new([a + b for a, b in zip(old.v, val.v)])
    elif arr.kind == "mat":
        arr.d[i] = old._new([[a + b for a, b in zip(r, s)] for r, s in zip(old.m, val.m)])
    else:
        arr.d[i] = old + val
    return old


def atomic_sub(arr, i, val):
    return atomic_add(arr, i, -val)


def atomic_min(arr, i, val):
    old = arr.d[i]
    if val < old:
        arr.d[i] = val
    return old


def atomic_max(arr, i, val):
    old = arr.d[i]
    if val > old:
        arr.d[i] = val
    return old


# ----------------------------------------------------------------------------- kernels
class Kernel:
    def __init__(self, fn):
        self.fn = fn
        self.key = fn.__name__


def kernel(fn=None, **kw):
    if fn is None:
        return lambda f: Kernel(f)
    return Kernel(fn)


LAUNCH_COUNTS = {}


def launch(kernel, dim, inputs=(), outputs=(), device=None, **kw):
    n = dim if isinstance(dim, int) else int(np.prod(dim))
    args = list(inputs) + list(outputs)
    fn = kernel.fn
    LAUNCH_COUNTS[kernel.key] = LAUNCH_COUNTS.get(kernel.key, 0) + 1
    for t in range(n):
        _TID[0] = t
        fn(*args)


# ----------------------------------------------------------------------------- hash grid
class HashGrid:
    """Broadphase stand-in: groups the points by their z coordinate (the reference puts
    each environment in its own z-slab) and answers a query with the whole slab."""

    def __init__(self, dim_x, dim_y, dim_z, device=None):
        self.groups = {}
        self.id = self

    def build(self, points, radius):
        self.groups = {}
        for i, p in enumerate(points.d):
            self.groups.setdefault(float(p.v[2]), []).append(i)


def hash_grid_query(grid, point, radius):
    return iter(grid.groups.get(float(point.v[2]), []))


def hash_grid_point_id(grid, i):
    return i


# ----------------------------------------------------------------------------- misc API
class _Config:
    quiet = True
    mode = "release"
    verify_fp = False


config = _Config()


def init():
    pass


def is_cuda_available():
    return False


def get_preferred_device():
    return "cpu"


def get_device(d=None):
    return "cpu"


def synchronize():
    pass


def synchronize_device(d=None):
    pass


def ScopedTimer(*a, **k):  # noqa: N802
    import contextlib
    return contextlib.nullcontext()


def install():
    """Register this module as `warp` (and `warp.types`) in sys.modules."""
    mod = sys.modules[__name__]
    mod.types = types_ns
    sys.modules["warp"] = mod
    tmod = _pytypes.ModuleType("warp.types")
    tmod.vector = types_ns.vector
    tmod.matrix = types_ns.matrix
    sys.modules["warp.types"] = tmod
    return mod
