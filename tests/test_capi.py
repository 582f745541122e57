"""The C ABI library builds, loads, and exports every symbol include/d2f.h declares; its
ctypes mirror of d2f_scene_desc matches the header field for field. No GPU needed: no
compute entry point is called."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT
from diff_2d_fem_gb300 import _lib, build

HDR = os.path.join(ROOT, "include", "d2f.h")


def _header_functions():
    txt = open(HDR).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z0-9_]+\s*\*?\s*(d2f_[a-z_]+)\s*\(", txt, re.M)))


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    lib = C.CDLL(path)
    names = _header_functions()
    assert set(names) == set(_lib.EXPORTS), f"header declares {names}"
    for n in names:
        assert hasattr(lib, n), f"{n} not exported"


def test_abi_version_and_error_string():
    L = _lib.load()
    assert L.d2f_abi_version() == _lib.D2F_ABI_VERSION
    assert isinstance(L.d2f_last_error(), bytes)


def test_create_rejects_bad_descriptors_without_a_gpu():
    L = _lib.load()
    d = _lib.SceneDesc()
    h = C.c_void_p()
    d.abi_version = 999
    assert L.d2f_create(C.byref(d), C.byref(h)) == -1
    assert b"ABI" in L.d2f_last_error()
    d.abi_version = _lib.D2F_ABI_VERSION
    d.precision = 7
    assert L.d2f_create(C.byref(d), C.byref(h)) == -1
    d.precision = 0
    assert L.d2f_create(C.byref(d), C.byref(h)) == -1      # empty scene
    assert L.d2f_create(None, C.byref(h)) == -1


def test_struct_mirrors_header():
    """Every field of d2f_scene_desc / d2f_seg in the header appears in the ctypes mirror in
    the same order."""
    txt = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    body = txt[txt.index("typedef struct d2f_scene_desc {"):txt.index("} d2f_scene_desc;")]
    names = []
    for line in body.splitlines()[1:]:
        line = line.strip()
        if not line:
            continue
        decl = re.sub(r"^(const\s+)?[a-z0-9_]+\s+", "", line.rstrip(";"))
        names += [re.sub(r"[\s*]", "", v) for v in decl.split(",")]
    assert names == [n for n, _ in _lib.DESC_FIELDS]
    seg = txt[txt.index("typedef struct d2f_seg {"):txt.index("} d2f_seg;")]
    sn = []
    for line in seg.splitlines()[1:]:
        line = line.strip().rstrip(";")
        if line:
            sn += [v.strip() for v in re.sub(r"^int32_t\s+", "", line).split(",")]
    assert sn == [n for n, _ in _lib.Seg._fields_]


def _valid_desc():
    """A descriptor that passes every check d2f_create makes before touching a device: one
    scene of one node and one triangle, every required pointer set (to a dummy address: the
    checks never dereference them)."""
    d = _lib.SceneDesc()
    d.abi_version = _lib.D2F_ABI_VERSION
    d.precision = _lib.D2F_FP64
    d.n_scenes, d.N, d.T = 1, 1, 1
    for name in ("segs", "x", "v", "xn", "xhat", "grad", "grad_prev", "p", "diagH", "mass", "free_mask",
                 "inc_ptr", "inc", "inc8", "node_bslot", "node_bc", "node_aff", "node_rig", "tri", "Bm", "area",
                 "mu", "lam", "iters", "active", "status", "escr", "ecache", "work"):
        setattr(d, name, 64)
    d.dt, d.iter_max = 1e-3, 1
    return d


@pytest.mark.parametrize("field,value,needle", [
    ("blocks_per_scene", 5, b"blocks_per_scene"),
    ("blocks_per_scene", 16, b"mixed precision only"),
    ("blocks_per_scene", -1, b"mixed precision only"),     # D2F_ALL_SMS, every SM on one scene
    ("blocks_per_scene", -2, b"D2F_ALL_SMS"),
    ("n_sp", 1, b"spring"),
    ("n_pe", 4, b"pressure"),
    ("threads", 96, b"threads"),
    ("line_search", 1, b"xu"),
])
def test_create_checks_the_new_fields_without_a_gpu(field, value, needle):
    """The checks of blocks_per_scene, the spring and pressure arrays, the launch width and
    the line search's buffer: D2F_EINVAL with a message naming the problem, before any device
    call (a descriptor that passes them all fails only for want of a device here)."""
    L = _lib.load()
    h = C.c_void_p()
    d = _valid_desc()
    rc = L.d2f_create(C.byref(d), C.byref(h))
    assert rc in (0, -2), L.d2f_last_error()          # created on a GPU machine; D2F_ECUDA without one
    if rc == 0:
        L.d2f_destroy(h)
    setattr(d, field, value)
    assert L.d2f_create(C.byref(d), C.byref(h)) == -1
    assert needle in L.d2f_last_error(), L.d2f_last_error()
