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
