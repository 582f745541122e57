"""ctypes binding of libd2f.so (include/d2f.h). Loading fails loudly: there is no CPU
fallback for the step."""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_LIB = None

_I = C.c_int32
_D = C.c_double
_P = C.c_void_p

D2F_ABI_VERSION = 7
D2F_FP64, D2F_MIXED = 0, 1
ERRORS = {0: "ok", -1: "D2F_EINVAL", -2: "D2F_ECUDA", -3: "D2F_ECAP", -4: "D2F_ENAN", -5: "D2F_ESPIN"}


class Seg(C.Structure):
    _fields_ = [(n, _I) for n in (
        "node0", "nn", "tri0", "nt", "bnd0", "nb", "edge0", "ne", "cand0", "ncap", "bc0", "nbc",
        "aff0", "naff", "affn0", "naffn", "rig0", "nrig", "rign0", "nrign", "ten0", "nten", "tent0", "ntent",
        "sp0", "nsp", "pe0", "npe")]


DESC_FIELDS = (
    [("abi_version", _I), ("precision", _I)]
    + [(n, _I) for n in ("n_scenes", "N", "T", "Nb", "Ne", "n_bc", "n_col", "n_aff", "n_affn", "n_rig",
                         "n_rign", "n_ten", "n_tent", "cand_total", "max_nb")]
    + [(n, _P) for n in (
        "segs", "x", "v", "xn", "xhat", "xu", "xrest", "grad", "grad_prev", "p", "diagH", "diag_el", "mass", "free_mask",
        "fext", "inc_ptr", "inc", "inc8", "node_bslot", "node_bc", "node_aff", "node_rig", "tri", "Bm", "area", "mu",
        "lam", "Dm", "escr", "ecache", "mscr", "bnd", "colliders", "col_mu_env", "bc_idx", "bc_target", "ea", "eb", "ela",
        "elb", "ca", "cb", "excl_ptr", "excl_idx", "mu_node", "cand", "cand_tr", "xref", "t_node", "t_prv", "t_nxt",
        "t_tid", "t_stiff", "t_L0", "t_Tcmd", "t_state", "a_node", "a_grp", "a_w", "a_Mu", "a_La", "a_q",
        "a_pq", "a_gq", "a_gq_prev", "a_zq", "a_H", "r_node", "r_grp", "r_acc", "r_zq", "iters", "active",
        "status", "work")]
    + [(n, _D) for n in ("dt", "drag", "dhat", "kappa", "epsv", "eps", "tol_x", "near_factor", "alpha_max",
                         "area_shrink", "ccd_eta", "cg_guard", "gtol", "ipc_mu", "ipc_dhat", "ipc_kappa",
                         "reach", "gap", "bc_floor", "skin")]
    + [(n, _I) for n in ("iter_max", "conv_check", "friction", "per_body", "threads", "blocks_per_sm")]
    + [("ls_tol", _D), ("line_search", _I), ("n_backtrack", _I), ("blocks_per_scene", _I),
       ("a_ptr", _P), ("n_sp", _I)] + [(n, _P) for n in ("sp_a", "sp_b", "sp_k", "sp_L0", "sp_anchor")]
    + [("n_pe", _I), ("n_ch", _I)] + [(n, _P) for n in ("pe_a", "pe_b", "pe_ch", "ch_p", "ch_ref")]
    + [("energy_out", _P)]
)


class SceneDesc(C.Structure):
    _fields_ = DESC_FIELDS


EXPORTS = ("d2f_abi_version", "d2f_create", "d2f_step", "d2f_set_dt", "d2f_stats", "d2f_destroy",
           "d2f_last_error", "d2f_kernels_per_step", "d2f_step_noalloc", "d2f_mixed_scratch_bytes",
           "d2f_adjoint_solve", "d2f_adjoint_vjp", "d2f_adjoint_work_doubles", "d2f_launch_shape",
           "d2f_element_fields", "d2f_adjoint_vjp_pressure", "d2f_contact_force", "d2f_energy")
NOALLOC_SCRATCH_BYTES = 16 << 20


def lib_path():
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libd2f.so (building it first if asked and absent). Raises if it cannot."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libd2f.so is not built ({path}); run python -m diff_2d_fem_gb300.build")
        _build.build()
    L = C.CDLL(path)
    L.d2f_abi_version.restype = _I
    L.d2f_create.argtypes = [C.POINTER(SceneDesc), C.POINTER(_P)]
    L.d2f_create.restype = _I
    L.d2f_step.argtypes = [_P, _P]
    L.d2f_step.restype = _I
    L.d2f_set_dt.argtypes = [_P, _D, _I]
    L.d2f_set_dt.restype = _I
    L.d2f_stats.argtypes = [_P, _P, _P, _P, _P]
    L.d2f_stats.restype = _I
    L.d2f_destroy.argtypes = [_P]
    L.d2f_destroy.restype = _I
    L.d2f_last_error.restype = C.c_char_p
    L.d2f_kernels_per_step.argtypes = [_P]
    L.d2f_kernels_per_step.restype = _I
    L.d2f_launch_shape.argtypes = [_P, _P, _P, _P]
    L.d2f_launch_shape.restype = _I
    L.d2f_element_fields.argtypes = [_I] + [_P] * 10
    L.d2f_element_fields.restype = _I
    L.d2f_adjoint_vjp_pressure.argtypes = [_P] * 5
    L.d2f_adjoint_vjp_pressure.restype = _I
    L.d2f_contact_force.argtypes = [_P, _I, _I, _I, _P, _P]
    L.d2f_contact_force.restype = _I
    L.d2f_energy.argtypes = [_P, _P, _P]
    L.d2f_energy.restype = _I
    L.d2f_step_noalloc.argtypes = [C.POINTER(SceneDesc), _P]
    L.d2f_step_noalloc.restype = _I
    L.d2f_mixed_scratch_bytes.argtypes = [_I, _I, _I, _I, _I]
    L.d2f_mixed_scratch_bytes.restype = C.c_size_t
    L.d2f_adjoint_solve.argtypes = [_P, _P, _P, _P, _P, _P, _D, _I, _I, _P, _P, _P]
    L.d2f_adjoint_solve.restype = _I
    L.d2f_adjoint_vjp.argtypes = [_P, _P, _P, _P, _P, _P]
    L.d2f_adjoint_vjp.restype = _I
    L.d2f_adjoint_work_doubles.argtypes = [_P]
    L.d2f_adjoint_work_doubles.restype = C.c_int64
    if L.d2f_abi_version() != D2F_ABI_VERSION:
        raise RuntimeError("libd2f.so ABI version mismatch; rebuild it")
    _LIB = L
    return L


def check(rc, what):
    if rc != 0:
        msg = _LIB.d2f_last_error().decode() if _LIB is not None else ""
        raise RuntimeError(f"{what} failed ({ERRORS.get(rc, rc)}): {msg}")
