"""CPU FP64 oracle of the implicit step — TEST INFRASTRUCTURE ONLY.

A ctypes front end to oracle.c, the serial C restatement of the reference's PNCG-IPC
solve. Only the tests, `__graft_entry__.smoke()` and `bench.py`'s CPU-baseline leg use it,
as the checker or the timed CPU baseline; the product path never imports it.

The input is a *problem*: a dict of numpy arrays and scalars describing one solver (every
environment of a scene), in the reference solver's own layout — see `problem_keys` below.
`diff_2d_fem_gb300.scene.solver_problem` produces it from a Model, and the golden
fixtures store the same dict as built by the reference itself.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_LIB = None

_I = C.c_int32
_D = C.c_double
_PD = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int32)

# (name, ctype) in the order of d2o_solver in oracle.h
_FIELDS = [
    ("N", _I), ("T", _I), ("B", _I), ("Nb", _I), ("n_bc", _I), ("n_col", _I),
    ("x", _PD), ("v", _PD), ("xn", _PD), ("xhat", _PD), ("grad", _PD), ("grad_prev", _PD),
    ("p", _PD), ("diagH", _PD), ("x0buf", _PD),
    ("mass", _PD), ("free_", _PD), ("node2env", _PI),
    ("tri", _PI), ("Bm", _PD), ("area", _PD), ("mu", _PD), ("lam", _PD), ("tri2env", _PI),
    ("bnd", _PI), ("b2e", _PI),
    ("bc_idx", _PI), ("bc_target", _PD),
    ("colliders", _PD),
    ("gPg", _PD), ("g_p", _PD), ("g_Py", _PD), ("y_p", _PD), ("y_Py", _PD), ("beta", _PD),
    ("gTp", _PD), ("pHp", _PD), ("alpha", _PD), ("p_inf", _PD), ("clr_min", _PD),
    ("dE", _PD), ("dE0", _PD), ("Ener", _PD), ("Els_prev", _PD), ("gn0", _PD),
    ("active", _PI), ("iters", _PI),
    ("dt", _D), ("h2", _D), ("inv_dt", _D), ("drag", _D), ("dhat", _D), ("kappa", _D), ("epsv", _D),
    ("eps", _D), ("tol_x", _D), ("near_factor", _D), ("alpha_max", _D), ("area_shrink", _D),
    ("ccd_eta", _D), ("cg_guard", _D), ("ls_tol", _D), ("gtol", _D),
    ("iter_max", _I), ("conv_check", _I), ("friction", _I), ("line_search", _I), ("n_bt", _I),
    ("has_ext", _I), ("fext", _PD),
    ("has_ipc", _I), ("Ne", _I), ("per_body", _I),
    ("ea", _PI), ("eb", _PI), ("ela", _PI), ("elb", _PI), ("e2env", _PI),
    ("ca", _PD), ("cb", _PD), ("bstart", _PI), ("bpe", _PI), ("excl_ptr", _PI), ("excl_idx", _PI),
    ("mu_node", _PD),
    ("ipc_mu", _D), ("ipc_dhat", _D), ("ipc_kappa", _D), ("reach", _D), ("gap", _D), ("bc_floor", _D),
    ("q", _PD), ("q_inf", _PD), ("sweep_beta", _PD), ("clr", _PD),
    ("pending", _I),
    ("n_tendon", _I), ("n_tent", _I),
    ("t_node", _PI), ("t_prv", _PI), ("t_nxt", _PI), ("t_tid", _PI), ("t2env", _PI),
    ("t_stiff", _PD), ("t_L0", _PD), ("t_Tcmd", _PD),
    ("t_L", _PD), ("t_dL", _PD), ("t_tau", _PD), ("t_keff", _PD),
    ("n_aff", _I), ("n_affn", _I),
    ("a_node", _PI), ("a_grp", _PI), ("a_env", _PI),
    ("a_w", _PD), ("a_Mu", _PD), ("a_La", _PD),
    ("a_q", _PD), ("a_q0", _PD), ("a_pq", _PD), ("a_gq", _PD), ("a_gq_prev", _PD), ("a_zq", _PD),
    ("a_Hx", _PD), ("a_Hy", _PD),
    ("n_rig", _I), ("n_rign", _I),
    ("r_node", _PI), ("r_grp", _PI), ("r_env", _PI),
    ("r_acc", _PD), ("r_gq", _PD), ("r_gq_prev", _PD), ("r_zq", _PD), ("r_Hc", _PD),
    ("diag_el", _PD),
    ("n_spring", _I), ("sp_a", _PI), ("sp_b", _PI), ("sp2env", _PI),
    ("sp_k", _PD), ("sp_L0", _PD), ("sp_anchor", _PD),
    ("n_pedge", _I), ("n_chamber", _I), ("pe_a", _PI), ("pe_b", _PI), ("pe_ch", _PI), ("ch2env", _PI),
    ("ch_p", _PD), ("ch_ref", _PD),
]


class _Solver(C.Structure):
    _fields_ = _FIELDS


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        _LIB = C.CDLL(path)
        _LIB.d2o_step.argtypes = [C.POINTER(_Solver)]
        _LIB.d2o_step.restype = C.c_int
        _LIB.d2o_energy.argtypes = [C.POINTER(_Solver), _PD]
        _LIB.d2o_energy.restype = None
        _LIB.d2o_ipc_energy.argtypes = [C.POINTER(_Solver), _PD]
        _LIB.d2o_ipc_energy.restype = None
        _LIB.d2o_term.argtypes = [C.POINTER(_Solver), C.c_int, _PD]
        _LIB.d2o_term.restype = None
        _LIB.d2o_sdf.argtypes = [C.c_int] + [C.c_double] * 5 + [_PD, C.c_int, _PD]
        _LIB.d2o_sdf.restype = None
        _LIB.d2o_sdf_full.argtypes = [C.c_int] + [C.c_double] * 5 + [_PD, C.c_int, _PD, _PD, _PD]
        _LIB.d2o_sdf_full.restype = None
        _LIB.d2o_affine_hessian.argtypes = [_PD, C.c_double, C.c_double, C.c_double, _PD, _PD, _PD]
        _LIB.d2o_affine_hessian.restype = None
        _LIB.d2o_chol6_solve.argtypes = [_PD, _PD, _PD]
        _LIB.d2o_chol6_solve.restype = None
    return _LIB


SCALARS = dict(dt=1e-3, drag=1.0, dhat=1e-4, kappa=0.0, epsv=1e-3, eps=1e-10, tol_x=0.0,
               near_factor=4.0, alpha_max=3.0, area_shrink=0.1, ccd_eta=0.9, cg_guard=0.0,
               ls_tol=1e-7, gtol=0.0, iter_max=40, conv_check=8, friction=1, line_search=0, n_bt=4)


def _f64(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, np.float64))
    if shape is not None:
        a = a.reshape(shape)
    return a


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, np.int32).reshape(-1))


class OracleSolver:
    """One oracle solver over a problem dict. State arrays live in self.state (numpy)."""

    def __init__(self, prob: dict):
        L = lib()
        self._lib = L
        self.prob = prob
        keep = self._keep = []
        s = self.s = _Solver()

        def P(a, kind="d"):
            a = _f64(a) if kind == "d" else _i32(a)
            keep.append(a)
            return a.ctypes.data_as(_PD if kind == "d" else _PI), a

        N = int(np.asarray(prob["x"]).shape[0])
        T = int(np.asarray(prob["tri"]).shape[0])
        B = int(prob["B"])
        Nb = int(np.asarray(prob["bnd"]).shape[0])
        bc_idx = _i32(prob.get("bc_idx", np.zeros(0)))
        cols = _f64(prob.get("colliders", np.zeros((0, 8))), (-1, 8)).copy()   # own copy: movable
        s.N, s.T, s.B, s.Nb, s.n_bc, s.n_col = N, T, B, Nb, len(bc_idx), cols.shape[0]
        self.N, self.B = N, B
        st = self.state = {}

        def state(name, shape, init=None, kind="d"):
            if init is None:
                a = np.zeros(shape, np.float64 if kind == "d" else np.int32)
            else:
                a = (_f64(init, shape) if kind == "d" else _i32(init).reshape(shape)).copy()
            st[name] = a
            keep.append(a)
            return a.ctypes.data_as(_PD if kind == "d" else _PI)

        s.x = state("x", (N, 2), prob["x"])
        s.v = state("v", (N, 2), prob.get("v"))
        for nm in ("xn", "xhat", "grad", "grad_prev", "p", "diagH", "x0buf"):
            setattr(s, nm, state(nm, (N, 2)))
        s.mass, _ = P(prob["mass"])
        s.free_ = state("free", (N, 2), prob["free"])
        s.node2env, _ = P(prob["node2env"], "i")
        s.tri, _ = P(prob["tri"], "i")
        s.Bm, _ = P(_f64(prob["Bm"], (T, 4)))
        s.area, _ = P(prob["area"])
        s.mu, _ = P(prob["mu"])
        s.lam, _ = P(prob["lam"])
        s.tri2env, _ = P(prob["tri2env"], "i")
        s.bnd, _ = P(prob["bnd"], "i")
        s.b2e, _ = P(prob["b2e"], "i")
        s.bc_idx, _ = P(bc_idx, "i")
        s.bc_target = state("bc_target", (len(bc_idx), 2))
        if len(bc_idx):
            st["bc_target"][:] = np.asarray(prob["x"], np.float64)[bc_idx]
        s.colliders, self._cols = P(cols)
        for nm in ("gPg", "g_p", "g_Py", "y_p", "y_Py", "beta", "gTp", "pHp", "alpha", "p_inf",
                   "clr_min", "dE", "dE0", "Ener", "Els_prev", "gn0"):
            setattr(s, nm, state(nm, (B,)))
        s.active = state("active", (B,), kind="i")
        s.iters = state("iters", (B,), kind="i")
        sc = dict(SCALARS)
        sc.update({k: prob[k] for k in SCALARS if k in prob})
        dt = float(sc["dt"])
        s.dt, s.h2, s.inv_dt = dt, dt * dt, 1.0 / dt
        for k in ("drag", "dhat", "kappa", "epsv", "eps", "tol_x", "near_factor", "alpha_max",
                  "area_shrink", "ccd_eta", "cg_guard", "ls_tol", "gtol"):
            setattr(s, k, float(sc[k]))
        for k in ("iter_max", "conv_check", "friction", "line_search", "n_bt"):
            setattr(s, k, int(sc[k]))

        fext = prob.get("fext")
        s.has_ext = 0 if fext is None else 1
        s.fext = state("fext", (N, 2), fext) if fext is not None else None

        ipc = prob.get("ipc")
        s.has_ipc = 0 if ipc is None else 1
        if ipc is not None:
            s.Ne = int(len(ipc["ea"]))
            for nm in ("ea", "eb", "ela", "elb", "e2env", "bstart", "bpe", "excl_ptr", "excl_idx"):
                setattr(s, nm, P(ipc[nm], "i")[0])
            s.ca, _ = P(ipc["ca"])
            s.cb, _ = P(ipc["cb"])
            mn = ipc.get("mu_node")
            s.per_body = 0 if mn is None else int(ipc.get("per_body", 1))
            s.mu_node, _ = P(np.zeros(1) if mn is None else mn)
            s.ipc_mu = float(ipc["mu"])
            s.ipc_dhat, s.ipc_kappa = float(ipc["dhat"]), float(ipc["kappa"])
            s.reach, s.gap = float(ipc["reach"]), float(ipc.get("gap", 0.1))
            s.bc_floor = float(ipc.get("bc_floor", 0.25))
            s.q = state("ipc_q", (N, 2))
            s.q_inf = state("ipc_q_inf", (B,))
            s.sweep_beta = state("ipc_beta", (B,))
            s.clr = state("ipc_clr", (B,))

        td = prob.get("tendon")
        if td is not None and len(td["t2env"]):
            s.n_tendon, s.n_tent = len(td["t2env"]), len(td["node"])
            for nm, key in (("t_node", "node"), ("t_prv", "prv"), ("t_nxt", "nxt"), ("t_tid", "tid"),
                            ("t2env", "t2env")):
                setattr(s, nm, P(td[key], "i")[0])
            s.t_stiff, _ = P(td["stiff"])
            s.t_L0 = state("t_L0", (s.n_tendon,), td["L0"])
            s.t_Tcmd = state("t_Tcmd", (s.n_tendon,), td["Tcmd"])
            for nm in ("t_L", "t_dL", "t_tau", "t_keff"):
                setattr(s, nm, state(nm, (s.n_tendon,)))

        af = prob.get("affine")
        if af is not None and len(af["env"]):
            na, nn = len(af["env"]), len(af["node"])
            s.n_aff, s.n_affn = na, nn
            s.a_node, _ = P(af["node"], "i")
            s.a_grp, _ = P(af["grp"], "i")
            s.a_env, _ = P(af["env"], "i")
            s.a_w, _ = P(_f64(af["w"], (nn, 3)))
            s.a_Mu, _ = P(af["Mu"])
            s.a_La, _ = P(af["La"])
            s.a_q = state("a_q", (na, 6), af["q"])
            for nm in ("a_q0", "a_pq", "a_gq", "a_gq_prev", "a_zq"):
                setattr(s, nm, state(nm, (na, 6)))
            s.a_Hx = state("a_Hx", (na, 9))
            s.a_Hy = state("a_Hy", (na, 9))

        sp = prob.get("springs")
        if sp is not None and len(sp["env"]):
            s.n_spring = len(sp["env"])
            s.sp_a, _ = P(sp["a"], "i")
            s.sp_b, _ = P(sp["b"], "i")
            s.sp2env, _ = P(sp["env"], "i")
            s.sp_k, _ = P(sp["k"])
            s.sp_L0 = state("sp_L0", (s.n_spring,), sp["L0"])
            s.sp_anchor = state("sp_anchor", (s.n_spring, 2), sp["anchor"])

        pr = prob.get("pressure")
        if pr is not None and len(pr["ea"]):
            s.n_pedge, s.n_chamber = len(pr["ea"]), len(pr["ch2env"])
            s.pe_a, _ = P(pr["ea"], "i")
            s.pe_b, _ = P(pr["eb"], "i")
            s.pe_ch, _ = P(pr["ch"], "i")
            s.ch2env, _ = P(pr["ch2env"], "i")
            s.ch_p = state("ch_p", (s.n_chamber,), pr["p"])
            s.ch_ref = state("ch_ref", (s.n_chamber, 2), pr["ref"])

        rg = prob.get("rigid")
        if rg is not None and len(rg["env"]):
            nr, nn = len(rg["env"]), len(rg["node"])
            s.n_rig, s.n_rign = nr, nn
            s.r_node, _ = P(rg["node"], "i")
            s.r_grp, _ = P(rg["grp"], "i")
            s.r_env, _ = P(rg["env"], "i")
            s.r_acc = state("r_acc", (nr, 3))
            for nm in ("r_gq", "r_gq_prev", "r_zq"):
                setattr(s, nm, state(nm, (nr, 3)))
            s.r_Hc = state("r_Hc", (nr, 9))
            s.diag_el = state("diag_el", (N, 2))

    # ---- commands ----
    def set_bc_target(self, t):
        if len(self.state["bc_target"]):
            self.state["bc_target"][:] = np.asarray(t, np.float64).reshape(-1, 2)

    def set_tendon(self, Tcmd=None, L0=None):
        if Tcmd is not None:
            self.state["t_Tcmd"][:] = np.asarray(Tcmd, np.float64)
        if L0 is not None:
            self.state["t_L0"][:] = np.asarray(L0, np.float64)

    def term(self, which, x, p=None, xn=None):
        """One term alone (which: "springs", "pressure" or "ipc") at positions x:
        (gradient (N, 2), diagonal (N, 2), curvature along p per environment, energy per
        environment) — for derivative checks."""
        st = self.state
        st["x"][:] = np.asarray(x, np.float64)
        if xn is not None:
            st["xn"][:] = np.asarray(xn, np.float64)
        st["p"][:] = 0.0 if p is None else np.asarray(p, np.float64)
        E = np.zeros(int(self.s.B))
        lib().d2o_term(C.byref(self.s), {"springs": 0, "pressure": 1, "ipc": 2}[which], E.ctypes.data_as(_PD))
        return st["grad"].copy(), st["diagH"].copy(), st["pHp"].copy(), E

    def set_pressure(self, p):
        """Gauge pressure of every chamber [Pa]."""
        self.state["ch_p"][:] = np.asarray(p, np.float64)

    def set_springs(self, anchor=None, L0=None):
        """World anchors (n, 2) and rest lengths of the springs."""
        if anchor is not None:
            self.state["sp_anchor"][:] = np.asarray(anchor, np.float64).reshape(-1, 2)
        if L0 is not None:
            self.state["sp_L0"][:] = np.asarray(L0, np.float64)

    def set_collider_centers(self, centers):
        """Move the colliders ((n_col, 2) centres) before the next step."""
        c = np.asarray(centers, np.float64).reshape(-1, 2)
        self._cols[: len(c), 1:3] = c

    def set_fext(self, f):
        self.state["fext"][:] = np.asarray(f, np.float64).reshape(-1, 2)

    def step(self):
        rc = self._lib.d2o_step(C.byref(self.s))
        if rc != 0:
            raise RuntimeError(f"oracle step failed: {rc}")

    def energy(self):
        out = np.zeros(self.B)
        self._lib.d2o_energy(C.byref(self.s), out.ctypes.data_as(_PD))
        return out

    def ipc_energy(self, x=None, xn=None):
        """The IPC contact energy per environment (barrier + lagged friction) at x, slip from
        xn; x and xn default to the solver's current state."""
        if x is not None:
            self.state["x"][:] = np.asarray(x, np.float64).reshape(-1, 2)
        if xn is not None:
            self.state["xn"][:] = np.asarray(xn, np.float64).reshape(-1, 2)
        out = np.zeros(self.B)
        self._lib.d2o_ipc_energy(C.byref(self.s), out.ctypes.data_as(_PD))
        return out

    @property
    def x(self):
        return self.state["x"]

    @property
    def v(self):
        return self.state["v"]


def run(prob: dict, steps: int, commands=None):
    """Run `steps` steps; commands(k) -> dict(bc_target=..., Tcmd=..., fext=...) or None.
    Returns (solver, list of x after each step, list of iters)."""
    s = OracleSolver(prob)
    xs, its = [], []
    for k in range(steps):
        c = commands(k) if commands is not None else None
        if c:
            if c.get("bc_target") is not None:
                s.set_bc_target(c["bc_target"])
            if c.get("Tcmd") is not None or c.get("L0") is not None:
                s.set_tendon(c.get("Tcmd"), c.get("L0"))
            if c.get("fext") is not None:
                s.set_fext(c["fext"])
        s.step()
        xs.append(s.x.copy())
        its.append(s.state["iters"].copy())
    return s, xs, its


def sdf(collider_row, pts):
    """A collider's level set (row of the problem's `colliders`: kind, cx, cy, rx, ry, rref,
    r, mu) at points (n, 2): the oracle's sdf_eval, the disc's |x - c| - r."""
    c = np.asarray(collider_row, np.float64)
    P = _f64(pts, (-1, 2))
    d = np.zeros(len(P))
    kind = int(c[0])
    rx = c[6] if kind == 0 else c[3]
    lib().d2o_sdf(kind, c[1], c[2], rx, c[4], c[5], P.ctypes.data_as(_PD), len(P), d.ctypes.data_as(_PD))
    return d


def sdf_full(collider_row, pts):
    """A collider's level set with its gradient and Hessian at points (n, 2): (d (n,),
    g (n, 2), H (n, 2, 2)) — the oracle's sdf_eval (any kind but the disc's closed form)."""
    c = np.asarray(collider_row, np.float64)
    P = _f64(pts, (-1, 2))
    d, g, H = np.zeros(len(P)), np.zeros((len(P), 2)), np.zeros((len(P), 4))
    lib().d2o_sdf_full(int(c[0]), c[1], c[2], c[3], c[4], c[5], P.ctypes.data_as(_PD), len(P),
                       d.ctypes.data_as(_PD), g.ctypes.data_as(_PD), H.ctypes.data_as(_PD))
    return d, g, H.reshape(-1, 2, 2)


def affine_hessian(A, Mu, La, h2=1.0, Hx=None, Hy=None):
    """The 6x6 reduced Hessian of an affine region (q = t_x, A11, A12, t_y, A21, A22) at the
    2x2 map A with the region's summed moduli: the mass blocks Hx, Hy (3x3, default 0) plus
    h2 times the elastic block, its negative twist curvature removed (the oracle's
    reduced_hessian)."""
    A4 = _f64(np.asarray(A, np.float64).reshape(4))
    Hx = _f64(np.zeros(9) if Hx is None else np.asarray(Hx, np.float64).reshape(9))
    Hy = _f64(np.zeros(9) if Hy is None else np.asarray(Hy, np.float64).reshape(9))
    out = np.zeros(36)
    lib().d2o_affine_hessian(A4.ctypes.data_as(_PD), float(Mu), float(La), float(h2), Hx.ctypes.data_as(_PD),
                             Hy.ctypes.data_as(_PD), out.ctypes.data_as(_PD))
    return out.reshape(6, 6)


def chol6_solve(H, b):
    """x with H x = b by the oracle's 6x6 Cholesky (diagonal fallback when H is not SPD)."""
    H36 = _f64(np.asarray(H, np.float64).reshape(36))
    bb = _f64(np.asarray(b, np.float64).reshape(6))
    x = np.zeros(6)
    lib().d2o_chol6_solve(H36.ctypes.data_as(_PD), bb.ctypes.data_as(_PD), x.ctypes.data_as(_PD))
    return x


def problem_keys():
    return ["B", "x", "v", "mass", "free", "node2env", "tri", "Bm", "area", "mu", "lam", "tri2env",
            "bnd", "b2e", "bc_idx", "colliders", "fext", "ipc", "tendon", "affine", "rigid", "springs",
            "pressure"] + list(SCALARS)


os.environ.setdefault("OMP_NUM_THREADS", "1")
