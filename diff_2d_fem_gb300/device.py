"""The GPU solver: a problem dict laid out in device memory (PyTorch tensors) and bound to
a libd2f handle.

Layout in HBM (all scenes back to back, scene by scene):
  node arrays      x, v, xn, xhat (FP64 pairs); grad, grad_prev, p, diagH, diag_el (real
                   pairs: FP64, or FP32 in mixed precision); mass, free mask, force
  triangle arrays  tri (int32 x3), Bm (real x4), area, mu, lam (real); per-corner scratch
                   (real x4 per corner) and a per-triangle cache (real x9)
  node -> corner   CSR (ascending triangle per node): the elastic gather
  boundary         slots, kinematic slots, IPC edges and the sparse exclusion lists
  per scene        a d2f_seg of index ranges; iters / active / status outputs
Index arrays are int32; everything that must not lose precision is FP64.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def _ranges(ids, B):
    """[start, count) per env of a nondecreasing env-id array."""
    ids = np.asarray(ids, np.int64)
    if len(ids) and np.any(np.diff(ids) < 0):
        raise ValueError("per-environment arrays must be grouped by environment")
    starts = np.searchsorted(ids, np.arange(B), side="left")
    ends = np.searchsorted(ids, np.arange(B), side="right")
    return starts, ends - starts


class DeviceSolver:
    """Binds a problem to device memory and a libd2f handle. `precision`: "fp64" or
    "mixed". threads / blocks_per_sm: the scene-block launch shape (0 = library default).
    blocks_per_scene (mixed): blocks of one cluster per scene, 1, 8, 12 or 16 (0 = library default)."""

    def __init__(self, prob, precision="fp64", threads=0, blocks_per_sm=0, device="cuda", stream=None,
                 blocks_per_scene=0):
        if torch is None:
            raise RuntimeError("PyTorch is required for device buffers")
        if not torch.cuda.is_available():
            raise RuntimeError("no CUDA device: the implicit step runs on the GPU only")
        self.L = _lib.load()
        self.dev = torch.device(device)
        self.mixed = precision == "mixed"
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.rdt = torch.float32 if self.mixed else torch.float64
        self.prob = prob
        self._t = {}
        B = int(prob["B"])
        self.B = B
        x = np.asarray(prob["x"], np.float64)
        N = x.shape[0]
        self.N = N
        tri = np.asarray(prob["tri"], np.int64)
        T = tri.shape[0]
        node2env = np.asarray(prob["node2env"], np.int64)
        n_s, n_c = _ranges(node2env, B)
        t_s, t_c = _ranges(prob["tri2env"], B)
        bnd = np.asarray(prob["bnd"], np.int64)
        b_s, b_c = _ranges(prob["b2e"], B)
        Nb = len(bnd)

        segs = np.zeros((B, 28), np.int32)
        segs[:, 0], segs[:, 1] = n_s, n_c
        segs[:, 2], segs[:, 3] = t_s, t_c
        segs[:, 4], segs[:, 5] = b_s, b_c

        node_bslot = np.full(N, -1, np.int64)
        node_bslot[bnd] = np.arange(Nb)

        # kinematic nodes, ascending (hence grouped by environment)
        bc = np.asarray(prob.get("bc_idx", np.zeros(0)), np.int64)
        self.bc_order = np.argsort(bc, kind="stable")
        bc_sorted = bc[self.bc_order]
        k_s, k_c = _ranges(node2env[bc_sorted], B)
        segs[:, 10], segs[:, 11] = k_s, k_c
        node_bc = np.full(N, -1, np.int64)
        node_bc[bc_sorted] = np.arange(len(bc_sorted))
        self.bc_sorted = bc_sorted

        # IPC edges and the candidate lists
        ipc = prob.get("ipc")
        Ne = 0
        cand_total = 0
        max_nb = int(b_c.max()) if B else 0
        if ipc is not None and len(ipc["ea"]):
            Ne = len(ipc["ea"])
            e_s, e_c = _ranges(ipc["e2env"], B)
            segs[:, 6], segs[:, 7] = e_s, e_c
            if e_c.max() >= 32768 or b_c.max() >= 65536:
                raise ValueError("a scene has too many boundary edges or nodes for the per-scene kernel")
            # every pair of a small scene, else 32 per edge (pixel outlines keep a handful)
            cap = np.where(e_c > 0, np.minimum(e_c * b_c, np.maximum(32 * e_c, 2048)), 0)
            segs[:, 8] = np.concatenate([[0], np.cumsum(cap)[:-1]])
            segs[:, 9] = cap
            cand_total = int(cap.sum())

        # affine regions, grouped by environment
        af = prob.get("affine")
        n_aff = n_affn = 0
        node_aff = np.full(N, -1, np.int64)
        if af is not None and len(af["env"]):
            env = np.asarray(af["env"], np.int64)
            rorder = np.argsort(env, kind="stable")
            rnew = np.empty_like(rorder)
            rnew[rorder] = np.arange(len(rorder))
            grp = rnew[np.asarray(af["grp"], np.int64)]
            eorder = np.argsort(grp, kind="stable")
            self.aff_order = rorder
            af = dict(node=np.asarray(af["node"], np.int64)[eorder], grp=grp[eorder],
                      w=np.asarray(af["w"], np.float64)[eorder], env=env[rorder],
                      Mu=np.asarray(af["Mu"], np.float64)[rorder], La=np.asarray(af["La"], np.float64)[rorder],
                      q=np.asarray(af["q"], np.float64)[rorder])
            n_aff, n_affn = len(af["env"]), len(af["node"])
            a_s, a_c = _ranges(af["env"], B)
            segs[:, 12], segs[:, 13] = a_s, a_c
            an_s, an_c = _ranges(af["env"][af["grp"]], B)
            segs[:, 14], segs[:, 15] = an_s, an_c
            node_aff[af["node"]] = np.arange(n_affn)
        self.af = af

        rg = prob.get("rigid")
        n_rig = n_rign = 0
        node_rig = np.full(N, -1, np.int64)
        if rg is not None and len(rg["env"]):
            env = np.asarray(rg["env"], np.int64)
            rorder = np.argsort(env, kind="stable")
            rnew = np.empty_like(rorder)
            rnew[rorder] = np.arange(len(rorder))
            grp = rnew[np.asarray(rg["grp"], np.int64)]
            eorder = np.argsort(grp, kind="stable")
            rg = dict(node=np.asarray(rg["node"], np.int64)[eorder], grp=grp[eorder], env=env[rorder])
            n_rig, n_rign = len(rg["env"]), len(rg["node"])
            r_s, r_c = _ranges(rg["env"], B)
            segs[:, 16], segs[:, 17] = r_s, r_c
            rn_s, rn_c = _ranges(rg["env"][rg["grp"]], B)
            segs[:, 18], segs[:, 19] = rn_s, rn_c
            node_rig[rg["node"]] = np.arange(n_rign)

        td = prob.get("tendon")
        n_ten = n_tent = 0
        if td is not None and len(td["t2env"]):
            t2env = np.asarray(td["t2env"], np.int64)
            torder = np.argsort(t2env, kind="stable")
            tnew = np.empty_like(torder)
            tnew[torder] = np.arange(len(torder))
            tid = tnew[np.asarray(td["tid"], np.int64)]
            eorder = np.argsort(tid, kind="stable")
            enew = np.empty_like(eorder)
            enew[eorder] = np.arange(len(eorder))
            remap = lambda a: np.where(np.asarray(a, np.int64) >= 0, enew[np.maximum(np.asarray(a, np.int64), 0)], -1)
            self.ten_order = torder
            td = dict(node=np.asarray(td["node"], np.int64)[eorder], prv=remap(td["prv"])[eorder],
                      nxt=remap(td["nxt"])[eorder], tid=tid[eorder], t2env=t2env[torder],
                      stiff=np.asarray(td["stiff"], np.float64)[torder],
                      L0=np.asarray(td["L0"], np.float64)[torder], Tcmd=np.asarray(td["Tcmd"], np.float64)[torder])
            n_ten, n_tent = len(td["t2env"]), len(td["node"])
            te_s, te_c = _ranges(td["t2env"], B)
            segs[:, 20], segs[:, 21] = te_s, te_c
            tn_s, tn_c = _ranges(td["t2env"][td["tid"]], B)
            segs[:, 22], segs[:, 23] = tn_s, tn_c
        self.td = td

        # springs and pins, grouped by environment
        sp = prob.get("springs")
        n_sp = 0
        self.sp_order = None
        if sp is not None and len(sp["env"]):
            self.sp_order = np.argsort(np.asarray(sp["env"], np.int64), kind="stable")
            sp = {k: np.asarray(v)[self.sp_order] for k, v in sp.items()}
            n_sp = len(sp["env"])
            segs[:, 24], segs[:, 25] = _ranges(sp["env"], B)
        # pressure boundary edges, grouped by their chamber's environment
        pr = prob.get("pressure")
        n_pe = n_ch = 0
        if pr is not None and len(pr["ea"]):
            ch2env = np.asarray(pr["ch2env"], np.int64)
            ch = np.asarray(pr["ch"], np.int64)
            eo = np.argsort(ch2env[ch], kind="stable")
            pr = dict(pr, ea=np.asarray(pr["ea"])[eo], eb=np.asarray(pr["eb"])[eo], ch=ch[eo])
            n_pe, n_ch = len(pr["ea"]), len(ch2env)
            segs[:, 26], segs[:, 27] = _ranges(ch2env[pr["ch"]], B)
        self.sp, self.pr = sp, pr

        # node -> corner CSR, ascending triangle per node
        corner_node = tri.reshape(-1)
        order = np.argsort(corner_node, kind="stable")
        inc_ptr = np.zeros(N + 1, np.int64)
        inc_ptr[1:] = np.cumsum(np.bincount(corner_node, minlength=N))

        free = np.asarray(prob["free"], np.float64)
        free_mask = ((free[:, 0] > 0.5).astype(np.uint8) | ((free[:, 1] > 0.5).astype(np.uint8) << 1))

        f64, i32, rdt = torch.float64, torch.int32, self.rdt
        T_ = self._put
        self.segs = T_("segs", segs, torch.int32)
        self.x = T_("x", x, f64)
        self.v = T_("v", np.asarray(prob.get("v", np.zeros_like(x)), np.float64), f64)
        self.xn = T_("xn", np.zeros_like(x), f64)
        if self.mixed:
            # the FP32 iterations work on increments from the step start and on displacements
            # from the rest shape (rest edge vectors per triangle)
            rest = np.asarray(prob.get("rest", x), np.float64)
            T_("xrest", rest, f64)
            Dm = prob.get("Dm")
            if Dm is None:
                Dm = np.concatenate([rest[tri[:, 1]] - rest[tri[:, 0]], rest[tri[:, 2]] - rest[tri[:, 0]]], 1)
            T_("Dm", np.asarray(Dm, np.float64).reshape(T, 4), f64)
        self.xhat = T_("xhat", np.zeros_like(x), f64)
        for nm in ("grad", "grad_prev", "p", "diagH", "diag_el"):
            T_(nm, np.zeros((N, 2)), rdt)
        T_("mass", prob["mass"], f64)
        T_("free_mask", free_mask, torch.uint8)
        fext = prob.get("fext")
        if fext is not None:
            T_("fext", fext, f64)
        T_("inc_ptr", inc_ptr, i32)
        T_("inc", order, i32)
        inc8 = np.full((N, 8), -1, np.int64)
        cnt = np.diff(inc_ptr)
        slot = np.arange(len(order)) - np.repeat(inc_ptr[:-1], cnt)
        first8 = slot < 8
        inc8[np.repeat(np.arange(N), cnt)[first8], slot[first8]] = order[first8]
        T_("inc8", inc8, i32)
        T_("node_bslot", node_bslot, i32)
        T_("node_bc", node_bc, i32)
        T_("node_aff", node_aff, i32)
        T_("node_rig", node_rig, i32)
        T_("tri", tri, i32)
        T_("Bm", np.asarray(prob["Bm"], np.float64).reshape(T, 4), rdt)
        T_("area", prob["area"], rdt)
        T_("mu", prob["mu"], rdt)
        T_("lam", prob["lam"], rdt)
        T_("escr", np.zeros((T, 12)), rdt)
        T_("ecache", np.zeros((T, 9)), rdt)
        T_("bnd", bnd, i32)
        cols = np.asarray(prob.get("colliders", np.zeros((0, 8))), np.float64).reshape(-1, 8)
        T_("colliders", cols if len(cols) else np.zeros((1, 8)), f64)
        if prob.get("col_mu_env") is not None:
            T_("col_mu_env", np.asarray(prob["col_mu_env"], np.float64), f64)
        T_("bc_idx", bc_sorted if len(bc_sorted) else np.zeros(1), i32)
        tg = x[bc_sorted] if len(bc_sorted) else np.zeros((1, 2))
        self.bc_target = T_("bc_target", tg, f64)
        if Ne:
            for nm in ("ea", "eb", "ela", "elb"):
                T_(nm, ipc[nm], i32)
            T_("ca", ipc["ca"], f64)
            T_("cb", ipc["cb"], f64)
            T_("excl_ptr", ipc["excl_ptr"], i32)
            T_("excl_idx", ipc["excl_idx"] if len(ipc["excl_idx"]) else np.zeros(1), i32)
            if ipc.get("mu_node") is not None and ipc.get("per_body", 1):
                T_("mu_node", ipc["mu_node"], f64)
            T_("cand", np.zeros(max(cand_total, 1)), i32)
            T_("cand_tr", np.zeros((max(cand_total, 1), 2)), f64)
            T_("xref", np.zeros((Nb, 2)), f64)
        if td is not None:
            for nm, key in (("t_node", "node"), ("t_prv", "prv"), ("t_nxt", "nxt"), ("t_tid", "tid")):
                T_(nm, td[key], i32)
            T_("t_stiff", td["stiff"], f64)
            T_("t_L0", td["L0"], f64)
            T_("t_Tcmd", td["Tcmd"], f64)
            T_("t_state", np.zeros((n_ten, 4)), f64)
        if sp is not None and n_sp:
            T_("sp_a", sp["a"], i32)
            T_("sp_b", sp["b"], i32)
            T_("sp_k", sp["k"], f64)
            T_("sp_L0", sp["L0"], f64)
            T_("sp_anchor", np.asarray(sp["anchor"], np.float64).reshape(-1, 2), f64)
        if pr is not None and n_pe:
            T_("pe_a", pr["ea"], i32)
            T_("pe_b", pr["eb"], i32)
            T_("pe_ch", pr["ch"], i32)
            T_("ch_p", pr["p"], f64)
            T_("ch_ref", np.asarray(pr["ref"], np.float64).reshape(-1, 2), f64)
        if af is not None:
            T_("a_node", af["node"], i32)
            T_("a_grp", af["grp"], i32)
            T_("a_ptr", np.searchsorted(af["grp"], np.arange(n_aff + 1)), i32)
            T_("a_w", af["w"], f64)
            T_("a_Mu", af["Mu"], f64)
            T_("a_La", af["La"], f64)
            T_("a_q", af["q"], f64)
            for nm in ("a_pq", "a_gq", "a_gq_prev", "a_zq"):
                T_(nm, np.zeros((n_aff, 6)), f64)
            T_("a_H", np.zeros((n_aff, 18)), f64)
        if rg is not None:
            T_("r_node", rg["node"], i32)
            T_("r_grp", rg["grp"], i32)
            T_("r_acc", np.zeros((n_rig, 3)), f64)
            T_("r_zq", np.zeros((n_rig, 3)), f64)
        if self.mixed:
            n_rig_ = len(rg["env"]) if rg is not None else 0
            ncol_ = len(np.asarray(prob.get("colliders", np.zeros((0, 8)))).reshape(-1, 8))
            nbytes = int(self.L.d2f_mixed_scratch_bytes(N, T, Nb, ncol_, n_rig_))
            self._t["mscr"] = torch.zeros(nbytes, dtype=torch.uint8, device=self.dev)
        T_("iters", np.zeros(B), i32)
        T_("active", np.zeros(B), i32)
        T_("status", np.zeros(B), i32)
        T_("work", np.zeros(4), i32)

        d = self.desc = _lib.SceneDesc()
        d.abi_version = _lib.D2F_ABI_VERSION
        d.precision = _lib.D2F_MIXED if self.mixed else _lib.D2F_FP64
        d.n_scenes, d.N, d.T, d.Nb, d.Ne, d.n_bc, d.n_col = B, N, T, Nb, Ne, len(bc_sorted), len(cols)
        d.n_aff, d.n_affn, d.n_rig, d.n_rign, d.n_ten, d.n_tent = n_aff, n_affn, n_rig, n_rign, n_ten, n_tent
        d.cand_total, d.max_nb = cand_total, max_nb
        d.n_sp, d.n_pe, d.n_ch = n_sp, n_pe, n_ch
        for name, _ in _lib.DESC_FIELDS:
            if _ is C.c_void_p and name in self._t:
                setattr(d, name, self._t[name].data_ptr())
        sc = prob
        d.dt, d.drag, d.dhat, d.kappa, d.epsv = sc["dt"], sc["drag"], sc["dhat"], sc["kappa"], sc["epsv"]
        d.eps, d.tol_x, d.near_factor, d.alpha_max = sc["eps"], sc["tol_x"], sc["near_factor"], sc["alpha_max"]
        d.area_shrink, d.ccd_eta, d.cg_guard, d.gtol = sc["area_shrink"], sc["ccd_eta"], sc.get("cg_guard", 0.0), sc.get("gtol", 0.0)
        d.iter_max, d.conv_check, d.friction = int(sc["iter_max"]), int(sc["conv_check"]), int(sc["friction"])
        if Ne:
            d.ipc_mu, d.ipc_dhat, d.ipc_kappa = float(ipc["mu"]), float(ipc["dhat"]), float(ipc["kappa"])
            d.reach, d.gap, d.bc_floor = float(ipc["reach"]), float(ipc.get("gap", 0.1)), float(ipc.get("bc_floor", 0.25))
            d.skin = d.reach
            d.per_body = int(ipc.get("per_body", 0)) if ipc.get("mu_node") is not None else 0
        d.threads = int(threads or 0)
        d.blocks_per_sm = int(blocks_per_sm or 0)
        d.blocks_per_scene = int(blocks_per_scene or 0)
        if int(sc.get("line_search", 0)):
            # saved positions (FP64 pairs; the mixed kernel keeps its FP32 offsets there), then
            # the affine bodies' coordinates
            self._t["xu"] = torch.zeros(2 * N + 6 * n_aff, dtype=torch.float64, device=self.dev)
            d.xu = self._t["xu"].data_ptr()
            d.line_search, d.n_backtrack, d.ls_tol = 1, int(sc.get("n_bt", 4)), float(sc.get("ls_tol", 1e-7))
        h = C.c_void_p()
        torch.cuda.synchronize(self.dev)
        _lib.check(self.L.d2f_create(C.byref(d), C.byref(h)), "d2f_create")
        self.h = h
        self.stream = stream

    def _put(self, name, arr, dtype):
        t = torch.as_tensor(np.ascontiguousarray(arr)).to(dtype=dtype, device=self.dev).contiguous()
        self._t[name] = t
        return t

    def tensor(self, name):
        return self._t[name]

    # ---- step
    def _stream_ptr(self):
        s = self.stream if self.stream is not None else torch.cuda.current_stream(self.dev)
        return C.c_void_p(s.cuda_stream)

    def step(self):
        _lib.check(self.L.d2f_step(self.h, self._stream_ptr()), "d2f_step")

    def step_noalloc(self):
        """The same step through d2f_step_noalloc: this solver's inputs and outputs, the
        library's static scratch instead of this solver's scratch buffers."""
        _lib.check(self.L.d2f_step_noalloc(C.byref(self.desc), self._stream_ptr()), "d2f_step_noalloc")

    def set_dt(self, dt, iter_max):
        self.desc.dt = float(dt)
        _lib.check(self.L.d2f_set_dt(self.h, float(dt), int(iter_max)), "d2f_set_dt")

    # ---- commands
    def set_targets(self, targets_full):
        if len(self.bc_sorted):
            tg = np.asarray(targets_full, np.float64)[self.bc_sorted]
            self._t["bc_target"].copy_(torch.as_tensor(tg))

    def set_fext(self, f):
        if "fext" not in self._t:
            raise RuntimeError("this solver was built without an external-force term")
        self._t["fext"].copy_(torch.as_tensor(np.asarray(f, np.float64)))

    def set_tendons(self, Tcmd=None, L0=None):
        if self.td is None:
            return
        if Tcmd is not None:
            self._t["t_Tcmd"].copy_(torch.as_tensor(np.asarray(Tcmd, np.float64)[self.ten_order]))
        if L0 is not None:
            self._t["t_L0"].copy_(torch.as_tensor(np.asarray(L0, np.float64)[self.ten_order]))

    def energy(self):
        """Total energy of every scene at the current state (PNCG2DSolver.energy,
        implicit/solver.py:500-502), (B,); FP64 solvers."""
        out = torch.empty(self.B, dtype=torch.float64, device=self.dev)
        _lib.check(self.L.d2f_energy(self.h, out.data_ptr(), self._stream_ptr()), "d2f_energy")
        return out.cpu().numpy()

    # ---- contact read-outs (implicit/solver.py:553-612), on the device
    def contact_force(self, friction=True, colliders=True, bodies=True):
        """Force that contact exerts ON each node [N/m], (N, 2): the colliders' barrier and
        the contact between bodies, with friction unless friction=False; kinematic nodes
        included. Evaluated where the bodies are now, with the slip of the last step."""
        out = torch.empty((self.N, 2), dtype=torch.float64, device=self.dev)
        flags = (1 if colliders else 0) | (2 if bodies else 0) | (4 if friction else 0)
        _lib.check(self.L.d2f_contact_force(self.h, 0, -1, flags, out.data_ptr(), self._stream_ptr()),
                   "d2f_contact_force")
        return out.cpu().numpy()

    def collider_force(self, index=None, include_friction=False):
        """Reaction on the colliders per environment (B, 2): on collider `index`, or on all of
        them together when index is None."""
        out = torch.empty((self.B, 2), dtype=torch.float64, device=self.dev)
        _lib.check(self.L.d2f_contact_force(self.h, 1, -1 if index is None else int(index),
                                            4 if include_friction else 0, out.data_ptr(), self._stream_ptr()),
                   "d2f_contact_force")
        return out.cpu().numpy()

    def set_collider_centers(self, centers):
        """Centres (n_col, 2) of the colliders, in the model's order, read by the next step
        (and by the contact read-outs)."""
        c = np.asarray(centers, np.float64).reshape(-1, 2)
        if len(c):
            self._t["colliders"][: len(c), 1:3].copy_(torch.as_tensor(c))

    def set_pressures(self, p):
        """Gauge pressure of every chamber [Pa], in the model's chamber order."""
        if self.pr is None:
            return
        self._t["ch_p"].copy_(torch.as_tensor(np.asarray(p, np.float64)))

    def set_springs(self, anchor=None, L0=None):
        """World anchors ((n, 2)) and rest lengths of the springs, in the model's order."""
        if self.sp_order is None:
            return
        if anchor is not None:
            a = np.asarray(anchor, np.float64).reshape(-1, 2)[self.sp_order]
            self._t["sp_anchor"].copy_(torch.as_tensor(a))
        if L0 is not None:
            self._t["sp_L0"].copy_(torch.as_tensor(np.asarray(L0, np.float64)[self.sp_order]))

    def set_rest_shape(self, Bm, area, Dm):
        """Every triangle's rest-shape inverse, rest area and rest edge vectors (the active
        regions' rest-shape change; ActiveStrain.set, implicit/actuation.py:335-341)."""
        T = self.desc.T
        self._t["Bm"].copy_(torch.as_tensor(np.asarray(Bm, np.float64).reshape(T, 4)))
        self._t["area"].copy_(torch.as_tensor(np.asarray(area, np.float64)))
        if "Dm" in self._t:
            self._t["Dm"].copy_(torch.as_tensor(np.asarray(Dm, np.float64).reshape(T, 4)))

    # ---- state
    def get_x(self):
        return self.x.cpu().numpy()

    def get_v(self):
        return self.v.cpu().numpy()

    def get_affine_q(self):
        if self.af is None:
            return np.zeros((0, 6))
        q = self._t["a_q"].cpu().numpy()
        out = np.empty_like(q)
        out[self.aff_order] = q
        return out

    def stats(self):
        B = self.B
        it = np.zeros(B, np.int32)
        ac = np.zeros(B, np.int32)
        st = np.zeros(B, np.int32)
        torch.cuda.synchronize(self.dev)
        _lib.check(self.L.d2f_stats(self.h, self._stream_ptr(), it.ctypes.data, ac.ctypes.data, st.ctypes.data),
                   "d2f_stats")
        return it, ac, st

    def launch_shape(self):
        """(blocks launched, threads per block, blocks per scene) of this solver's step."""
        b, t, c = C.c_int32(), C.c_int32(), C.c_int32()
        _lib.check(self.L.d2f_launch_shape(self.h, C.byref(b), C.byref(t), C.byref(c)), "d2f_launch_shape")
        return b.value, t.value, c.value

    def set_nodes(self, nodes, x=None, v=None, xn=False):
        idx = torch.as_tensor(np.asarray(nodes, np.int64), device=self.dev)
        if x is not None:
            xt = torch.as_tensor(np.asarray(x, np.float64), device=self.dev)
            self.x[idx] = xt
            if xn:
                self.xn[idx] = xt
        if v is not None:
            self.v[idx] = torch.as_tensor(np.asarray(v, np.float64), device=self.dev)

    def sync_affine(self, regions=None):
        """Fit each affine region's q to its nodes' positions (least squares, on the host)
        and move the slaved nodes to J q (implicit/affine.py:331-344)."""
        if self.af is None:
            return
        x = self.get_x()
        q = self._t["a_q"].cpu().numpy()
        af = self.af
        sel = range(len(af["env"])) if regions is None else [int(np.nonzero(self.aff_order == r)[0][0]) for r in regions]
        for b in sel:
            k = af["grp"] == b
            sol = np.linalg.lstsq(af["w"][k], x[af["node"][k]], rcond=None)[0]
            q[b, :3], q[b, 3:] = sol[:, 0], sol[:, 1]
        self._t["a_q"].copy_(torch.as_tensor(q))
        for nm in ("a_pq", "a_gq", "a_gq_prev"):
            self._t[nm].zero_()
        w, qg = af["w"], q[af["grp"]]
        x[af["node"], 0] = w[:, 0] * qg[:, 0] + w[:, 1] * qg[:, 1] + w[:, 2] * qg[:, 2]
        x[af["node"], 1] = w[:, 0] * qg[:, 3] + w[:, 1] * qg[:, 4] + w[:, 2] * qg[:, 5]
        self.x.copy_(torch.as_tensor(x))

    def reset_envs(self, pick, rest=None):
        """Environments flagged in pick ((B,) 0/1, or None = all) back to rest at zero
        velocity (solver.py:34-43, 535-542)."""
        rest = np.asarray(self.prob["rest"] if rest is None else rest, np.float64)
        if pick is None:
            self.x.copy_(torch.as_tensor(rest))
            self.v.zero_()
            self.xn.zero_()
        else:
            nodes = np.nonzero(np.asarray(pick)[np.asarray(self.prob["node2env"])] != 0)[0]
            self.set_nodes(nodes, x=rest[nodes], v=np.zeros((len(nodes), 2)), xn=True)
        self.sync_affine()

    def close(self):
        if getattr(self, "h", None):
            self.L.d2f_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
