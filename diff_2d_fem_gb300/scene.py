"""The solver problem of a finalized Model: every array the step needs, host side.

This is the reference's ImplicitIntegrator._build (implicit/integrator.py:252-311) together
with the constructors it calls — PNCG2DSolver.__init__ (implicit/solver.py:97-226),
AffineBodies.__init__ (implicit/affine.py:282-328), IPCContact.__init__
(implicit/ipc_contact.py:353-386), RigidModes.build (implicit/affine.py:503-523) and the
actuation sync (implicit/integrator.py:151-229) — producing the same arrays in the same
order. The result is a plain dict (the "problem"), consumed by the GPU solver
(device.py); the test suite's oracle reads the same dict.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.sparse import coo_matrix
from scipy.sparse.csgraph import connected_components


def cfl_number(model, dt):
    """The acoustic CFL number of a step: the largest c_p dt / h over the bodies that are
    not kinematic, c_p = sqrt((lambda + 2 mu) / rho) of their stiffest non-rigid element and
    h the body's CFL length (implicit/integrator.py:88-122)."""
    me = model.me
    wave = (np.asarray(me.lam, np.float64) + 2.0 * np.asarray(me.mu, np.float64))
    rigid = np.zeros(len(wave), bool)
    for piece in model._affine:
        rigid[piece.elems] = True
    C = 0.0
    for h, b in enumerate(model._bodies):
        el = model._tri_range[h]
        el = el[~rigid[el]]
        if b.role == "kinematic" or not len(el):
            continue
        C = max(C, np.sqrt(wave[el].max() / b.rho) * dt / model._cfl_length(h))
    return float(C)


def iters_for(model, integ, dt):
    """Iteration budget of a step (implicit/integrator.py:88-122): iters_per_cfl x the
    acoustic CFL number of the stiffest soft body, clipped to [40 (120 with IPC contact
    between bodies), max_iter_cap]. Batch-global, as in the reference."""
    if integ.max_iter is not None:
        return int(integ.max_iter)
    C = cfl_number(model, dt)
    n = int(np.ceil(integ.iters_per_cfl * C))
    lo = 120 if integ.self_collision and model.body_contact == "ipc" else 40
    return int(np.clip(n, lo, integ.max_iter_cap))


def _affine_arrays(model, mu_s, lam_s, free, x):
    """AffineBodies (implicit/affine.py:282-344): slaved node lists, the 6-DOF maps, the
    region moduli summed over area; zeroes the regions' own elements in mu_s/lam_s and
    returns q fitted to x (least squares), with x's slaved nodes moved to J q."""
    me = model.me
    tri = np.asarray(me.tri)
    mass = np.asarray(me.mass, np.float64)
    X = np.asarray(me.rest_pos, np.float64)
    area = np.asarray(me.rest_area, np.float64)
    node, grp, w, Mu, La, env = [], [], [], [], [], []
    owner = np.full(X.shape[0], -1)
    for b, g in enumerate(model._affine):
        el = np.asarray(g.elems, np.int64)
        nd = np.unique(tri[el].reshape(-1))
        if (owner[nd] >= 0).any():
            raise ValueError("two rigid regions share a node; merge them or leave a gap of "
                             "at least one soft element between them")
        if (free[nd] == 0).any():
            raise ValueError("a rigid region contains kinematically constrained nodes. A "
                             "body whose motion is PRESCRIBED needs no rigid region")
        owner[nd] = b
        c = (mass[nd, None] * X[nd]).sum(0) / mass[nd].sum()
        node += list(nd)
        grp += [b] * len(nd)
        w.append(np.c_[np.ones(len(nd)), X[nd] - c])
        Mu.append(float((area[el] * np.asarray(me.mu, np.float64)[el]).sum()))
        La.append(float((area[el] * np.asarray(me.lam, np.float64)[el]).sum()))
        env.append(int(np.asarray(me.tri2env)[el[0]]))
        mu_s[el] = 0.0
        lam_s[el] = 0.0
    w_np = np.concatenate(w, 0)
    node = np.asarray(node, np.int64)
    grp = np.asarray(grp, np.int64)
    q = np.zeros((len(model._affine), 6))
    first = np.concatenate([[0], np.cumsum([len(a) for a in w])])
    for b in range(len(model._affine)):
        k = slice(first[b], first[b + 1])
        sol = np.linalg.lstsq(w_np[k], x[node[k]], rcond=None)[0]
        q[b, :3], q[b, 3:] = sol[:, 0], sol[:, 1]
    qg = q[grp]
    x[node, 0] = w_np[:, 0] * qg[:, 0] + w_np[:, 1] * qg[:, 1] + w_np[:, 2] * qg[:, 2]
    x[node, 1] = w_np[:, 0] * qg[:, 3] + w_np[:, 1] * qg[:, 4] + w_np[:, 2] * qg[:, 5]
    return dict(node=node, grp=grp, env=np.asarray(env, np.int64), w=w_np,
                Mu=np.asarray(Mu), La=np.asarray(La), q=q), owner >= 0


def _rigid_arrays(model, free, skip_nodes):
    """RigidModes.build (implicit/affine.py:503-523): one 3-mode coarse space per connected
    piece of soft material with no kinematic node and no rigid region, of >= 3 nodes."""
    me = model.me
    N = me.rest_pos.shape[0]
    tri = np.asarray(me.tri)
    a = np.concatenate([tri[:, 0], tri[:, 1], tri[:, 2]])
    b = np.concatenate([tri[:, 1], tri[:, 2], tri[:, 0]])
    ncomp, lab = connected_components(coo_matrix((np.ones(len(a)), (a, b)), shape=(N, N)), directed=False)
    held = np.zeros(ncomp, bool)
    held[np.unique(lab[(free == 0).any(1)])] = True
    if skip_nodes is not None and np.any(skip_nodes):
        held[np.unique(lab[np.asarray(skip_nodes, bool)])] = True
    size = np.bincount(lab, minlength=ncomp)
    keep = np.where(~held & (size >= 3))[0]
    if len(keep) == 0:
        return None
    newid = np.full(ncomp, -1)
    newid[keep] = np.arange(len(keep))
    nodes = np.where(newid[lab] >= 0)[0]
    grp = newid[lab[nodes]]
    first = np.zeros(len(keep), np.int64)
    first[grp[::-1]] = nodes[::-1]
    return dict(node=nodes.astype(np.int64), grp=grp.astype(np.int64),
                env=np.asarray(me.node2env)[first].astype(np.int64))


def _ipc_arrays(model, integ):
    """IPCContact.__init__ (implicit/ipc_contact.py:353-386)."""
    me = model.me
    N = me.rest_pos.shape[0]
    edges = np.asarray(me.boundary_edges, np.int64)
    env = np.asarray(me.node2env)[edges[:, 0]]
    bn = np.asarray(me.boundary_nodes)
    pos = np.full(N, -1, np.int64)
    pos[bn] = np.arange(len(bn)) - np.asarray(me.boundary_starts)[np.asarray(me.boundary2env)]
    m = np.bincount(edges.reshape(-1), minlength=N).astype(np.float64)
    share = (m - 1.0) / np.maximum(m, 1.0)
    ptr, idx = model.exclusion_csr()
    friction = integ.friction
    mu_node = None
    if friction and any(b.mu is not None for b in model._bodies):
        mu_node = np.zeros(N, np.float64)
        for h, b in enumerate(model._bodies):
            mu_node[model._node_range[h]] = model.body_friction if b.mu is None else b.mu
    return dict(ea=edges[:, 0], eb=edges[:, 1], ela=pos[edges[:, 0]], elb=pos[edges[:, 1]], e2env=env,
                ca=share[edges[:, 0]], cb=share[edges[:, 1]],
                bstart=np.asarray(me.boundary_starts[:-1], np.int64),
                bpe=np.asarray(me.boundary_per_env, np.int64), excl_ptr=ptr, excl_idx=idx,
                mu=(model.body_friction if friction else 0.0), per_body=0 if mu_node is None else 1,
                mu_node=mu_node, dhat=float(model.dhat), kappa=float(model.body_kappa),
                reach=max(2.0 * model.dx, 2.0 * model.dhat), gap=0.1, bc_floor=0.25)


def _tendon_arrays(model):
    node, prv, nxt, tid = [], [], [], []
    for i, t in enumerate(model._tendons):
        o, n = len(node), len(t.nodes)
        node += list(t.nodes)
        tid += [i] * n
        prv += [-1] + list(range(o, o + n - 1))
        nxt += list(range(o + 1, o + n)) + [-1]
    T = model._tendons
    return dict(node=np.asarray(node, np.int64), prv=np.asarray(prv, np.int64), nxt=np.asarray(nxt, np.int64),
                tid=np.asarray(tid, np.int64), t2env=np.asarray([model.body_env(t.body) for t in T], np.int64),
                stiff=np.asarray([t.stiffness for t in T], np.float64),
                L0=np.asarray([t.length for t in T], np.float64),
                Tcmd=np.asarray([t.tension for t in T], np.float64))


def _spring_arrays(model):
    """Springs and pins (implicit/actuation.py:381-476): node b = -1 ties node a to `anchor`."""
    S = model._springs
    return dict(a=np.asarray([k.a for k in S], np.int64), b=np.asarray([k.b for k in S], np.int64),
                k=np.asarray([k.stiffness for k in S], np.float64),
                L0=np.asarray([k.length for k in S], np.float64),
                anchor=np.asarray([k.anchor for k in S], np.float64).reshape(-1, 2),
                env=np.asarray([k.env for k in S], np.int64))


def _pressure_arrays(model):
    """Pressure boundaries (implicit/actuation.py:80-152): every chamber's directed edges
    (fluid on the left), its environment, gauge pressure and shoelace reference point."""
    Cs = model._chambers
    return dict(ea=np.concatenate([c.ea for c in Cs]).astype(np.int64),
                eb=np.concatenate([c.eb for c in Cs]).astype(np.int64),
                ch=np.concatenate([np.full(len(c.ea), i) for i, c in enumerate(Cs)]).astype(np.int64),
                ch2env=np.asarray([model.body_env(c.body) for c in Cs], np.int64),
                p=np.asarray([c.pressure for c in Cs], np.float64),
                ref=np.asarray([c.ref for c in Cs], np.float64).reshape(-1, 2))


def rest_shape(model):
    """(Bm, area, Dm) of every triangle with the active regions' rest-shape change A applied
    (ActiveStrain, implicit/actuation.py:318-345): the rest edge vectors become A Dm0, so
    Bm = Bm0 A^-1 and area = area0 det A. Dm: (T, 4) rest edge vectors (e1x, e1y, e2x, e2y)."""
    me = model.me
    Bm0 = np.asarray(me.D_m_inv, np.float64)
    shape = Bm0.shape
    Bm = Bm0.reshape(-1, 2, 2).copy()
    area = np.asarray(me.rest_area, np.float64).copy()
    rest = np.asarray(me.rest_pos, np.float64)
    tri = np.asarray(me.tri, np.int64)
    e1, e2 = rest[tri[:, 1]] - rest[tri[:, 0]], rest[tri[:, 2]] - rest[tri[:, 0]]
    for r in model._regions:
        A = np.asarray(r.A, np.float64)
        if np.array_equal(A, np.eye(2)):
            continue
        el = r.elems
        Bm[el] = Bm[el] @ np.linalg.inv(A)
        area[el] = area[el] * np.linalg.det(A)
        e1[el], e2[el] = e1[el] @ A.T, e2[el] @ A.T
    return Bm.reshape(shape), area, np.concatenate([e1, e2], 1)


def external_force(model):
    """The ExternalForce field f = fext + m g (implicit/integrator.py:205-211), or None."""
    g = model._gravity
    if model._fext is None and g == (0.0, 0.0):
        return None
    f = np.zeros((model.n_nodes, 2)) if model._fext is None else model._fext.copy()
    f += np.asarray(model.me.mass, np.float64)[:, None] * np.asarray(g, np.float64)[None, :]
    return f


def solver_problem(model, integ, dt):
    """The problem dict of a finalized Model for a step of size dt."""
    me = model.me
    if me is None:
        raise RuntimeError("call model.finalize() before simulating")
    if model.body_contact not in ("ipc", "node"):
        raise ValueError(f"model.body_contact must be 'ipc' or 'node', not {model.body_contact!r}")
    if model.body_contact == "node" and integ.self_collision:
        raise NotImplementedError("the 'node' penalty contact is not implemented; use body_contact='ipc'")
    N = me.rest_pos.shape[0]
    cfg = model.cfg
    x = np.asarray(model._x_host, np.float64).copy()
    v = np.asarray(model._v0, np.float64).copy() if model._v0 is not None else np.zeros_like(x)
    bc = model.all_constrained()
    free = np.ones((N, 2), np.float64)
    free[bc] = 0.0
    mu_s = np.asarray(me.mu, np.float64).copy()
    lam_s = np.asarray(me.lam, np.float64).copy()
    prob = dict(
        B=int(me.n_envs), x=x, v=v, rest=np.asarray(me.rest_pos, np.float64),
        mass=np.asarray(me.mass, np.float64), free=free,
        node2env=np.asarray(me.node2env, np.int64), tri=np.asarray(me.tri, np.int64),
        Bm=None, area=None,
        mu=mu_s, lam=lam_s, tri2env=np.asarray(me.tri2env, np.int64),
        bnd=np.asarray(me.boundary_nodes, np.int64), b2e=np.asarray(me.boundary2env, np.int64),
        bc_idx=np.asarray(bc, np.int64),
        colliders=np.array([c.row() for c in model._colliders], np.float64).reshape(-1, 8),
        dt=float(dt), drag=math.exp(-float(dt) * cfg.damping), dhat=float(cfg.ipc_d_hat),
        kappa=float(cfg.obstacle_stiffness), epsv=float(cfg.obstacle_friction_epsv), eps=integ.eps,
        tol_x=integ.tol_x, near_factor=integ.near_factor, alpha_max=integ.alpha_max,
        area_shrink=integ.area_shrink, ccd_eta=integ.ccd_eta, ls_tol=integ.ls_tol, gtol=integ.gtol,
        iter_max=iters_for(model, integ, dt), conv_check=integ.conv_check, friction=int(integ.friction),
        line_search=int(integ.line_search), n_bt=integ.n_backtrack)
    prob["Bm"], prob["area"], prob["Dm"] = rest_shape(model)
    if model._col_mu_env:
        cm = np.repeat(prob["colliders"][None, :, 7], prob["B"], axis=0)
        for k, arr in model._col_mu_env.items():
            cm[:, k] = arr
        prob["col_mu_env"] = cm
    slaved = None
    if model._affine:
        prob["affine"], slaved = _affine_arrays(model, mu_s, lam_s, free, x)
    ipc = None
    if integ.self_collision and model.body_contact == "ipc":
        ipc = prob["ipc"] = _ipc_arrays(model, integ)
    f = external_force(model)
    if f is not None:
        prob["fext"] = f
    if model._tendons:
        prob["tendon"] = _tendon_arrays(model)
    if model._springs:
        prob["springs"] = _spring_arrays(model)
    if model._chambers:
        prob["pressure"] = _pressure_arrays(model)
    prob["active_regions"] = len(model._regions)
    prob["cg_guard"] = float((0.5 if ipc is not None else 0.0) if integ.cg_restart is None else integ.cg_restart)
    if integ.rigid_modes:
        rg = _rigid_arrays(model, free, slaved)
        if rg is not None:
            prob["rigid"] = rg
    return prob


def min_distance(prob):
    """Smallest node-edge distance per environment at the problem's positions (1e30 where
    no pair is within reach) — the reference's IPCContact.min_distance
    (implicit/ipc_contact.py:441-447), computed on the host: KD-tree candidates, then the
    exact point-segment distance, vectorised over all environments."""
    from scipy.spatial import cKDTree
    ipc = prob["ipc"]
    B = int(prob["B"])
    out = np.full(B, 1.0e30)
    ea, eb = np.asarray(ipc["ea"], np.int64), np.asarray(ipc["eb"], np.int64)
    if len(ea) == 0:
        return out
    x = np.asarray(prob["x"], np.float64)
    bnd = np.asarray(prob["bnd"], np.int64)
    b2e = np.asarray(prob["b2e"], np.int64)
    e2env = np.asarray(ipc["e2env"], np.int64)
    reach = float(ipc["reach"])
    L = np.linalg.norm(x[eb] - x[ea], axis=1)
    span = float(np.ptp(x, 0).max()) + 4.0 * (float(L.max()) + reach)
    shift = lambda e: np.stack([np.asarray(e, np.float64) * 2.0 * span, np.zeros(len(e))], 1)
    tn = cKDTree(x[bnd] + shift(b2e))
    te = cKDTree(0.5 * (x[ea] + x[eb]) + shift(e2env))
    D = te.sparse_distance_matrix(tn, 0.5 * float(L.max()) + reach, output_type="ndarray")
    k, jb = D["i"].astype(np.int64), D["j"].astype(np.int64)
    pn = bnd[jb]
    ok = (pn != ea[k]) & (pn != eb[k]) & (b2e[jb] == e2env[k])
    k, jb, pn = k[ok], jb[ok], pn[ok]
    ptr, idx = np.asarray(ipc["excl_ptr"], np.int64), np.asarray(ipc["excl_idx"], np.int64)
    M = int(idx.max()) + 2 if len(idx) else 1
    rows = np.repeat(np.arange(len(ptr) - 1), np.diff(ptr))
    keys = np.sort(rows * M + idx)

    def is_excl(slot, loc):
        q = slot * M + np.asarray(loc, np.int64)
        pos = np.minimum(np.searchsorted(keys, q), len(keys) - 1)
        return keys[pos] == q if len(keys) else np.zeros(len(q), bool)
    ok = ~is_excl(jb, np.asarray(ipc["ela"], np.int64)[k]) & ~is_excl(jb, np.asarray(ipc["elb"], np.int64)[k])
    k, pn = k[ok], pn[ok]
    a, b = x[ea[k]], x[eb[k]]
    ab = b - a
    t = np.clip(((x[pn] - a) * ab).sum(1) / np.maximum((ab * ab).sum(1), 1e-30), 0.0, 1.0)
    dd = np.linalg.norm(x[pn] - a - t[:, None] * ab, axis=1)
    near = dd < reach
    np.minimum.at(out, e2env[k][near], dd[near])
    return out


def subset_problem(prob, envs):
    """The problem restricted to the environments `envs` (renumbered 0..len-1), with every
    batch-global parameter (iteration budget, contact scales) kept as it is."""
    envs = np.asarray(envs, np.int64)
    B = int(prob["B"])
    newenv = np.full(B, -1, np.int64)
    newenv[envs] = np.arange(len(envs))
    node2env = np.asarray(prob["node2env"], np.int64)
    keep_n = np.nonzero(newenv[node2env] >= 0)[0]
    # order nodes by the new environment order, stable
    keep_n = keep_n[np.argsort(newenv[node2env[keep_n]], kind="stable")]
    nmap = np.full(len(node2env), -1, np.int64)
    nmap[keep_n] = np.arange(len(keep_n))
    tri2env = np.asarray(prob["tri2env"], np.int64)
    keep_t = np.nonzero(newenv[tri2env] >= 0)[0]
    keep_t = keep_t[np.argsort(newenv[tri2env[keep_t]], kind="stable")]
    b2e = np.asarray(prob["b2e"], np.int64)
    keep_b = np.nonzero(newenv[b2e] >= 0)[0]
    keep_b = keep_b[np.argsort(newenv[b2e[keep_b]], kind="stable")]
    out = {k: v for k, v in prob.items() if np.ndim(v) == 0 and not isinstance(v, dict)}
    out["B"] = len(envs)
    for k in ("x", "v", "mass", "free", "rest", "fext"):
        if prob.get(k) is not None:
            out[k] = np.asarray(prob[k])[keep_n]
    out["node2env"] = newenv[node2env[keep_n]]
    out["tri"] = nmap[np.asarray(prob["tri"], np.int64)[keep_t]]
    for k in ("Bm", "area", "mu", "lam", "Dm"):
        if prob.get(k) is not None:
            out[k] = np.asarray(prob[k])[keep_t]
    out["tri2env"] = newenv[tri2env[keep_t]]
    out["bnd"] = nmap[np.asarray(prob["bnd"], np.int64)[keep_b]]
    out["b2e"] = newenv[b2e[keep_b]]
    bc = np.asarray(prob.get("bc_idx", np.zeros(0)), np.int64)
    out["bc_idx"] = np.sort(nmap[bc[nmap[bc] >= 0]])
    out["colliders"] = np.asarray(prob["colliders"])
    if prob.get("col_mu_env") is not None:
        out["col_mu_env"] = np.asarray(prob["col_mu_env"])[envs]
    if prob.get("ipc") is not None:
        ip = prob["ipc"]
        e2env = np.asarray(ip["e2env"], np.int64)
        ke = np.nonzero(newenv[e2env] >= 0)[0]
        ke = ke[np.argsort(newenv[e2env[ke]], kind="stable")]
        ptr = np.asarray(ip["excl_ptr"], np.int64)
        idx = np.asarray(ip["excl_idx"], np.int64)
        rows = [idx[ptr[s]:ptr[s + 1]] for s in keep_b]
        nptr = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int64)
        bpe = np.bincount(out["b2e"], minlength=len(envs)).astype(np.int64)
        q = dict(ip)
        q.update(ea=nmap[np.asarray(ip["ea"], np.int64)[ke]], eb=nmap[np.asarray(ip["eb"], np.int64)[ke]],
                 ela=np.asarray(ip["ela"])[ke], elb=np.asarray(ip["elb"])[ke], e2env=newenv[e2env[ke]],
                 ca=np.asarray(ip["ca"])[ke], cb=np.asarray(ip["cb"])[ke],
                 bstart=np.concatenate([[0], np.cumsum(bpe)[:-1]]).astype(np.int64), bpe=bpe,
                 excl_ptr=nptr, excl_idx=(np.concatenate(rows) if rows else np.zeros(0, np.int64)),
                 mu_node=(None if ip.get("mu_node") is None else np.asarray(ip["mu_node"])[keep_n]))
        out["ipc"] = q
    if prob.get("rigid") is not None:
        rg = prob["rigid"]
        renv = np.asarray(rg["env"], np.int64)
        kp = np.nonzero(newenv[renv] >= 0)[0]
        kp = kp[np.argsort(newenv[renv[kp]], kind="stable")]
        pmap = np.full(len(renv), -1, np.int64)
        pmap[kp] = np.arange(len(kp))
        grp = np.asarray(rg["grp"], np.int64)
        kn = np.nonzero(pmap[grp] >= 0)[0]
        kn = kn[np.argsort(pmap[grp[kn]], kind="stable")]
        out["rigid"] = dict(node=nmap[np.asarray(rg["node"], np.int64)[kn]], grp=pmap[grp[kn]], env=newenv[renv[kp]])
    def pick(env_of):
        """Items whose environment is kept, in the new environment order (stable), and the
        old -> new item map."""
        env_of = np.asarray(env_of, np.int64)
        k = np.nonzero(newenv[env_of] >= 0)[0]
        k = k[np.argsort(newenv[env_of[k]], kind="stable")]
        m = np.full(len(env_of), -1, np.int64)
        m[k] = np.arange(len(k))
        return k, m

    def members(owner, omap):
        """Entries whose owner is kept, grouped in the owners' new order (stable)."""
        owner = np.asarray(owner, np.int64)
        k = np.nonzero(omap[owner] >= 0)[0]
        return k[np.argsort(omap[owner[k]], kind="stable")]

    remap = lambda ids: np.where(np.asarray(ids, np.int64) >= 0, nmap[np.asarray(ids, np.int64)], -1)
    if prob.get("affine") is not None:
        af = prob["affine"]
        kr, rmap = pick(af["env"])
        ke = members(af["grp"], rmap)
        out["affine"] = dict(node=nmap[np.asarray(af["node"], np.int64)[ke]], grp=rmap[np.asarray(af["grp"], np.int64)[ke]],
                             env=newenv[np.asarray(af["env"], np.int64)[kr]],
                             w=np.asarray(af["w"], np.float64).reshape(-1, 3)[ke],
                             Mu=np.asarray(af["Mu"])[kr], La=np.asarray(af["La"])[kr],
                             q=np.asarray(af["q"], np.float64).reshape(-1, 6)[kr])
    if prob.get("tendon") is not None:
        td = prob["tendon"]
        kt, tmap = pick(td["t2env"])
        kj = members(td["tid"], tmap)
        jmap = np.full(len(np.asarray(td["tid"])), -1, np.int64)
        jmap[kj] = np.arange(len(kj))
        link = lambda a: np.where(np.asarray(a, np.int64)[kj] >= 0, jmap[np.asarray(a, np.int64)[kj]], -1)
        out["tendon"] = dict(node=nmap[np.asarray(td["node"], np.int64)[kj]], prv=link(td["prv"]), nxt=link(td["nxt"]),
                             tid=tmap[np.asarray(td["tid"], np.int64)[kj]], t2env=newenv[np.asarray(td["t2env"], np.int64)[kt]],
                             stiff=np.asarray(td["stiff"])[kt], L0=np.asarray(td["L0"])[kt], Tcmd=np.asarray(td["Tcmd"])[kt])
    if prob.get("springs") is not None:
        sp = prob["springs"]
        ks, _ = pick(sp["env"])
        out["springs"] = dict(a=nmap[np.asarray(sp["a"], np.int64)[ks]], b=remap(np.asarray(sp["b"], np.int64)[ks]),
                              k=np.asarray(sp["k"])[ks], L0=np.asarray(sp["L0"])[ks],
                              anchor=np.asarray(sp["anchor"], np.float64).reshape(-1, 2)[ks],
                              env=newenv[np.asarray(sp["env"], np.int64)[ks]])
    if prob.get("pressure") is not None:
        pr = prob["pressure"]
        kc, cmap = pick(pr["ch2env"])
        kq = members(pr["ch"], cmap)
        out["pressure"] = dict(ea=nmap[np.asarray(pr["ea"], np.int64)[kq]], eb=nmap[np.asarray(pr["eb"], np.int64)[kq]],
                               ch=cmap[np.asarray(pr["ch"], np.int64)[kq]], ch2env=newenv[np.asarray(pr["ch2env"], np.int64)[kc]],
                               p=np.asarray(pr["p"])[kc], ref=np.asarray(pr["ref"], np.float64).reshape(-1, 2)[kc])
    return out
