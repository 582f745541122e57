"""CPU FP64 oracle of the step adjoint — TEST INFRASTRUCTURE ONLY.

A numpy restatement of the reference's adjoint (implicit/adjoint.py) that the GPU adjoint is
checked against. Where the reference runs matrix-free MINRES, this assembles the tangent
H = M + h^2 (K_elastic + K_collider + K_tendon) as a sparse matrix on the free DOFs and solves
it directly (scipy), so its solution carries no Krylov tolerance:

  element tangent      assemble_Ke_kernel       implicit/adjoint.py:145-160 (nh_d2PsidF2_dir,
                                                core/math.py:85-93)
  collider tangent     chvp_disc_kernel /       implicit/adjoint.py:88-114, frozen gate
                       chvp_sdf_kernel          d in (0, dhat); every collider kind
  element force        drho_kernel              implicit/adjoint.py:164-178 (nh_dPsidF,
                                                core/math.py:76-81)
  recursion            transient_adjoint        implicit/adjoint.py:371-399
  affine bodies        AffineBodies             implicit/affine.py:60-101, 156-269: the
                                                system in the reduced coordinates (x = J q
                                                on a region's nodes) plus each region's
                                                exact elastic block; not in the reference's
                                                adjoint, which refuses affine bodies
  IPC tangent          ipc_pair_kernel terms    implicit/ipc_contact.py:174-296: barrier
                                                terms frozen at x, frictionless, exact
                                                Hessian of each distance; not in the
                                                reference's adjoint, which refuses IPC
  tendon tangent       pHp_tendon_kernel        implicit/actuation.py:229-248 (tension-
                                                controlled: T / len (I - d d^T) per segment);
                                                not in the reference's adjoint, which refuses
                                                tendons

Only the tests use it. Input: a solver problem dict (the layout `oracle.OracleSolver` takes).
"""
from __future__ import annotations

import numpy as np

LOG_EPS = 1.0e-6


def bp(d, dhat):
    """b'(d) of b = -(d - dhat)^2 log(d / dhat) (core/math.py:118-122)."""
    u = d - dhat
    return -2.0 * u * np.log(d / dhat) - u * u / d


def bpp(d, dhat):
    """b''(d) (core/math.py:125-129)."""
    u = d - dhat
    return -2.0 * np.log(d / dhat) - 4.0 * u / d + u * u / (d * d)


def _F(x, prob):
    tri = np.asarray(prob["tri"], np.int64)
    B = np.asarray(prob["Bm"], np.float64).reshape(-1, 2, 2)
    x0, x1, x2 = x[tri[:, 0]], x[tri[:, 1]], x[tri[:, 2]]
    Ds = np.stack([x1 - x0, x2 - x0], axis=2)            # (T, 2, 2): columns = edges
    return Ds @ B, B, tri


def _inv_T(F):
    J = F[:, 0, 0] * F[:, 1, 1] - F[:, 0, 1] * F[:, 1, 0]
    inv = np.empty_like(F)
    inv[:, 0, 0], inv[:, 0, 1] = F[:, 1, 1], -F[:, 0, 1]
    inv[:, 1, 0], inv[:, 1, 1] = -F[:, 1, 0], F[:, 0, 0]
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.where(J[:, None, None] != 0.0, inv / J[:, None, None], 0.0)
    return np.transpose(inv, (0, 2, 1)), J


def element_forces(x, prob, mu=None, lam=None):
    """(T, 3, 2): each corner's share of the element's elastic force dE/dx (no h^2)."""
    F, B, tri = _F(x, prob)
    mu = np.asarray(prob["mu"] if mu is None else mu, np.float64)
    la = np.asarray(prob["lam"] if lam is None else lam, np.float64)
    G, J = _inv_T(F)
    logJ = np.log(np.maximum(J, LOG_EPS))
    P = mu[:, None, None] * F + (la * logJ - mu)[:, None, None] * G
    HH = np.asarray(prob["area"], np.float64)[:, None, None] * (P @ np.transpose(B, (0, 2, 1)))
    g1, g2 = HH[:, :, 0], HH[:, :, 1]
    return np.stack([-(g1 + g2), g1, g2], axis=1)


def element_hessians(x, prob, mu=None, lam=None):
    """(T, 6, 6) element tangents, node-major DOFs (x0, y0, x1, y1, x2, y2); unclamped."""
    F, B, tri = _F(x, prob)
    mu = np.asarray(prob["mu"] if mu is None else mu, np.float64)
    la = np.asarray(prob["lam"] if lam is None else lam, np.float64)
    A = np.asarray(prob["area"], np.float64)
    G, J = _inv_T(F)
    logJ = np.log(np.maximum(J, LOG_EPS))
    c1 = la * logJ - mu
    Bt = np.transpose(B, (0, 2, 1))
    K = np.zeros((len(A), 6, 6))
    for j in range(6):
        n, c = divmod(j, 2)
        a, b = {0: (-1.0, -1.0), 1: (1.0, 0.0), 2: (0.0, 1.0)}[n]
        dDs = np.zeros((2, 2))
        dDs[c, 0], dDs[c, 1] = a, b
        dF = dDs[None] @ B
        GdF = np.einsum("tij,tij->t", G, dF)
        W = G @ np.transpose(dF, (0, 2, 1)) @ G
        dP = mu[:, None, None] * dF + (la * GdF)[:, None, None] * G - c1[:, None, None] * W
        HH = A[:, None, None] * (dP @ Bt)
        f1, f2 = HH[:, :, 0], HH[:, :, 1]
        f0 = -(f1 + f2)
        K[:, 0:2, j], K[:, 2:4, j], K[:, 4:6, j] = f0, f1, f2
    return K


def collider_blocks(x, prob):
    """(Nb, 2, 2): kappa (b'' g g^T + b' H_phi) per boundary node summed over the colliders,
    gate frozen at d in (0, dhat). Every collider kind: the disc and the half-space in closed
    form, the other shapes through the oracle's level set, gradient and Hessian."""
    bnd = np.asarray(prob["bnd"], np.int64)
    dhat, kappa = float(prob["dhat"]), float(prob["kappa"])
    out = np.zeros((len(bnd), 2, 2))
    for c in np.asarray(prob.get("colliders", np.zeros((0, 8))), np.float64).reshape(-1, 8):
        kind = int(c[0])
        p = x[bnd]
        if kind == 0:
            e = p - c[1:3]
            dc = np.linalg.norm(e, axis=1)
            d = dc - c[6]
            n = e / dc[:, None]
            Hphi = (np.eye(2)[None] - n[:, :, None] * n[:, None, :]) / dc[:, None, None]
        elif kind == 4:
            n = np.broadcast_to(c[3:5], p.shape)
            d = (p - c[1:3]) @ c[3:5]
            Hphi = np.zeros((len(p), 2, 2))
        else:  # any other level set: kappa (b'' g g^T + b' H_phi), chvp_sdf_kernel (:101-114)
            from . import sdf_full
            d, n, Hphi = sdf_full(c, p)
        on = (d > 0.0) & (d < dhat)
        dd = np.where(on, d, dhat * 0.5)
        blk = kappa * (bpp(dd, dhat)[:, None, None] * n[:, :, None] * n[:, None, :]
                       + bp(dd, dhat)[:, None, None] * Hphi)
        out += np.where(on[:, None, None], blk, 0.0)
    return out


def _line_ddd(ab, w, Ll, c0, v):
    """Directional second derivative of the point-line distance |cross(ab, w)| / |ab| along
    v = (v_p, v_a, v_b) (the curvature of the oracle's pHp mode 1, ipc_contact.py:150-160) —
    a quadratic form in v."""
    vp, va, vb = v[0:2], v[2:4], v[4:6]
    de, dw = vb - va, vp - va
    cr = lambda u, q: u[0] * q[1] - u[1] * q[0]
    c1 = cr(de, w) + cr(ab, dw)
    c2 = 2.0 * cr(de, dw)
    L1 = float(ab @ de) / Ll
    Lq = (float(de @ de) - L1 * L1) / Ll
    s0 = c0 / Ll
    s1 = (c1 - s0 * L1) / Ll
    ddd = (c2 - 2.0 * s1 * L1 - s0 * Lq) / Ll
    return -ddd if c0 < 0.0 else ddd


def ipc_terms(x, prob):
    """The frozen-active-set tangent of the IPC barrier between bodies, frictionless: every
    barrier term the pair loop evaluates (ipc_contact.py:174-296 — the edge interior with
    weights (1 - t, t), and each end with its vertex-correction coefficient) as
    (node ids, coef kappa (b'' g g^T + b' H_d)), g = grad d and H_d its exact Hessian (the
    interior's by polarisation of the directional second derivative). Not in the
    reference's adjoint, which refuses IPC contact."""
    ipc = prob.get("ipc")
    if ipc is None or len(ipc.get("ea", [])) == 0:
        return []
    ea, eb = np.asarray(ipc["ea"], np.int64), np.asarray(ipc["eb"], np.int64)
    ela, elb = np.asarray(ipc["ela"], np.int64), np.asarray(ipc["elb"], np.int64)
    e2env = np.asarray(ipc["e2env"], np.int64)
    ca, cb = np.asarray(ipc["ca"], np.float64), np.asarray(ipc["cb"], np.float64)
    bstart, bpe = np.asarray(ipc["bstart"], np.int64), np.asarray(ipc["bpe"], np.int64)
    ptr, idx = np.asarray(ipc["excl_ptr"], np.int64), np.asarray(ipc["excl_idx"], np.int64)
    bnd, b2e = np.asarray(prob["bnd"], np.int64), np.asarray(prob["b2e"], np.int64)
    dhat, kappa, reach = float(ipc["dhat"]), float(ipc["kappa"]), float(ipc["reach"])
    dlo = 1.0e-9 * dhat
    excl = lambda jb, loc: loc in set(idx[ptr[jb]:ptr[jb + 1]].tolist())
    eye = np.eye(6)
    out = []

    def point_term(nodes, coef, wv, d):
        dd = max(d, dlo)
        n = wv / dd
        K = (np.eye(2) - np.outer(n, n)) / dd
        g = np.concatenate([n, -n])
        Hd = np.block([[K, -K], [-K, K]])
        out.append((nodes, coef * kappa * (bpp(dd, dhat) * np.outer(g, g) + bp(dd, dhat) * Hd)))

    for k in range(len(ea)):
        a, b, e = int(ea[k]), int(eb[k]), int(e2env[k])
        xa, xb = x[a], x[b]
        ab = xb - xa
        L2 = max(float(ab @ ab), 1.0e-30)
        Ll = np.sqrt(L2)
        for jb in range(int(bstart[e]), int(bstart[e]) + int(bpe[e])):
            pn = int(bnd[jb])
            if b2e[jb] != e or pn == a or pn == b or excl(jb, int(ela[k])) or excl(jb, int(elb[k])):
                continue
            w = x[pn] - xa
            tt = float(w @ ab) / L2
            dvec = w if tt <= 0.0 else (x[pn] - xb if tt >= 1.0 else w - tt * ab)
            if not np.linalg.norm(dvec) < reach:
                continue
            d = float(np.linalg.norm(dvec))
            if 0.0 < tt < 1.0 and d < dhat:
                dd = max(d, dlo)
                n = dvec / dd
                g = np.concatenate([n, -(1.0 - tt) * n, -tt * n])
                c0 = ab[0] * w[1] - ab[1] * w[0]
                q = [_line_ddd(ab, w, Ll, c0, eye[i]) for i in range(6)]
                Hd = np.diag(q)
                for i in range(6):
                    for j in range(i + 1, 6):
                        Hd[i, j] = Hd[j, i] = 0.5 * (_line_ddd(ab, w, Ll, c0, eye[i] + eye[j]) - q[i] - q[j])
                out.append(((pn, a, b), kappa * (bpp(dd, dhat) * np.outer(g, g) + bp(dd, dhat) * Hd)))
            coef_a = -ca[k] + (1.0 if tt <= 0.0 else 0.0)
            if coef_a != 0.0 and np.linalg.norm(w) < dhat:
                point_term((pn, a), coef_a, w, float(np.linalg.norm(w)))
            wb = x[pn] - xb
            coef_b = -cb[k] + (1.0 if tt >= 1.0 else 0.0)
            if coef_b != 0.0 and np.linalg.norm(wb) < dhat:
                point_term((pn, b), coef_b, wb, float(np.linalg.norm(wb)))
    return out


def tendon_segments(prob):
    """(a, b, tendon) node pairs of every tendon segment (eyelet -> next eyelet)."""
    td = prob.get("tendon")
    if td is None or len(td.get("t2env", [])) == 0:
        return np.zeros((0, 3), np.int64)
    node = np.asarray(td["node"], np.int64)
    nxt = np.asarray(td["nxt"], np.int64)
    tid = np.asarray(td["tid"], np.int64)
    j = np.nonzero(nxt >= 0)[0]
    return np.stack([node[j], node[nxt[j]], tid[j]], 1)


def assemble(x, prob, tension=None, mu=None, lam=None):
    """Sparse H = M + h^2 (K_el + K_col + K_tendon) over all 2N DOFs (scipy CSR)."""
    import scipy.sparse as sp
    N = x.shape[0]
    h2 = float(prob["dt"]) ** 2
    tri = np.asarray(prob["tri"], np.int64)
    K = element_hessians(x, prob, mu, lam)
    dof = np.stack([2 * tri[:, 0], 2 * tri[:, 0] + 1, 2 * tri[:, 1], 2 * tri[:, 1] + 1,
                    2 * tri[:, 2], 2 * tri[:, 2] + 1], 1)
    rows = [np.repeat(dof, 6, axis=1).ravel()]
    cols = [np.tile(dof, (1, 6)).ravel()]
    vals = [h2 * K.reshape(len(tri), 36).ravel()]
    m = np.asarray(prob["mass"], np.float64)
    rows.append(np.arange(2 * N)); cols.append(np.arange(2 * N)); vals.append(np.repeat(m, 2))
    bnd = np.asarray(prob["bnd"], np.int64)
    Cb = collider_blocks(x, prob)
    for a in range(2):
        for b in range(2):
            rows.append(2 * bnd + a); cols.append(2 * bnd + b); vals.append(h2 * Cb[:, a, b])
    seg = tendon_segments(prob)
    if len(seg):
        td = prob["tendon"]
        Tc = np.asarray(td["Tcmd"] if tension is None else tension, np.float64)
        tau = np.maximum(Tc, 0.0)[seg[:, 2]]
        t = x[seg[:, 1]] - x[seg[:, 0]]
        ln = np.maximum(np.linalg.norm(t, axis=1), 1e-12)
        s = t / ln[:, None]
        k = (tau / ln)[:, None, None] * (np.eye(2)[None] - s[:, :, None] * s[:, None, :])
        for (na, nb, sg) in ((seg[:, 0], seg[:, 0], 1.0), (seg[:, 1], seg[:, 1], 1.0),
                             (seg[:, 0], seg[:, 1], -1.0), (seg[:, 1], seg[:, 0], -1.0)):
            for a in range(2):
                for b in range(2):
                    rows.append(2 * na + a); cols.append(2 * nb + b); vals.append(sg * h2 * k[:, a, b])
    for nodes, blk in ipc_terms(x, prob):
        dof = np.array([2 * n + c for n in nodes for c in range(2)])
        rows.append(np.repeat(dof, len(dof))); cols.append(np.tile(dof, len(dof))); vals.append(h2 * blk.ravel())
    H = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(2 * N, 2 * N)).tocsr()
    return H


def free_dofs(prob):
    return np.asarray(prob["free"], np.float64).reshape(-1) > 0.5


def _nh_dP(A, dA, mu, la):
    """Directional derivative of the Neo-Hookean P at A along dA (moduli mu, la)."""
    J = A[0, 0] * A[1, 1] - A[0, 1] * A[1, 0]
    G = np.linalg.inv(A).T
    logJ = np.log(max(J, LOG_EPS))
    return mu * dA + la * float((G * dA).sum()) * G - (la * logJ - mu) * (G @ dA.T @ G)


def affine_reduction(x, prob):
    """The affine bodies' reduced coordinates at the state x (AffineBodies, implicit/
    affine.py:60-101, 156-269): S (2N x n_u, sparse) maps the unknowns u — every free DOF of a
    node no rigid region owns, then q = (t_x, A11, A12, t_y, A21, A22) of each region — to
    node displacements (x = J q on a region's nodes); and each region's exact elastic block
    d2 Psi / dq2 at its current A with the region's summed moduli (6x6, in q), to be added
    times h^2. q is recovered from the region's node positions (x = J q holds exactly)."""
    import scipy.sparse as sp
    af = prob["affine"]
    node, grp = np.asarray(af["node"], np.int64), np.asarray(af["grp"], np.int64)
    w = np.asarray(af["w"], np.float64).reshape(-1, 3)
    Mu, La = np.asarray(af["Mu"], np.float64), np.asarray(af["La"], np.float64)
    N = x.shape[0]
    nreg = len(Mu)
    ff = free_dofs(prob)
    slaved = np.zeros(2 * N, bool)
    slaved[2 * node], slaved[2 * node + 1] = True, True
    plain = np.flatnonzero(ff & ~slaved)
    nu = len(plain) + 6 * nreg
    rows = [plain]
    cols = [np.arange(len(plain))]
    vals = [np.ones(len(plain))]
    base = len(plain) + 6 * grp
    for c in range(3):
        rows += [2 * node, 2 * node + 1]
        cols += [base + c, base + 3 + c]
        vals += [w[:, c], w[:, c]]
    S = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(2 * N, nu))
    blocks = []
    idx = (1, 2, 4, 5)
    for b in range(nreg):
        k = grp == b
        sol = np.linalg.lstsq(w[k], x[node[k]], rcond=None)[0]          # (3, 2): q_x, q_y columns
        A = np.array([[sol[1, 0], sol[2, 0]], [sol[1, 1], sol[2, 1]]])
        K = np.zeros((6, 6))
        for j in range(4):
            dA = np.zeros(4)
            dA[j] = 1.0
            dP = _nh_dP(A, dA.reshape(2, 2), Mu[b], La[b]).reshape(4)
            for r in range(4):
                K[idx[r], idx[j]] = dP[r]
        blocks.append((len(plain) + 6 * b, K))
    return S, blocks


def adjoint_solve(x, prob, rhs, tension=None, mu=None, lam=None):
    """Solve H(x) lam = rhs on the free DOFs (direct); lam = 0 on the held DOFs. With affine
    bodies the system is solved in the reduced coordinates, S^T H S + h^2 K_A, and mapped
    back: lam = S u."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    H = assemble(x, prob, tension, mu, lam)
    b = np.asarray(rhs, np.float64).reshape(-1)
    if prob.get("affine") is not None and len(prob["affine"].get("Mu", [])):
        S, blocks = affine_reduction(x, prob)
        Hr = (S.T @ H @ S).tolil()
        h2 = float(prob["dt"]) ** 2
        for o, K in blocks:
            Hr[o:o + 6, o:o + 6] = Hr[o:o + 6, o:o + 6].toarray() + h2 * K
        u = spl.spsolve(sp.csc_matrix(Hr), S.T @ b)
        return (S @ u).reshape(-1, 2)
    ff = free_dofs(prob)
    out = np.zeros(2 * x.shape[0])
    out[ff] = spl.spsolve(H[ff][:, ff].tocsc(), b[ff])
    return out.reshape(-1, 2)


def tendon_length_grad(x, prob):
    """(n_ten, N, 2): d len_k / dx."""
    td = prob["tendon"]
    seg = tendon_segments(prob)
    n_ten = len(td["t2env"])
    g = np.zeros((n_ten, x.shape[0], 2))
    t = x[seg[:, 1]] - x[seg[:, 0]]
    s = t / np.maximum(np.linalg.norm(t, axis=1), 1e-12)[:, None]
    np.add.at(g, (seg[:, 2], seg[:, 1]), s)
    np.add.at(g, (seg[:, 2], seg[:, 0]), -s)
    return g


def rollout_adjoint(prob, xs, seed, E=None, tensions=None):
    """The damped backward-Euler recursion over forward states xs = [x_0 .. x_T]:
        H_k lam_k = seed_k + (1 + drag) M lam_{k+1} - drag M lam_{k+2}
    Returns dict(dE (T_tri,), dT (steps, n_ten) or None, dx0, dv0 (N, 2), lams).
    E: per-element multipliers of prob's moduli (the forward ran with mu = E mu, lam = E lam);
    tensions: (steps, n_ten) tension commands per step (tendon order of prob)."""
    T = len(xs) - 1
    h = float(prob["dt"])
    h2, dr = h * h, float(prob["drag"])
    mu0, la0 = np.asarray(prob["mu"], np.float64), np.asarray(prob["lam"], np.float64)
    E = np.ones(len(mu0)) if E is None else np.asarray(E, np.float64)
    mu, la = E * mu0, E * la0
    m2 = np.asarray(prob["mass"], np.float64)[:, None]
    free = np.asarray(prob["free"], np.float64)
    tri = np.asarray(prob["tri"], np.int64)
    has_t = prob.get("tendon") is not None and len(prob["tendon"].get("t2env", [])) > 0
    n_ten = len(prob["tendon"]["t2env"]) if has_t else 0
    lam1 = np.zeros_like(xs[0])
    lam2 = np.zeros_like(xs[0])
    dE = np.zeros(len(mu0))
    dT = np.zeros((T, n_ten)) if has_t else None
    lams = {}
    for k in range(T, 0, -1):
        rhs = (1.0 + dr) * m2 * lam1 - dr * m2 * lam2
        if k in seed:
            rhs = rhs + np.asarray(seed[k], np.float64)
        tk = None if tensions is None else np.asarray(tensions[k - 1], np.float64)
        lam_k = adjoint_solve(xs[k], prob, rhs, tk, mu, la)
        f = element_forces(xs[k], prob, mu0, la0)               # unit-multiplier force
        dE += -h2 * np.einsum("tcd,tcd->t", f, lam_k[tri])
        if has_t:
            gl = tendon_length_grad(xs[k], prob)
            tc = np.asarray(prob["tendon"]["Tcmd"] if tk is None else tk, np.float64)
            dT[k - 1] = -h2 * np.einsum("knd,nd->k", gl, lam_k) * (tc > 0)
        lams[k] = lam_k
        lam2, lam1 = lam1, lam_k
    dx0 = (m2 * lam1 - dr * m2 * lam2) * free
    dv0 = h * dr * m2 * lam1 * free
    return dict(dE=dE, dT=dT, dx0=dx0, dv0=dv0, lams=lams)
