"""Static equilibrium by Newton's method — TEST INFRASTRUCTURE ONLY.

An independent check of the implicit step's physics, in the role the reference's
tests/reference_static.py (`solve_static`) plays for its own tests: a converged static
state that the dynamic PNCG solve, run until it comes to rest, must reach. It shares no
code with the PNCG solve. The total potential

    Pi(x) = sum_t area_t Psi(F_t) - f . (x - X) + T L(x)

is minimised over the free nodes, with

  * Psi = mu/2 (|F|^2 - 2) - mu log J + lam/2 log^2 J, the plane-strain Neo-Hookean
    energy of core/math.py:75-93, and F = Ds Bm with Ds = [x1 - x0, x2 - x0];
  * f fixed nodal loads [N/m] (set_external_force);
  * T L the work of a tension-controlled tendon through a chain of nodes, L the length of
    the chain (implicit/actuation.py:169-316).

The element tangent is exact:
dP = mu dF + lam tr(F^-1 dF) F^-T - (lam log J - mu) F^-T dF^T F^-T, assembled into a
sparse matrix; each Newton step is a sparse solve followed by a backtracking line search
on Pi that keeps every J positive, and the loads are ramped in. Only the tests use it.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# d Ds / d x for each of a triangle's 6 coordinates (node n, component c): the row c of
# Ds moves by (-1, -1) for node 0, (1, 0) for node 1 and (0, 1) for node 2
_DDS = np.zeros((6, 2, 2))
for _n, _ab in enumerate(((-1.0, -1.0), (1.0, 0.0), (0.0, 1.0))):
    for _c in range(2):
        _DDS[2 * _n + _c, _c] = _ab


def _F(x, tri, Bm):
    p0, p1, p2 = x[tri[:, 0]], x[tri[:, 1]], x[tri[:, 2]]
    Ds = np.stack([np.stack([p1[:, 0] - p0[:, 0], p2[:, 0] - p0[:, 0]], -1),
                   np.stack([p1[:, 1] - p0[:, 1], p2[:, 1] - p0[:, 1]], -1)], 1)
    return Ds @ Bm


def _nodal(G):
    """(T, 2, 2) matrices A P Bm^T -> (T, 6) forces on the three nodes (x0, y0, x1, ...)."""
    g1, g2 = G[:, :, 0], G[:, :, 1]
    return np.concatenate([-(g1 + g2), g1, g2], 1)


def elastic(x, tri, Bm, area, mu, lam, tangent=True):
    """(energy, gradient (N, 2), sparse tangent or None); energy inf if any J <= 0."""
    F = _F(x, tri, Bm)
    J = np.linalg.det(F)
    if (J <= 0.0).any():
        return np.inf, None, None
    logJ = np.log(J)
    Fi = np.linalg.inv(F)
    FiT = Fi.transpose(0, 2, 1)
    E = float((area * (0.5 * mu * ((F * F).sum((1, 2)) - 2.0) - mu * logJ + 0.5 * lam * logJ ** 2)).sum())
    P = mu[:, None, None] * F + (lam * logJ - mu)[:, None, None] * FiT
    BmT = Bm.transpose(0, 2, 1)
    ge = _nodal(area[:, None, None] * P @ BmT)
    dofs = np.stack([2 * tri[:, k] + c for k in range(3) for c in range(2)], 1)
    g = np.bincount(dofs.ravel(), ge.ravel(), minlength=x.size).reshape(-1, 2)
    if not tangent:
        return E, g, None
    Ke = np.empty((len(tri), 6, 6))
    c1 = (lam * logJ - mu)[:, None, None]
    for j in range(6):
        dF = _DDS[j][None] @ Bm
        trFidF = np.einsum("tij,tji->t", Fi, dF)
        dP = mu[:, None, None] * dF + (lam * trFidF)[:, None, None] * FiT - c1 * (FiT @ dF.transpose(0, 2, 1) @ FiT)
        Ke[:, :, j] = _nodal(area[:, None, None] * dP @ BmT)
    rows = np.repeat(dofs, 6, 1).ravel()
    cols = np.tile(dofs, (1, 6)).ravel()
    K = sp.csr_matrix((Ke.ravel(), (rows, cols)), shape=(x.size, x.size))
    return E, g, K


def tendon(x, nodes, T):
    """(T L, gradient, sparse tangent) of a tendon of tension T through `nodes` in order."""
    n = np.asarray(nodes, np.int64)
    N = x.shape[0]
    if len(n) < 2 or T == 0.0:
        return 0.0, np.zeros_like(x), sp.csr_matrix((x.size, x.size))
    d = x[n[1:]] - x[n[:-1]]
    ell = np.linalg.norm(d, axis=1)
    u = d / ell[:, None]
    g = np.zeros_like(x)
    np.add.at(g, n[1:], T * u)
    np.add.at(g, n[:-1], -T * u)
    Hs = T * (np.eye(2)[None] - u[:, :, None] * u[:, None, :]) / ell[:, None, None]   # (S, 2, 2)
    a, b = n[:-1], n[1:]
    rows, cols, vals = [], [], []
    for (p, q, sgn) in ((a, a, 1.0), (b, b, 1.0), (a, b, -1.0), (b, a, -1.0)):
        for i in range(2):
            for j in range(2):
                rows.append(2 * p + i)
                cols.append(2 * q + j)
                vals.append(sgn * Hs[:, i, j])
    K = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(2 * N, 2 * N))
    return float(T * ell.sum()), g, K


def solve_static(X, tri, Bm, area, mu, lam, fixed, fext=None, tendon_nodes=None, T=0.0, ramps=6,
                 tol=1e-10, max_newton=60):
    """Equilibrium positions (N, 2) of the free nodes with `fixed` held at X, loads ramped in
    over `ramps` stages; returns (x, residual) with the residual the largest free-node force
    imbalance relative to the largest elastic nodal force."""
    X = np.asarray(X, np.float64)
    tri = np.asarray(tri, np.int64)
    Bm, area = np.asarray(Bm, np.float64), np.asarray(area, np.float64)
    mu, lam = np.asarray(mu, np.float64), np.asarray(lam, np.float64)
    f = np.zeros_like(X) if fext is None else np.asarray(fext, np.float64)
    free = np.ones(X.size, bool)
    fx = np.asarray(fixed, np.int64)
    free[2 * fx] = False
    free[2 * fx + 1] = False
    x = X.copy()

    def total(xx, s, tangent=True):
        E, g, K = elastic(xx, tri, Bm, area, mu, lam, tangent)
        if not np.isfinite(E):
            return np.inf, None, None
        Et, gt, Kt = tendon(xx, tendon_nodes if tendon_nodes is not None else [], s * T)
        E = E + Et - s * float((f * (xx - X)).sum())
        g = g + gt - s * f
        return E, g, (K + Kt if tangent else None)

    res = np.inf
    for r in range(1, ramps + 1):
        s = r / ramps
        for _ in range(max_newton):
            E, g, K = total(x, s)
            gf = g.ravel()[free]
            scale = max(np.abs(elastic(x, tri, Bm, area, mu, lam, False)[1]).max(), np.abs(s * f).max(), 1e-300)
            res = float(np.abs(gf).max() / scale)
            if res < tol:
                break
            Kff = K[free][:, free].tocsc()
            dx = np.zeros(X.size)
            dx[free] = spla.spsolve(Kff, -gf)
            t = 1.0
            while t > 1e-8:
                xn = x + t * dx.reshape(-1, 2)
                En = total(xn, s, tangent=False)[0]
                if np.isfinite(En) and En <= E + 1e-4 * t * float(gf @ dx[free]):
                    break
                t *= 0.5
            x = xn
    return x, res
