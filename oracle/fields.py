"""Per-element strain and stress from node positions (numpy) — TEST INFRASTRUCTURE ONLY:
the checker of the device read-outs (d2f_element_fields). A restatement of the reference's
core/fields.py (deformation_gradient :22-26, green_lagrange :36-38, cauchy_stress :41-49,
von Mises :52-61, principal values :64-76, element_field :79-92)."""
from __future__ import annotations

import numpy as np


def deformation_gradient(tri, Bm, x):
    p = np.asarray(x, np.float64)[np.asarray(tri)]
    Ds = np.stack([p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]], -1)       # edge vectors as columns
    return Ds @ np.asarray(Bm, np.float64).reshape(-1, 2, 2)


def _in_3d(T2, zz):
    T = np.zeros((len(T2), 3, 3))
    T[:, :2, :2] = T2
    T[:, 2, 2] = zz
    return T


def _dev_norm2(T):
    dev = T - np.trace(T, axis1=1, axis2=2)[:, None, None] / 3.0 * np.eye(3)
    return np.einsum("nij,nij->n", dev, dev)


def _signed_principal(T):
    a, b, d = T[:, 0, 0], T[:, 0, 1], T[:, 1, 1]
    m, r = 0.5 * (a + d), np.sqrt(0.25 * (a - d) ** 2 + b * b)
    hi, lo = m + r, m - r
    return np.where(np.abs(hi) >= np.abs(lo), hi, lo)


def element_field(tri, Bm, mu, lam, x, field, signed=False):
    F = deformation_gradient(tri, Bm, x)
    if field == "strain":
        T = _in_3d(0.5 * (F.transpose(0, 2, 1) @ F - np.eye(2)), 0.0)
        return _signed_principal(T) if signed else np.sqrt(2.0 / 3.0 * _dev_norm2(T))
    J = np.linalg.det(F)
    lnJ = np.log(np.maximum(J, 1e-12))
    mu, lam = np.asarray(mu, np.float64), np.asarray(lam, np.float64)
    s2 = (mu[:, None, None] * (F @ F.transpose(0, 2, 1)) + ((lam * lnJ - mu)[:, None, None]) * np.eye(2)) / J[:, None, None]
    T = _in_3d(s2, lam * lnJ / J)
    return _signed_principal(T) if signed else np.sqrt(1.5 * _dev_norm2(T))
