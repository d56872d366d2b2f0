"""Oracle nodal Green-Lagrange strain by weighted least squares (FP64).

Test infrastructure only (see oracle/__init__.py).

Reference: d2ic/strain.py:11-114.
"""
from __future__ import annotations

import numpy as np


def green_lagrange_nodes_lsq(u, nodes, nbr_index, nbr_degree, gauge_length=0.0, eps=1e-8):
    """Per node: LSQ displacement gradient, F = I + grad u, E = (F^T F - I)/2.

    d2ic/strain.py:11-92: neighbours beyond the degree get weight 0 (their
    index replaced by 0), Gaussian weight ``exp(-(r/(L+1e-12))^2)`` when L > 0,
    normal matrix ``sum w dX dX^T + eps I``.  Returns ``(F, E)`` each (Nn,2,2).
    """
    u = np.asarray(u, dtype=np.float64)
    X = np.asarray(nodes, dtype=np.float64)
    idx = np.asarray(nbr_index)
    Nn, md = idx.shape
    mask = np.arange(md)[None, :] < np.asarray(nbr_degree)[:, None]
    nid = np.where(mask, idx, 0)
    dX = X[nid] - X[:, None, :]
    du = u[nid] - u[:, None, :]
    w = mask.astype(np.float64)
    L = float(gauge_length)
    if L > 0.0:
        r = np.linalg.norm(dX, axis=2)
        w = w * np.exp(-(r / (L + 1e-12)) ** 2)
    Xw = dX * w[..., None]
    A = np.einsum("nki,nkj->nij", Xw, dX) + eps * np.eye(2)
    b0 = np.einsum("nki,nk->ni", Xw, du[..., 0])
    b1 = np.einsum("nki,nk->ni", Xw, du[..., 1])
    gx = np.linalg.solve(A, b0[..., None])[..., 0]
    gy = np.linalg.solve(A, b1[..., None])[..., 0]
    G = np.stack([gx, gy], axis=1)
    F = np.eye(2)[None] + G
    C = np.einsum("nki,nkj->nij", F, F)
    E = 0.5 * (C - np.eye(2)[None])
    return F, E


def to_voigt(E):
    """``[E11, E22, E12]`` of the symmetric part (d2ic/strain.py:95-114)."""
    E = np.asarray(E)
    s = 0.5 * (E + np.swapaxes(E, 1, 2))
    return np.stack([s[:, 0, 0], s[:, 1, 1], s[:, 0, 1]], axis=1)
