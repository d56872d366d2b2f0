"""Oracle implicit-function derivative of the converged solve (FP64).

Test infrastructure only (see oracle/__init__.py).

The reference propagates image noise with ``jax.jvp`` through a fixed, 25
iteration unrolled nonlinear CG (doc/11_Advanced_Use_Uncertainty_Propagation.ipynb,
cells 14, 22, 30).  The derivative of the *converged* solution u*(I2), defined
by grad_u J(u*, I2) = 0, is the implicit-function derivative

    du*/dI2 . dI = -H^-1 (d grad_u J / dI2) . dI,

with H the exact Hessian of J at u*:
    H_ab = (1/Np) sum_p N_a N_b (grad I2 grad I2^T + r hess I2) + alpha * spring Hessian,
and the mixed term
    (d grad_u J / dI2 . dI)_a = (1/Np) sum_p N_a (dI(x_def) grad I2 + r grad dI(x_def)),
dI sampled with the same cubic B-spline (linear in dI).  The FD check solves
to machine precision with Newton steps on the same Hessian.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .cubic import ORACLE_PAD, bspline_coefficients, cubic_sample, cubic_sample_hessian
from .objective import Problem, J_total_and_grad


def _pixel_state(u, pb: Problem):
    N = pb.pixel_shapeN
    u_pix = np.einsum("pa,pac->pc", N, np.asarray(u, np.float64)[pb.pixel_nodes])
    xd = pb.pixel_coords + u_pix
    s = cubic_sample_hessian(pb.coeff2, ORACLE_PAD, xd[:, 0] - 0.5, xd[:, 1] - 0.5)
    I1 = cubic_sample(pb.coeff1, ORACLE_PAD, pb.pixel_coords[:, 0] - 0.5, pb.pixel_coords[:, 1] - 0.5)
    return xd, s, s["v"] - I1


def spring_hessian(pb: Problem, n_nodes: int) -> sp.csr_matrix:
    """Hessian of the spring energy 0.25 sum_i sum_k w_ik |u_i - u_j|^2 (one component; same for x and y)."""
    idx = pb.nbr_index
    md = idx.shape[1]
    mask = np.arange(md)[None, :] < pb.nbr_degree[:, None]
    nid = np.where(mask, idx, 0)
    w = np.where(mask, pb.nbr_weight, 0.0) * 0.5 * (pb.node_reg_weight[:, None] + pb.node_reg_weight[nid])
    i = np.repeat(np.arange(n_nodes), md)[mask.ravel()]
    j = nid.ravel()[mask.ravel()]
    ww = w.ravel()[mask.ravel()]
    rows = np.concatenate([i, j, i, j])
    cols = np.concatenate([i, j, j, i])
    vals = np.concatenate([0.5 * ww, 0.5 * ww, -0.5 * ww, -0.5 * ww])
    return sp.csr_matrix((vals, (rows, cols)), shape=(n_nodes, n_nodes))


def hessian(u, pb: Problem, alpha_reg: float, exact: bool = True) -> sp.csr_matrix:
    """Exact (or Gauss-Newton) Hessian of J_total at u, dofs ordered (node, component)."""
    n_nodes = np.asarray(u).shape[0]
    _, s, r = _pixel_state(u, pb)
    Np = max(r.shape[0], 1)
    mxx = s["gx"] * s["gx"]
    mxy = s["gx"] * s["gy"]
    myy = s["gy"] * s["gy"]
    if exact:
        mxx = mxx + r * s["hxx"]
        mxy = mxy + r * s["hxy"]
        myy = myy + r * s["hyy"]
    N = pb.pixel_shapeN
    pn = pb.pixel_nodes
    rows, cols, vals = [], [], []
    for a in range(4):
        for b in range(4):
            nab = N[:, a] * N[:, b] / Np
            for (ca, cb, m) in ((0, 0, mxx), (0, 1, mxy), (1, 0, mxy), (1, 1, myy)):
                rows.append(2 * pn[:, a] + ca)
                cols.append(2 * pn[:, b] + cb)
                vals.append(nab * m)
    Hp = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                       shape=(2 * n_nodes, 2 * n_nodes))
    L = spring_hessian(pb, n_nodes)
    return (Hp + alpha_reg * sp.kron(L, sp.eye(2))).tocsr()


def mixed_term(u, pb: Problem, dI) -> np.ndarray:
    """(d grad_u J / dI2) . dI as an (Nn, 2) array."""
    xd, s, r = _pixel_state(u, pb)
    Np = max(r.shape[0], 1)
    cd = bspline_coefficients(np.asarray(dI, np.float64))
    dv, dgx, dgy = cubic_sample(cd, ORACLE_PAD, xd[:, 0] - 0.5, xd[:, 1] - 0.5, with_grad=True)
    tx = (dv * s["gx"] + r * dgx) / Np
    ty = (dv * s["gy"] + r * dgy) / Np
    n_nodes = np.asarray(u).shape[0]
    out = np.zeros((n_nodes, 2))
    for a in range(4):
        out[:, 0] += np.bincount(pb.pixel_nodes[:, a], weights=pb.pixel_shapeN[:, a] * tx, minlength=n_nodes)
        out[:, 1] += np.bincount(pb.pixel_nodes[:, a], weights=pb.pixel_shapeN[:, a] * ty, minlength=n_nodes)
    return out


def _active(H: sp.csr_matrix) -> np.ndarray:
    """Dofs with any Hessian entry (nodes outside every element and spring have none)."""
    return np.flatnonzero(np.asarray(abs(H).sum(axis=1)).ravel() > 0)


def implicit_jvp(u, pb: Problem, alpha_reg: float, dI, exact: bool = True) -> np.ndarray:
    H = hessian(u, pb, alpha_reg, exact)
    rhs = mixed_term(u, pb, dI).reshape(-1)
    act = _active(H)
    du = np.zeros_like(rhs)
    du[act] = -spla.spsolve(H[act][:, act].tocsc(), rhs[act])
    return du.reshape(-1, 2)


def newton_solve(u0, pb: Problem, alpha_reg: float, tol: float = 1e-13, max_iter: int = 30):
    """Minimiser of J_total by exact Newton steps (oracle-side convenience for finite differences)."""
    u = np.array(u0, dtype=np.float64)
    for _ in range(max_iter):
        J, g = J_total_and_grad(u, pb, alpha_reg)
        if np.linalg.norm(g) < tol:
            break
        H = hessian(u, pb, alpha_reg, True)
        act = _active(H)
        step = np.zeros(g.size)
        step[act] = spla.spsolve(H[act][:, act].tocsc(), g.reshape(-1)[act])
        u = u - step.reshape(-1, 2)
    return u


def with_image(pb: Problem, image) -> Problem:
    """A copy of the problem with another deformed image."""
    img = np.asarray(image, np.float64)
    return Problem(pb.coeff1, bspline_coefficients(img), pb.im1, img, pb.pixel_coords, pb.pixel_nodes,
                   pb.pixel_shapeN, pb.nbr_index, pb.nbr_degree, pb.nbr_weight, pb.node_reg_weight,
                   pb.interpolation)


def fd_jvp(u_star, pb: Problem, alpha_reg: float, dI, h: float) -> np.ndarray:
    """Central finite difference of the converged solution along the image direction dI."""
    up = newton_solve(u_star, with_image(pb, pb.im2 + h * dI), alpha_reg)
    um = newton_solve(u_star, with_image(pb, pb.im2 - h * dI), alpha_reg)
    return (up - um) / (2 * h)
