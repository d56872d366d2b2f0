"""Oracle objective, analytic gradient and nonlinear CG solve (FP64).

Test infrastructure only (see oracle/__init__.py).

Reference: d2ic/solver_global_cg.py:205-469.  The reference obtains the
gradient with ``jax.value_and_grad``; here it is written out analytically
(chain rule through the Q4 interpolation and the sampler) and the tests check
it against central finite differences.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .cubic import ORACLE_PAD, bspline_coefficients, cubic_sample, linear_sample


@dataclass
class Problem:
    """Inputs of one frame, in the reference's asset layout (FP64)."""
    coeff1: np.ndarray | None      # B-spline coefficients of the reference image (cubic)
    coeff2: np.ndarray | None      # ... of the deformed image
    im1: np.ndarray                # raw images (used by 'linear')
    im2: np.ndarray
    pixel_coords: np.ndarray       # (Np,2) pixel centres, x = col + 0.5
    pixel_nodes: np.ndarray        # (Np,4)
    pixel_shapeN: np.ndarray       # (Np,4)
    nbr_index: np.ndarray          # (Nn,maxdeg), -1 padded
    nbr_degree: np.ndarray         # (Nn,)
    nbr_weight: np.ndarray         # (Nn,maxdeg)
    node_reg_weight: np.ndarray    # (Nn,)
    interpolation: str = "cubic"

    @staticmethod
    def build(ref_image, def_image, assets, interpolation="cubic"):
        c1 = c2 = None
        if interpolation == "cubic":
            c1 = bspline_coefficients(ref_image)
            c2 = bspline_coefficients(def_image)
        return Problem(c1, c2, np.asarray(ref_image, np.float64), np.asarray(def_image, np.float64),
                       assets["pixel_coords_ref"], assets["pixel_nodes"], assets["pixel_shapeN"],
                       assets["node_neighbor_index"], assets["node_neighbor_degree"],
                       assets["node_neighbor_weight"], assets["node_reg_weight"], interpolation)

    def sample(self, which, xy, with_grad=False):
        """Sample image 1 or 2 at pixel-centre coordinates (shift by -0.5 as the reference)."""
        if self.interpolation == "cubic":
            c = self.coeff1 if which == 1 else self.coeff2
            return cubic_sample(c, ORACLE_PAD, xy[:, 0] - 0.5, xy[:, 1] - 0.5, with_grad)
        im = self.im1 if which == 1 else self.im2
        return linear_sample(im, xy[:, 0], xy[:, 1], with_grad)


def residuals(u, pb: Problem, with_grad=False):
    """``r = I2(x + sum_a N_a u_a) - I1(x)`` (d2ic/solver_global_cg.py:205-234)."""
    u = np.asarray(u, dtype=np.float64)
    N = pb.pixel_shapeN
    u_pix = np.einsum("pa,pac->pc", N, u[pb.pixel_nodes])
    x_def = pb.pixel_coords + u_pix
    I1 = pb.sample(1, pb.pixel_coords)
    if with_grad:
        I2, gx, gy = pb.sample(2, x_def, True)
        return I2 - I1, gx, gy
    return pb.sample(2, x_def) - I1


def reg_energy(u, pb: Problem):
    """Spring energy (d2ic/solver_global_cg.py:261-286).

    ``0.25 * sum_i sum_{k<deg_i} w_ik * 0.5 (rho_i + rho_j) * |u_i - u_j|^2``.
    """
    u = np.asarray(u, dtype=np.float64)
    idx = pb.nbr_index
    Nn, md = idx.shape
    mask = np.arange(md)[None, :] < pb.nbr_degree[:, None]
    nid = np.where(mask, idx, 0)
    w = np.where(mask, pb.nbr_weight, 0.0) * 0.5 * (pb.node_reg_weight[:, None] + pb.node_reg_weight[nid])
    diff = np.where(mask[..., None], u[:, None, :] - u[nid], 0.0)
    return 0.25 * np.sum(w * np.sum(diff ** 2, axis=2))


def reg_energy_grad(u, pb: Problem):
    """Gradient of :func:`reg_energy` for any (not necessarily symmetric) table."""
    u = np.asarray(u, dtype=np.float64)
    idx = pb.nbr_index
    Nn, md = idx.shape
    mask = np.arange(md)[None, :] < pb.nbr_degree[:, None]
    nid = np.where(mask, idx, 0)
    w = np.where(mask, pb.nbr_weight, 0.0) * 0.5 * (pb.node_reg_weight[:, None] + pb.node_reg_weight[nid])
    diff = np.where(mask[..., None], u[:, None, :] - u[nid], 0.0)       # (Nn,md,2)
    g = 0.5 * np.sum(w[..., None] * diff, axis=1)
    contrib = -0.5 * w[..., None] * diff
    np.add.at(g, nid.ravel(), contrib.reshape(-1, 2))
    return g


def J_total(u, pb: Problem, alpha_reg):
    """``0.5 * sum r^2 / max(Np,1) + alpha * E_reg`` (d2ic/solver_global_cg.py:237-320)."""
    r = residuals(u, pb)
    denom = max(r.shape[0], 1)
    return 0.5 * np.sum(r ** 2) / denom + alpha_reg * reg_energy(u, pb)


def J_total_and_grad(u, pb: Problem, alpha_reg):
    """Value and analytic gradient of :func:`J_total`.

    ``dJ/du_n = (1/Np) sum_{p: n in p} r_p N_n(p) grad I2(x_def,p) + alpha dE/du_n``.
    """
    r, gx, gy = residuals(u, pb, with_grad=True)
    Np = r.shape[0]
    denom = max(Np, 1)
    J = 0.5 * np.sum(r ** 2) / denom + alpha_reg * reg_energy(u, pb)
    Nn = np.asarray(u).shape[0]
    g = np.zeros((Nn, 2))
    w = pb.pixel_shapeN * (r / denom)[:, None]
    for a in range(pb.pixel_nodes.shape[1]):
        g[:, 0] += np.bincount(pb.pixel_nodes[:, a], weights=w[:, a] * gx, minlength=Nn)
        g[:, 1] += np.bincount(pb.pixel_nodes[:, a], weights=w[:, a] * gy, minlength=Nn)
    g += alpha_reg * reg_energy_grad(u, pb)
    return J, g


def cg_solve(u0, pb: Problem, alpha_reg, max_iter, tol, value_and_grad=None, value=None):
    """Nonlinear Polak-Ribiere+ CG with Armijo backtracking.

    Literal control flow of ``_cg_solve`` (d2ic/solver_global_cg.py:326-469):

    * stop when ``|g|_2 < tol`` at the start of an iteration: history row
      ``[J, |g|, 0]`` at index k, k not incremented;
    * ``d = -g`` at k = 0, else ``-g + max(0, g.(g-g_prev)/(g_prev.g_prev + 1e-16)) d``;
      restart ``d = -g`` (and ``g.d = -g.g``) when ``g.d >= 0``;
    * Armijo ``J(u + a d) <= J + 1e-4 a g.d`` from a = 1, halving, 10 tries; after
      10 failures a = 2**-10 is applied anyway (history keeps the last tried J);
    * history rows ``[J_trial, |g|, a]``, NaN elsewhere.

    Returns ``(u, hist (max_iter,3), k, n_evals)``.
    """
    if value_and_grad is None:
        value_and_grad = lambda uu: J_total_and_grad(uu, pb, alpha_reg)
    if value is None:
        value = lambda uu: J_total(uu, pb, alpha_reg)
    max_iter = int(max_iter)
    u = np.array(u0, dtype=np.float64)
    hist = np.full((max_iter, 3), np.nan)
    d = np.zeros_like(u)
    g_prev = np.zeros_like(u)
    k = 0
    n_evals = 0
    while k < max_iter:
        J, g = value_and_grad(u)
        n_evals += 1
        gn = float(np.linalg.norm(g))
        if gn < tol:
            hist[k] = [J, gn, 0.0]
            break
        if k == 0:
            dn = -g
        else:
            beta = max(np.sum(g * (g - g_prev)) / (np.sum(g_prev * g_prev) + 1e-16), 0.0)
            dn = -g + beta * d
        gd = np.sum(g * dn)
        if gd >= 0:
            dn = -g
            gd = -np.sum(g * g)
        alpha = 1.0
        J_c = J
        done = False
        for _ in range(10):
            if done:
                continue
            J_c = value(u + alpha * dn)
            n_evals += 1
            if J_c <= J + 1e-4 * alpha * gd:
                done = True
            else:
                alpha *= 0.5
        u = u + alpha * dn
        hist[k] = [J_c, gn, alpha]
        d = dn
        g_prev = g
        k += 1
    return u, hist, k, n_evals
