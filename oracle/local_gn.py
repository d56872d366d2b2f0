"""Oracle (test infrastructure only): the local Gauss-Newton sweeps in FP64.

Restates d2ic/solver_local_gn.py:
* ``_compute_image_gradient_np`` (:195-201): central differences, zero on the
  first/last column (x) and row (y);
* ``_pixel_state`` (:214-256): r = I2(x_def) - I1(x_ref), and the gradient
  images sampled at x_def with the same interpolator (cubic: B-spline with
  edge replication, at (x - 0.5, y - 0.5));
* ``jacobi_nodal_step_spring`` (:316-414): per node the 2x2 Gauss-Newton
  normal equations of its pixels (J = grad * N), Levenberg term lam * trace,
  spring term alpha * rho_i * sum_j w_ij (u_i - u_j), +1e-8 I, a relaxed
  (omega) step clipped to max_step; nodes without pixels and springs stay put;
* ``_local_sweeps`` (:259-313): n_sweeps sweeps, history [rms r, rms step].
"""
from __future__ import annotations

import numpy as np

from .cubic import ORACLE_PAD, bspline_coefficients, cubic_sample, linear_sample


def central_gradient(im):
    im = np.asarray(im, dtype=np.float64)
    gx = np.zeros_like(im)
    gy = np.zeros_like(im)
    gx[:, 1:-1] = 0.5 * (im[:, 2:] - im[:, :-2])
    gy[1:-1, :] = 0.5 * (im[2:, :] - im[:-2, :])
    return gx, gy


def local_sweeps(u0, pb, lam, max_step, alpha_reg, omega, n_sweeps):
    """``pb``: an :class:`oracle.objective.Problem`; returns (u, history (n_sweeps, 2))."""
    u = np.asarray(u0, dtype=np.float64).copy()
    gx2, gy2 = central_gradient(pb.im2)
    if pb.interpolation == "cubic":
        cgx, cgy = bspline_coefficients(gx2), bspline_coefficients(gy2)
        samp = lambda c, xy: cubic_sample(c, ORACLE_PAD, xy[:, 0] - 0.5, xy[:, 1] - 0.5)
        sgx = lambda xy: samp(cgx, xy)
        sgy = lambda xy: samp(cgy, xy)
    else:
        sgx = lambda xy: linear_sample(gx2, xy[:, 0], xy[:, 1])
        sgy = lambda xy: linear_sample(gy2, xy[:, 0], xy[:, 1])
    N = pb.pixel_shapeN
    pn = pb.pixel_nodes
    Nn = u.shape[0]
    idx = np.asarray(pb.nbr_index)
    deg = np.asarray(pb.nbr_degree)
    wts = np.asarray(pb.nbr_weight, dtype=np.float64)
    rho = np.asarray(pb.node_reg_weight, dtype=np.float64)
    md = idx.shape[1]
    nmask = np.arange(md)[None, :] < deg[:, None]
    nid = np.where(nmask, idx, 0)
    w = np.where(nmask, wts, 0.0)
    has_pix = np.zeros(Nn, dtype=bool)
    has_pix[np.unique(pn)] = True
    hist = np.full((n_sweeps, 2), np.nan)
    I1 = pb.sample(1, pb.pixel_coords)
    for k in range(n_sweeps):
        x_def = pb.pixel_coords + np.einsum("pa,pac->pc", N, u[pn])
        r = pb.sample(2, x_def) - I1
        gx, gy = sgx(x_def), sgy(x_def)
        Jx = gx[:, None] * N
        Jy = gy[:, None] * N
        acc = np.zeros((Nn, 5))
        for a in range(N.shape[1]):
            np.add.at(acc, pn[:, a], np.stack([r * Jx[:, a], r * Jy[:, a], Jx[:, a] ** 2, Jx[:, a] * Jy[:, a],
                                               Jy[:, a] ** 2], axis=1))
        g0, g1, H00, H01, H11 = acc.T
        lam_loc = lam * (H00 + H11 + 1e-12)
        diff = u[:, None, :] - np.where(nmask[..., None], u[nid], 0.0)
        alpha_loc = alpha_reg * rho
        g_reg = alpha_loc[:, None] * np.sum(w[..., None] * diff, axis=1)
        hreg = alpha_loc * w.sum(axis=1)
        a11 = H00 + lam_loc + hreg + 1e-8
        a22 = H11 + lam_loc + hreg + 1e-8
        a12 = H01
        b0, b1 = g0 + g_reg[:, 0], g1 + g_reg[:, 1]
        det = a11 * a22 - a12 * a12
        dx = -(a22 * b0 - a12 * b1) / det
        dy = -(a11 * b1 - a12 * b0) / det
        upd = has_pix | ((alpha_reg != 0.0) & (deg > 0))
        delta = np.where(upd[:, None], np.stack([dx, dy], axis=1), 0.0)
        nrm = np.linalg.norm(delta, axis=1)
        delta = delta * np.minimum(1.0, max_step / (nrm + 1e-12))[:, None]
        step = omega * delta
        hist[k] = [np.sqrt(np.mean(r * r)), np.sqrt(np.mean(step * step))]
        u = u + step
    return u, hist
