"""Oracle image samplers (FP64).

Test infrastructure only (see oracle/__init__.py).

The reference samples images with ``im_jax.flat_nd_cubic_interpolate(image_T,
coords - 0.5, mode="nearest", cval=0.0, layout="HW")``
(d2ic/solver_global_cg.py:512-518).  im_jax is a third-party package that is
neither vendored in the reference nor pinned to a version (pyproject.toml:19),
and no reference test pins its output, so its exact cubic kernel is unknown:
CUBIC PARITY WITH THE REFERENCE IS UNPINNED.

This oracle defines the cubic sampler as the interpolating cubic B-spline
(prefiltered coefficients, pole z = sqrt(3) - 2) of the image extended by
edge replication ('nearest'), evaluated at image-index coordinates
``(x - 0.5, y - 0.5)`` (x = column, y = row).  It is checked against the
independent ``scipy.ndimage.map_coordinates(order=3, mode='nearest')``.

The bilinear sampler restates the reference's in-repo fallback
``_bilinear_sample`` (d2ic/solver_global_cg.py:481-509) with edge clamping.
"""
from __future__ import annotations

import numpy as np

POLE = np.sqrt(3.0) - 2.0
ORACLE_PAD = 40           # z**40 ~ 1e-23: the truncated boundary is invisible


def _prefilter_axis0(a: np.ndarray) -> np.ndarray:
    """Exact cubic B-spline prefilter along axis 0 (causal + anti-causal IIR).

    Mirror-symmetric initialisation at both ends; applied to a signal that was
    edge-padded by ORACLE_PAD samples, the boundary rule has no visible effect
    on the original samples.
    """
    z = POLE
    n = a.shape[0]
    c = np.empty_like(a)
    # causal init: sum_k z^k s[k] (truncated at machine precision)
    K = min(n, 60)
    zk = z ** np.arange(K)
    c[0] = np.tensordot(zk, a[:K], axes=(0, 0))
    for i in range(1, n):
        c[i] = a[i] + z * c[i - 1]
    out = np.empty_like(a)
    out[n - 1] = (z / (z * z - 1.0)) * (c[n - 1] + z * c[n - 2])
    for i in range(n - 2, -1, -1):
        out[i] = z * (out[i + 1] - c[i])
    return 6.0 * out


def bspline_coefficients(image: np.ndarray, pad: int = ORACLE_PAD) -> np.ndarray:
    """Cubic B-spline coefficients of the edge-extended image, with a ``pad`` halo.

    Returns an array of shape (H + 2 pad, W + 2 pad) in which entry
    ``[pad + i, pad + j]`` is the coefficient at pixel (i, j).
    """
    img = np.asarray(image, dtype=np.float64)
    ext = np.pad(img, pad, mode="edge")
    c = _prefilter_axis0(ext)
    c = _prefilter_axis0(c.T).T
    return c


def bspline_weights(t):
    """Cubic B-spline weights and their derivatives for taps -1, 0, 1, 2."""
    t2 = t * t
    t3 = t2 * t
    omt = 1.0 - t
    w = np.stack([omt ** 3 / 6.0, (3 * t3 - 6 * t2 + 4) / 6.0, (-3 * t3 + 3 * t2 + 3 * t + 1) / 6.0, t3 / 6.0])
    dw = np.stack([-0.5 * omt * omt, 1.5 * t2 - 2 * t, -1.5 * t2 + t + 0.5, 0.5 * t2])
    return w, dw


def cubic_sample(coeff: np.ndarray, pad: int, x, y, with_grad: bool = False):
    """Evaluate the B-spline at image-index coordinates ``(x, y)`` (column, row).

    Taps outside the coefficient array are clamped to its border, where the
    coefficients equal the edge value (constant extension).  With ``with_grad``
    also returns the analytic derivatives d/dx and d/dy.
    """
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    Hc, Wc = coeff.shape
    ix = np.floor(x).astype(np.int64)
    iy = np.floor(y).astype(np.int64)
    wx, dwx = bspline_weights(x - ix)
    wy, dwy = bspline_weights(y - iy)
    val = np.zeros_like(x)
    gx = np.zeros_like(x)
    gy = np.zeros_like(x)
    for a in range(4):
        rr = np.clip(iy - 1 + a + pad, 0, Hc - 1)
        rv = np.zeros_like(x)
        rd = np.zeros_like(x)
        for b in range(4):
            cc = np.clip(ix - 1 + b + pad, 0, Wc - 1)
            cv = coeff[rr, cc]
            rv += wx[b] * cv
            rd += dwx[b] * cv
        val += wy[a] * rv
        gx += wy[a] * rd
        gy += dwy[a] * rv
    if with_grad:
        return val, gx, gy
    return val


def bspline_weights2(t):
    """Second derivatives of the cubic B-spline weights for taps -1, 0, 1, 2."""
    return np.stack([1.0 - t, 3.0 * t - 2.0, -3.0 * t + 1.0, t])


def cubic_sample_hessian(coeff: np.ndarray, pad: int, x, y):
    """Value, gradient and Hessian (d2/dx2, d2/dxdy, d2/dy2) of the spline at (x, y)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    Hc, Wc = coeff.shape
    ix = np.floor(x).astype(np.int64)
    iy = np.floor(y).astype(np.int64)
    tx, ty = x - ix, y - iy
    wx, dwx = bspline_weights(tx)
    wy, dwy = bspline_weights(ty)
    ddwx, ddwy = bspline_weights2(tx), bspline_weights2(ty)
    out = {k: np.zeros_like(x) for k in ("v", "gx", "gy", "hxx", "hxy", "hyy")}
    for a in range(4):
        rr = np.clip(iy - 1 + a + pad, 0, Hc - 1)
        rv = np.zeros_like(x)
        rd = np.zeros_like(x)
        rdd = np.zeros_like(x)
        for b in range(4):
            cv = coeff[rr, np.clip(ix - 1 + b + pad, 0, Wc - 1)]
            rv += wx[b] * cv
            rd += dwx[b] * cv
            rdd += ddwx[b] * cv
        out["v"] += wy[a] * rv
        out["gx"] += wy[a] * rd
        out["gy"] += dwy[a] * rv
        out["hxx"] += wy[a] * rdd
        out["hxy"] += dwy[a] * rd
        out["hyy"] += ddwy[a] * rv
    return out


def linear_sample(image: np.ndarray, x, y, with_grad: bool = False):
    """Bilinear sample at pixel-centre coordinates ``(x, y)`` (x = col + 0.5).

    Restates d2ic/solver_global_cg.py:481-509: ``x0 = floor(x - 0.5)``, taps
    clamped into the image.  (The reference clamps the column with the row
    count and vice versa; the two agree for square images, which is all the
    benchmark uses.)  The derivative is that of the bilinear form (clamping
    contributes nothing), as autodiff gives.
    """
    img = np.asarray(image, dtype=np.float64)
    H, W = img.shape
    xs = np.asarray(x, dtype=np.float64) - 0.5
    ys = np.asarray(y, dtype=np.float64) - 0.5
    x0 = np.floor(xs).astype(np.int64)
    y0 = np.floor(ys).astype(np.int64)
    fx = xs - x0
    fy = ys - y0
    cx0 = np.clip(x0, 0, W - 1); cx1 = np.clip(x0 + 1, 0, W - 1)
    cy0 = np.clip(y0, 0, H - 1); cy1 = np.clip(y0 + 1, 0, H - 1)
    i00 = img[cy0, cx0]; i10 = img[cy0, cx1]; i01 = img[cy1, cx0]; i11 = img[cy1, cx1]
    val = (1 - fx) * (1 - fy) * i00 + fx * (1 - fy) * i10 + (1 - fx) * fy * i01 + fx * fy * i11
    if not with_grad:
        return val
    gx = (1 - fy) * (i10 - i00) + fy * (i11 - i01)
    gy = (1 - fx) * (i01 - i00) + fx * (i11 - i10)
    return val, gx, gy
