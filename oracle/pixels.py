"""Oracle restatement of the pixel-level assets (FP64).

Test infrastructure only (see oracle/__init__.py).

Reference: d2ic/pixel_assets.py:21-526.
"""
from __future__ import annotations

import numpy as np


def sample_pixels_in_bbox(nodes, H, W, pad=2.0):
    """Pixel centres ``(j+0.5, i+0.5)`` inside the padded node bounding box.

    d2ic/pixel_assets.py:115-132: rows outer, columns inner (meshgrid order).
    """
    nodes = np.asarray(nodes, dtype=np.float64)
    j0 = max(0, int(np.floor(nodes[:, 0].min() - pad)))
    j1 = min(W, int(np.ceil(nodes[:, 0].max() + pad)))
    i0 = max(0, int(np.floor(nodes[:, 1].min() - pad)))
    i1 = min(H, int(np.ceil(nodes[:, 1].max() + pad)))
    jj, ii = np.meshgrid(np.arange(j0, j1), np.arange(i0, i1))
    return np.stack([jj.ravel() + 0.5, ii.ravel() + 0.5], axis=1)


def _quad_geometry(nodes, elements):
    quad = np.asarray(nodes, dtype=np.float64)[np.asarray(elements)]      # (Ne,4,2)
    nxt = np.roll(quad, -1, axis=1)
    edges = nxt - quad
    area2 = np.sum(quad[:, :, 0] * nxt[:, :, 1] - quad[:, :, 1] * nxt[:, :, 0], axis=1)
    orient = np.where(area2 >= 0.0, 1.0, -1.0)
    return quad, edges, orient, quad.min(axis=1), quad.max(axis=1)


def pixel_to_element_bruteforce(pixel_coords, nodes, elements, tol=1e-6, chunk=2048):
    """First element (lowest index) whose bbox and half-plane test accept the pixel.

    d2ic/pixel_assets.py:135-237: ``valid = in_bbox & all(orient*cross >= -tol)``,
    ``first = argmax(valid)``, -1 when no element is valid; node ids of the
    chosen element, zeros for rejected pixels.  O(Np*Ne): small cases only.
    """
    pc = np.asarray(pixel_coords, dtype=np.float64)
    elements = np.asarray(elements, dtype=np.int64)
    Np, Ne = pc.shape[0], elements.shape[0]
    if Np == 0 or Ne == 0:
        return -np.ones(Np, dtype=np.int64), np.zeros((Np, 4), dtype=np.int64)
    quad, edges, orient, bmin, bmax = _quad_geometry(nodes, elements)
    elts = np.empty(Np, dtype=np.int64)
    for s in range(0, Np, chunk):
        p = pc[s:s + chunk]
        x = p[:, 0][:, None]
        y = p[:, 1][:, None]
        in_bb = (x >= bmin[:, 0]) & (x <= bmax[:, 0]) & (y >= bmin[:, 1]) & (y <= bmax[:, 1])
        vec = p[:, None, None, :] - quad[None]
        cross = edges[None, :, :, 0] * vec[..., 1] - edges[None, :, :, 1] * vec[..., 0]
        inside = np.all(orient[None, :, None] * cross >= -tol, axis=-1)
        valid = in_bb & inside
        anyv = valid.any(axis=1)
        elts[s:s + chunk] = np.where(anyv, np.argmax(valid, axis=1), -1)
    nodes_out = np.where((elts >= 0)[:, None], elements[np.maximum(elts, 0)], 0)
    return elts, nodes_out


def pixel_to_element_hashed(pixel_coords, nodes, elements, tol=1e-6, cell=None):
    """Same semantics as :func:`pixel_to_element_bruteforce`, bbox-culled.

    A pixel can only be accepted by an element whose bounding box contains it
    (the bbox test is part of ``valid``), so testing only those candidates and
    keeping the lowest valid element index gives the identical answer.
    Candidates come from a uniform grid over element bounding boxes.
    """
    pc = np.asarray(pixel_coords, dtype=np.float64)
    elements = np.asarray(elements, dtype=np.int64)
    Np, Ne = pc.shape[0], elements.shape[0]
    if Np == 0 or Ne == 0:
        return -np.ones(Np, dtype=np.int64), np.zeros((Np, 4), dtype=np.int64)
    quad, edges, orient, bmin, bmax = _quad_geometry(nodes, elements)
    if cell is None:
        cell = max(1.0, float(np.median(bmax - bmin)))
    ox, oy = float(bmin[:, 0].min()), float(bmin[:, 1].min())
    cx0 = np.floor((bmin[:, 0] - ox) / cell).astype(np.int64)
    cx1 = np.floor((bmax[:, 0] - ox) / cell).astype(np.int64)
    cy0 = np.floor((bmin[:, 1] - oy) / cell).astype(np.int64)
    cy1 = np.floor((bmax[:, 1] - oy) / cell).astype(np.int64)
    ncx = int(cx1.max()) + 1
    # (cell, element) pairs
    pairs_c, pairs_e = [], []
    for e in range(Ne):
        for cy in range(cy0[e], cy1[e] + 1):
            for cx in range(cx0[e], cx1[e] + 1):
                pairs_c.append(cy * ncx + cx)
                pairs_e.append(e)
    pairs_c = np.asarray(pairs_c, dtype=np.int64)
    pairs_e = np.asarray(pairs_e, dtype=np.int64)
    order = np.lexsort((pairs_e, pairs_c))
    pairs_c, pairs_e = pairs_c[order], pairs_e[order]
    ncell = int(pairs_c.max()) + 1
    start = np.searchsorted(pairs_c, np.arange(ncell + 1))
    pcx = np.floor((pc[:, 0] - ox) / cell).astype(np.int64)
    pcy = np.floor((pc[:, 1] - oy) / cell).astype(np.int64)
    ok = (pcx >= 0) & (pcy >= 0) & (pcx < ncx)
    pcell = np.where(ok, pcy * ncx + pcx, -1)
    ok &= (pcell >= 0) & (pcell < ncell)
    elts = -np.ones(Np, dtype=np.int64)
    pidx = np.nonzero(ok)[0]
    if pidx.size:
        cs = pcell[pidx]
        cnt = start[cs + 1] - start[cs]
        rep_p = np.repeat(pidx, cnt)
        offs = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
        rep_e = pairs_e[np.repeat(start[cs], cnt) + offs]
        x = pc[rep_p, 0]
        y = pc[rep_p, 1]
        valid = (x >= bmin[rep_e, 0]) & (x <= bmax[rep_e, 0]) & (y >= bmin[rep_e, 1]) & (y <= bmax[rep_e, 1])
        vx = pc[rep_p, None, 0] - quad[rep_e, :, 0]
        vy = pc[rep_p, None, 1] - quad[rep_e, :, 1]
        cross = edges[rep_e, :, 0] * vy - edges[rep_e, :, 1] * vx
        valid &= np.all(orient[rep_e, None] * cross >= -tol, axis=1)
        cand = np.where(valid, rep_e, np.iinfo(np.int64).max)
        best = np.full(Np, np.iinfo(np.int64).max, dtype=np.int64)
        np.minimum.at(best, rep_p, cand)
        elts = np.where(best == np.iinfo(np.int64).max, -1, best)
    nodes_out = np.where((elts >= 0)[:, None], elements[np.maximum(elts, 0)], 0)
    return elts, nodes_out


def solve2x2_pivot(a11, a12, a21, a22, b1, b2):
    """2x2 solve by LU with partial pivoting, elementwise (vectorised).

    Stands in for ``jnp.linalg.solve`` (LAPACK getrf/getrs) in
    d2ic/pixel_assets.py:291.  Row swap when ``|a21| > |a11|``; multiplier by
    division.  The product builder uses the same operation sequence.
    """
    swap = np.abs(a21) > np.abs(a11)
    p11 = np.where(swap, a21, a11)
    p12 = np.where(swap, a22, a12)
    p21 = np.where(swap, a11, a21)
    p22 = np.where(swap, a12, a22)
    q1 = np.where(swap, b2, b1)
    q2 = np.where(swap, b1, b2)
    l21 = p21 / p11
    u22 = p22 - l21 * p12
    y2 = q2 - l21 * q1
    x2 = y2 / u22
    x1 = (q1 - p12 * x2) / p11
    return x1, x2


def shape_functions(xi, eta):
    """Q4 bilinear shape functions (d2ic/pixel_assets.py:297-306)."""
    return np.stack([0.25 * (1 - xi) * (1 - eta), 0.25 * (1 + xi) * (1 - eta),
                     0.25 * (1 + xi) * (1 + eta), 0.25 * (1 - xi) * (1 + eta)], axis=-1)


def newton_local_coords(pixel_coords, pixel_nodes, nodes, iters=10):
    """Local (xi, eta) of each pixel by 10 Newton steps from (0, 0).

    d2ic/pixel_assets.py:240-294 (FP64 as under x64).  Dot products are summed
    left to right over the 4 element nodes.
    """
    pc = np.asarray(pixel_coords, dtype=np.float64)
    Xe = np.asarray(nodes, dtype=np.float64)[np.asarray(pixel_nodes)]      # (Np,4,2)
    X0, X1, X2, X3 = Xe[:, 0, 0], Xe[:, 1, 0], Xe[:, 2, 0], Xe[:, 3, 0]
    Y0, Y1, Y2, Y3 = Xe[:, 0, 1], Xe[:, 1, 1], Xe[:, 2, 1], Xe[:, 3, 1]
    xi = np.zeros(pc.shape[0])
    eta = np.zeros(pc.shape[0])
    for _ in range(iters):
        n0 = 0.25 * (1 - xi) * (1 - eta)
        n1 = 0.25 * (1 + xi) * (1 - eta)
        n2 = 0.25 * (1 + xi) * (1 + eta)
        n3 = 0.25 * (1 - xi) * (1 + eta)
        dx0 = -0.25 * (1 - eta); dx1 = 0.25 * (1 - eta); dx2 = 0.25 * (1 + eta); dx3 = -0.25 * (1 + eta)
        de0 = -0.25 * (1 - xi); de1 = -0.25 * (1 + xi); de2 = 0.25 * (1 + xi); de3 = 0.25 * (1 - xi)
        x = ((n0 * X0 + n1 * X1) + n2 * X2) + n3 * X3
        y = ((n0 * Y0 + n1 * Y1) + n2 * Y2) + n3 * Y3
        j11 = ((dx0 * X0 + dx1 * X1) + dx2 * X2) + dx3 * X3
        j21 = ((dx0 * Y0 + dx1 * Y1) + dx2 * Y2) + dx3 * Y3
        j12 = ((de0 * X0 + de1 * X1) + de2 * X2) + de3 * X3
        j22 = ((de0 * Y0 + de1 * Y1) + de2 * Y2) + de3 * Y3
        d1, d2 = solve2x2_pivot(j11, j12, j21, j22, x - pc[:, 0], y - pc[:, 1])
        xi = xi - d1
        eta = eta - d2
    return xi, eta


def node_neighbor_dense(elements, nodes, n_nodes):
    """Regularisation neighbour table (d2ic/pixel_assets.py:330-409).

    Unique directed element edges, lexsorted by (src, dst); slot = rank within
    the src group; weight ``1/(|x_j-x_i| + 1e-6)``; -1 / 0 padding.
    """
    el = np.asarray(elements, dtype=np.int64)
    X = np.asarray(nodes, dtype=np.float64)
    if el.size == 0 or n_nodes == 0:
        return (np.full((n_nodes, 0), -1, np.int32), np.zeros(n_nodes, np.int32), np.zeros((n_nodes, 0)))
    k = el.shape[1]
    li = np.arange(k)
    s_idx = np.repeat(li, k)
    d_idx = np.tile(li, k)
    m = s_idx != d_idx
    src = el[:, s_idx[m]].reshape(-1)
    dst = el[:, d_idx[m]].reshape(-1)
    e = np.unique(np.stack([src, dst], axis=1), axis=0)
    src, dst = e[:, 0], e[:, 1]
    o = np.lexsort((dst, src))
    src, dst = src[o], dst[o]
    deg = np.bincount(src, minlength=n_nodes).astype(np.int32)
    maxd = int(deg.max(initial=0))
    w = 1.0 / (np.linalg.norm(X[dst, :2] - X[src, :2], axis=1) + 1e-6)
    mlen = src.shape[0]
    change = np.empty(mlen, dtype=bool)
    change[0] = True
    change[1:] = src[1:] != src[:-1]
    gstart = np.maximum.accumulate(np.where(change, np.arange(mlen), 0))
    slot = np.arange(mlen) - gstart
    idx = -np.ones((n_nodes, maxd), dtype=np.int32)
    wt = np.zeros((n_nodes, maxd), dtype=np.float64)
    idx[src, slot] = dst
    wt[src, slot] = w
    return idx, deg, wt


def node_pixel_dense(pixel_nodes, pixel_shapeN, n_nodes):
    """Node -> pixel ELL table (d2ic/pixel_assets.py:459-526).

    Slots follow the flattened ``(pixel, local node)`` order (the ``lax.scan``
    counter), i.e. ascending pixel id within each node.
    """
    pn = np.asarray(pixel_nodes, dtype=np.int64)
    N = np.asarray(pixel_shapeN)
    if pn.size == 0:
        return np.full((n_nodes, 0), -1, np.int32), np.zeros((n_nodes, 0)), np.zeros(n_nodes, np.int32)
    flat = pn.reshape(-1)
    deg = np.bincount(flat, minlength=n_nodes)
    maxd = int(deg.max(initial=0))
    Np, kl = pn.shape
    pix = np.repeat(np.arange(Np), kl)
    # the scan's counter value for an entry = its rank among equal node ids, in flat order
    slot = np.empty(flat.size, dtype=np.int64)
    o = np.argsort(flat, kind="stable")
    starts = np.cumsum(deg) - deg
    slot[o] = np.arange(flat.size) - np.repeat(starts, deg)
    idx = -np.ones((n_nodes, maxd), dtype=np.int32)
    wt = np.zeros((n_nodes, maxd), dtype=N.dtype)
    idx[flat, slot] = pix
    wt[flat, slot] = N.reshape(-1)
    return idx, wt, deg.astype(np.int32)


def build_pixel_assets(nodes, elements, H, W, roi_mask=None, bbox_pad=2.0, bruteforce=False):
    """All pixel assets (d2ic/pixel_assets.py:21-112), FP64.

    Returns a dict with the reference's PixelAssets fields plus ``pixel_elts``
    (the element chosen for each kept pixel) and ``xi_eta``.
    """
    nodes = np.asarray(nodes, dtype=np.float64)
    elements = np.asarray(elements)
    pc = sample_pixels_in_bbox(nodes, H, W, bbox_pad)
    if roi_mask is not None and pc.size > 0:
        roi_mask = np.asarray(roi_mask, dtype=bool)
        rows = np.clip(np.floor(pc[:, 1] - 0.5).astype(int), 0, H - 1)
        cols = np.clip(np.floor(pc[:, 0] - 0.5).astype(int), 0, W - 1)
        pc = pc[roi_mask[rows, cols]]
    f = pixel_to_element_bruteforce if bruteforce else pixel_to_element_hashed
    elts, pn = f(pc, nodes, elements)
    keep = elts >= 0
    pc, pn, elts = pc[keep], pn[keep], elts[keep]
    xi, eta = newton_local_coords(pc, pn, nodes)
    N = shape_functions(xi, eta)
    nidx, ndeg, nw = node_neighbor_dense(elements, nodes, nodes.shape[0])
    npi, npw, npd = node_pixel_dense(pn, N, nodes.shape[0])
    rows = np.clip(np.floor(pc[:, 1] - 0.5).astype(int), 0, H - 1)
    cols = np.clip(np.floor(pc[:, 0] - 0.5).astype(int), 0, W - 1)
    return dict(
        pixel_coords_ref=pc, pixel_nodes=pn.astype(np.int32), pixel_shapeN=N,
        node_neighbor_index=nidx, node_neighbor_degree=ndeg, node_neighbor_weight=nw,
        node_reg_weight=np.ones(nodes.shape[0], dtype=np.float64),
        node_pixel_index=npi, node_N_weight=npw, node_pixel_degree=npd,
        roi_mask_flat=rows * W + cols, image_shape=(H, W),
        pixel_elts=elts, xi_eta=np.stack([xi, eta], axis=1),
    )
