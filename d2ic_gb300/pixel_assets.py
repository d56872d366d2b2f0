"""Pixel-level assets: pixel -> element map, Q4 local coordinates and shape
functions, spring neighbour table, node -> pixel table.

Reference: d2ic/pixel_assets.py:21-526.  The reference assigns pixels by a
dense (pixels x elements) inside test (O(Np*Ne), infeasible at 4096^2).  Here:

* structured grids (the mesher's output: a tensor grid of nodes and
  axis-aligned cells) use a direct cell lookup.  For an axis-aligned
  rectangle the reference's test "inside the element's bounding box and on
  the inner side (within 1e-6) of every edge" is exactly "inside the closed
  rectangle", so every pixel gets the lowest-index element whose closed
  rectangle contains it (at most 4 candidate cells, on shared edges);
* any other quad mesh uses a uniform grid over element bounding boxes and
  runs the reference's test on the candidates only, keeping the lowest valid
  element index (a pixel outside an element's bbox is never valid, so the
  answer is identical).

Local coordinates come from the reference's 10 Newton steps from (0, 0),
vectorised in FP64 with the same operation sequence on every path.
"""
from __future__ import annotations

import numpy as np

from .mesh_assets import Mesh, PixelAssets, unique_sorted

_TOL = 1e-6


def _bbox(nodes: np.ndarray, H: int, W: int, pad: float):
    """Pixel rows [i0, i1) and columns [j0, j1) of the padded node bbox, inside the image."""
    j0 = max(0, int(np.floor(nodes[:, 0].min() - pad)))
    j1 = min(W, int(np.ceil(nodes[:, 0].max() + pad)))
    i0 = max(0, int(np.floor(nodes[:, 1].min() - pad)))
    i1 = min(H, int(np.ceil(nodes[:, 1].max() + pad)))
    return i0, i1, j0, j1


def _sample_pixels_in_bbox(nodes: np.ndarray, H: int, W: int, pad: float) -> np.ndarray:
    """Pixel centres ``(j+0.5, i+0.5)`` of the padded node bbox, rows outer (d2ic/pixel_assets.py:115-132)."""
    i0, i1, j0, j1 = _bbox(nodes, H, W, pad)
    jj, ii = np.meshgrid(np.arange(j0, j1), np.arange(i0, i1))
    return np.stack([jj.ravel() + 0.5, ii.ravel() + 0.5], axis=1)


def _roi_pixels(nodes: np.ndarray, H: int, W: int, pad: float, roi_mask):
    """The bbox pixels kept by the ROI mask (all of them without one), rows outer, as integer
    rows and columns: the same pixels and order as sampling the bbox and then testing the mask at
    ``floor(centre - 0.5)`` (d2ic/pixel_assets.py:115-132), without forming the whole bbox."""
    i0, i1, j0, j1 = _bbox(nodes, H, W, pad)
    if i1 <= i0 or j1 <= j0:
        z = np.zeros((0,), dtype=np.int64)
        return z, z
    if roi_mask is None:
        ii, jj = np.divmod(np.arange((i1 - i0) * (j1 - j0), dtype=np.int64), j1 - j0)
    else:
        ii, jj = np.nonzero(roi_mask[i0:i1, j0:j1])
    return ii.astype(np.int64) + i0, jj.astype(np.int64) + j0


def structured_grid(nodes: np.ndarray, elements: np.ndarray):
    """``(gx, gy, cell_elem)`` if the mesh is a tensor grid of axis-aligned cells, else None.

    cell_elem[iy, ix] = lowest element index on cell (ix, iy), -1 for none.
    """
    nodes = np.asarray(nodes, dtype=np.float64)
    el = np.asarray(elements, dtype=np.int64)
    if el.ndim != 2 or el.shape[1] != 4 or el.shape[0] == 0:
        return None
    gx = np.unique(nodes[:, 0])
    gy = np.unique(nodes[:, 1])
    nx, ny = gx.size, gy.size
    if nx < 2 or ny < 2 or nx * ny != nodes.shape[0]:
        return None
    xx, yy = np.meshgrid(gx, gy)
    if not (np.array_equal(nodes[:, 0], xx.ravel()) and np.array_equal(nodes[:, 1], yy.ravel())):
        return None
    n0 = el[:, 0]
    iy, ix = n0 // nx, n0 % nx
    ok = (ix < nx - 1) & (iy < ny - 1)
    ok &= (el[:, 1] == n0 + 1) & (el[:, 2] == n0 + nx + 1) & (el[:, 3] == n0 + nx)
    if not ok.all():
        return None
    cell = np.full((ny - 1, nx - 1), -1, dtype=np.int64)
    order = np.arange(el.shape[0])[::-1]                 # write high ids first so the lowest id wins
    cell[iy[order], ix[order]] = order
    return gx, gy, cell


def grid_cells(nodes: np.ndarray, elements: np.ndarray):
    """``(gx, gy, cell, elem_cell)`` for a tensor grid whose every element is a distinct cell (the
    meshes mask_to_mesh builds), else None; elem_cell[e] = ix | iy << 16 of element e's cell."""
    sg = structured_grid(nodes, elements)
    if sg is None:
        return None
    gx, gy, cell = sg
    if gx.size >= 65536 or gy.size >= 65536:
        return None
    el = np.asarray(elements, dtype=np.int64)
    n0 = el[:, 0]
    iy, ix = n0 // gx.size, n0 % gx.size
    if not np.array_equal(cell[iy, ix], np.arange(el.shape[0])):      # two elements on one cell
        return None
    return gx, gy, cell, (ix | (iy << 16)).astype(np.int64)


class GridPixelData:
    """Pixel assets of a tensor-grid mesh kept as their recipe -- mesh, ROI mask, image shape --
    for the device layout builder (FrameLayout.from_grid): no per-pixel host array is formed.

    Attribute access to the host fields of :class:`PixelAssets` (``pixel_coords_ref``,
    ``pixel_shapeN``, ...) builds them once with :func:`build_pixel_assets` (identical values)."""

    def __init__(self, mesh: Mesh, image_shape, roi_mask=None, binning: float = 1.0, bbox_pad: float = 2.0):
        self.mesh = mesh
        self.image_shape = tuple(int(v) for v in image_shape)
        self.roi_mask = None if roi_mask is None else np.asarray(roi_mask, dtype=bool)
        self.binning = float(binning)
        self.bbox_pad = float(bbox_pad)
        self._host = None
        self._counts = None

    def device_ok(self) -> bool:
        return _gpu_available() and grid_cells(np.asarray(self.mesh.nodes_xy, np.float64) / self.binning,
                                              np.asarray(self.mesh.elements, np.int64)) is not None

    def element_pixel_counts(self) -> np.ndarray:
        """ROI pixels of each element (the device count pass, or the host assets without a GPU)."""
        if self._counts is None:
            if self._host is None and self.device_ok():
                from .engine import grid_element_counts
                self._counts = grid_element_counts(self.mesh, self.roi_mask, self.image_shape, self.bbox_pad,
                                                   self.binning)
            else:
                e = np.asarray(self.to_host().pixel_elts, np.int64)
                self._counts = np.bincount(e, minlength=np.asarray(self.mesh.elements).shape[0])
        return self._counts

    @property
    def n_pixels(self) -> int:
        return int(self.element_pixel_counts().sum())

    def to_host(self) -> "PixelAssets":
        if self._host is None:
            self._host = build_pixel_assets(self.mesh, np.zeros(self.image_shape, np.float32), self.binning,
                                            self.roi_mask, self.bbox_pad)
        return self._host

    def __getattr__(self, name):
        if name.startswith("_") or name in ("mesh", "image_shape", "roi_mask", "binning", "bbox_pad"):
            raise AttributeError(name)
        return getattr(self.to_host(), name)


def build_pixel_assets_device(mesh: Mesh, ref_image, binning: float, roi_mask=None, bbox_pad: float = 2.0):
    """Pixel assets for the device path: a :class:`GridPixelData` recipe when the mesh is a tensor
    grid and a GPU is present (the solvers then build their layout on the device), else the host
    :func:`build_pixel_assets`."""
    H, W = (int(s) for s in np.shape(ref_image)[:2])
    gp = GridPixelData(mesh, (H, W), roi_mask, binning, bbox_pad)
    if gp.device_ok():
        return gp
    return build_pixel_assets(mesh, ref_image, binning, roi_mask, bbox_pad)


def _structured_assign(pc: np.ndarray, gx, gy, cell):
    """Lowest element index whose closed cell rectangle contains each pixel, -1 if none."""
    nx, ny = gx.size, gy.size
    best = np.full(pc.shape[0], np.iinfo(np.int64).max, dtype=np.int64)
    ixr = np.searchsorted(gx, pc[:, 0], side="right") - 1          # last line <= x
    iyr = np.searchsorted(gy, pc[:, 1], side="right") - 1
    for dx in (0, 1):
        cx = ixr - dx
        okx = (cx >= 0) & (cx <= nx - 2)
        cxs = np.clip(cx, 0, nx - 2)
        okx &= (gx[cxs] <= pc[:, 0]) & (pc[:, 0] <= gx[cxs + 1])
        for dy in (0, 1):
            cy = iyr - dy
            ok = okx & (cy >= 0) & (cy <= ny - 2)
            cys = np.clip(cy, 0, ny - 2)
            ok &= (gy[cys] <= pc[:, 1]) & (pc[:, 1] <= gy[cys + 1])
            e = np.where(ok, cell[cys, cxs], -1)
            e = np.where(e < 0, np.iinfo(np.int64).max, e)
            best = np.minimum(best, e)
    return np.where(best == np.iinfo(np.int64).max, -1, best)


def _generic_assign(pc: np.ndarray, nodes: np.ndarray, el: np.ndarray):
    """Reference inside test on bbox-grid candidates; lowest valid element index."""
    quad = nodes[el]                                           # (Ne,4,2)
    nxt = np.roll(quad, -1, axis=1)
    edges = nxt - quad
    area2 = np.sum(quad[:, :, 0] * nxt[:, :, 1] - quad[:, :, 1] * nxt[:, :, 0], axis=1)
    orient = np.where(area2 >= 0.0, 1.0, -1.0)
    bmin, bmax = quad.min(axis=1), quad.max(axis=1)
    Np, Ne = pc.shape[0], el.shape[0]
    cellsz = max(1.0, float(np.median(bmax - bmin)))
    ox, oy = float(bmin[:, 0].min()), float(bmin[:, 1].min())
    cx0 = np.floor((bmin[:, 0] - ox) / cellsz).astype(np.int64)
    cx1 = np.floor((bmax[:, 0] - ox) / cellsz).astype(np.int64)
    cy0 = np.floor((bmin[:, 1] - oy) / cellsz).astype(np.int64)
    cy1 = np.floor((bmax[:, 1] - oy) / cellsz).astype(np.int64)
    ncx = int(cx1.max()) + 1
    ncy = int(cy1.max()) + 1
    spanx = cx1 - cx0 + 1
    spany = cy1 - cy0 + 1
    cnt = spanx * spany
    e_rep = np.repeat(np.arange(Ne), cnt)
    k = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    c_rep = (cy0[e_rep] + k // spanx[e_rep]) * ncx + (cx0[e_rep] + k % spanx[e_rep])
    o = np.lexsort((e_rep, c_rep))
    c_rep, e_rep = c_rep[o], e_rep[o]
    start = np.searchsorted(c_rep, np.arange(ncx * ncy + 1))
    pcx = np.floor((pc[:, 0] - ox) / cellsz).astype(np.int64)
    pcy = np.floor((pc[:, 1] - oy) / cellsz).astype(np.int64)
    ok = (pcx >= 0) & (pcy >= 0) & (pcx < ncx) & (pcy < ncy)
    best = np.full(Np, np.iinfo(np.int64).max, dtype=np.int64)
    pidx = np.nonzero(ok)[0]
    step = 1 << 20
    for s in range(0, pidx.size, step):
        pi = pidx[s:s + step]
        cs = pcy[pi] * ncx + pcx[pi]
        n = start[cs + 1] - start[cs]
        rp = np.repeat(pi, n)
        off = np.arange(n.sum()) - np.repeat(np.cumsum(n) - n, n)
        re = e_rep[np.repeat(start[cs], n) + off]
        x, y = pc[rp, 0], pc[rp, 1]
        valid = (x >= bmin[re, 0]) & (x <= bmax[re, 0]) & (y >= bmin[re, 1]) & (y <= bmax[re, 1])
        vx = x[:, None] - quad[re, :, 0]
        vy = y[:, None] - quad[re, :, 1]
        cross = edges[re, :, 0] * vy - edges[re, :, 1] * vx
        valid &= np.all(orient[re, None] * cross >= -_TOL, axis=1)
        np.minimum.at(best, rp[valid], re[valid])
    return np.where(best == np.iinfo(np.int64).max, -1, best)


def build_pixel_to_element_mapping_numpy(pixel_coords, nodes_coord, elements, chunk_size: int = 4096):
    """``(pixel_elts, pixel_nodes)``: element per pixel (-1 outside), its nodes (zeros outside).

    Same contract as d2ic/pixel_assets.py:135-237 (``chunk_size`` accepted for
    API parity; no dense chunks are formed).
    """
    if chunk_size < 1:
        raise ValueError("chunk_size must be >= 1")
    pc = np.asarray(pixel_coords, dtype=np.float64).reshape(-1, 2)
    nodes = np.asarray(nodes_coord, dtype=np.float64)
    el = np.asarray(elements, dtype=np.int64)
    Np = pc.shape[0]
    if Np == 0 or el.size == 0:
        return -np.ones((Np,), dtype=int), np.zeros((Np, 4), dtype=int)
    sg = structured_grid(nodes, el)
    elts = _structured_assign(pc, *sg) if sg is not None else _generic_assign(pc, nodes, el)
    pn = np.where((elts >= 0)[:, None], el[np.maximum(elts, 0)], 0)
    return elts, pn


def structured_assign_device(pc: np.ndarray, gx, gy, cell, device=None) -> np.ndarray:
    """:func:`_structured_assign` on the GPU (``d2ic_structured_assign``): the same FP64
    comparisons, so the element map is identical."""
    import torch

    from . import _lib
    from ._lib import ptr
    dev = torch.device(device if device is not None else "cuda")
    n = int(pc.shape[0])
    if n == 0:
        return np.zeros((0,), dtype=np.int64)
    t_pc = torch.from_numpy(np.ascontiguousarray(pc, dtype=np.float64)).to(dev)
    t_gx = torch.from_numpy(np.ascontiguousarray(gx, dtype=np.float64)).to(dev)
    t_gy = torch.from_numpy(np.ascontiguousarray(gy, dtype=np.float64)).to(dev)
    t_cell = torch.from_numpy(np.ascontiguousarray(cell, dtype=np.int64)).to(dev)
    out = torch.empty(n, dtype=torch.int64, device=dev)
    _lib.call("d2ic_structured_assign", ptr(t_pc), n, ptr(t_gx), int(gx.size), ptr(t_gy), int(gy.size), ptr(t_cell),
              ptr(out), _lib.stream_handle())
    return out.cpu().numpy()


def _pixel_element_ids(pc: np.ndarray, nodes: np.ndarray, el: np.ndarray) -> np.ndarray:
    """The element of each pixel (-1 outside), as ``build_pixel_to_element_mapping_numpy``, with
    the tensor-grid search on the GPU when one is present (identical results)."""
    if pc.shape[0] == 0 or el.size == 0:
        return -np.ones((pc.shape[0],), dtype=np.int64)
    sg = structured_grid(nodes, el)
    if sg is not None:
        return structured_assign_device(pc, *sg) if _gpu_available() else _structured_assign(pc, *sg)
    return _generic_assign(pc, nodes, el)


def _solve2(a11, a12, a21, a22, b1, b2):
    # LU with partial pivoting on a 2x2 system (row swap when |a21| > |a11|)
    swap = np.abs(a21) > np.abs(a11)
    p11 = np.where(swap, a21, a11)
    p12 = np.where(swap, a22, a12)
    p21 = np.where(swap, a11, a21)
    p22 = np.where(swap, a12, a22)
    q1 = np.where(swap, b2, b1)
    q2 = np.where(swap, b1, b2)
    l21 = p21 / p11
    x2 = (q2 - l21 * q1) / (p22 - l21 * p12)
    x1 = (q1 - p12 * x2) / p11
    return x1, x2


def _newton_step(xi, eta, X, Y, px, py):
    om_x, op_x, om_e, op_e = 1 - xi, 1 + xi, 1 - eta, 1 + eta
    n0 = 0.25 * om_x * om_e
    n1 = 0.25 * op_x * om_e
    n2 = 0.25 * op_x * op_e
    n3 = 0.25 * om_x * op_e
    dx0, dx1, dx2, dx3 = -0.25 * om_e, 0.25 * om_e, 0.25 * op_e, -0.25 * op_e
    de0, de1, de2, de3 = -0.25 * om_x, -0.25 * op_x, 0.25 * op_x, 0.25 * om_x
    X0, X1, X2, X3 = X
    Y0, Y1, Y2, Y3 = Y
    fx = (((n0 * X0 + n1 * X1) + n2 * X2) + n3 * X3) - px
    fy = (((n0 * Y0 + n1 * Y1) + n2 * Y2) + n3 * Y3) - py
    j11 = ((dx0 * X0 + dx1 * X1) + dx2 * X2) + dx3 * X3
    j21 = ((dx0 * Y0 + dx1 * Y1) + dx2 * Y2) + dx3 * Y3
    j12 = ((de0 * X0 + de1 * X1) + de2 * X2) + de3 * X3
    j22 = ((de0 * Y0 + de1 * Y1) + de2 * Y2) + de3 * Y3
    return _solve2(j11, j12, j21, j22, fx, fy)


def local_coordinates(pixel_coords, pixel_nodes, nodes_coord, iters: int = 10):
    """(xi, eta) of each pixel in its element by Newton from (0,0) (d2ic/pixel_assets.py:277-294).

    A pixel whose update is exactly zero keeps (xi, eta), so every later
    iteration repeats the same zero update: such pixels drop out of the
    remaining iterations, which gives bit-for-bit the result of all ``iters``
    steps at a fraction of the cost (axis-aligned elements settle in 2-3).
    """
    pc = np.asarray(pixel_coords, dtype=np.float64)
    Xe = np.asarray(nodes_coord, dtype=np.float64)[np.asarray(pixel_nodes)]
    n = pc.shape[0]
    xi = np.zeros(n)
    eta = np.zeros(n)
    live = np.arange(n)
    for _ in range(iters):
        if live.size == 0:
            break
        X = tuple(Xe[live, a, 0] for a in range(4))
        Y = tuple(Xe[live, a, 1] for a in range(4))
        d1, d2 = _newton_step(xi[live], eta[live], X, Y, pc[live, 0], pc[live, 1])
        xi[live] = xi[live] - d1
        eta[live] = eta[live] - d2
        moving = (d1 != 0) | (d2 != 0) | ~np.isfinite(d1) | ~np.isfinite(d2)
        live = live[moving]
    return xi, eta


def shape_functions(xi, eta) -> np.ndarray:
    """Q4 shape functions, node order (-1,-1), (1,-1), (1,1), (-1,1)."""
    xi, eta = np.asarray(xi), np.asarray(eta)
    if xi.ndim != 1 or eta.ndim != 1:
        return np.stack([0.25 * (1 - xi) * (1 - eta), 0.25 * (1 + xi) * (1 - eta),
                         0.25 * (1 + xi) * (1 + eta), 0.25 * (1 - xi) * (1 + eta)], axis=-1)
    a0, a1 = 0.25 * (1 - xi), 0.25 * (1 + xi)       # the same products, left to right
    b0, b1 = 1 - eta, 1 + eta
    N = np.empty((xi.shape[0], 4), dtype=np.result_type(a0, b0))
    np.multiply(a0, b0, out=N[:, 0])
    np.multiply(a1, b0, out=N[:, 1])
    np.multiply(a1, b1, out=N[:, 2])
    np.multiply(a0, b1, out=N[:, 3])
    return N


def local_coordinates_device(pixel_coords, pixel_nodes, nodes_coord, iters: int = 10, device=None):
    """:func:`local_coordinates` on the GPU (``d2ic_local_coordinates``): the same FP64 operation
    sequence with correctly rounded operations, so the results are bit-identical."""
    import torch

    from . import _lib
    from ._lib import ptr
    dev = torch.device(device if device is not None else "cuda")
    pc = torch.from_numpy(np.ascontiguousarray(pixel_coords, dtype=np.float64)).to(dev)
    pn = torch.from_numpy(np.ascontiguousarray(pixel_nodes, dtype=np.int32)).to(dev)
    X = torch.from_numpy(np.ascontiguousarray(nodes_coord, dtype=np.float64)).to(dev)
    n = int(pc.shape[0])
    xi = torch.empty(max(n, 1), dtype=torch.float64, device=dev)
    eta = torch.empty_like(xi)
    _lib.call("d2ic_local_coordinates", ptr(pc), ptr(pn), ptr(X), n, int(iters), ptr(xi), ptr(eta),
              _lib.stream_handle())
    return xi[:n].cpu().numpy(), eta[:n].cpu().numpy()


def _gpu_available() -> bool:
    try:
        import torch

        from . import _lib
        if not torch.cuda.is_available():
            return False
        _lib.load()
        return True
    except Exception:
        return False


def compute_pixel_shape_functions(pixel_coords, pixel_nodes, nodes_coord):
    """``(pixel_N (Np,4), xi_eta (Np,2))`` (d2ic/pixel_assets.py:240-274).

    The Newton inverse map runs on the GPU when one is present (bit-identical to
    the host form, which runs otherwise)."""
    if _gpu_available() and np.asarray(pixel_coords).shape[0] > 0:
        xi, eta = local_coordinates_device(pixel_coords, pixel_nodes, nodes_coord)
    else:
        xi, eta = local_coordinates(pixel_coords, pixel_nodes, nodes_coord)
    return shape_functions(xi, eta), np.stack([xi, eta], axis=1)


def build_node_neighbor_dense(elements, nodes_coord, n_nodes):
    """Spring neighbour table (d2ic/pixel_assets.py:330-409): lexsorted unique
    directed element edges, weight ``1/(|x_j - x_i| + 1e-6)``, -1 / 0 padded."""
    el = np.asarray(elements, dtype=np.int64)
    X = np.asarray(nodes_coord, dtype=np.float64)
    n_nodes = int(n_nodes)
    empty = (np.full((n_nodes, 0), -1, np.int32), np.zeros(n_nodes, np.int32), np.zeros((n_nodes, 0), X.dtype))
    if el.size == 0 or n_nodes == 0:
        return empty
    k = el.shape[1]
    a, b = np.meshgrid(np.arange(k), np.arange(k), indexing="ij")
    m = (a != b).ravel()
    src = el[:, a.ravel()[m]].ravel()
    dst = el[:, b.ravel()[m]].ravel()
    key = unique_sorted(src * n_nodes + dst)        # unique pairs, ordered by (src, dst)
    src, dst = key // n_nodes, key % n_nodes
    deg = np.bincount(src, minlength=n_nodes).astype(np.int32)
    maxd = int(deg.max(initial=0))
    if maxd == 0:
        return empty
    w = (1.0 / (np.linalg.norm(X[dst, :2] - X[src, :2], axis=1) + 1e-6)).astype(X.dtype)
    start = np.cumsum(deg) - deg
    slot = np.arange(src.size) - np.repeat(start, deg)
    idx = -np.ones((n_nodes, maxd), dtype=np.int32)
    wt = np.zeros((n_nodes, maxd), dtype=X.dtype)
    idx[src, slot] = dst
    wt[src, slot] = w
    return idx, deg, wt


def build_node_pixel_dense(pixel_nodes, pixel_shapeN, n_nodes):
    """Dense node -> pixel table (d2ic/pixel_assets.py:459-526): slots in ascending pixel order."""
    pn = np.asarray(pixel_nodes, dtype=np.int64)
    N = np.asarray(pixel_shapeN)
    n_nodes = int(n_nodes)
    if pn.size == 0:
        return np.full((n_nodes, 0), -1, np.int32), np.zeros((n_nodes, 0), N.dtype), np.zeros(n_nodes, np.int32)
    flat = pn.reshape(-1)
    deg = np.bincount(flat, minlength=n_nodes)
    maxd = int(deg.max(initial=0))
    Np, kl = pn.shape
    order = np.argsort(flat, kind="stable")
    start = np.cumsum(deg) - deg
    slot = np.empty(flat.size, dtype=np.int64)
    slot[order] = np.arange(flat.size) - np.repeat(start, deg)
    idx = -np.ones((n_nodes, maxd), dtype=np.int32)
    wt = np.zeros((n_nodes, maxd), dtype=N.dtype)
    idx[flat, slot] = np.repeat(np.arange(Np, dtype=np.int32), kl)
    wt[flat, slot] = N.reshape(-1)
    return idx, wt, deg.astype(np.int32)


def build_pixel_assets(mesh: Mesh, ref_image, binning: float, roi_mask=None, bbox_pad: float = 2.0,
                       chunk_size: int = 4096) -> PixelAssets:
    """Pixel assets of a mesh over a reference image (d2ic/pixel_assets.py:21-112)."""
    nodes = np.asarray(mesh.nodes_xy, dtype=np.float64) / float(binning)
    elements = np.asarray(mesh.elements, dtype=np.int64)
    H, W = (int(s) for s in np.shape(ref_image)[:2])
    if roi_mask is not None:
        roi_mask = np.asarray(roi_mask, dtype=bool)
        if roi_mask.shape != (H, W):
            raise ValueError(f"roi_mask shape {roi_mask.shape} does not match ref_image shape {(H, W)}")
    if chunk_size < 1:
        raise ValueError("chunk_size must be >= 1")
    rows, cols = _roi_pixels(nodes, H, W, bbox_pad, roi_mask)
    pc = np.empty((rows.size, 2), dtype=np.float64)
    pc[:, 0] = cols + 0.5
    pc[:, 1] = rows + 0.5
    elts = _pixel_element_ids(pc, nodes, elements)
    keep = elts >= 0
    pc, elts, rows, cols = pc[keep], elts[keep], rows[keep], cols[keep]
    pn = elements[elts]
    N, xe = compute_pixel_shape_functions(pc, pn, nodes)
    nidx, ndeg, nw = build_node_neighbor_dense(elements, nodes, nodes.shape[0])
    return PixelAssets(
        pixel_coords_ref=pc, pixel_nodes=pn.astype(np.int32), pixel_shapeN=N,
        node_neighbor_index=nidx, node_neighbor_degree=ndeg, node_neighbor_weight=nw,
        node_reg_weight=np.ones(nodes.shape[0], dtype=nodes.dtype),
        roi_mask_flat=rows * W + cols, image_shape=(H, W), pixel_elts=elts, xi_eta=xe,
    )
