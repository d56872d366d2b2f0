"""Oracle restatement of the structured mask mesher and mesh tables (FP64).

Test infrastructure only (see oracle/__init__.py).

Reference: d2ic/mask2mesh.py, d2ic/mesh_assets.py.
"""
from __future__ import annotations

import numpy as np
from scipy import ndimage


def build_axis_coords(size: int, step: int) -> np.ndarray:
    """Grid-line positions along one image axis.

    Follows d2ic/mask2mesh.py:391-397: ``count = max(2, floor((size-1)/step)+1)``
    equally spaced lines from 0, plus a last line at ``size-1`` when the regular
    spacing stops short of it.
    """
    count = max(2, int(np.floor((size - 1) / step)) + 1)
    coords = np.arange(count, dtype=np.float64) * step
    if coords[-1] < size - 1:
        coords = np.append(coords, float(size - 1))
    return coords


def remove_small_components_floodfill(mask: np.ndarray, min_area: int) -> np.ndarray:
    """4-connected island removal by explicit flood fill.

    Literal restatement of d2ic/mask2mesh.py:400-432 (stack-based fill, raster
    seed order, components with area < max(1, min_area) dropped).  Pure Python:
    use only on small masks.
    """
    mask = np.asarray(mask, dtype=bool)
    h, w = mask.shape
    labels = -np.ones(mask.shape, dtype=np.int64)
    areas = []
    label = 0
    for y in range(h):
        for x in range(w):
            if not mask[y, x] or labels[y, x] != -1:
                continue
            stack = [(y, x)]
            labels[y, x] = label
            count = 0
            while stack:
                cy, cx = stack.pop()
                count += 1
                for ny, nx in ((cy - 1, cx), (cy + 1, cx), (cy, cx - 1), (cy, cx + 1)):
                    if 0 <= ny < h and 0 <= nx < w and mask[ny, nx] and labels[ny, nx] == -1:
                        labels[ny, nx] = label
                        stack.append((ny, nx))
            areas.append(count)
            label += 1
    if label == 0:
        return mask
    keep = np.asarray(areas) >= max(1, min_area)
    return keep[labels.clip(min=0)] & (labels >= 0)


def remove_small_components(mask: np.ndarray, min_area: int) -> np.ndarray:
    """Same result as :func:`remove_small_components_floodfill` via scipy labelling.

    The set of 4-connected components (and so each component's area) does not
    depend on the labelling order, so the kept set is identical; the tests
    check this equality on random masks.
    """
    mask = np.asarray(mask, dtype=bool)
    if not mask.any():
        return mask
    labels, n = ndimage.label(mask, structure=[[0, 1, 0], [1, 1, 1], [0, 1, 0]])
    areas = np.bincount(labels.ravel(), minlength=n + 1)
    keep = areas >= max(1, min_area)
    keep[0] = False
    return keep[labels]


def downsample_mask(mask: np.ndarray, binning: int) -> np.ndarray:
    """Block-OR downsampling with zero padding (d2ic/mask2mesh.py:26-57)."""
    mask = np.asarray(mask, dtype=bool)
    if binning <= 1:
        return mask
    h, w = mask.shape
    mask = np.pad(mask, ((0, (-h) % binning), (0, (-w) % binning)))
    return mask.reshape(mask.shape[0] // binning, binning, mask.shape[1] // binning, binning).any(axis=(1, 3))


def mask_to_mesh(mask, element_size_px, binning=1, origin_xy=(0.0, 0.0),
                 remove_islands=True, min_island_area_px=64):
    """Structured Q4 mesh over the whole (binned) mask grid.

    Restates d2ic/mask2mesh.py:60-142: grid lines from build_axis_coords on
    both axes, ALL grid nodes kept (orphans included), a cell becomes an
    element when the mask is set at ``(min(round(cy), h-1), min(round(cx), w-1))``
    of its centre (Python ``round``: half to even); element node order
    ``[n0, n0+1, n0+nx+1, n0+nx]``, cells visited row by row.
    Returns ``(nodes (Nn,2) f64, elements (Ne,4) i32)``.
    """
    if element_size_px <= 0:
        raise ValueError("element_size_px must be positive")
    m = np.asarray(mask, dtype=bool)
    if remove_islands:
        m = remove_small_components(m, min_island_area_px)
    mds = downsample_mask(m, binning)
    if not mds.any():
        raise ValueError("mask_to_mesh: no ROI pixels remain after preprocessing.")
    step = max(1, int(round(element_size_px / max(1, binning))))
    h, w = mds.shape
    gx = build_axis_coords(w, step)
    gy = build_axis_coords(h, step)
    nx, ny = gx.size, gy.size
    xx, yy = np.meshgrid(gx, gy)
    nodes = np.stack([xx.ravel(), yy.ravel()], axis=1).astype(np.float64)
    nodes[:, 0] = origin_xy[0] + nodes[:, 0] * binning
    nodes[:, 1] = origin_xy[1] + nodes[:, 1] * binning
    elements = []
    for iy in range(ny - 1):
        cy = 0.5 * (gy[iy] + gy[iy + 1])
        my = min(int(round(cy)), h - 1)
        for ix in range(nx - 1):
            cx = 0.5 * (gx[ix] + gx[ix + 1])
            mx = min(int(round(cx)), w - 1)
            if not mds[my, mx]:
                continue
            n0 = iy * nx + ix
            elements.append([n0, n0 + 1, n0 + nx + 1, n0 + nx])
    if not elements:
        raise ValueError("mask_to_mesh: no elements found inside the ROI.")
    return nodes, np.asarray(elements, dtype=np.int32)


def mask_to_mesh_assets(mask, element_size_px, binning=1, origin_xy=(0.0, 0.0),
                        remove_islands=True, min_island_area_px=64):
    """Mesh plus element centres and the binned ROI mask (d2ic/mask2mesh.py:145-182)."""
    nodes, elements = mask_to_mesh(mask, element_size_px, binning, origin_xy,
                                   remove_islands, min_island_area_px)
    m = np.asarray(mask, dtype=bool)
    if remove_islands:
        m = remove_small_components(m, min_island_area_px)
    roi = downsample_mask(m, binning)
    return dict(nodes=nodes, elements=elements, centers=element_centers(nodes, elements), roi_mask=roi)


def element_centers(nodes, elements):
    """Mean of the element's node coordinates (d2ic/mesh_assets.py:77-92)."""
    return np.asarray(nodes, dtype=np.float64)[np.asarray(elements)].mean(axis=1)


def node_neighbor_tables(nodes, elements, max_degree=16):
    """Strain neighbour tables (d2ic/mesh_assets.py:95-132).

    For each node the sorted set of other nodes sharing an element, truncated
    to ``max_degree``, zero-padded; returns ``(index (Nn,max_degree) i32, degree (Nn,) i32)``.
    """
    n_nodes = np.asarray(nodes).shape[0]
    neigh = [set() for _ in range(n_nodes)]
    for elt in np.asarray(elements):
        e = [int(i) for i in elt]
        for ni in e:
            for nj in e:
                if nj != ni:
                    neigh[ni].add(nj)
    idx = np.zeros((n_nodes, max_degree), dtype=np.int32)
    deg = np.zeros((n_nodes,), dtype=np.int32)
    for i, s in enumerate(neigh):
        srt = sorted(s)
        d = min(len(srt), max_degree)
        deg[i] = d
        if d:
            idx[i, :d] = srt[:d]
    return idx, deg
