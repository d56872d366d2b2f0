"""Structured Q4 meshing of a binary ROI mask.

Reference: d2ic/mask2mesh.py:26-182,391-432.  The unstructured gmsh mesher
(mask_to_mesh_gmsh, :185-388) needs gmsh/meshio, which are not available; the
functions exist for API parity and raise ImportError like the reference does
without gmsh.
"""
from __future__ import annotations

from typing import Tuple

import numpy as np
from scipy import ndimage

from .mesh_assets import Mesh, MeshAssets, compute_element_centers


def downsample_mask(mask: np.ndarray, binning: int) -> np.ndarray:
    """Block-OR binning with zero padding to a multiple of ``binning``."""
    mask = np.asarray(mask, dtype=bool)
    if binning <= 1:
        return mask
    h, w = mask.shape
    mask = np.pad(mask, ((0, (-h) % binning), (0, (-w) % binning)))
    return mask.reshape(mask.shape[0] // binning, binning, mask.shape[1] // binning, binning).any(axis=(1, 3))


def _build_axis_coords(size: int, step: int) -> np.ndarray:
    """Grid lines 0, step, 2 step, ... and a last line at size-1 if the spacing stops short."""
    count = max(2, int(np.floor((size - 1) / step)) + 1)
    coords = np.arange(count, dtype=np.float64) * step
    if coords[-1] < size - 1:
        coords = np.append(coords, float(size - 1))
    return coords


def _remove_small_components(mask: np.ndarray, min_area: int) -> np.ndarray:
    """Drop 4-connected components smaller than ``max(1, min_area)`` pixels."""
    mask = np.asarray(mask, dtype=bool)
    if not mask.any():
        return mask
    labels, n = ndimage.label(mask, structure=[[0, 1, 0], [1, 1, 1], [0, 1, 0]])
    if n == 1:                                       # one component: its area is the mask's
        return mask if int(np.count_nonzero(mask)) >= max(1, min_area) else np.zeros_like(mask)
    area = np.bincount(labels.ravel(), minlength=n + 1)
    keep = area >= max(1, min_area)
    if keep[1:].all():
        return mask                                  # every component is kept: the mask as it is
    keep[0] = False
    return keep[labels]


def mask_to_mesh(mask: np.ndarray, element_size_px: float, binning: int = 1,
                 origin_xy: Tuple[float, float] = (0.0, 0.0), enforce_quads: bool = True,
                 remove_islands: bool = True, min_island_area_px: int = 64) -> Mesh:
    """Regular Q4 grid over the whole (binned) mask; cells whose rounded centre is in the ROI become elements.

    All grid nodes are kept (including nodes of no element), node index
    ``iy * nx + ix``, element nodes ``[n0, n0+1, n0+nx+1, n0+nx]`` row by row.
    """
    if not enforce_quads:
        raise NotImplementedError("Only quadrilateral meshes are supported at the moment.")
    if element_size_px <= 0:
        raise ValueError("element_size_px must be positive")
    m = np.asarray(mask, dtype=bool)
    if remove_islands:
        m = _remove_small_components(m, min_island_area_px)
    mds = downsample_mask(m, binning)
    if not mds.any():
        raise ValueError("mask_to_mesh: no ROI pixels remain after preprocessing.")
    step = max(1, int(round(element_size_px / max(1, binning))))
    h, w = mds.shape
    gx = _build_axis_coords(w, step)
    gy = _build_axis_coords(h, step)
    nx, ny = gx.size, gy.size
    xx, yy = np.meshgrid(gx, gy)
    nodes = np.stack([xx.ravel(), yy.ravel()], axis=1).astype(np.float64)
    nodes[:, 0] = origin_xy[0] + nodes[:, 0] * binning
    nodes[:, 1] = origin_xy[1] + nodes[:, 1] * binning
    cx = 0.5 * (gx[:-1] + gx[1:])
    cy = 0.5 * (gy[:-1] + gy[1:])
    mx = np.minimum(np.round(cx).astype(np.int64), w - 1)      # round half to even, as Python round()
    my = np.minimum(np.round(cy).astype(np.int64), h - 1)
    inside = mds[my[:, None], mx[None, :]]                       # (ny-1, nx-1)
    iy, ix = np.nonzero(inside)                                  # row-major = the reference's loop order
    if iy.size == 0:
        raise ValueError("mask_to_mesh: no elements found inside the ROI.")
    n0 = iy * nx + ix
    elements = np.stack([n0, n0 + 1, n0 + nx + 1, n0 + nx], axis=1).astype(np.int32)
    return Mesh(nodes_xy=nodes, elements=elements)


def mask_to_mesh_assets(mask: np.ndarray, element_size_px: float, binning: int = 1,
                        origin_xy: Tuple[float, float] = (0.0, 0.0), enforce_quads: bool = True,
                        remove_islands: bool = True, min_island_area_px: int = 64):
    """``(mesh, MeshAssets(mesh, centres, roi_mask=binned mask))`` (d2ic/mask2mesh.py:145-182)."""
    m = np.asarray(mask, dtype=bool)
    if remove_islands:                               # islands removed once, for the mesh and the ROI
        m = _remove_small_components(m, min_island_area_px)
    mesh = mask_to_mesh(m, element_size_px, binning, origin_xy, enforce_quads, False, min_island_area_px)
    roi = downsample_mask(m, binning)
    return mesh, MeshAssets(mesh=mesh, element_centers_xy=compute_element_centers(mesh), pixel_data=None,
                            roi_mask=roi)


def mask_to_mesh_gmsh(*args, **kwargs) -> Mesh:
    """Unstructured gmsh mesher of the reference: requires gmsh and meshio."""
    try:
        import gmsh  # noqa: F401
        import meshio  # noqa: F401
    except Exception as exc:
        raise ImportError("mask_to_mesh_gmsh requires gmsh and meshio, which are not installed") from exc
    raise NotImplementedError("the gmsh mesher is outside the GPU hot path of this package")


def mask_to_mesh_assets_gmsh(*args, **kwargs):
    mask_to_mesh_gmsh(*args, **kwargs)
