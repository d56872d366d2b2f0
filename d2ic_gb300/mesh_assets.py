"""Mesh, mesh-level assets and pixel-level assets.

Reference: d2ic/mesh_assets.py:12-164.  Host-side numpy containers; the GPU
layout derived from them lives in :mod:`d2ic_gb300.engine`.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np

from .types import Array


@dataclass(frozen=True)
class Mesh:
    """2D mesh in image coordinates (x = column, y = row): nodes (Nn,2), elements (Ne,4)."""
    nodes_xy: Array
    elements: Array


@dataclass(frozen=True)
class MeshAssets:
    """Mesh plus element centres, optional strain neighbour tables, pixel assets and ROI mask."""
    mesh: Mesh
    element_centers_xy: Array
    node_neighbor_index: Optional[Array] = None
    node_neighbor_degree: Optional[Array] = None
    pixel_data: "PixelAssets | None" = None
    roi_mask: Optional[Array] = None


class PixelAssets:
    """Pixel-level caches (reference fields of d2ic/mesh_assets.py:55-75).

    ``node_pixel_index / node_N_weight / node_pixel_degree`` (the dense
    node -> pixel tables) are built on first access: the GPU solver gathers
    through a node -> chunk table instead and never needs them.
    ``pixel_elts`` (element of each pixel) and ``xi_eta`` (local coordinates)
    are extra fields kept from the build.
    """

    _LAZY = ("node_pixel_index", "node_N_weight", "node_pixel_degree")

    def __init__(self, pixel_coords_ref, pixel_nodes, pixel_shapeN, node_neighbor_index, node_neighbor_degree,
                 node_neighbor_weight, node_reg_weight, node_pixel_index=None, node_N_weight=None,
                 node_pixel_degree=None, roi_mask_flat=None, image_shape=None, pixel_elts=None, xi_eta=None):
        self.pixel_coords_ref = pixel_coords_ref
        self.pixel_nodes = pixel_nodes
        self.pixel_shapeN = pixel_shapeN
        self.node_neighbor_index = node_neighbor_index
        self.node_neighbor_degree = node_neighbor_degree
        self.node_neighbor_weight = node_neighbor_weight
        self.node_reg_weight = node_reg_weight
        self._np_tables = None
        if node_pixel_index is not None:
            self._np_tables = (node_pixel_index, node_N_weight, node_pixel_degree)
        self.roi_mask_flat = roi_mask_flat
        self.image_shape = tuple(image_shape) if image_shape is not None else None
        self.pixel_elts = pixel_elts
        self.xi_eta = xi_eta

    def _tables(self):
        if self._np_tables is None:
            from .pixel_assets import build_node_pixel_dense
            self._np_tables = build_node_pixel_dense(self.pixel_nodes, self.pixel_shapeN,
                                                     np.asarray(self.node_reg_weight).shape[0])
        return self._np_tables

    @property
    def node_pixel_index(self):
        return self._tables()[0]

    @property
    def node_N_weight(self):
        return self._tables()[1]

    @property
    def node_pixel_degree(self):
        return self._tables()[2]

    @property
    def n_pixels(self) -> int:
        return int(np.asarray(self.pixel_coords_ref).shape[0])



def unique_sorted(a: np.ndarray) -> np.ndarray:
    """``np.unique`` of a 1-D integer array (sorted distinct values) by one sort and a neighbour
    comparison; the same result, and much faster than the hash-based path of recent numpy on
    millions of keys."""
    s = np.sort(np.asarray(a).ravel())
    if s.size == 0:
        return s
    keep = np.empty(s.size, dtype=bool)
    keep[0] = True
    np.not_equal(s[1:], s[:-1], out=keep[1:])
    return s[keep]

def compute_element_centers(mesh: Mesh) -> np.ndarray:
    """Mean of each element's node coordinates (d2ic/mesh_assets.py:77-92)."""
    return np.asarray(mesh.nodes_xy, dtype=np.float64)[np.asarray(mesh.elements)].mean(axis=1)


def build_node_neighbor_tables(mesh: Mesh, max_degree: int = 16):
    """Strain neighbour tables (d2ic/mesh_assets.py:95-132).

    For each node: the ascending list of other nodes sharing an element,
    truncated to ``max_degree``, zero padded.  Vectorised: unique (src, dst)
    pairs sorted by (src, dst), rank within src < max_degree.
    """
    nodes = np.asarray(mesh.nodes_xy)
    n = nodes.shape[0]
    el = np.asarray(mesh.elements, dtype=np.int64)
    idx = np.zeros((n, max_degree), dtype=np.int32)
    deg = np.zeros((n,), dtype=np.int32)
    if el.size == 0:
        return idx, deg
    k = el.shape[1]
    a, b = np.meshgrid(np.arange(k), np.arange(k), indexing="ij")
    m = (a != b).ravel()
    src = el[:, a.ravel()[m]].ravel()
    dst = el[:, b.ravel()[m]].ravel()
    key = unique_sorted(src * n + dst)
    src, dst = key // n, key % n
    cnt = np.bincount(src, minlength=n)
    start = np.cumsum(cnt) - cnt
    rank = np.arange(src.size) - np.repeat(start, cnt)
    keep = rank < max_degree
    idx[src[keep], rank[keep]] = dst[keep]
    deg[:] = np.minimum(cnt, max_degree)
    return idx, deg


def make_mesh_assets(mesh: Mesh, with_neighbors: bool = True, max_degree: int = 16) -> MeshAssets:
    """Element centres and (optionally) strain neighbour tables (d2ic/mesh_assets.py:135-164)."""
    centers = compute_element_centers(mesh)
    ni = nd = None
    if with_neighbors:
        ni, nd = build_node_neighbor_tables(mesh, max_degree=max_degree)
    return MeshAssets(mesh=mesh, element_centers_xy=centers, node_neighbor_index=ni, node_neighbor_degree=nd,
                      pixel_data=None)
