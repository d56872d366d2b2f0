"""Product asset builder against the FP64 oracle (CPU): maps, shape functions, tables bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

import d2ic_gb300 as d2
from d2ic_gb300 import pixel_assets as pp
from d2ic_gb300.mesh_assets import Mesh, build_node_neighbor_tables
from d2ic_gb300.synthetic import ellipse_mask, rect_mask
from oracle import mesh as om
from oracle import pixels as op

FIELDS = ["pixel_coords_ref", "pixel_nodes", "pixel_shapeN", "node_neighbor_index", "node_neighbor_degree",
          "node_neighbor_weight", "node_pixel_index", "node_N_weight", "node_pixel_degree", "roi_mask_flat"]


def _compare(prod, orc):
    for k in FIELDS:
        a, b = np.asarray(getattr(prod, k)), np.asarray(orc[k])
        assert a.shape == b.shape, k
        assert np.array_equal(a, b), k


@pytest.mark.parametrize("H,W,elem,binning", [(96, 80, 16, 1), (120, 100, 12, 1), (128, 128, 8, 2)])
def test_structured_assets_bit_exact_vs_bruteforce(H, W, elem, binning):
    rng = np.random.default_rng(H + elem)
    mask = ellipse_mask(H, W, rng, 0.5, 0.8)
    mesh, assets = d2.mask_to_mesh_assets(mask, elem, binning=binning)
    nodes, elements = om.mask_to_mesh(mask, elem, binning=binning)
    assert np.array_equal(mesh.nodes_xy, nodes) and np.array_equal(mesh.elements, elements)
    roi = assets.roi_mask if binning == 1 else None
    prod = d2.build_pixel_assets(mesh, np.zeros((H, W)), 1.0, roi)
    orc = op.build_pixel_assets(nodes, elements, H, W, roi, bruteforce=True)
    _compare(prod, orc)


def test_generic_quad_mesh_bit_exact_vs_bruteforce():
    mesh, _ = d2.mask_to_mesh_assets(np.ones((90, 110), bool), 15)
    rng = np.random.default_rng(3)
    nodes = np.asarray(mesh.nodes_xy) + rng.uniform(-2.5, 2.5, np.asarray(mesh.nodes_xy).shape)
    m2 = Mesh(nodes, mesh.elements)
    assert pp.structured_grid(nodes, mesh.elements) is None
    prod = d2.build_pixel_assets(m2, np.zeros((90, 110)), 1.0, None)
    orc = op.build_pixel_assets(nodes, np.asarray(mesh.elements), 90, 110, None, bruteforce=True)
    _compare(prod, orc)


def test_config0_assets_bit_exact():
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(512, 512, 448, 448), 16)
    prod = d2.build_pixel_assets(mesh, np.zeros((512, 512)), 1.0, assets.roi_mask)
    orc = op.build_pixel_assets(np.asarray(mesh.nodes_xy), np.asarray(mesh.elements), 512, 512, assets.roi_mask)
    assert prod.n_pixels == 200704
    _compare(prod, orc)


def test_strain_neighbor_tables_match_reference_rule():
    rng = np.random.default_rng(1)
    mesh, _ = d2.mask_to_mesh_assets(ellipse_mask(80, 90, rng), 8)
    i1, d1 = build_node_neighbor_tables(mesh)
    i2, d2_ = om.node_neighbor_tables(np.asarray(mesh.nodes_xy), np.asarray(mesh.elements))
    assert np.array_equal(i1, i2) and np.array_equal(d1, d2_)


def test_build_errors_match_reference():
    mesh, _ = d2.mask_to_mesh_assets(np.ones((40, 40), bool), 8)
    with pytest.raises(ValueError):
        d2.build_pixel_assets(mesh, np.zeros((40, 40)), 1.0, np.ones((30, 40), bool))
    with pytest.raises(ValueError):
        d2.mask_to_mesh(np.zeros((20, 20), bool), 8)
    with pytest.raises(ValueError):
        d2.mask_to_mesh(np.ones((20, 20), bool), 0)


def test_host_helpers_match_numpy_forms():
    """The host fast paths give exactly what the plain numpy forms give: sort-based unique of
    edge keys, shape functions without the stacking copy, ROI pixels from the mask window."""
    from d2ic_gb300.mesh_assets import unique_sorted
    from d2ic_gb300.pixel_assets import _roi_pixels, _sample_pixels_in_bbox, shape_functions
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 10 ** 9, 100000)
    assert np.array_equal(unique_sorted(keys), np.unique(keys)) and unique_sorted(keys[:0]).size == 0
    xi, eta = rng.uniform(-1, 1, 1000), rng.uniform(-1, 1, 1000)
    ref = np.stack([0.25 * (1 - xi) * (1 - eta), 0.25 * (1 + xi) * (1 - eta),
                    0.25 * (1 + xi) * (1 + eta), 0.25 * (1 - xi) * (1 + eta)], axis=-1)
    assert np.array_equal(shape_functions(xi, eta), ref)
    H, W = 61, 47
    nodes = np.array([[3.2, 4.9], [40.1, 4.9], [40.1, 55.3], [3.2, 55.3]])
    roi = rng.random((H, W)) > 0.3
    for mask in (roi, None):
        pc = _sample_pixels_in_bbox(nodes, H, W, 2.0)
        if mask is not None:
            rows = np.clip(np.floor(pc[:, 1] - 0.5).astype(int), 0, H - 1)
            cols = np.clip(np.floor(pc[:, 0] - 0.5).astype(int), 0, W - 1)
            pc = pc[mask[rows, cols]]
        r, c = _roi_pixels(nodes, H, W, 2.0, mask)
        assert np.array_equal(np.stack([c + 0.5, r + 0.5], axis=1), pc)


def test_island_removal_fast_paths_equal_the_general_rule():
    """One component (kept or dropped) and several components all kept take shortcuts in
    _remove_small_components; each must equal the flood-fill rule of the oracle."""
    from d2ic_gb300.mask2mesh import _remove_small_components
    one = np.zeros((40, 50), bool)
    one[5:30, 8:40] = True
    two = one.copy()
    two[33:38, 44:49] = True                      # a second component of 25 pixels
    tiny = np.zeros((40, 50), bool)
    tiny[3:5, 3:5] = True                         # one component of 4 pixels
    for m, a in ((one, 64), (one, 2000), (two, 10), (two, 64), (tiny, 3), (tiny, 5)):
        got = _remove_small_components(m, a)
        assert np.array_equal(got, om.remove_small_components_floodfill(m, a)), (int(m.sum()), a)


def test_mask_to_mesh_assets_removes_islands_once():
    """The mesh and the ROI of mask_to_mesh_assets come from the same cleaned mask."""
    m = ellipse_mask(300, 260, np.random.default_rng(3))
    m[5:9, 5:9] = True                            # an island below the default 64 pixels
    mesh, assets = d2.mask_to_mesh_assets(m, 12)
    ref_mesh = d2.mask_to_mesh(m, 12)
    assert np.array_equal(mesh.nodes_xy, ref_mesh.nodes_xy) and np.array_equal(mesh.elements, ref_mesh.elements)
    assert not assets.roi_mask[5:9, 5:9].any() and assets.roi_mask.sum() == (m.sum() - 16)


def test_tile_shape_uses_the_90th_percentile_when_the_largest_box_does_not_fit():
    """Coefficient tile per chunk: the largest pixel box when it fits in TILE_MAX_FLOATS, else the
    90th percentile of the boxes' sides (chunks beyond it read the rest from global memory)."""
    from d2ic_gb300 import _lib
    from d2ic_gb300.engine import FrameLayout

    def boxes(sizes):
        b = []
        for k, (w, h) in enumerate(sizes):
            x0, y0 = 40 * k, 10
            b.append([x0 | (y0 << 16), (x0 + w - 1) | ((y0 + h - 1) << 16)])
        return np.asarray(b, np.int64).astype(np.uint32).view(np.int32)

    regular = boxes([(16, 16)] * 20)
    assert FrameLayout._tile_shape(_lib.INTERP_CUBIC, regular, 512, 512) == (28, 24)
    outliers = boxes([(32, 8)] * 30 + [(32, 18), (30, 24)])          # the largest needs 44 x 32 > 736
    assert FrameLayout._tile_shape(_lib.INTERP_CUBIC, outliers, 1024, 1024) == (44, 16)
    huge = boxes([(60, 60)] * 10)
    assert FrameLayout._tile_shape(_lib.INTERP_CUBIC, huge, 1024, 1024) == (0, 0)
    assert FrameLayout._tile_shape(_lib.INTERP_LINEAR, regular, 512, 512) == (0, 0)
