"""The frame layout built on the device from the ROI mask (FrameLayout.from_grid: d2ic_grid_count,
d2ic_grid_layout, d2ic_grid_springs) against the layout built from the host pixel assets
(build_pixel_assets, d2ic/pixel_assets.py:21-526): every table bit-exact -- pixel records (element
map, FP64 Newton coordinates, I1), chunks, node slots, group counts and spring tables."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _masks():
    from d2ic_gb300.synthetic import ellipse_mask, plate_hole_mask, rect_mask
    out = [("plate_hole_512_e16", plate_hole_mask(512, 512, 450, 75.0), 16, 512),
           ("corner_cells_160_e16", rect_mask(160, 160, 114, 114), 16, 160),
           ("whole_image_96_e12", None, 12, 96)]
    for i, e in enumerate((8, 12, 24, 32)):
        out.append((f"ellipse_384_e{e}", ellipse_mask(384, 384, np.random.default_rng(70 + i)), e, 384))
    # a mask with an island (removed by the mesher) and a cut through the plate
    m = plate_hole_mask(256, 256, 240, 40.0)
    m[5:9, 5:9] = True
    m[:, 120:124] = False
    out.append(("islands_256_e16", m, 16, 256))
    return out


@pytest.mark.parametrize("case", _masks(), ids=lambda c: c[0])
@pytest.mark.parametrize("interpolation", ["cubic", "linear"])
def test_device_layout_equals_host_layout(cuda, case, interpolation):
    import d2ic_gb300 as d2
    from d2ic_gb300.engine import FrameLayout
    from d2ic_gb300.synthetic import Translation, speckle_sequence
    name, mask, elem, H = case
    ref, _ = speckle_sequence(H, H, [Translation(0.0, 0.0)], seed=9, noise_seeds=[9, 10])
    if mask is None:
        mesh, assets = d2.mask_to_mesh_assets(np.ones((H, H), bool), elem)
        roi = None
    else:
        mesh, assets = d2.mask_to_mesh_assets(mask, elem)
        roi = assets.roi_mask
    pix = d2.build_pixel_assets(mesh, ref, 1.0, roi)
    for chunk in (256, 64):
        host = FrameLayout(pix, mesh.nodes_xy.shape[0], ref, interpolation, cuda, chunk_max=chunk)
        dev = FrameLayout.from_grid(mesh, roi, ref, interpolation, cuda, chunk_max=chunk)
        assert (dev.n_pix, dev.n_chunks, dev.node_chunk_k, dev.max_deg) == \
            (host.n_pix, host.n_chunks, host.node_chunk_k, host.max_deg)
        assert (dev.tile_w, dev.tile_h) == (host.tile_w, host.tile_h)
        for f in ("pix", "chunk_begin", "chunk_nodes", "chunk_box", "chunk_slot", "group_need", "nbr_index",
                  "nbr_weight"):
            a, b = getattr(dev, f), getattr(host, f)
            assert a.shape == b.shape and a.dtype == b.dtype, f
            assert torch.equal(a, b), f"{name} chunk {chunk}: {f} differs"


def test_grid_pixel_data_drives_the_solver(cuda):
    """GlobalCGSolver on assets from build_pixel_assets_device (no per-pixel host arrays) gives the
    same solve as on the host pixel assets."""
    from dataclasses import replace

    import d2ic_gb300 as d2
    from d2ic_gb300.pixel_assets import GridPixelData, build_pixel_assets_device
    from d2ic_gb300.synthetic import Translation, plate_hole_mask, speckle_sequence
    H = 256
    ref, frames = speckle_sequence(H, H, [Translation(0.4, -0.3)], seed=12, noise_seeds=[12, 13])
    mesh, assets = d2.mask_to_mesh_assets(plate_hole_mask(H, H, 220, 40.0), 16)
    cfg = d2.MeshDICConfig(max_iters=100, tol=1e-3, reg_strength=0.1)
    out = []
    for pd in (d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask),
               build_pixel_assets_device(mesh, ref, 1.0, assets.roi_mask)):
        dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(), cfg)
        dic.prepare(ref, replace(assets, pixel_data=pd))
        out.append((pd, dic.run(frames[0])))
    assert isinstance(out[1][0], GridPixelData)
    assert out[1][0].n_pixels == out[0][0].pixel_coords_ref.shape[0]
    assert out[0][1].diagnostics.info["n_iters"] == out[1][1].diagnostics.info["n_iters"]
    assert np.array_equal(np.asarray(out[0][1].u_nodal), np.asarray(out[1][1].u_nodal))
