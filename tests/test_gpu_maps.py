"""Discrepancy map (d2ic/discrepancy.py:86-127): oracle sanity on CPU, GPU kernel vs oracle."""
from __future__ import annotations

import numpy as np
import pytest


def test_oracle_discrepancy_known_answers():
    from oracle.discrepancy import bilinear_sample, discrepancy_map_ref
    img = np.arange(30, dtype=np.float64).reshape(5, 6)            # I(i, j) = 6 i + j: bilinear is exact
    xy = np.array([[1.5, 1.5], [2.25, 3.75], [5.5, 1.5], [0.4, 2.0]])
    v = bilinear_sample(img, xy)
    assert v[0] == 7.0 and v[1] == pytest.approx(6 * 3.25 + 1.75)
    assert np.isnan(v[2]) and np.isnan(v[3])                         # last column / left of the image
    # a pure translation by (0.5, 0): residual = +0.5 grey levels where valid
    pc = np.array([[1.5, 1.5], [3.5, 2.5], [5.5, 4.5]])
    m, rms = discrepancy_map_ref(img, img, np.array([[0.5, 0.0]]), pc, np.zeros((3, 1), int), np.ones((3, 1)),
                                 np.array([1 * 6 + 1, 2 * 6 + 3, 4 * 6 + 5]), (5, 6))
    assert m[1, 1] == 0.5 and m[2, 3] == 0.5 and np.isnan(m[4, 5]) and np.isnan(m[0, 0])
    assert rms == 0.5


@pytest.mark.gpu
def test_discrepancy_map_matches_oracle(cuda):
    from dataclasses import replace

    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    from oracle.discrepancy import discrepancy_map_ref
    H = W = 160
    ref, frames = speckle_sequence(H, W, [Translation(0.6, -0.3)], seed=8, noise_seeds=[8, 9])
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, W, 144, 144), 16)
    pix = d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask)
    assets = replace(assets, pixel_data=pix)
    cfg = d2.MeshDICConfig(max_iters=200, tol=1e-3, reg_strength=0.1, compute_discrepancy_map=True)
    dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(device=cuda), cfg)
    dic.prepare(ref, assets)
    res = dic.run(frames[0])
    assert res.diagnostics.info["discrepancy"] == "discrepancy_ref"
    gmap = res.pixel_maps["discrepancy_ref"].cpu().numpy()
    omap, orms = discrepancy_map_ref(ref, frames[0], res.u_nodal, pix.pixel_coords_ref, pix.pixel_nodes,
                                     pix.pixel_shapeN, pix.roi_mask_flat, (H, W))
    assert np.array_equal(np.isnan(gmap), np.isnan(omap))            # same ROI / validity pattern
    ok = ~np.isnan(omap)
    assert ok.sum() > 0.8 * 144 * 144
    assert np.abs(gmap[ok] - omap[ok]).max() <= 2e-3                  # grey levels (FP32 weights vs FP64)
    assert abs(res.diagnostics.info["discrepancy_rms"] - orms) <= 1e-4 * max(orms, 1.0)


@pytest.mark.gpu
def test_batch_writes_per_frame_fields(cuda, tmp_path):
    """BatchMeshBased(save_per_frame=True) writes frame_XXXX.npz with u_nodal, strain and the
    discrepancy map (d2ic/batch_mesh_based.py:174-185)."""
    from dataclasses import replace

    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    H = W = 128
    ref, frames = speckle_sequence(H, W, [Translation(0.3, 0.1), Translation(0.5, 0.2)], seed=9,
                                   noise_seeds=[9, 10, 11])
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, W, 96, 96), 16)
    assets = replace(assets, pixel_data=d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))
    cfg = d2.MeshDICConfig(max_iters=100, tol=1e-3, reg_strength=0.1, compute_discrepancy_map=True)
    dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(device=cuda), cfg)
    batch = d2.BatchMeshBased(ref, assets, dic, d2.BatchConfig(warm_start_from_previous=True, save_per_frame=True,
                                                               per_frame_dir=str(tmp_path)))
    batch.before(frames)
    out = batch.sequence(frames)
    for k in range(2):
        z = np.load(tmp_path / f"frame_{k:04d}.npz")
        assert np.array_equal(z["u_nodal"], np.asarray(out.results[k].u_nodal))
        assert z["strain"].shape == (mesh.nodes_xy.shape[0], 3)
        assert z["discrepancy_ref"].shape == (H, W) and np.isfinite(z["discrepancy_ref"]).sum() > 0.5 * 96 * 96
    seq = np.load(d2.save_fields_sequence(tmp_path, mesh.nodes_xy, out.results))
    assert seq["u_nodal"].shape == (2, mesh.nodes_xy.shape[0], 2)
    assert seq["discrepancy_ref"].shape == (2, H, W)
    assert np.array_equal(seq["u_nodal"][1], np.asarray(out.results[1].u_nodal))
