"""Launch-shape autotuner: signatures and cache on the host; measured choice and solve parity on the GPU."""
from __future__ import annotations

import json

import numpy as np
import pytest


def _frame(H=128, elem=16, seed=5):
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    ref, frames = speckle_sequence(H, H, [Translation(0.4, -0.3)], seed=seed, noise_seeds=[seed, seed + 1])
    # ROI on the element grid (16..112): every element lies inside it, no weakly held corner nodes
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, H - 32, H - 32), elem)
    pix = d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask)
    return ref, frames[0], mesh, assets, pix


def test_signature_and_cache_roundtrip(tmp_path):
    from d2ic_gb300.autotune import Autotuner, LaunchShape, frame_signature
    ref, _, _, _, pix = _frame()
    key = frame_signature(pix, 128, 128, "cubic")
    assert key == frame_signature(pix, 128, 128, "cubic")
    assert key != frame_signature(pix, 128, 128, "linear")
    assert ":e16:" in key                                   # element size recovered from the pixel map
    path = tmp_path / "tune.json"
    t = Autotuner(device="cpu", cache_path=str(path))
    t.cache[key] = LaunchShape(128, 0, 12.5)
    t._save()
    assert json.loads(path.read_text())[key]["chunk_pixels"] == 128
    t2 = Autotuner(device="cpu", cache_path=str(path))
    assert t2.cache[key] == LaunchShape(128, 0, 12.5)
    with pytest.raises(ValueError):
        Autotuner(device="cpu", chunk_candidates=(0, 300))


def test_only_distinct_chunk_sizes_are_timed():
    """Chunks hold pixels of one element: sizes at or above the largest element give one layout."""
    from d2ic_gb300.autotune import distinct_chunk_sizes
    assert distinct_chunk_sizes((64, 128, 256), 64) == (64,)          # 8-px elements
    assert distinct_chunk_sizes((64, 128, 256), 144) == (64, 128, 256)   # 12-px elements
    assert distinct_chunk_sizes((64, 128, 256), 256) == (64, 128, 256)
    assert distinct_chunk_sizes((64, 128, 256), 1024) == (64, 128, 256)
    assert distinct_chunk_sizes((256,), 16) == (256,)


@pytest.mark.gpu
def test_tuned_solve_matches_oracle(cuda):
    import d2ic_gb300 as d2
    from oracle import fast
    ref, deformed, mesh, assets, pix = _frame()
    from dataclasses import replace
    assets = replace(assets, pixel_data=pix)
    cfg = d2.MeshDICConfig(max_iters=1000, tol=1e-5, reg_strength=0.1)
    solver = d2.GlobalCGSolver(device=cuda, autotune=True)
    dic = d2.DICMeshBased(mesh, solver, cfg)
    dic.prepare(ref, assets)
    res = dic.run(deformed)
    shape = solver.launch_shape
    assert shape is not None and shape.chunk_pixels in (64, 128, 256) and shape.us_per_round > 0
    from d2ic_gb300.autotune import default_tuner, frame_signature
    trials = default_tuner(cuda).trials[frame_signature(pix, 128, 128, "cubic")]
    assert len(trials) >= 3 and min(t.us_per_round for t in trials) == shape.us_per_round
    from oracle import objective, pixels
    oa = pixels.build_pixel_assets(np.asarray(mesh.nodes_xy), np.asarray(mesh.elements), 128, 128, assets.roi_mask)
    pb = objective.Problem.build(ref, deformed, oa)
    u_ref, _, _, _ = fast.FastProblem(pb).cg_solve(np.zeros((mesh.nodes_xy.shape[0], 2)), 0.1, 1000, 1e-5)
    used = np.unique(np.asarray(mesh.elements))
    assert np.abs(np.asarray(res.u_nodal, np.float64)[used] - u_ref[used]).max() <= 1e-3
