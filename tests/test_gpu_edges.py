"""Edge cases of the CG path against the FP64 oracle (d2ic/solver_global_cg.py:326-469):
no iterations, a start at the solution (stop branch on the first evaluation), a ragged image
whose size no element divides (bilinear and cubic sampling), and motion that pushes stencils past
the image border (edge-replicated taps)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(H, W, mask_hw, elem, warp, seed):
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import rect_mask, speckle_sequence
    ref, frames = speckle_sequence(H, W, [warp], seed=seed, noise_seeds=[seed, seed + 1])
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, W, *mask_hw), elem)
    pix = d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask)
    a = d2.MeshAssets(mesh=mesh, element_centers_xy=assets.element_centers_xy, pixel_data=pix,
                      roi_mask=assets.roi_mask)
    return ref, frames[0], mesh, assets, a


def _oracle(ref, dfm, mesh, assets, interpolation="cubic"):
    from oracle import objective, pixels
    oa = pixels.build_pixel_assets(np.asarray(mesh.nodes_xy), np.asarray(mesh.elements), ref.shape[0], ref.shape[1],
                                   assets.roi_mask)
    return objective.Problem.build(ref, dfm, oa, interpolation=interpolation)


def _run(mesh, a, ref, dfm, cfg, interpolation="cubic", u0=None):
    import d2ic_gb300 as d2
    dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(interpolation=interpolation), cfg)
    dic.prepare(ref, a)
    if u0 is not None:
        dic.set_initial_guess(u0)
    return dic.run(dfm)


def test_zero_iterations_return_the_initial_guess(cuda):
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation
    ref, dfm, mesh, assets, a = _case(128, 128, (96, 96), 16, Translation(0.3, 0.2), seed=31)
    u0 = np.random.default_rng(0).normal(0, 0.1, (mesh.nodes_xy.shape[0], 2)).astype(np.float32)
    res = _run(mesh, a, ref, dfm, d2.MeshDICConfig(max_iters=0, tol=1e-3, reg_strength=0.1), u0=u0)
    assert res.diagnostics.info["n_iters"] == 0
    assert np.array_equal(np.asarray(res.u_nodal), u0)


def test_start_at_the_solution_stops_on_the_first_evaluation(cuda):
    """Identical images and u0 = 0: g = 0 at the start, so the stop branch fires with k = 0 and
    history row 0 = [J, |g|, 0] (the reference writes the stop row without advancing k)."""
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation
    ref, _, mesh, assets, a = _case(128, 128, (96, 96), 16, Translation(0.0, 0.0), seed=32)
    res = _run(mesh, a, ref, ref, d2.MeshDICConfig(max_iters=50, tol=1e-3, reg_strength=0.1))
    assert res.diagnostics.info["n_iters"] == 0
    assert np.abs(np.asarray(res.u_nodal)).max() == 0.0
    h = np.asarray(res.history)
    assert h[0, 0] == 0.0 and h[0, 1] < 1e-3 and h[0, 2] == 0.0 and np.isnan(h[1:]).all()


@pytest.mark.parametrize("interpolation", ["linear", "cubic"])
def test_ragged_image_matches_oracle(cuda, interpolation):
    """257 x 389 image, 12-px elements over a centred 240 x 372 ROI: no element size divides the
    image, rows and pitch are odd.  The tolerance is the headline one (1e-3): below ~1e-4 the FP32
    pixel sums of the objective cannot resolve the Armijo decrease, as in the reference's FP32
    solve.  (Partly covered elements are covered by tests/test_gpu_parity_masks.py.)"""
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation
    from oracle import fast
    ref, dfm, mesh, assets, a = _case(257, 389, (240, 372), 12, Translation(0.45, -0.3), seed=33)
    cfg = d2.MeshDICConfig(max_iters=300, tol=1e-3, reg_strength=0.1)
    res = _run(mesh, a, ref, dfm, cfg, interpolation=interpolation)
    pb = _oracle(ref, dfm, mesh, assets, interpolation)
    u = np.asarray(res.u_nodal, np.float64)
    if interpolation == "cubic":
        ur, _, kr, _ = fast.FastProblem(pb).cg_solve(np.zeros_like(u), 0.1, 300, 1e-3)
    else:
        from oracle import objective
        ur, _, kr, _ = objective.cg_solve(np.zeros_like(u), pb, 0.1, 300, 1e-3)
    used = np.unique(np.asarray(mesh.elements))
    print(f"{interpolation}: n_iters gpu={res.diagnostics.info['n_iters']} oracle={kr} "
          f"max|du|={np.abs(u[used] - ur[used]).max():.2e}")
    assert np.abs(u[used] - ur[used]).max() <= 1e-3
    assert abs(res.diagnostics.info["n_iters"] - kr) <= max(3, 0.05 * kr)


def test_motion_past_the_border_matches_oracle(cuda):
    """A ROI reaching the image edge and a 2.6 px translation: stencils of the edge pixels leave
    the image and read the edge-replicated coefficients of the halo (the reference's nearest-edge
    boundary)."""
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation
    from oracle import fast
    ref, dfm, mesh, assets, a = _case(128, 128, (128, 128), 16, Translation(2.6, -1.7), seed=34)
    cfg = d2.MeshDICConfig(max_iters=400, tol=1e-4, reg_strength=0.1)
    u0 = np.tile(np.array([[2.5, -1.5]], np.float32), (mesh.nodes_xy.shape[0], 1))
    res = _run(mesh, a, ref, dfm, cfg, u0=u0)
    pb = _oracle(ref, dfm, mesh, assets)
    u = np.asarray(res.u_nodal, np.float64)
    ur, _, kr, _ = fast.FastProblem(pb).cg_solve(u0.astype(np.float64), 0.1, 400, 1e-4)
    used = np.unique(np.asarray(mesh.elements))
    assert np.abs(u[used] - ur[used]).max() <= 1e-3
