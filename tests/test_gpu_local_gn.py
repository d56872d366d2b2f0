"""Local Gauss-Newton refinement (d2ic/solver_local_gn.py) on the GPU vs the FP64 oracle sweeps."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(interp):
    from dataclasses import replace

    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Affine, rect_mask, speckle_sequence
    H = 128
    ref, frames = speckle_sequence(H, H, [Affine([[0.004, 0.001], [0.0, -0.003]], [0.45, -0.3], [64, 64])], seed=12,
                                   noise_seeds=[12, 13])
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, 112, 112), 16)
    assets = replace(assets, pixel_data=d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))
    return ref, frames[0], mesh, assets


@pytest.mark.parametrize("interp", ["cubic", "linear"])
def test_local_gn_sweeps_match_oracle(cuda, interp):
    import d2ic_gb300 as d2
    from oracle import local_gn, objective, pixels
    ref, deformed, mesh, assets = _case(interp)
    n_sweeps = 6
    cfg = d2.MeshDICConfig(max_iters=n_sweeps, tol=1e-3, reg_strength=0.1, save_history=True)
    dic = d2.DICMeshBased(mesh, d2.LocalGaussNewtonSolver(lam=1e-3, max_step=0.2, omega=0.5, interpolation=interp,
                                                          device=cuda), cfg)
    dic.prepare(ref, assets)
    u0 = np.tile(np.array([[0.4, -0.25]], np.float32), (mesh.nodes_xy.shape[0], 1))
    dic.set_initial_guess(u0)
    res = dic.run(deformed)
    oa = pixels.build_pixel_assets(np.asarray(mesh.nodes_xy), np.asarray(mesh.elements), 128, 128, assets.roi_mask)
    pb = objective.Problem.build(ref, deformed, oa, interpolation=interp)
    u_ref, h_ref = local_gn.local_sweeps(u0, pb, 1e-3, 0.2, 0.1, 0.5, n_sweeps)
    err = np.abs(np.asarray(res.u_nodal, np.float64) - u_ref).max()
    assert err <= 1e-3, err                                          # nodal tolerance, px
    hist = np.asarray(res.history)
    assert hist.shape == (n_sweeps, 2)
    assert np.allclose(hist, h_ref, rtol=1e-3, atol=1e-6)            # [rms r, rms step] per sweep


def test_cg_then_local_chain(cuda):
    """BatchMeshBased(dic_local=...): CG, then local sweeps from the CG solution (the reference pipeline)."""
    import d2ic_gb300 as d2
    ref, deformed, mesh, assets = _case("cubic")
    cg = d2.DICMeshBased(mesh, d2.GlobalCGSolver(device=cuda), d2.MeshDICConfig(max_iters=200, tol=1e-3,
                                                                                reg_strength=0.1))
    loc = d2.DICMeshBased(mesh, d2.LocalGaussNewtonSolver(device=cuda), d2.MeshDICConfig(max_iters=3, tol=1e-3,
                                                                                         reg_strength=0.1))
    batch = d2.BatchMeshBased(ref, assets, cg, d2.BatchConfig(warm_start_from_previous=True), dic_local=loc)
    batch.before([deformed])
    out = batch.sequence([deformed])
    u_cg = cg.run(deformed).u_nodal
    u = np.asarray(out.results[0].u_nodal)
    assert np.isfinite(u).all()
    assert 0 < np.abs(u - np.asarray(u_cg)).max() < 0.2                 # a few relaxed local steps from CG


def test_device_local_coordinates_bit_exact(cuda):
    """GPU Newton inverse map == host restatement, bit for bit, on distorted quads."""
    from d2ic_gb300.pixel_assets import local_coordinates, local_coordinates_device
    rng = np.random.default_rng(21)
    n_el = 400
    base = np.array([[0.0, 0.0], [10.0, 0.0], [10.0, 10.0], [0.0, 10.0]])
    nodes = (base[None] + rng.normal(0, 1.2, (n_el, 4, 2)) + 20 * rng.integers(0, 30, (n_el, 1, 2))).reshape(-1, 2)
    pn = np.arange(4 * n_el).reshape(n_el, 4).repeat(50, axis=0)
    w = rng.uniform(0.05, 0.95, (n_el * 50, 2))
    q = nodes[pn]
    pc = ((1 - w[:, :1]) * (1 - w[:, 1:]) * q[:, 0] + w[:, :1] * (1 - w[:, 1:]) * q[:, 1]
          + w[:, :1] * w[:, 1:] * q[:, 2] + (1 - w[:, :1]) * w[:, 1:] * q[:, 3])
    xh, eh = local_coordinates(pc, pn, nodes)
    xd, ed = local_coordinates_device(pc, pn, nodes, device=cuda)
    assert np.array_equal(xh.view(np.int64), xd.view(np.int64)) and np.array_equal(eh.view(np.int64), ed.view(np.int64))


def test_device_structured_assign_exact(cuda):
    """GPU tensor-grid pixel -> element search == host search, including pixels on grid lines
    (shared edges: lowest element wins), in holes and outside the grid."""
    import d2ic_gb300 as d2
    from d2ic_gb300.pixel_assets import _structured_assign, structured_assign_device, structured_grid
    from d2ic_gb300.synthetic import ellipse_mask
    H = W = 256
    mask = ellipse_mask(H, W, np.random.default_rng(3))
    mesh, _ = d2.mask_to_mesh_assets(mask, 12)
    nodes = np.asarray(mesh.nodes_xy, np.float64)
    sg = structured_grid(nodes, np.asarray(mesh.elements, np.int64))
    assert sg is not None
    gx, gy, _cell = sg
    rng = np.random.default_rng(4)
    pc = np.concatenate([
        rng.uniform(-5, W + 5, (20000, 2)),                                   # anywhere, also outside
        np.stack([rng.choice(gx, 4000), rng.uniform(0, H, 4000)], 1),        # on vertical grid lines
        np.stack([rng.uniform(0, W, 4000), rng.choice(gy, 4000)], 1),        # on horizontal grid lines
        np.stack([rng.choice(gx, 2000), rng.choice(gy, 2000)], 1),           # on grid nodes
    ])
    host = _structured_assign(pc, *sg)
    dev = structured_assign_device(pc, *sg, device=cuda)
    assert (host >= 0).sum() > 10000 and (host < 0).sum() > 1000
    assert np.array_equal(host, dev)
    # and through build_pixel_assets (device path) against the host mapping function
    ref = rng.random((H, W)).astype(np.float32)
    pix = d2.build_pixel_assets(mesh, ref, 1.0)
    elts, _ = d2.pixel_assets.build_pixel_to_element_mapping_numpy(pix.pixel_coords_ref, nodes, mesh.elements)
    assert np.array_equal(elts, pix.pixel_elts)
