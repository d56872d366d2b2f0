"""Golden vectors (tests/golden/translation_128.npz, made by tests/golden/make_golden.py from the oracle).

CPU: the oracle reproduces the fixture from the fixture's own images (a
regression pin of the restatement, independent of the speckle renderer).
GPU: the product path against the fixture without running the oracle.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "translation_128.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def test_oracle_reproduces_golden(gold):
    from oracle import cubic, fast, mesh, objective, pixels
    a = mesh.mask_to_mesh_assets(gold["roi_mask"], 16)
    assert np.array_equal(a["nodes"], gold["nodes"]) and np.array_equal(a["elements"], gold["elements"])
    pa = pixels.build_pixel_assets(a["nodes"], a["elements"], 128, 128, a["roi_mask"])
    for k in ("pixel_coords_ref", "pixel_nodes", "pixel_shapeN", "node_neighbor_index", "node_neighbor_weight",
              "node_pixel_index", "node_pixel_degree"):
        assert np.array_equal(pa[k], gold[k]), k
    c2 = cubic.bspline_coefficients(gold["deformed"].astype(np.float64))
    p = gold["sample_points"].astype(np.float64)
    v = cubic.cubic_sample(c2, cubic.ORACLE_PAD, p[:, 0], p[:, 1])
    np.testing.assert_allclose(v, gold["sample_val"], rtol=1e-12, atol=1e-10)
    pb = objective.Problem.build(gold["ref"].astype(np.float64), gold["deformed"].astype(np.float64), pa)
    J1, g1 = objective.J_total_and_grad(gold["u_rand"], pb, 0.1)
    np.testing.assert_allclose(J1, gold["J1"], rtol=1e-12)
    np.testing.assert_allclose(g1, gold["g1"], rtol=1e-9, atol=1e-14)
    u5, h5, _, _ = fast.FastProblem(pb, nthreads=1).cg_solve(np.zeros_like(a["nodes"]), 0.1, 5, 1e-3)
    np.testing.assert_allclose(u5, gold["u_iter5"], rtol=1e-9, atol=1e-12)


@pytest.mark.gpu
def test_gpu_path_against_golden(cuda, gold):
    from dataclasses import replace

    import d2ic_gb300 as d2
    mesh, assets = d2.mask_to_mesh_assets(gold["roi_mask"], 16)
    pix = d2.build_pixel_assets(mesh, gold["ref"], 1.0, assets.roi_mask)
    for k in ("pixel_coords_ref", "pixel_nodes", "pixel_shapeN", "node_pixel_index"):
        assert np.array_equal(np.asarray(getattr(pix, k)), gold[k]), k        # bit-exact maps / N / tables
    assets = replace(assets, pixel_data=pix)
    cfg = d2.MeshDICConfig(max_iters=200, tol=1e-3, reg_strength=0.1)
    dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(), cfg)
    dic.prepare(gold["ref"], assets)
    res = dic.run(gold["deformed"])
    used = np.unique(gold["elements"])
    u = np.asarray(res.u_nodal, np.float64)
    err = np.abs(u[used] - gold["u_conv"][used]).max()
    assert err <= 1e-3, err                                                    # nodal tolerance, px
    assert abs(res.diagnostics.info["n_iters"] - int(gold["k_conv"])) <= 2
    # strain kernel parity: the GPU strain against the FP64 strain of the GPU's own displacement
    from oracle import mesh as om, strain as ostrain
    sidx, sdeg = om.node_neighbor_tables(gold["nodes"], gold["elements"])
    _, E = ostrain.green_lagrange_nodes_lsq(u, gold["nodes"], sidx, sdeg)
    assert np.abs(np.asarray(res.strain) - ostrain.to_voigt(E)).max() <= 1e-5   # strain tolerance
    # end to end: the two solves stop at tol 1e-3 within an iteration or two of each other; a strain is a
    # difference quotient of nodal values over the 16 px element, so its gap is bounded by ~2 err / 16
    e2e = np.abs(np.asarray(res.strain) - gold["strain_voigt"]).max()
    print(f"golden: n_iters gpu={res.diagnostics.info['n_iters']} oracle={int(gold['k_conv'])} "
          f"max|du|={err:.2e} px max|dE|={e2e:.2e}")
    assert e2e <= 1e-5 + 2 * err / 16
    J, g = dic.solver.objective_and_gradient(dic.state, gold["deformed"], gold["u_rand"])
    assert abs(J - float(gold["J1"])) <= 1e-5 * abs(float(gold["J1"]))
    assert np.abs(g - gold["g1"]).max() <= 1e-4 * np.abs(gold["g1"]).max()
