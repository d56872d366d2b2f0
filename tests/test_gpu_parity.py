"""GPU parity of the sm_103a kernels against the FP64 oracle (through the C ABI).

Tolerances (stated per test): bicubic samples 1e-5 relative to the grey
range; objective/gradient within FP32 accumulation error; converged nodal
displacements <= 1e-3 px; strain <= 1e-5.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _speckle_case(H, W, mask_hw, elem, warp, seed=0):
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import rect_mask, speckle_sequence
    ref, frames = speckle_sequence(H, W, [warp], seed=seed, noise_seeds=[seed, seed + 1])
    mask = rect_mask(H, W, *mask_hw)
    mesh, assets = d2.mask_to_mesh_assets(mask, elem)
    pix = d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask)
    return ref, frames[0], mesh, assets, pix


@pytest.fixture(scope="module")
def config0():
    from d2ic_gb300.synthetic import Translation
    return _speckle_case(512, 512, (448, 448), 16, Translation(0.35, -0.62), seed=0)


def _oracle_problem(ref, dfm, mesh, assets):
    from oracle import objective, pixels
    oa = pixels.build_pixel_assets(np.asarray(mesh.nodes_xy), np.asarray(mesh.elements), ref.shape[0], ref.shape[1],
                                   assets.roi_mask)
    return objective.Problem.build(ref, dfm, oa)


def test_cubic_sampler_matches_oracle(cuda):
    from d2ic_gb300 import engine
    from oracle.cubic import ORACLE_PAD, bspline_coefficients, cubic_sample
    rng = np.random.default_rng(3)
    img = rng.uniform(20, 230, (97, 131)).astype(np.float32)
    c = engine.prepare_coefficients(engine.as_device_image(img, cuda), engine.interp_kind("cubic"))
    # points given to both sides as float32 (the kernel's coordinate type)
    xy = np.stack([rng.uniform(-6, 137, 10000), rng.uniform(-6, 103, 10000)], axis=1).astype(np.float32)
    v, gx, gy = engine.sample_points(c, 97, 131, engine.interp_kind("cubic"), torch.tensor(xy))
    co = bspline_coefficients(img.astype(np.float64))
    xy64 = xy.astype(np.float64)
    rv, rgx, rgy = cubic_sample(co, ORACLE_PAD, xy64[:, 0], xy64[:, 1], with_grad=True)
    # tolerance: samples within 1e-5 of the grey range, gradients within 1e-5 of the largest gradient
    scale = float(img.max() - img.min())
    gscale = float(max(np.abs(rgx).max(), np.abs(rgy).max()))
    assert np.abs(v.cpu().numpy() - rv).max() <= 1e-5 * scale
    assert np.abs(gx.cpu().numpy() - rgx).max() <= 1e-5 * gscale
    assert np.abs(gy.cpu().numpy() - rgy).max() <= 1e-5 * gscale


def test_linear_sampler_matches_oracle(cuda):
    from d2ic_gb300 import engine
    from oracle.cubic import linear_sample
    rng = np.random.default_rng(4)
    img = rng.uniform(20, 230, (64, 64)).astype(np.float32)
    c = engine.prepare_coefficients(engine.as_device_image(img, cuda), engine.interp_kind("linear"))
    xy = np.stack([rng.uniform(-3, 67, 5000), rng.uniform(-3, 67, 5000)], axis=1)
    v, gx, gy = engine.sample_points(c, 64, 64, engine.interp_kind("linear"), torch.tensor(xy))
    rv, rgx, rgy = linear_sample(img.astype(np.float64), xy[:, 0] + 0.5, xy[:, 1] + 0.5, with_grad=True)
    assert np.abs(v.cpu().numpy() - rv).max() <= 1e-5 * 210
    assert np.abs(gx.cpu().numpy() - rgx).max() <= 1e-4 * 210
    assert np.abs(gy.cpu().numpy() - rgy).max() <= 1e-4 * 210


def test_objective_and_gradient_match_oracle(cuda, config0):
    import d2ic_gb300 as d2
    from d2ic_gb300.dic_mesh_based import MeshDICState
    from oracle import objective
    ref, dfm, mesh, assets, pix = config0
    a = d2.MeshAssets(mesh=mesh, element_centers_xy=assets.element_centers_xy, pixel_data=pix, roi_mask=assets.roi_mask)
    cfg = d2.MeshDICConfig(max_iters=10, tol=1e-3, reg_strength=0.1)
    st = MeshDICState(ref_image=ref, nodes_xy_device=None, assets=a, config=cfg)
    solver = d2.GlobalCGSolver()
    solver.compile(a)
    rng = np.random.default_rng(5)
    u = rng.normal(0, 0.3, (mesh.nodes_xy.shape[0], 2)).astype(np.float32)
    J, g = solver.objective_and_gradient(st, dfm, u)
    pb = _oracle_problem(ref, dfm, mesh, assets)
    Jr, gr = objective.J_total_and_grad(u.astype(np.float64), pb, 0.1)
    assert abs(J - Jr) <= 1e-5 * abs(Jr)
    # FP32 sample/accumulate: gradient within 1e-4 of its max magnitude
    assert np.abs(g - gr).max() <= 1e-4 * np.abs(gr).max()


def test_cg_solve_config0_matches_oracle(cuda, config0):
    import d2ic_gb300 as d2
    from oracle import fast
    ref, dfm, mesh, assets, pix = config0
    a = d2.MeshAssets(mesh=mesh, element_centers_xy=assets.element_centers_xy, pixel_data=pix, roi_mask=assets.roi_mask)
    cfg = d2.MeshDICConfig(max_iters=200, tol=1e-3, reg_strength=0.1)
    dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(), cfg)
    dic.prepare(ref, a)
    res = dic.run(dfm)
    u = np.asarray(res.u_nodal, dtype=np.float64)
    pb = _oracle_problem(ref, dfm, mesh, assets)
    ur, hr, kr, _ = fast.FastProblem(pb).cg_solve(np.zeros_like(u), 0.1, 200, 1e-3)
    used = np.unique(np.asarray(mesh.elements))
    err = np.abs(u[used] - ur[used]).max()
    print(f"config0: n_iters gpu={res.diagnostics.info['n_iters']} oracle={kr} max|du|={err:.3e}px")
    assert err <= 1e-3          # spec tolerance, px
    assert abs(res.diagnostics.info["n_iters"] - kr) <= max(3, 0.05 * kr)
    h = np.asarray(res.history)
    k = res.diagnostics.info["n_iters"]
    assert np.isfinite(h[:k]).all() and np.isnan(h[k + 1:]).all()


def test_cg_solve_is_deterministic(cuda, config0):
    import d2ic_gb300 as d2
    ref, dfm, mesh, assets, pix = config0
    a = d2.MeshAssets(mesh=mesh, element_centers_xy=assets.element_centers_xy, pixel_data=pix, roi_mask=assets.roi_mask)
    cfg = d2.MeshDICConfig(max_iters=60, tol=1e-4, reg_strength=0.1)
    dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(), cfg)
    dic.prepare(ref, a)
    r1 = dic.run(dfm)
    r2 = dic.run(dfm)
    assert np.array_equal(np.asarray(r1.u_nodal), np.asarray(r2.u_nodal))
    assert np.array_equal(np.asarray(r1.history), np.asarray(r2.history), equal_nan=True)


def test_zncc_reference_known_answer(cuda):
    """tests/test_solver_translation_zncc.py:8-33 of the reference, on the GPU kernel."""
    from d2ic_gb300.solver_translation_zncc import _match_centers
    rng = np.random.default_rng(0)
    ref = rng.normal(size=(64, 64)).astype(np.float32)
    dx, dy = 3, 2
    deformed = np.zeros_like(ref)
    deformed[dy:, dx:] = ref[:-dy, :-dx]
    centers = np.array([[32.0, 32.0], [40.0, 24.0], [24.0, 40.0]], dtype=np.float32)
    u, s = _match_centers(centers, ref, deformed, win=9, search=6)
    assert u.shape == (3, 2) and s.shape == (3,)
    assert np.isfinite(s).all()
    assert np.allclose(u, np.array([dx, dy], dtype=np.float32), atol=0.5)


@pytest.mark.parametrize("win,search,n", [(17, 8, 300), (41, 24, 40), (13, 5, 200)])
def test_zncc_matches_oracle_on_speckle(cuda, win, search, n):
    """The bench's window (17, search 8), the reference's default (41, 24: 2,401 offsets, more
    than one block's threads) and a small one."""
    from d2ic_gb300.solver_translation_zncc import _match_centers
    from d2ic_gb300.synthetic import Translation, speckle_sequence
    from oracle.init_motion import match_centers
    ref, fr = speckle_sequence(256, 256, [Translation(4.3, -2.6)], seed=7, noise_seeds=[7, 8])
    rng = np.random.default_rng(1)
    centers = rng.uniform(0, 256, (n, 2)).astype(np.float32)
    u, s = _match_centers(centers, ref, fr[0], win=win, search=search)
    ur, sr = match_centers(centers, ref, fr[0], win, search)
    assert np.isfinite(sr).sum() >= n // 4
    ok = np.isfinite(sr)
    assert np.array_equal(np.isfinite(s), ok)
    assert np.array_equal(u[ok], ur[ok])             # integer shifts: exact
    assert np.abs(s[ok] - sr[ok]).max() <= 1e-4      # FP32 scores


def test_idw_matches_oracle(cuda):
    from d2ic_gb300.dic_init_motion import project_centers_to_nodes_idw_device
    from oracle.init_motion import project_centers_to_nodes_idw
    rng = np.random.default_rng(2)
    nodes = np.stack(np.meshgrid(np.arange(0, 400, 16.0), np.arange(0, 300, 16.0)), -1).reshape(-1, 2)
    centers = nodes[:200] + 8.0
    centers[5] = nodes[7]                       # exact match path
    disp = rng.normal(0, 2, (200, 2))
    disp[3] = np.nan                            # dropped centre
    out = project_centers_to_nodes_idw_device(nodes, centers, disp).cpu().numpy()
    ref = project_centers_to_nodes_idw(nodes, centers, disp)
    assert np.abs(out - ref).max() <= 1e-5


@pytest.mark.parametrize("nx,ny", [(52, 35), (176, 168)])
def test_idw_many_centres_matches_oracle(cuda, nx, ny):
    """Several 256-centre tiles (lanes split each tile), two exact centres for one node (the first in
    centre order wins), dropped NaN centres in several tiles, and node counts that are not multiples
    of a block's nodes; 176 x 168 nodes take the four-nodes-per-warp kernel."""
    from d2ic_gb300.dic_init_motion import project_centers_to_nodes_idw_device
    from oracle.init_motion import project_centers_to_nodes_idw
    rng = np.random.default_rng(5)
    nodes = np.stack(np.meshgrid(np.arange(nx) * 12.0, np.arange(ny) * 12.0), -1).reshape(-1, 2)[:-3]
    hi = 12 * max(nx, ny)
    centers = rng.integers(0, hi * 8, (1100, 2)) / 8.0      # exact in float32, as pixel-grid centres are
    disp = rng.normal(0, 2, (1100, 2))
    centers[700] = nodes[40]
    centers[900] = nodes[40]
    centers[300] = nodes[41]
    disp[[10, 333, 1000]] = np.nan
    out = project_centers_to_nodes_idw_device(nodes, centers, disp).cpu().numpy()
    ref = project_centers_to_nodes_idw(nodes, centers, disp)
    assert np.array_equal(out[40], disp[700].astype(np.float32))
    assert np.array_equal(out[41], disp[300].astype(np.float32))
    assert np.abs(out - ref).max() <= 1e-5


def test_strain_matches_oracle(cuda):
    import d2ic_gb300 as d2
    from oracle.mesh import node_neighbor_tables
    from oracle.strain import green_lagrange_nodes_lsq, to_voigt
    mesh, _ = d2.mask_to_mesh_assets(np.ones((200, 240), bool), 16)
    X = np.asarray(mesh.nodes_xy)
    rng = np.random.default_rng(9)
    u = 0.01 * X[:, [0]] * np.array([1.0, -0.3]) + 0.002 * X[:, [1]] + rng.normal(0, 0.01, X.shape)
    idx, deg = node_neighbor_tables(X, np.asarray(mesh.elements))
    for L in (0.0, 40.0):
        F, E = d2.compute_green_lagrange_strain_nodes_lsq(u.astype(np.float32), X, idx, deg, gauge_length=L)
        Fr, Er = green_lagrange_nodes_lsq(u, X, idx, deg, gauge_length=L)
        assert np.abs(d2.green_lagrange_to_voigt(E) - to_voigt(Er)).max() <= 1e-5
        assert np.abs(F - Fr).max() <= 1e-5
