"""Pins of the FP64 oracle (CPU, no GPU).

The reference's own known-answer tests are restated here against the oracle
(the reference itself cannot run without jax): pixel -> element on a unit
quad (tests/test_pixel_assets.py:6-36), ZNCC integer shift on seeded noise
(tests/test_solver_translation_zncc.py:8-33), Green-Lagrange strain of a 1%
stretch (tests/test_strain_smoke.py:10-40), island removal
(tests/test_mask2mesh_smoke.py:8-25).  The cubic sampler is pinned against
scipy.ndimage.map_coordinates and the analytic gradient against central
finite differences.
"""
from __future__ import annotations

import numpy as np
import pytest
from scipy import ndimage

from oracle import cubic, init_motion, mesh, objective, pixels, strain


def test_pixel_to_element_unit_quad():
    """tests/test_pixel_assets.py:6-36 of the reference."""
    nodes = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    elements = np.array([[0, 1, 2, 3]], dtype=np.int32)
    pc = np.array([[0.5, 0.5], [0.1, 0.9], [1.5, 1.5]])
    for f in (pixels.pixel_to_element_bruteforce, pixels.pixel_to_element_hashed):
        elts, pn = f(pc, nodes, elements)
        assert elts.tolist() == [0, 0, -1]
        assert pn.shape == (3, 4)
        assert pn[0].tolist() == [0, 1, 2, 3]
        assert pn[2].tolist() == [0, 0, 0, 0]


def test_zncc_integer_shift_on_noise():
    """tests/test_solver_translation_zncc.py:8-33 of the reference."""
    rng = np.random.default_rng(0)
    ref = rng.normal(size=(64, 64)).astype(np.float32)
    dx, dy = 3, 2
    deformed = np.zeros_like(ref)
    deformed[dy:, dx:] = ref[:-dy, :-dx]
    centers = np.array([[32.0, 32.0], [40.0, 24.0], [24.0, 40.0]], dtype=np.float32)
    u, scores = init_motion.match_centers(centers, ref, deformed, win=9, search=6)
    assert u.shape == (3, 2) and scores.shape == (3,)
    assert np.isfinite(scores).all()
    assert np.allclose(u, [dx, dy], atol=0.5)


def test_green_lagrange_uniform_extension():
    """tests/test_strain_smoke.py:10-40 of the reference."""
    nodes = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0]])
    elements = np.array([[0, 1, 3, 2]], dtype=np.int32)
    idx, deg = mesh.node_neighbor_tables(nodes, elements)
    eps = 0.01
    u = np.stack([nodes[:, 0] * eps, np.zeros(4)], axis=1)
    _, E = strain.green_lagrange_nodes_lsq(u, nodes, idx, deg)
    v = strain.to_voigt(E)
    np.testing.assert_allclose(v[:, 0], eps + 0.5 * eps ** 2, atol=5e-4)
    np.testing.assert_allclose(v[:, 1], 0.0, atol=5e-4)
    np.testing.assert_allclose(v[:, 2], 0.0, atol=5e-4)


def test_mask_to_mesh_filters_small_islands():
    """tests/test_mask2mesh_smoke.py:8-25 of the reference (oracle and product mesher)."""
    import d2ic_gb300 as d2
    m = np.zeros((64, 64), dtype=bool)
    m[8:48, 10:50] = True
    m[2, 2] = True
    nodes, elements = mesh.mask_to_mesh(m, 8, remove_islands=True, min_island_area_px=10)
    prod = d2.mask_to_mesh(m, element_size_px=8, binning=1, remove_islands=True, min_island_area_px=10)
    assert np.array_equal(nodes, prod.nodes_xy) and np.array_equal(elements, prod.elements)
    assert nodes.shape[1] == 2 and nodes.shape[0] > 0 and elements.shape[1] == 4 and elements.shape[0] > 0
    centers = nodes[elements].mean(axis=1).astype(int)
    assert not np.any((centers[:, 0] == 2) & (centers[:, 1] == 2))


def test_island_removal_label_equals_flood_fill():
    rng = np.random.default_rng(5)
    for _ in range(5):
        m = rng.random((40, 50)) < 0.45
        for a in (1, 3, 10):
            assert np.array_equal(mesh.remove_small_components(m, a), mesh.remove_small_components_floodfill(m, a))


@pytest.mark.parametrize("H,W,h,w,elem,nn,ne", [(512, 512, 448, 448, 16, 1089, 784)])
def test_benchmark_mesh_sizes(H, W, h, w, elem, nn, ne):
    from d2ic_gb300.synthetic import rect_mask
    a = mesh.mask_to_mesh_assets(rect_mask(H, W, h, w), elem)
    assert a["nodes"].shape[0] == nn and a["elements"].shape[0] == ne


def test_plate_hole_mesh_sizes():
    from d2ic_gb300.synthetic import plate_hole_mask
    a = mesh.mask_to_mesh_assets(plate_hole_mask(), 16)
    assert a["nodes"].shape[0] == 16641 and a["elements"].shape[0] == 11430


def test_cubic_matches_scipy_map_coordinates():
    rng = np.random.default_rng(0)
    img = rng.uniform(20, 230, (48, 61))
    c = cubic.bspline_coefficients(img)
    x = rng.uniform(-8, 68, 4000)
    y = rng.uniform(-8, 55, 4000)
    v = cubic.cubic_sample(c, cubic.ORACLE_PAD, x, y)
    s = ndimage.map_coordinates(img, [y, x], order=3, mode="nearest")
    assert np.abs(v - s).max() <= 1e-9 * np.abs(s).max()
    ii, jj = np.mgrid[0:48, 0:61]
    assert np.abs(cubic.cubic_sample(c, cubic.ORACLE_PAD, jj.ravel() * 1.0, ii.ravel() * 1.0) - img.ravel()).max() < 1e-10


def _small_problem(seed=0, H=96):
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    ref, fr = speckle_sequence(H, H, [Translation(0.3, -0.4)], seed=seed, noise_seeds=[seed, seed + 1])
    a = mesh.mask_to_mesh_assets(rect_mask(H, H, H - 16, H - 16), 16)
    pa = pixels.build_pixel_assets(a["nodes"], a["elements"], H, H, a["roi_mask"])
    return a, pa, objective.Problem.build(ref.astype(np.float64), fr[0].astype(np.float64), pa)


def test_analytic_gradient_matches_finite_differences():
    a, pa, pb = _small_problem()
    rng = np.random.default_rng(1)
    u = rng.normal(0, 0.3, a["nodes"].shape)
    J, g = objective.J_total_and_grad(u, pb, 0.1)
    used = np.unique(a["elements"])
    for n in rng.choice(used, 6, replace=False):
        for c in (0, 1):
            e = np.zeros_like(u)
            e[n, c] = 1e-5
            fd = (objective.J_total(u + e, pb, 0.1) - objective.J_total(u - e, pb, 0.1)) / 2e-5
            assert abs(fd - g[n, c]) <= 1e-6 * max(1.0, abs(g[n, c])) + 1e-8


def test_c_pixel_term_matches_numpy():
    from oracle import fast
    a, pa, pb = _small_problem(seed=3)
    rng = np.random.default_rng(2)
    u = rng.normal(0, 0.3, a["nodes"].shape)
    J1, g1 = objective.J_total_and_grad(u, pb, 0.1)
    J2, g2 = fast.FastProblem(pb, nthreads=2).value_and_grad(u, 0.1)
    assert abs(J1 - J2) <= 1e-12 * abs(J1)
    assert np.abs(g1 - g2).max() <= 1e-12 * np.abs(g1).max()


def test_c_pixel_term_f32_is_the_same_objective_in_float32():
    """The x32-equivalent timing variant computes the same objective to float32 accuracy."""
    from oracle import fast
    a, pa, pb = _small_problem(seed=3)
    rng = np.random.default_rng(2)
    u = rng.normal(0, 0.3, a["nodes"].shape)
    J1, g1 = fast.FastProblem(pb, nthreads=2).value_and_grad(u, 0.1)
    J2, g2 = fast.FastProblem(pb, nthreads=2, precision="f32").value_and_grad(u, 0.1)
    assert abs(J1 - J2) <= 1e-5 * abs(J1)
    assert np.abs(g1 - g2).max() <= 1e-4 * np.abs(g1).max()


def test_cg_control_flow_quirks():
    """Stop row keeps k; 10 failed halvings apply alpha = 2**-10 anyway (d2ic/solver_global_cg.py:374-459)."""
    calls = {"v": 0}

    def vg(u):
        return float(np.sum(u * u)), 2 * u

    def value_never_decreasing(u):          # Armijo always fails
        calls["v"] += 1
        return 1e9

    pb = None
    u, h, k, ne = objective.cg_solve(np.array([[1.0, 2.0]]), pb, 0.0, 3, 1e-12, value_and_grad=vg,
                                     value=value_never_decreasing)
    assert k == 3 and calls["v"] == 30
    assert np.allclose(h[:, 2], 2.0 ** -10) and np.all(h[:, 0] == 1e9)
    u, h, k, ne = objective.cg_solve(np.zeros((1, 2)), pb, 0.0, 5, 1e-3, value_and_grad=vg, value=lambda u: 0.0)
    assert k == 0 and h[0, 2] == 0.0 and np.isnan(h[1:]).all()


def test_oracle_local_gn_recovers_translation():
    """Local Gauss-Newton sweeps (d2ic/solver_local_gn.py:259-414) restated: a noiseless rigid
    translation is recovered and the residual RMS falls sweep after sweep."""
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    from oracle import local_gn, objective, pixels
    H = 96
    ref, fr = speckle_sequence(H, H, [Translation(0.3, -0.2)], seed=1, noise_seeds=[1, 2], noise_sigma=0.0)
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, 64, 64), 16)
    oa = pixels.build_pixel_assets(np.asarray(mesh.nodes_xy), np.asarray(mesh.elements), H, H, assets.roi_mask)
    pb = objective.Problem.build(ref, fr[0], oa)
    u, h = local_gn.local_sweeps(np.zeros((mesh.nodes_xy.shape[0], 2)), pb, 1e-3, 0.2, 0.1, 0.5, 20)
    used = np.unique(np.asarray(mesh.elements))
    assert np.abs(u[used] - [0.3, -0.2]).max() < 5e-3
    assert np.all(np.diff(h[:, 0]) < 0)                  # residual RMS decreases every sweep
