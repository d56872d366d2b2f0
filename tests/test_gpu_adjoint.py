"""Implicit adjoint of the converged solve (GPU) against the FP64 oracle.

Tolerances: JVP vs the oracle's implicit JVP at the same linearisation point
1e-3 relative (FP32 pixel arithmetic and matvec); vs central finite
differences (h = 1e-2 grey level) of the oracle's exactly converged solve
2e-3 relative; <VJP(w), dI> = <w, JVP(dI)> to 1e-4 relative.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem(cuda):
    from dataclasses import replace

    import d2ic_gb300 as d2
    from d2ic_gb300.adjoint import newton_polish
    from d2ic_gb300.synthetic import Affine, rect_mask, speckle_sequence
    from oracle import objective, pixels
    H = 128
    ref, fr = speckle_sequence(H, H, [Affine([[0.005, 0], [0, 0]], [0.3, -0.2], [64, 64])], seed=3, noise_seeds=[3, 4])
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, 112, 112), 12)
    assets = replace(assets, pixel_data=d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))
    cfg = d2.MeshDICConfig(max_iters=400, tol=1e-5, reg_strength=0.1)
    dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(), cfg)
    dic.prepare(ref, assets)
    res = dic.run(fr[0])
    img = torch.as_tensor(fr[0], device=cuda)
    u = newton_polish(dic.solver, dic.state, img, res.u_nodal, 0.1, steps=3)
    oa = pixels.build_pixel_assets(np.asarray(mesh.nodes_xy), np.asarray(mesh.elements), H, H, assets.roi_mask)
    pb = objective.Problem.build(ref.astype(np.float64), fr[0].astype(np.float64), oa)
    return dict(dic=dic, img=img, u=u, pb=pb, mesh=mesh, H=H)


def _adj(p):
    from d2ic_gb300.adjoint import ImplicitAdjoint
    slot = p["dic"].solver._ensure(p["dic"].state)
    slot.load_image(p["img"])
    return ImplicitAdjoint(slot, p["u"], 0.1, exact=True)


def test_newton_polish_reaches_the_minimiser(problem):
    from oracle import objective
    J, g = objective.J_total_and_grad(problem["u"].cpu().numpy().astype(np.float64), problem["pb"], 0.1)
    assert np.linalg.norm(g) < 1e-5          # FP32 floor of the objective's gradient (the CG tol was 1e-5)


def test_jvp_matches_oracle_and_finite_differences(problem):
    from oracle import adjoint as oadj
    adj = _adj(problem)
    rng = np.random.default_rng(0)
    dI = rng.normal(0, 2.0, (2, problem["H"], problem["H"]))
    du = adj.jvp(torch.as_tensor(dI, device=problem["u"].device)).cpu().numpy()
    u64 = problem["u"].cpu().numpy().astype(np.float64)
    for k in range(2):
        ref = oadj.implicit_jvp(u64, problem["pb"], 0.1, dI[k])
        rel = np.linalg.norm(du[k] - ref) / np.linalg.norm(ref)
        assert rel <= 1e-3, rel
    u_star = oadj.newton_solve(u64, problem["pb"], 0.1)
    fd = oadj.fd_jvp(u_star, problem["pb"], 0.1, dI[0], 1e-2)
    rel_fd = np.linalg.norm(du[0] - fd) / np.linalg.norm(fd)
    print(f"adjoint: jvp vs FD(h=1e-2) rel {rel_fd:.2e}, CG iters {adj.last_iters}")
    assert rel_fd <= 2e-3


def test_vjp_is_the_transpose_of_jvp(problem):
    adj = _adj(problem)
    g = torch.Generator(device="cpu").manual_seed(1)
    dI = torch.randn((1, problem["H"], problem["H"]), generator=g, dtype=torch.float64).to(problem["u"].device)
    w = torch.randn((1,) + tuple(problem["u"].shape), generator=g, dtype=torch.float64).to(problem["u"].device)
    lhs = float((adj.vjp(w, rtol=1e-9).to(torch.float64) * dI).sum())
    rhs = float((w * adj.jvp(dI, rtol=1e-9)).sum())
    assert abs(lhs - rhs) <= 1e-4 * max(abs(lhs), abs(rhs))


def test_autograd_function_backward_and_jvp(problem):
    from d2ic_gb300.adjoint import DifferentiableSolve
    p = problem
    ds = DifferentiableSolve(p["dic"].solver, p["dic"].state, u0=p["u"].cpu().numpy(), polish=2)
    img = p["img"].clone().requires_grad_(True)
    u = ds(img)
    w = torch.linspace(-1, 1, u.numel(), device=u.device).reshape(u.shape)
    (u * w).sum().backward()
    ref = ds.adj.vjp(w[None].to(torch.float64))[0]
    assert torch.allclose(img.grad.to(torch.float64), ref.to(torch.float64), rtol=1e-4, atol=1e-9)
    import torch.autograd.forward_ad as fwAD
    d = torch.ones_like(p["img"]) * 0.5
    fw = DifferentiableSolve(p["dic"].solver, p["dic"].state, u0=p["u"].cpu().numpy(), polish=2)
    with fwAD.dual_level():
        tangent = fwAD.unpack_dual(fw(fwAD.make_dual(p["img"], d))).tangent
    direct = ds.adj.jvp(d[None])[0]
    assert torch.allclose(tangent.to(torch.float64), direct.to(torch.float64), rtol=1e-3, atol=1e-7)


def test_strain_jvp_matches_finite_difference(problem):
    from d2ic_gb300.adjoint import strain_jvp
    from oracle import mesh as om, strain as ostrain
    X = np.asarray(problem["mesh"].nodes_xy)
    idx, deg = om.node_neighbor_tables(X, np.asarray(problem["mesh"].elements))
    u = problem["u"].cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(4)
    du = rng.normal(0, 0.01, u.shape)
    d = strain_jvp(u, torch.as_tensor(du[None], device=problem["u"].device), X, idx, deg, 8.0)[0].cpu().numpy()
    h = 1e-4
    Ep = ostrain.to_voigt(ostrain.green_lagrange_nodes_lsq(u + h * du, X, idx, deg, 8.0)[1])
    Em = ostrain.to_voigt(ostrain.green_lagrange_nodes_lsq(u - h * du, X, idx, deg, 8.0)[1])
    assert np.abs(d - (Ep - Em) / (2 * h)).max() <= 1e-8


@pytest.mark.parametrize("K", [1, 37, 256])
def test_assembled_operator_equals_chunk_matvec(problem, K):
    """The assembled node operator (d2ic_hessian_assemble / d2ic_hessian_apply) applies the same
    Hessian as the chunk-block product through node slots (d2ic_hessian_matvec), to FP32 rounding."""
    adj = _adj(problem)
    Nn = problem["u"].shape[0]
    g = torch.Generator(device=problem["u"].device).manual_seed(7)
    V = torch.randn((Nn, 2, K), generator=g, device=problem["u"].device, dtype=torch.float64)
    V[~adj.active] = 0.0
    a = adj.matvec(V)
    b = adj.matvec_chunks(V)
    scale = float(b.abs().max())
    assert float((a - b).abs().max()) <= 1e-5 * scale


def test_pcg_solves_with_four_column_tiles(problem):
    """K a multiple of 4 takes the vectorised product inside the PCG; each column's solution must
    equal the one-column solve (the same operations per column), and H X = B must hold."""
    adj = _adj(problem)
    Nn = problem["u"].shape[0]
    g = torch.Generator(device=problem["u"].device).manual_seed(9)
    B = torch.randn((Nn, 2, 8), generator=g, device=problem["u"].device, dtype=torch.float64)
    B[~adj.active] = 0.0
    X = adj.solve(B, rtol=1e-9)
    for k in (0, 5):
        Xk = adj.solve(B[:, :, k:k + 1].contiguous(), rtol=1e-9)
        assert float((X[:, :, k] - Xk[:, :, 0]).abs().max()) <= 1e-6 * float(X[:, :, k].abs().max())
    R = adj.matvec(X) - B
    assert float(R[adj.active].norm()) <= 1e-5 * float(B.norm())
