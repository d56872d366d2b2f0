"""Generate the golden vectors in tests/golden/ from the FP64 oracle.

    python tests/golden/make_golden.py

Case ``translation_128``: 128^2 seeded speckle (seed 0), uniform translation
(0.35, -0.62) px, centred 96^2 mask, 16 px elements, MeshDICConfig(200, 1e-3, 0.1):
mesh and pixel assets, cubic samples at 10^4 seeded points, J and its gradient
at zero and at a seeded random displacement, the first 5 CG iterates with
their history, the converged displacement and its Green-Lagrange strain.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def make_translation_128():
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    from oracle import cubic, fast, mesh, objective, pixels, strain
    H = W = 128
    ref, fr = speckle_sequence(H, W, [Translation(0.35, -0.62)], seed=0, noise_seeds=[0, 1])
    a = mesh.mask_to_mesh_assets(rect_mask(H, W, 96, 96), 16)
    pa = pixels.build_pixel_assets(a["nodes"], a["elements"], H, W, a["roi_mask"], bruteforce=True)
    pb = objective.Problem.build(ref.astype(np.float64), fr[0].astype(np.float64), pa)
    rng = np.random.default_rng(123)
    pts = np.stack([rng.uniform(-4, W + 3, 10000), rng.uniform(-4, H + 3, 10000)], axis=1).astype(np.float32)
    c2 = cubic.bspline_coefficients(fr[0].astype(np.float64))
    sv, sgx, sgy = cubic.cubic_sample(c2, cubic.ORACLE_PAD, pts[:, 0].astype(np.float64), pts[:, 1].astype(np.float64),
                                      with_grad=True)
    u_rand = rng.normal(0, 0.3, a["nodes"].shape)
    J0, g0 = objective.J_total_and_grad(np.zeros_like(a["nodes"]), pb, 0.1)
    J1, g1 = objective.J_total_and_grad(u_rand, pb, 0.1)
    fp = fast.FastProblem(pb, nthreads=1)
    u5, h5, k5, _ = fp.cg_solve(np.zeros_like(a["nodes"]), 0.1, 5, 1e-3)
    u, h, k, _ = fp.cg_solve(np.zeros_like(a["nodes"]), 0.1, 200, 1e-3)
    sidx, sdeg = mesh.node_neighbor_tables(a["nodes"], a["elements"])
    _, E = strain.green_lagrange_nodes_lsq(u, a["nodes"], sidx, sdeg)
    return dict(
        ref=ref, deformed=fr[0], roi_mask=a["roi_mask"], nodes=a["nodes"], elements=a["elements"],
        pixel_coords_ref=pa["pixel_coords_ref"], pixel_nodes=pa["pixel_nodes"], pixel_shapeN=pa["pixel_shapeN"],
        node_neighbor_index=pa["node_neighbor_index"], node_neighbor_weight=pa["node_neighbor_weight"],
        node_pixel_index=pa["node_pixel_index"], node_pixel_degree=pa["node_pixel_degree"],
        sample_points=pts, sample_val=sv, sample_gx=sgx, sample_gy=sgy,
        u_rand=u_rand, J0=J0, g0=g0, J1=J1, g1=g1,
        u_iter5=u5, hist_iter5=h5, u_conv=u, hist_conv=h, k_conv=k, strain_voigt=strain.to_voigt(E),
    )


if __name__ == "__main__":
    d = make_translation_128()
    out = os.path.join(HERE, "translation_128.npz")
    np.savez_compressed(out, **d)
    print(out, os.path.getsize(out), "bytes; k_conv =", d["k_conv"])
