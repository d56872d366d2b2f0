"""Device rendering of benchmark frames and the 8-bit frame path (GPU).

The serving stream's frames are rendered on the device (d2ic_render_speckle, a fixed summation
order per pixel in FP32) and delivered as 8-bit camera images; the coefficient preparation reads
8-bit pixels directly (d2ic_bspline_prefilter_u8 / d2ic_pad_image_u8).
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_device_render_matches_float64_render(cuda):
    """Raw speckle fields of an affine warp: device FP32 vs the FP64 torch renderer, within 1e-4
    of the field's range (FP32 sums of a few dozen dots)."""
    from d2ic_gb300.synthetic import Affine, DeviceSpeckle, make_dots, render_dots
    H, W = 160, 192
    dots = make_dots(H, W, 7)
    warp = Affine(np.array([[0.015, 0.004], [-0.006, -0.01]]), np.array([1.3, -0.8]), [W / 2, H / 2])
    sp = DeviceSpeckle(H, W, dots, cuda)
    for w in (None, warp):
        ref = render_dots(H, W, dots, w, "cpu").numpy()
        got = sp.raw(w).cpu().numpy().astype(np.float64)
        assert np.abs(got - ref).max() <= 1e-4 * (ref.max() - ref.min())


def test_speckle_finish_noise_and_quantisation(cuda):
    from d2ic_gb300.synthetic import DeviceSpeckle, make_dots
    H = W = 256
    sp = DeviceSpeckle(H, W, make_dots(H, W, 3), cuda)
    raw = sp.raw(None)
    lo, hi = (float(v) for v in torch.aminmax(raw))
    scale = 210.0 / (hi - lo)
    clean = sp.finish(raw, lo, scale, 0.0, 1, u8=False)
    noisy = sp.finish(raw, lo, scale, 2.0, 1, u8=False)
    again = sp.finish(raw, lo, scale, 2.0, 1, u8=False)
    other = sp.finish(raw, lo, scale, 2.0, 2, u8=False)
    assert torch.equal(noisy, again) and not torch.equal(noisy, other)       # seeded, deterministic
    n = (noisy - clean).double()
    assert abs(float(n.mean())) < 0.05 and abs(float(n.std()) - 2.0) < 0.05
    assert float(clean.min()) == pytest.approx(20.0, abs=1e-3) and float(clean.max()) == pytest.approx(230.0, abs=1e-3)
    q = sp.finish(raw, lo, scale, 0.5, 1, u8=True)
    assert q.dtype == torch.uint8
    assert float((q.double() - sp.finish(raw, lo, scale, 0.5, 1, u8=False).double()).abs().max()) <= 0.5 + 1e-4


@pytest.mark.parametrize("interpolation", ["cubic", "linear"])
def test_u8_frames_prepare_like_float_frames(cuda, interpolation):
    """The 8-bit path widens on the device: coefficients bitwise those of the same values in float32."""
    from d2ic_gb300 import engine
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (97, 131)).astype(np.uint8)
    kind = engine.interp_kind(interpolation)
    a = engine.prepare_coefficients(torch.from_numpy(img).to(cuda), kind)
    b = engine.prepare_coefficients(torch.from_numpy(img.astype(np.float32)).to(cuda), kind)
    w = img.shape[1] + 2 * engine.PAD                  # columns past the halo are row-pitch padding
    assert torch.equal(a[:, :w], b[:, :w])


def test_u8_frame_solves_like_float_frame(cuda):
    """A solve from an 8-bit pinned host frame equals the solve from the same frame as float32."""
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    H = 192
    ref, frames = speckle_sequence(H, H, [Translation(0.4, -0.3)], seed=61, noise_seeds=[61, 62])
    ref8 = np.clip(np.rint(ref), 0, 255).astype(np.uint8)
    f8 = np.clip(np.rint(frames[0]), 0, 255).astype(np.uint8)
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, 160, 160), 16)
    cfg = d2.MeshDICConfig(max_iters=100, tol=1e-3, reg_strength=0.1)
    out = []
    for img in (torch.from_numpy(f8).pin_memory(), f8.astype(np.float32)):
        dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(), cfg)
        dic.prepare(ref8, assets)
        out.append(dic.run(img))
    assert out[0].diagnostics.info["n_iters"] == out[1].diagnostics.info["n_iters"]
    assert np.array_equal(np.asarray(out[0].u_nodal), np.asarray(out[1].u_nodal))
