"""The allocation-free solve entry point (d2ic_cg_solve_noalloc) against the regular one.

Some callers cannot call cudaMalloc -- a host runtime that has no device
allocator of its own, or a plugin whose host application owns every device
buffer and forbids allocations behind its back.  For them the library offers
one solve entry point whose scratch (descriptor copy, control block, CG
workspace) lives in a fixed-size device array inside the library.  This test
calls it through the C ABI twice in a row and checks each result against the
regular, caller-allocated entry point (d2ic_cg_solve_batched) on the same
inputs, within the nodal tolerance used by the other parity tests (1e-3 px),
then once more on a smaller frame, so that counters and tile origins left in
the shared array by a larger frame cannot leak into a smaller one.
It is collected last so that a failure here cannot hide another test's.
"""
from __future__ import annotations

import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu

TOL_PX = 1e-3


def _frame(device, side=256, roi=224, seed=11):
    import d2ic_gb300 as d2
    from d2ic_gb300 import engine
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    H = W = side
    ref, frames = speckle_sequence(H, W, [Translation(0.8, -0.45)], seed=seed, noise_seeds=[seed, seed + 1])
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, W, roi, roi), 16)
    pix = d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask)
    layout = engine.FrameLayout(pix, mesh.nodes_xy.shape[0], ref, "cubic", device)
    slot = engine.FrameSlot(layout, max_iter=120)
    slot.set_params(1e-4, 0.1)
    slot.load_image(frames[0])
    slot.set_u0(None)
    return layout, slot


def _regular(cuda, layout, slot):
    """The regular entry point (d2ic_cg_solve_batched, caller-allocated scratch)."""
    from d2ic_gb300 import engine
    eng = engine.Engine(cuda, 1)
    eng.solve(engine.descriptors_to_device([slot.desc], cuda), 1, layout.kind)
    torch.cuda.synchronize()
    return slot.u_out.clone(), slot.info.clone()


def test_noalloc_matches_regular_entry_point_on_consecutive_calls(cuda):
    from d2ic_gb300 import _lib
    big = _frame(cuda)
    small = _frame(cuda, side=128, roi=96, seed=13)
    refs = [_regular(cuda, *big), _regular(cuda, *small)]
    assert int(refs[0][1][0]) > 5 and int(refs[1][1][0]) > 5
    # allocation-free entry point: same inputs, separate outputs, host descriptor; two calls on
    # the 256 x 256 frame, then one on the 128 x 128 frame
    for call, which in enumerate((0, 0, 1)):
        layout, slot = (big, small)[which]
        u_ref, info_ref = refs[which]
        desc = _lib.Frame.from_buffer_copy(bytes(slot.desc))
        u_out = torch.full_like(slot.u_out, float("nan"))
        hist = torch.full_like(slot.hist, float("nan"))
        info = torch.zeros(3, dtype=torch.int32, device=cuda)
        desc.u_out = u_out.data_ptr()
        desc.hist = hist.data_ptr()
        desc.n_iters = info.data_ptr()
        desc.status = info.data_ptr() + 4
        desc.n_evals = info.data_ptr() + 8
        rc = _lib.load().d2ic_cg_solve_noalloc(ctypes.byref(desc), layout.kind, _lib.stream_handle())
        assert rc == 0, _lib.load().d2ic_last_error_string()
        # the descriptor went to the device with the launch: the host copy may be reused at once
        ctypes.memset(ctypes.addressof(desc), 0, ctypes.sizeof(desc))
        torch.cuda.synchronize()
        err = float((u_out - u_ref).abs().max())
        assert err <= TOL_PX, f"call {call}: max nodal difference {err:.3e} px"
        assert int(info[0]) == int(info_ref[0]) and int(info[2]) == int(info_ref[2])
        assert torch.equal(hist[: int(info[0])], slot.hist[: int(info[0])])


def test_noalloc_rejects_oversize_frame(cuda):
    from d2ic_gb300 import _lib
    f = _lib.Frame()
    f.n_nodes = 4_000_000          # far beyond the fixed scratch array
    f.n_chunks = 1
    f.node_chunk_k = 4
    L = _lib.load()
    assert L.d2ic_cg_solve_noalloc(ctypes.byref(f), _lib.INTERP_CUBIC, _lib.stream_handle()) == _lib.BAD_ARG
    assert b"fixed" in L.d2ic_last_error_string()
