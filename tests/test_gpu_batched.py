"""Batched and served solves against the plain single-frame path (GPU).

Every reduction in the engine is per frame and in a fixed order, so a frame's
result must be bitwise the same alone, in a batch of uneven frames, and when
it is admitted into a running server and advanced across several slices.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(H, elem, warp, seed, mask_frac=0.85):
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import rect_mask, speckle_sequence
    ref, frames = speckle_sequence(H, H, [warp], seed=seed, noise_seeds=[seed, seed + 1])
    side = int(H * mask_frac)
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, side, side), elem)
    pix = d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask)
    return ref, frames[0], mesh, assets, pix


@pytest.fixture(scope="module")
def uneven(cuda):
    from d2ic_gb300.synthetic import Affine, Translation
    return [
        _case(192, 12, Translation(0.4, -0.3), 21),
        _case(256, 16, Affine([[0.01, 0.002], [-0.001, -0.008]], [0.6, 0.2], [128, 128]), 22),
        _case(320, 24, Translation(-0.7, 0.5), 23),
    ]


def test_batch_alone_equals_mix(cuda, uneven):
    import d2ic_gb300 as d2
    from d2ic_gb300 import engine
    from d2ic_gb300.serving import solve_batch
    cfg = d2.MeshDICConfig(max_iters=80, tol=1e-4, reg_strength=0.1)
    items = []
    for ref, dfm, mesh, assets, pix in uneven:
        L = engine.FrameLayout(pix, mesh.nodes_xy.shape[0], ref, "cubic", cuda)
        items.append((L, dfm, None, cfg))
    alone = [solve_batch([it], cuda)[0] for it in items]
    mixed = solve_batch(items, cuda)
    for a, m in zip(alone, mixed):
        assert a[1] == m[1] and a[2] == m[2]
        assert np.array_equal(a[0], m[0])                      # bitwise
        assert np.array_equal(a[3], m[3], equal_nan=True)


def test_server_equals_plain_sequences(cuda):
    """Two sequences, three frames each, interleaved; frames cross several engine slices."""
    import d2ic_gb300 as d2
    from d2ic_gb300.serving import DICServer, Request, ServeConfig
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    seqs = {}
    for sid, (H, elem, seed) in enumerate([(192, 16, 31), (256, 12, 32)]):
        warps = [Translation(0.2 * (k + 1), -0.15 * (k + 1)) for k in range(3)]
        ref, frames = speckle_sequence(H, H, warps, seed=seed, noise_seeds=[seed, seed + 1, seed + 2, seed + 3])
        mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, H - 32, H - 32), elem)
        from dataclasses import replace
        assets = replace(assets, pixel_data=d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))
        seqs[sid] = (ref, frames, mesh, assets)
    cfg = d2.MeshDICConfig(max_iters=60, tol=1e-4, reg_strength=0.1)
    # plain: one DICMeshBased per sequence, frame by frame, warm start from the previous frame
    plain = {}
    for sid, (ref, frames, mesh, assets) in seqs.items():
        dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(), cfg)
        dic.prepare(ref, assets)
        u_prev, out = None, []
        for f in frames:
            if u_prev is not None:
                dic.set_initial_guess(u_prev)
            r = dic.run(f)
            out.append(r)
            u_prev = r.u_nodal
        plain[sid] = out
    # served: both sequences at once, slices of 7 rounds (short slices only)
    srv = DICServer(cuda, ServeConfig(max_slots=4, slice_rounds=7, light_load_frames=0))
    for sid, (ref, frames, mesh, assets) in seqs.items():
        srv.add_sequence(sid, ref, mesh, assets, cfg)
    for k in range(3):
        for sid, (ref, frames, mesh, assets) in seqs.items():
            srv.submit(Request(sid, k, frames[k]))
    done = srv.run_until_idle()
    assert len(done) == 6
    assert srv.slices > 3
    for r in done:
        p = plain[r.seq_id][r.frame_index]
        assert r.n_iters == p.diagnostics.info["n_iters"]
        assert np.array_equal(r.u, np.asarray(p.u_nodal))      # bitwise, alone vs in the mix
        assert np.abs(r.strain - np.asarray(p.strain)).max() <= 1e-6
    st = srv.stats()
    assert st["frames"] == 6 and st["latency_ms_p99"] >= st["latency_ms_p50"] > 0


def test_overlapped_sequence_equals_frame_by_frame(cuda):
    """BatchMeshBased queues frame k + 1 before collecting frame k when it can (built-in
    propagator, device warm starts); the frame-by-frame loop (a user propagator) must give
    bitwise the same displacements, strains and iteration counts."""
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    H = 192
    warps = [Translation(0.2 * k, -0.1 * k) for k in range(1, 6)]
    ref, frames = speckle_sequence(H, H, warps, seed=41, noise_seeds=list(range(41, 47)))
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, 160, 160), 16)
    from dataclasses import replace
    assets = replace(assets, pixel_data=d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))
    cfg = d2.MeshDICConfig(max_iters=150, tol=1e-3, reg_strength=0.1)

    class UserCV(d2.ConstantVelocityPropagator):      # a user type: the frame-by-frame loop
        pass

    out = {}
    for name, prop in (("overlapped", d2.ConstantVelocityPropagator()), ("frame_by_frame", UserCV())):
        dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(device=cuda), cfg)
        batch = d2.BatchMeshBased(ref, assets, dic, d2.BatchConfig(), propagator=prop)
        assert batch._can_pipeline() == (name == "overlapped")
        batch.before(frames)
        out[name] = batch.sequence(frames).results
    for a, b in zip(out["overlapped"], out["frame_by_frame"]):
        assert np.array_equal(np.asarray(a.u_nodal), np.asarray(b.u_nodal))
        assert np.array_equal(np.asarray(a.strain), np.asarray(b.strain))
        assert a.diagnostics.info["n_iters"] == b.diagnostics.info["n_iters"]


def _two_sequences():
    import d2ic_gb300 as d2
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    from dataclasses import replace
    seqs = {}
    for sid, (H, elem, seed) in enumerate([(192, 16, 51), (256, 12, 52)]):
        warps = [Translation(0.2 * (k + 1), -0.15 * (k + 1)) for k in range(3)]
        ref, frames = speckle_sequence(H, H, warps, seed=seed, noise_seeds=[seed, seed + 1, seed + 2, seed + 3])
        mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, H - 32, H - 32), elem)
        assets = replace(assets, pixel_data=d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))
        seqs[sid] = (ref, frames, mesh, assets)
    return seqs


def _served(cuda, seqs, cfg, scfg, offsets=None):
    from d2ic_gb300.serving import DICServer, Request
    srv = DICServer(cuda, scfg)
    for sid, (ref, frames, mesh, assets) in seqs.items():
        srv.add_sequence(sid, ref, mesh, assets, cfg)
    reqs = [Request(sid, k, seqs[sid][1][k]) for k in range(3) for sid in seqs]
    if offsets is None:
        for r in reqs:
            srv.submit(r)
        srv.run_until_idle()
    else:
        srv.run_stream(reqs, offsets)
    return srv, {(r.seq_id, r.frame_index): r for r in srv.completed}


def test_light_load_slices_equal_short_slices(cuda):
    """Under light load the server runs one long slice at a time that ends when a frame finishes
    (D2IC_STOP_ON_FINISH) or when the host raises the irq word for a new arrival
    (D2IC_STOP_ON_IRQ); the results must be bitwise those of fixed short slices."""
    import d2ic_gb300 as d2
    from d2ic_gb300.serving import ServeConfig
    seqs = _two_sequences()
    cfg = d2.MeshDICConfig(max_iters=60, tol=1e-4, reg_strength=0.1)
    _, short = _served(cuda, seqs, cfg, ServeConfig(max_slots=4, slice_rounds=5, light_load_frames=0))
    # staggered arrivals: frames arrive while others run, so the irq path is taken as well
    offs = [0.0, 0.001, 0.002, 0.004, 0.006, 0.008]
    srv, light = _served(cuda, seqs, cfg, ServeConfig(max_slots=4, slice_rounds=5, light_load_frames=4), offs)
    assert srv.long_slices >= 3
    assert set(light) == set(short)
    for key, r in short.items():
        q = light[key]
        assert q.n_iters == r.n_iters
        assert np.array_equal(q.u, r.u)
        assert np.array_equal(q.strain, r.strain)


@pytest.mark.parametrize("light", [0, 4])
def test_held_frames_equal_short_slices(cuda, light):
    """Size priority (ServeConfig.hold_pixels): the larger sequence's frames sit out slices while a
    smaller frame is in flight (D2IC_CMD_HOLD) and resume where they stopped; every result must be
    bitwise that of plain short slices, with fixed and with light-load (long) slices."""
    import d2ic_gb300 as d2
    from d2ic_gb300.serving import ServeConfig
    seqs = _two_sequences()                        # ROI 160^2 = 25,600 px and 224^2 = 50,176 px
    cfg = d2.MeshDICConfig(max_iters=60, tol=1e-4, reg_strength=0.1)
    _, short = _served(cuda, seqs, cfg, ServeConfig(max_slots=4, slice_rounds=5, light_load_frames=0))
    srv, held = _served(cuda, seqs, cfg, ServeConfig(max_slots=4, slice_rounds=5, light_load_frames=light,
                                                     hold_pixels=40_000, hold_max_slices=3))
    assert set(held) == set(short)
    for key, r in short.items():
        q = held[key]
        assert q.n_iters == r.n_iters
        assert np.array_equal(q.u, r.u)
        assert np.array_equal(q.strain, r.strain)


def test_slice_stops_when_a_frame_finishes(cuda, uneven):
    """d2ic_cg_slice_ex with D2IC_STOP_ON_FINISH ends after the first round in which a frame
    finishes: that frame's outputs are written, the others report RUNNING, and continuing in
    further slices gives bitwise the one-launch result."""
    import torch

    import d2ic_gb300 as d2
    from d2ic_gb300 import _lib, engine
    from d2ic_gb300.serving import solve_batch
    # different iteration caps, so that the frames finish in different rounds
    cfgs = [d2.MeshDICConfig(max_iters=m, tol=1e-4, reg_strength=0.1) for m in (30, 55, 80)]
    layouts = [engine.FrameLayout(pix, mesh.nodes_xy.shape[0], ref, "cubic", cuda)
               for ref, dfm, mesh, assets, pix in uneven]
    one = solve_batch([(L, c[1], None, cfg) for L, c, cfg in zip(layouts, uneven, cfgs)], cuda)
    slots = []
    for L, c, cfg in zip(layouts, uneven, cfgs):
        s = engine.FrameSlot(L, cfg.max_iters)
        s.set_params(cfg.tol, cfg.reg_strength)
        s.load_image(c[1])
        s.set_u0(None)
        slots.append(s)
    eng = engine.Engine(cuda, len(slots))
    desc = engine.descriptors_to_device([s.desc for s in slots], cuda)
    eng.commands(len(slots)).fill_(_lib.CMD_INIT)
    finished_per_slice = []
    for _ in range(10):
        eng.run_slice(desc, len(slots), _lib.INTERP_CUBIC, 1 << 20, stop_flags=_lib.STOP_ON_FINISH)
        torch.cuda.synchronize()
        st = [int(s.info[1]) for s in slots]
        finished_per_slice.append(sum(x != _lib.RUNNING for x in st))
        if all(x != _lib.RUNNING for x in st):
            break
        eng.commands(len(slots)).fill_(_lib.CMD_RUN)
    assert 1 <= finished_per_slice[0] < len(slots) and len(finished_per_slice) >= 2
    assert finished_per_slice[-1] == len(slots)
    for s, o in zip(slots, one):
        assert int(s.info[0]) == o[1]
        assert np.array_equal(s.u_out.cpu().numpy(), o[0])


def test_batch_beyond_the_shared_list_equals_alone(cuda):
    """More active frames than the engine keeps in shared memory (64): the rounds then look the
    active list up in HBM, and frames that finish in different rounds rebuild it while other
    warps still walk it.  Every frame must still be bitwise its solve alone."""
    import d2ic_gb300 as d2
    from d2ic_gb300 import engine
    from d2ic_gb300.serving import solve_batch
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    items = []
    for k, (H, elem) in enumerate([(96, 12), (112, 16), (128, 12), (96, 16)]):
        warps = [Translation(0.05 * j - 0.4, 0.3 - 0.03 * j) for j in range(21)]
        ref, frames = speckle_sequence(H, H, warps, seed=50 + k, noise_seeds=list(range(60, 82)))
        mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, H - 16, H - 16), elem)
        pix = d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask)
        L = engine.FrameLayout(pix, mesh.nodes_xy.shape[0], ref, "cubic", cuda)
        for j, img in enumerate(frames):
            # caps from 12 to 60 iterations: frames leave the list in many different rounds
            cfg = d2.MeshDICConfig(max_iters=12 + 2 * ((7 * j + 5 * k) % 25), tol=1e-5, reg_strength=0.1)
            items.append((L, img, None, cfg))
    assert len(items) == 84
    mixed = solve_batch(items, cuda)
    for it, m in zip(items, mixed):
        a = solve_batch([it], cuda)[0]
        assert a[1] == m[1] and a[2] == m[2]
        assert np.array_equal(a[0], m[0])                      # bitwise
        assert np.array_equal(a[3], m[3], equal_nan=True)
