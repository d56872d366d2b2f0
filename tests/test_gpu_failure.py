"""Failure detection without a GPU fault (GPU).

A node group whose chunk count can never be reached makes the engine's bounded wait (5 s) run out:
the warp that waits sets the launch's abort flag and D2IC_WAIT_TIMEOUT, every other wait of the
launch sees the flag and returns, copies in flight are drained, and the host reads the status.
Nothing faults, traps or spins unboundedly, and the context stays usable: with the table restored
the next solve equals the one before the failure.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_group_wait_times_out_and_the_context_survives(cuda):
    import d2ic_gb300 as d2
    from d2ic_gb300 import _lib
    from d2ic_gb300.synthetic import Translation, rect_mask, speckle_sequence
    H = 128
    ref, frames = speckle_sequence(H, H, [Translation(0.4, -0.3)], seed=61, noise_seeds=[61, 62])
    mesh, assets = d2.mask_to_mesh_assets(rect_mask(H, H, 112, 112), 16)
    from dataclasses import replace
    assets = replace(assets, pixel_data=d2.build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))
    dic = d2.DICMeshBased(mesh, d2.GlobalCGSolver(device=cuda), d2.MeshDICConfig(max_iters=50, tol=1e-4))
    dic.prepare(ref, assets)
    before = dic.run(frames[0])
    layout = dic.solver._layout
    saved = layout.group_need.clone()
    layout.group_need[0] += 1_000_000            # a count that the group's chunks never reach
    with pytest.raises(_lib.D2ICError) as err:
        dic.run(frames[0])
    assert err.value.code == _lib.WAIT_TIMEOUT
    layout.group_need.copy_(saved)
    after = dic.run(frames[0])
    assert after.diagnostics.info["n_iters"] == before.diagnostics.info["n_iters"]
    assert np.array_equal(np.asarray(after.u_nodal), np.asarray(before.u_nodal))
