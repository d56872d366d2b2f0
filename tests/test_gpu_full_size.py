"""The full-size headline workload (2048^2 plate with a hole: 2.92 M ROI pixels, 16,641 nodes),
checked through properties that need no oracle run at this size:

* accuracy against the known displacement field of the synthetic frames, with the reference's
  validation threshold (mean nodal error < 0.1 px, tests/test_validation_imageserie_full.py:52);
* the CG history: the objective never increases over steps that pass the Armijo test, and each
  frame stops below the gradient tolerance;
* determinism: a second run of the sequence gives bitwise the same displacements.
"""
from __future__ import annotations

import numpy as np
import pytest


@pytest.mark.gpu
def test_plate_hole_2048_sequence_properties(cuda):
    import torch

    import d2ic_gb300 as d2
    from d2ic_gb300 import workloads
    wl = workloads.plate_hole_2048(n_frames=3, seed=1, device=cuda)
    assert wl.n_pix == 2923392 and wl.n_nodes == 16641
    # the workload's own cap (200 iterations) stops the stretch frames before the large-scale modes
    # have converged; the accuracy property is checked on converged solves
    cfg = d2.MeshDICConfig(max_iters=4000, tol=wl.config.tol, reg_strength=wl.config.reg_strength, save_history=True)
    dic = d2.DICMeshBased(wl.mesh, d2.GlobalCGSolver(device=cuda), cfg)
    init = d2.DICInitMotion(wl.init, d2.TranslationZNCCSolver(wl.init, device=cuda))
    init.prepare(wl.ref, wl.assets)
    batch = d2.BatchMeshBased(wl.ref, wl.assets, dic, d2.BatchConfig(warm_start_from_previous=True))
    batch.before(wl.frames)

    def run():
        dic.set_initial_guess(init.run(wl.frames[0]).u_nodal)
        return batch.sequence(wl.frames).results

    res = run()
    nodes = np.asarray(wl.mesh.nodes_xy, np.float64)
    used = np.unique(np.asarray(wl.mesh.elements))
    for k, r in enumerate(res):
        u_true = wl.fields[k].displacement(torch.as_tensor(nodes[used])).numpy()
        err = np.linalg.norm(np.asarray(r.u_nodal, np.float64)[used] - u_true, axis=1)
        assert err.mean() < 0.1, (k, err.mean())
        h = np.asarray(r.history)
        rows = h[~np.isnan(h[:, 0])]
        assert rows.shape[0] >= 1
        # J never increases over a step that passed the Armijo test (a forced 2^-10 step may)
        armijo = rows[1:, 2] > 1.5 * 2.0 ** -10
        rise = np.diff(rows[:, 0]) > 1e-6 * np.abs(rows[:-1, 0]) + 1e-12
        assert not np.any(rise & armijo), k
        n_it = int(r.diagnostics.info.get("n_iters", rows.shape[0]))
        assert n_it < cfg.max_iters and rows[-1, 1] < cfg.tol, (k, n_it)    # converged below tol
    again = run()
    for a, b in zip(res, again):
        assert np.array_equal(np.asarray(a.u_nodal), np.asarray(b.u_nodal))
