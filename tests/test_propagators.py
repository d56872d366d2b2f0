"""Warm-start propagators (d2ic/propagator_previous.py:15-20, d2ic/propagator_constant_velocity.py:23-32):
the extrapolation rule and its fallbacks, on numpy arrays and torch tensors."""
from __future__ import annotations

import numpy as np
import pytest


@pytest.mark.parametrize("as_torch", [False, True])
def test_constant_velocity_and_previous(as_torch):
    import torch

    import d2ic_gb300 as d2
    u1 = np.array([[1.0, -2.0], [0.5, 0.25]], dtype=np.float32)
    u2 = np.array([[0.5, -1.0], [1.5, 0.0]], dtype=np.float32)
    if as_torch:
        u1, u2 = torch.from_numpy(u1), torch.from_numpy(u2)
    cv = d2.ConstantVelocityPropagator()
    assert cv.propagate(None) is None and cv.propagate(None, u2) is None
    assert cv.propagate(u1) is u1                               # no second history frame: previous
    w = cv.propagate(u1, u2)
    assert np.array_equal(np.asarray(w), np.array([[1.5, -3.0], [-0.5, 0.5]], dtype=np.float32))
    prev = d2.PreviousDisplacementPropagator()
    assert prev.propagate(u1, u2) is u1 and prev.propagate(None) is None


def test_batch_uses_the_propagator_for_warm_starts():
    """BatchMeshBased asks the propagator for each frame's warm start with the two previous
    solutions (d2ic/batch_mesh_based.py:150-160); recorded here with a stand-in DIC."""
    import d2ic_gb300 as d2
    from d2ic_gb300.batch_mesh_based import BatchMeshBased
    from d2ic_gb300.dataclasses import BatchConfig, DICDiagnostics, DICResult

    class Rec(d2.DisplacementPropagatorBase):
        def __init__(self):
            self.calls = []

        def propagate(self, u_prev, u_prevprev=None):
            self.calls.append((None if u_prev is None else float(u_prev[0, 0]),
                               None if u_prevprev is None else float(u_prevprev[0, 0])))
            return None if u_prev is None else 2.0 * u_prev - (u_prev if u_prevprev is None else u_prevprev)

    class FakeDIC:
        def __init__(self):
            self.k, self.guesses = 0, []

        def prepare(self, ref, assets):
            pass

        def set_initial_guess(self, u):
            self.guesses.append(float(u[0, 0]))

        def run(self, img):
            self.k += 1
            return DICResult(u_nodal=np.full((3, 2), float(self.k), np.float32), strain=np.zeros((3, 3)),
                             diagnostics=DICDiagnostics(info={}))

    prop, dic = Rec(), FakeDIC()
    b = BatchMeshBased(np.zeros((4, 4), np.float32), None, dic, BatchConfig(), propagator=prop)
    frames = [np.zeros((4, 4), np.float32)] * 4
    b.before(frames)
    b.sequence(frames)
    assert prop.calls == [(None, None), (1.0, None), (2.0, 1.0), (3.0, 2.0)]
    assert dic.guesses == [1.0, 3.0, 4.0]                      # 2*1-1, 2*2-1, 2*3-2
