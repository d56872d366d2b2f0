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


def test_overlapped_loop_order_and_warm_starts():
    """The overlapped sequence loop (run on the host here with a stand-in DIC): frame k + 1 is
    queued before frame k is collected, the warm start of frame k + 1 is the constant-velocity
    extrapolation of the two previous solutions, and results come back in frame order."""
    import torch

    import d2ic_gb300 as d2
    from d2ic_gb300.batch_mesh_based import BatchMeshBased
    from d2ic_gb300.dataclasses import BatchConfig, DICDiagnostics, DICResult

    events = []

    class Pending:
        def __init__(self, k, u):
            self.k, self.u_device = k, u

    class FakeDIC:
        def __init__(self):
            self.k, self.guess = 0, None

        def prepare(self, ref, assets):
            pass

        def set_initial_guess(self, u):
            self.guess = u

        def run_begin(self, img):
            self.k += 1
            events.append(("begin", self.k, None if self.guess is None else float(self.guess[0, 0])))
            return Pending(self.k, torch.full((3, 2), float(self.k * self.k)))

        def run_end(self, p):
            events.append(("end", p.k))
            return DICResult(u_nodal=p.u_device.numpy().copy(), strain=np.zeros((3, 3)),
                             diagnostics=DICDiagnostics(info={"frame": p.k}))

    dic = FakeDIC()
    b = BatchMeshBased(np.zeros((4, 4), np.float32), None, dic, BatchConfig(),
                       propagator=d2.ConstantVelocityPropagator())
    per_frame, lat = [], []
    b._sequence_pipelined([np.zeros((4, 4), np.float32)] * 4, per_frame, lat, False, None, False, 4)
    # solutions k^2: warm starts none, 1 (previous only), 2*4-1 = 7, 2*9-4 = 14
    assert events == [("begin", 1, None), ("begin", 2, 1.0), ("end", 1), ("begin", 3, 7.0), ("end", 2),
                      ("begin", 4, 14.0), ("end", 3), ("end", 4)]
    assert [r.diagnostics.info["frame"] for r in per_frame] == [1, 2, 3, 4] and len(lat) == 4
