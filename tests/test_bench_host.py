"""Host-side pieces of bench.py and of the serving stream's arrival process (no GPU)."""
from __future__ import annotations

import importlib.util
import os

import numpy as np


def _bench():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(root, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_fifo_latency_is_a_single_server_queue():
    b = _bench()
    arrivals = np.array([0.0, 0.5, 0.6, 3.0])
    service = np.array([1.0, 1.0, 1.0, 0.5])
    # frame 0: 0 -> 1; frame 1 waits to 1, ends 2; frame 2 waits to 2, ends 3; frame 3 starts at 3
    assert np.allclose(b._fifo_latency(arrivals, service), [1.0, 1.5, 2.4, 0.5])


def test_stream_offsets_are_seeded_poisson_arrivals():
    from d2ic_gb300.workloads import ServingStream
    st = ServingStream(sequences=[], order=[(0, k) for k in range(20000)], seed=4)
    a = st.offsets(50.0)
    assert a.shape == (20000,) and np.all(np.diff(a) > 0)
    assert abs(np.mean(np.diff(a)) - 1 / 50.0) < 0.02 / 50.0 * 10      # mean gap 1 / rate
    assert np.array_equal(a, st.offsets(50.0))                          # same seed, same arrivals
    assert not np.array_equal(a[:100], st.offsets(100.0)[:100] * 2.0)   # each rate its own draw
    assert st.offsets(50.0, 10).shape == (10,)
