"""bench.py's multi-rank plumbing on CPU: two gloo ranks, max-over-ranks timing and barriers.

The GPU path shards by replica (one independent sequence per rank, no data-path
collective); what needs checking without GPUs is the rendezvous, the MAX
reduction of the per-rank step time and the barrier around the timed region.
"""
from __future__ import annotations

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank: int, ws: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    w, r, _ = bench.dist_init()
    t = bench.max_over_ranks(0.5 + r, w)          # rank r "took" 0.5 + r seconds
    bench.barrier(w)
    # a rank that is not rank 0 runs no reference work and prints nothing
    done = bench.run_reference(None, w, r) if r != 0 else None
    q.put((r, w, t, done))
    dist.destroy_process_group()


def test_two_gloo_ranks_max_and_barrier():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[2] == pytest.approx(1.5) for o in out)   # both ranks report the slowest rank's time
    assert out[1][3] is None
