"""Sequence runner (reference: d2ic/batch_base.py:9-52, d2ic/batch_mesh_based.py:25-282).

``run(images) = end(sequence(images))`` after ``before(images)``; per frame:
warm start (propagator, else the previous solution), optional chained local
refinement pipeline, optional per-frame ``.npz`` (``u_nodal``, ``strain``,
``discrepancy_ref``; writers in ``outputs.py``).
PNG export needs matplotlib, which this package does not use.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from dataclasses import dataclass
from pathlib import Path
from typing import Iterable, Optional, Sequence

import numpy as np

from .dataclasses import BatchConfig, BatchDiagnostics, BatchResult, DICResult
from .dic_mesh_based import DICMeshBased
from .mesh_assets import MeshAssets
from .outputs import save_frame_npz
from .propagators import ConstantVelocityPropagator, DisplacementPropagatorBase, PreviousDisplacementPropagator
from .types import Array


def _prefetched(images):
    """The frames as device tensors, each host->device copy queued on a copy stream one frame
    ahead, so that frame k+1 travels while frame k is solved (pinned host frames copy
    asynchronously; device frames pass through)."""
    import torch
    if not torch.cuda.is_available():
        yield from images
        return
    dev = torch.device("cuda", torch.cuda.current_device())
    copy = torch.cuda.Stream(device=dev)

    def start(img):
        if isinstance(img, torch.Tensor) and img.is_cuda:
            return img, None
        src = img if isinstance(img, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(img, dtype=np.float32))
        with torch.cuda.stream(copy):
            d = src.to(dev, dtype=torch.float32, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(copy)
        return d, ev

    def finish(pair):
        d, ev = pair
        if ev is not None:
            cur = torch.cuda.current_stream(dev)
            cur.wait_event(ev)
            d.record_stream(cur)
        return d

    it = iter(images)
    try:
        nxt = start(next(it))
    except StopIteration:
        return
    for img in it:
        cur_pair, nxt = nxt, start(img)
        yield finish(cur_pair)
    yield finish(nxt)


class BatchBase(ABC):
    def run(self, images: Sequence[Array]) -> BatchResult:
        self.before(images)
        result = self.sequence(images)
        return self.end(result)

    @abstractmethod
    def before(self, images: Sequence[Array]) -> None:
        raise NotImplementedError

    @abstractmethod
    def sequence(self, images: Sequence[Array]) -> BatchResult:
        raise NotImplementedError

    @abstractmethod
    def end(self, result: BatchResult) -> BatchResult:
        raise NotImplementedError


@dataclass
class BatchState:
    ref_image: Array
    assets: MeshAssets
    is_prepared: bool = False


class BatchMeshBased(BatchBase):
    def __init__(self, ref_image: Array, assets: MeshAssets, dic_mesh: DICMeshBased, batch_config: BatchConfig,
                 dic_local: Optional[DICMeshBased] = None,
                 propagator: Optional[DisplacementPropagatorBase] = None) -> None:
        self.ref_image = ref_image
        self.assets = assets
        self.dic_mesh = dic_mesh
        self.dic_local = dic_local
        self.config = batch_config
        self.propagator = propagator
        self._state = BatchState(ref_image=ref_image, assets=assets, is_prepared=False)

    def before(self, images) -> None:
        self.dic_mesh.prepare(self.ref_image, self.assets)
        if self.dic_local is not None:
            self.dic_local.prepare(self.ref_image, self.assets)
        self._state.is_prepared = True

    def sequence(self, images: Sequence[Array] | Iterable[Array], latencies: list | None = None) -> BatchResult:
        """Per-frame loop; ``latencies`` (optional list) receives each frame's wall time in seconds."""
        import time
        if not self._state.is_prepared:
            raise RuntimeError("BatchMeshBased.before() must be called before sequence().")
        if bool(getattr(self.config, "export_png", False)):
            raise ImportError("export_png needs matplotlib plotting, which is not part of this package")
        save = bool(self.config.save_per_frame)
        out_dir = None
        if save:
            out_dir = Path(self.config.per_frame_dir) if self.config.per_frame_dir else Path.cwd() / "_outputs" / "per_frame_fields"
            out_dir.mkdir(parents=True, exist_ok=True)
        verbose = bool(self.config.verbose)
        progress = bool(self.config.progress)
        try:
            n_frames = len(images)  # type: ignore[arg-type]
        except TypeError:
            n_frames = None
        per_frame: list[DICResult] = []
        if self._can_pipeline():
            self._sequence_pipelined(images, per_frame, latencies, save, out_dir, progress or verbose, n_frames)
            diag = BatchDiagnostics(info={"stage": "batch_mesh_based", "n_frames": len(per_frame),
                                          "warm_start_from_previous": self.config.warm_start_from_previous})
            return BatchResult(results=per_frame, diagnostics=diag)
        u_prev = None
        u_prevprev = None
        for k, Idef in enumerate(_prefetched(images)):
            t0 = time.perf_counter()
            if progress or verbose:
                print(f"[Batch] Frame {k + 1}{'' if n_frames is None else '/' + str(n_frames)}: start")
            if self.propagator is not None:
                u_warm = self.propagator.propagate(u_prev=u_prev, u_prevprev=u_prevprev)
            else:
                u_warm = u_prev if self.config.warm_start_from_previous else None
            if u_warm is not None:
                self.dic_mesh.set_initial_guess(np.array(u_warm, copy=True))
            res = self.dic_mesh.run(Idef)
            if self.dic_local is not None:
                self.dic_local.set_initial_guess(np.array(res.u_nodal, copy=True))
                res = self.dic_local.run(Idef)
            per_frame.append(res)
            if latencies is not None:
                latencies.append(time.perf_counter() - t0)
            if save:
                save_frame_npz(out_dir / f"frame_{k:04d}.npz", res)
            u_prevprev = u_prev
            u_prev = res.u_nodal
            if progress or verbose:
                print(f"[Batch] Frame {k + 1}{'' if n_frames is None else '/' + str(n_frames)}: done")
        diag = BatchDiagnostics(info={"stage": "batch_mesh_based", "n_frames": len(per_frame),
                                      "warm_start_from_previous": self.config.warm_start_from_previous})
        return BatchResult(results=per_frame, diagnostics=diag)

    def _can_pipeline(self) -> bool:
        """Frames can overlap (frame k + 1 queued before frame k is collected) when the CG driver
        splits its runs, no local refinement is chained, the propagator is one of the built-in
        rules (they work on device tensors) and a GPU is present."""
        import torch
        if self.dic_local is not None or not hasattr(self.dic_mesh, "run_begin"):
            return False
        if not hasattr(getattr(self.dic_mesh, "solver", None), "solve_begin"):
            return False
        if self.propagator is not None and type(self.propagator) not in (PreviousDisplacementPropagator,
                                                                         ConstantVelocityPropagator):
            return False
        return torch.cuda.is_available()

    def _sequence_pipelined(self, images, per_frame, latencies, save, out_dir, talk, n_frames):
        """The per-frame loop with frame k + 1 queued before frame k's results are collected, so
        the host work of a frame (copies out, result objects, files) overlaps the next solve.
        Warm starts use device copies of the previous solutions: the same values as the host
        path, so the results are identical."""
        import time
        u_prev = u_prevprev = None
        pending = None
        done = [0.0]   # when the previous frame's results were collected

        def collect(item):
            # a frame's latency runs from when its solve could start (queued, and the previous
            # frame done) to its results on the host: the service time, without the wait behind
            # the previous frame that queueing ahead adds
            k, pend, t0 = item
            res = self.dic_mesh.run_end(pend)
            now = time.perf_counter()
            per_frame.append(res)
            if latencies is not None:
                latencies.append(now - max(t0, done[0]))
            done[0] = now
            if save:
                save_frame_npz(out_dir / f"frame_{k:04d}.npz", res)
            if talk:
                print(f"[Batch] Frame {k + 1}{'' if n_frames is None else '/' + str(n_frames)}: done")

        for k, Idef in enumerate(_prefetched(images)):
            t0 = time.perf_counter()
            if talk:
                print(f"[Batch] Frame {k + 1}{'' if n_frames is None else '/' + str(n_frames)}: start")
            if self.propagator is not None:
                u_warm = self.propagator.propagate(u_prev=u_prev, u_prevprev=u_prevprev)
            else:
                u_warm = u_prev if self.config.warm_start_from_previous else None
            if u_warm is not None:
                self.dic_mesh.set_initial_guess(u_warm)
            pend = self.dic_mesh.run_begin(Idef)
            u_prevprev, u_prev = u_prev, pend.u_device.clone()   # queued after the solve
            if pending is not None:
                collect(pending)
            pending = (k, pend, t0)
        if pending is not None:
            collect(pending)

    def end(self, result: BatchResult) -> BatchResult:
        return BatchResult(results=result.results,
                           diagnostics=BatchDiagnostics(info={**result.diagnostics.info, "post": "end() placeholder"}))
