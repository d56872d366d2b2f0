"""Serving and batching form of the global CG solve.

The reference solves one frame per ``GlobalCGSolver.solve`` call with a host
sync per frame (d2ic/solver_global_cg.py:151-198) inside a per-sequence frame
loop (d2ic/batch_mesh_based.py:140-225).  Here many sequences of uneven image
and mesh sizes are served at once:

* each registered sequence keeps its resident state in HBM: the reference
  image's pixel layout (records, tables), strain tables and the warm start
  (the previous frame's solution);
* a request (sequence, frame image) is admitted into a free engine slot when
  the HBM budget allows: its image is copied in (pinned -> device), its
  B-spline coefficients are computed, and the slot is marked for admission;
* the engine runs in slices: one persistent cooperative launch advances every
  admitted frame by at most ``slice_rounds`` objective evaluations and keeps
  all CG state in HBM; frames that finish free their slot, new requests join
  at the next slice (continuous batching: work of requests that arrive while
  others are on the GPU overlaps on the device);
* the slice launch is captured once in a CUDA graph and replayed;
* host work overlaps the device: while slice k runs, the host harvests slice
  k-1 (status copied back asynchronously into pinned memory), queues the
  finished frames' strain kernels and result copies (pinned, completed by
  event polling), admits new requests and queues slice k+1 behind slice k;
* each sequence owns one device slot (coefficients, node buffers, workspace)
  reused by its frames, so admission allocates nothing;
* frames of one sequence are solved in order (frame k+1 starts from frame k's
  solution, as BatchMeshBased with warm_start_from_previous), so a frame's
  result is the same whether it is solved alone or in the mix: every reduction
  inside the engine is per frame and in a fixed order.

``solve_batch`` is the one-shot batched launch (all frames start together).
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field
from typing import Any

import numpy as np
import torch

from . import _lib
from ._lib import ptr
from .dataclasses import InitMotionConfig, MeshDICConfig
from .engine import PAD, Engine, FrameLayout, FrameSlot, as_device_image, descriptors_to_device, interp_kind
from .mesh_assets import build_node_neighbor_tables
from .strain import strain_device

DESC_BYTES = 0


def _desc_bytes() -> int:
    import ctypes
    return ctypes.sizeof(_lib.Frame)


@dataclass
class ServeConfig:
    """Serving knobs: engine slots, HBM budget for admitted frames, rounds per slice, graph replay."""
    max_slots: int = 64
    hbm_budget_bytes: int | None = None      # default: 80% of the free device memory at start
    slice_rounds: int = 16
    use_graphs: bool = True
    grid_blocks: int = 0
    autotune: bool = False                   # chunk size per sequence from the launch-shape autotuner
    # light load: with at most this many frames in flight and none waiting, one long slice runs at a
    # time and ends when a frame finishes or a new request can be admitted (0 turns this off)
    light_load_frames: int = 4
    # size priority: while a frame with fewer than hold_pixels ROI pixels is in flight, frames with
    # at least that many sit out slices (D2IC_CMD_HOLD; their state is kept, so results do not
    # change), for at most hold_max_slices slices in a row; the engine advances all admitted frames
    # by one evaluation per round, so this lets small frames finish at their own pace (0: off)
    hold_pixels: int = 0
    hold_max_slices: int = 8


@dataclass
class Request:
    seq_id: Any
    frame_index: int
    image: Any
    t_arrival: float = 0.0
    t_admit: float | None = None
    t_done: float | None = None
    u: np.ndarray | None = None
    strain: np.ndarray | None = None
    n_iters: int | None = None
    status: str | None = None

    @property
    def latency(self) -> float | None:
        return None if self.t_done is None else self.t_done - self.t_arrival


@dataclass
class _Sequence:
    seq_id: Any
    layout: FrameLayout
    config: MeshDICConfig
    nodes: torch.Tensor
    strain_idx: torch.Tensor | None
    strain_deg: torch.Tensor | None
    u_prev: torch.Tensor | None = None
    init: InitMotionConfig | None = None
    centers: np.ndarray | None = None
    in_flight: bool = False
    queue: collections.deque = field(default_factory=collections.deque)
    frames_done: int = 0
    slot: Any = None                     # the sequence's device slot, reused by its frames
    centers_dev: Any = None
    out_u: Any = None                    # pinned result buffers
    out_strain: Any = None


class DICServer:
    """Continuous-batching server of global-CG DIC frames on one GPU."""

    def __init__(self, device=None, config: ServeConfig | None = None, interpolation: str = "cubic"):
        self.device = torch.device(device if device is not None else "cuda")
        self.cfg = config or ServeConfig()
        self.kind = interp_kind(interpolation)
        self.interpolation = interpolation
        S = self.cfg.max_slots
        if not 1 <= S <= _lib.MAX_FRAMES:
            raise ValueError(f"max_slots must be in [1, {_lib.MAX_FRAMES}]")
        self.engine = Engine(self.device, S)
        self.cmd = self.engine.commands(S)
        self.cmd.fill_(_lib.CMD_IDLE)
        self.cmd_host = [_lib.CMD_IDLE] * S        # the host's copy of the command words
        self.held = [0] * S                          # consecutive slices a slot's frame was held
        nb = _desc_bytes()
        self.desc_dev = torch.zeros(S * nb, dtype=torch.uint8, device=self.device)
        self.slots: list[tuple[FrameSlot, Request, _Sequence] | None] = [None] * S
        self.status_dev = torch.zeros((S, 3), dtype=torch.int32, device=self.device)   # n_iters, status, n_evals
        self.status_host = [torch.zeros((S, 3), dtype=torch.int32).pin_memory() for _ in range(2)]
        self.status_event = [torch.cuda.Event(), torch.cuda.Event()]
        self.desc_host = torch.zeros(S * nb, dtype=torch.uint8).pin_memory()
        self.pending_slices: collections.deque = collections.deque()   # parities of slices not harvested
        self.parity = 0
        self.awaiting: list = []                                       # (request, sequence, event)
        self.seqs: dict[Any, _Sequence] = {}
        self.ready: collections.deque = collections.deque()     # sequences with queued frames, FIFO
        self.completed: list[Request] = []
        free, _ = torch.cuda.mem_get_info(self.device)
        self.budget = int(self.cfg.hbm_budget_bytes or 0.8 * free)
        self.bytes_in_use = 0
        self.copy_stream = torch.cuda.Stream(device=self.device)
        self.graphs: dict = {}                  # slice mode -> captured CUDA graph
        self.graph_failed = False
        self.slices = 0
        self.busy_time = 0.0
        # light-load slices: the host interrupts a running slice by writing the control block's irq word
        # from a side stream (the kernel reads it at each round end; every launch clears it)
        self.irq_stream = torch.cuda.Stream(device=self.device)
        self.irq_dev = self.engine.irq_word()
        self.irq_one = torch.ones(1, dtype=torch.int32).pin_memory()
        self.irq_sent = False
        self.long_running = False
        self.long_slices = 0

    @property
    def graph(self):
        """The short-slice graph (None until captured)."""
        return self.graphs.get("short")

    # -- sequences -----------------------------------------------------------------------------------
    def add_sequence(self, seq_id, ref_image, mesh, assets, config: MeshDICConfig,
                     init: InitMotionConfig | None = None, chunk_pixels: int | None = None):
        """Make a sequence resident: pixel layout of its reference image and mesh, strain tables.

        ``chunk_pixels``: pixels per engine chunk; by default the autotuner's choice for the
        sequence's frame signature when ``ServeConfig.autotune`` is set, else 256."""
        if seq_id in self.seqs:
            raise ValueError(f"sequence {seq_id!r} already registered")
        if assets.pixel_data is None:
            raise ValueError("assets must carry pixel_data (build_pixel_assets)")
        nn = int(np.asarray(mesh.nodes_xy).shape[0])
        if chunk_pixels is None:
            chunk_pixels = _lib.CHUNK_MAX
            if self.cfg.autotune:
                from .autotune import default_tuner
                ref = as_device_image(ref_image, self.device)
                chunk_pixels = default_tuner(self.device).tune(assets.pixel_data, nn, ref, torch.roll(ref, 1, dims=1),
                                                               self.interpolation).chunk_pixels
        layout = FrameLayout(assets.pixel_data, nn, ref_image, self.interpolation, self.device, chunk_max=chunk_pixels)
        T = lambda a, dt: torch.as_tensor(np.ascontiguousarray(np.asarray(a)), dtype=dt, device=self.device)
        idx, deg = assets.node_neighbor_index, assets.node_neighbor_degree
        if idx is None or deg is None:
            idx, deg = build_node_neighbor_tables(mesh)
        seq = _Sequence(seq_id, layout, config, T(mesh.nodes_xy, torch.float32), T(idx, torch.int32),
                        T(deg, torch.int32), init=init,
                        centers=np.asarray(assets.element_centers_xy, dtype=np.float32))
        self.seqs[seq_id] = seq
        self.bytes_in_use += self._layout_bytes(layout)
        return seq

    @staticmethod
    def _layout_bytes(L: FrameLayout) -> int:
        return int(L.pix.numel() * 4 + L.ref_image.numel() * 4 + L.chunk_begin.numel() * 4 * 4
                   + (L.nbr_index.numel() + L.nbr_weight.numel()) * 4)

    @staticmethod
    def _slot_bytes(L: FrameLayout, max_iter: int) -> int:
        coeff = (L.H + 2 * PAD) * L.cpitch * 4 * 2
        ws = _lib.load().d2ic_frame_workspace_bytes(L.n_nodes, L.n_chunks, L.node_chunk_k)
        return int(coeff + ws + L.n_nodes * 16 + max(max_iter, 1) * 12 + L.H * L.W * 4)

    # -- requests ------------------------------------------------------------------------------------
    def submit(self, req: Request):
        seq = self.seqs[req.seq_id]
        if not req.t_arrival:
            req.t_arrival = time.perf_counter()
        seq.queue.append(req)
        if not seq.in_flight and len(seq.queue) == 1:
            self.ready.append(seq)

    def reset_sequences(self):
        """Forget warm starts and completed requests (resident layouts are kept)."""
        if any(x is not None for x in self.slots) or self.pending_slices:
            raise RuntimeError("reset while frames are in flight")
        self._complete(wait=True)
        for s in self.seqs.values():
            s.u_prev = None
            s.queue.clear()
            s.in_flight = False
            s.frames_done = 0
        self.ready.clear()
        self.completed = []

    def run_stream(self, requests, offsets):
        """Online serving: request i arrives ``offsets[i]`` seconds after the call (sorted)."""
        t0 = time.perf_counter()
        i = 0
        n = len(requests)
        while i < n or self.pending() or self.pending_slices:
            now = time.perf_counter() - t0
            while i < n and offsets[i] <= now:
                requests[i].t_arrival = t0 + offsets[i]
                self.submit(requests[i])
                i += 1
            if self.pending() or self.pending_slices:
                self.step()
            elif i < n:
                time.sleep(max(0.0, offsets[i] - (time.perf_counter() - t0)))
        self._complete(wait=True)
        return self.completed

    def pending(self) -> int:
        return sum(len(s.queue) for s in self.seqs.values()) + sum(x is not None for x in self.slots)

    # -- scheduling ----------------------------------------------------------------------------------
    def _admit(self):
        free_slots = [i for i, x in enumerate(self.slots) if x is None]
        admitted = 0
        stream = torch.cuda.current_stream(self.device)
        nb = _desc_bytes()
        while free_slots and self.ready:
            seq = self.ready[0]
            L = seq.layout
            if seq.slot is None:                             # first frame: the sequence's resident slot
                need = self._slot_bytes(L, seq.config.max_iters)
                if self.bytes_in_use + need > self.budget:
                    break                                    # wait for memory to free up
                seq.slot = FrameSlot(L, seq.config.max_iters)
                seq.slot.set_params(seq.config.tol, seq.config.reg_strength)
                seq.out_u = torch.empty((L.n_nodes, 2), dtype=torch.float32).pin_memory()
                seq.out_strain = torch.empty((L.n_nodes, 3), dtype=torch.float32).pin_memory()
                if seq.centers is not None:
                    seq.centers_dev = torch.as_tensor(seq.centers, device=self.device).reshape(-1, 2).contiguous()
                self.bytes_in_use += need
            self.ready.popleft()
            req = seq.queue.popleft()
            i = free_slots.pop(0)
            slot = seq.slot
            # image: pinned host -> device on the copy stream, then coefficients on the compute stream
            # (8-bit camera frames cross the host link as bytes and are widened by the prefilter)
            if isinstance(req.image, torch.Tensor) and req.image.is_cuda:
                img = req.image if req.image.dtype == torch.uint8 else req.image.to(torch.float32)
            else:
                src = req.image if isinstance(req.image, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(
                    req.image if np.asarray(req.image).dtype == np.uint8 else np.asarray(req.image, np.float32)))
                if src.dtype != torch.uint8:
                    src = src.to(torch.float32)
                img = torch.empty((L.H, L.W), dtype=src.dtype, device=self.device)
                with torch.cuda.stream(self.copy_stream):
                    img.copy_(src, non_blocking=True)
                stream.wait_stream(self.copy_stream)
                img.record_stream(stream)
            slot.load_image(img)
            if seq.u_prev is not None:
                slot.u0.copy_(seq.u_prev)
            elif seq.init is not None:                      # first frame: ZNCC at centres + IDW, on the device
                from .dic_init_motion import project_centers_to_nodes_idw_device
                from .solver_translation_zncc import match_centers_device
                u_c, sc = match_centers_device(seq.centers_dev, L.ref_image, img, seq.init.win, seq.init.search,
                                               self.device)
                if seq.init.score_min is not None:
                    u_c = torch.where((sc >= float(seq.init.score_min))[:, None], u_c, torch.zeros_like(u_c))
                slot.u0.copy_(project_centers_to_nodes_idw_device(seq.nodes, seq.centers_dev, u_c, 2.0, self.device))
            else:
                slot.u0.zero_()
            # per-slot status words live in one array that is copied back after every slice
            slot.desc.n_iters = ptr(self.status_dev[i])
            slot.desc.status = ptr(self.status_dev[i]) + 4
            slot.desc.n_evals = ptr(self.status_dev[i]) + 8
            hb = self.desc_host[i * nb:(i + 1) * nb]
            hb.copy_(torch.frombuffer(bytearray(bytes(slot.desc)), dtype=torch.uint8))
            self.desc_dev[i * nb:(i + 1) * nb].copy_(hb, non_blocking=True)
            self.cmd[i] = _lib.CMD_INIT
            self.cmd_host[i] = _lib.CMD_INIT
            self.held[i] = 0
            self.status_dev[i, 1] = _lib.RUNNING
            self.slots[i] = (slot, req, seq, self.slices)    # first slice that sees the frame
            seq.in_flight = True
            req.t_admit = time.perf_counter()
            admitted += 1
        return admitted

    LONG_ROUNDS = 1 << 20

    def _launch_slice(self, mode: str = "short"):
        """Queue one slice: ``short`` = slice_rounds rounds; ``long`` = until a frame finishes or the
        host raises the irq word (light load)."""
        n = self.cfg.max_slots
        if mode == "long":
            rounds, flags = self.LONG_ROUNDS, _lib.STOP_ON_FINISH | _lib.STOP_ON_IRQ
        else:
            rounds, flags = self.cfg.slice_rounds, 0

        def launch():
            self.engine.run_slice(self.desc_dev, n, self.kind, rounds, self.cfg.grid_blocks, stop_flags=flags)

        if self.cfg.use_graphs and not self.graph_failed:
            g = self.graphs.get(mode)
            if g is None:
                try:
                    launch()                                 # this slice runs directly; later ones replay
                    if mode == "long":
                        return                               # captured at its next use, when no slice runs
                    torch.cuda.synchronize(self.device)
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g):
                        launch()
                    self.graphs[mode] = g
                except Exception:
                    self.graph_failed = True
                    self.graphs.clear()
                return
            g.replay()
        else:
            launch()

    def _capture_long(self):
        """Capture the long-slice graph while nothing runs (a capture launches nothing)."""
        if not self.cfg.use_graphs or self.graph_failed or "long" in self.graphs or self.slices == 0:
            return
        try:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self.engine.run_slice(self.desc_dev, self.cfg.max_slots, self.kind, self.LONG_ROUNDS,
                                      self.cfg.grid_blocks, stop_flags=_lib.STOP_ON_FINISH | _lib.STOP_ON_IRQ)
            self.graphs["long"] = g
        except Exception:
            self.graph_failed = True
            self.graphs.clear()

    def _admissible(self) -> bool:
        """A queued request could be admitted now (a free slot and a sequence with no frame in flight)."""
        return bool(self.ready) and any(x is None for x in self.slots)

    def _harvest(self, parity: int, slice_no: int):
        """Frames that finished by slice ``slice_no`` (status copy of parity ``parity``)."""
        self.status_event[parity].synchronize()
        status = self.status_host[parity]
        done = 0
        for i, entry in enumerate(self.slots):
            if entry is None or entry[3] > slice_no:        # admitted after that slice was queued
                continue
            n_iters, st, _ = (int(x) for x in status[i])
            if st == _lib.RUNNING:
                continue
            slot, req, seq, _ = entry
            u = slot.u_out
            voigt, _ = strain_device(u, seq.nodes, seq.strain_idx, seq.strain_deg, seq.config.strain_gauge_length,
                                     seq.config.strain_eps, self.device)
            if seq.u_prev is None:
                seq.u_prev = torch.empty_like(u)
            seq.u_prev.copy_(u)
            seq.out_u.copy_(u, non_blocking=True)
            seq.out_strain.copy_(voigt, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record()
            req.n_iters = n_iters
            req.status = _lib.STATUS_NAMES.get(st, str(st))
            self.awaiting.append((req, seq, ev))
            self.slots[i] = None
            self.cmd[i] = _lib.CMD_IDLE
            self.cmd_host[i] = _lib.CMD_IDLE
            seq.in_flight = False
            seq.frames_done += 1
            if seq.queue:
                self.ready.append(seq)
            done += 1
        return done

    def _complete(self, wait: bool = False):
        """Requests whose result copies have landed in pinned memory."""
        keep = []
        for req, seq, ev in self.awaiting:
            if wait or ev.query():
                ev.synchronize()
                req.u = seq.out_u.numpy().copy()
                req.strain = seq.out_strain.numpy().copy()
                req.t_done = time.perf_counter()
                self.completed.append(req)
            else:
                keep.append((req, seq, ev))
        self.awaiting = keep

    def _apply_holds(self):
        """Command words of the next slice under the size priority (ServeConfig.hold_pixels).  Only
        frames admitted in an earlier slice are touched: that slice consumed their CMD_INIT."""
        hp = self.cfg.hold_pixels
        if not hp:
            return
        occ = [(i, e) for i, e in enumerate(self.slots) if e is not None and e[3] < self.slices]
        small = any(e[0].layout.n_pix < hp for _, e in self.slots_in_flight())
        for i, e in occ:
            hold = small and e[0].layout.n_pix >= hp and self.held[i] < self.cfg.hold_max_slices
            want = _lib.CMD_HOLD if hold else _lib.CMD_RUN
            if self.cmd_host[i] != want:
                self.cmd[i] = want
                self.cmd_host[i] = want
            self.held[i] = self.held[i] + 1 if hold else 0

    def slots_in_flight(self):
        return [(i, e) for i, e in enumerate(self.slots) if e is not None]

    def _queue_slice(self, mode: str):
        self._apply_holds()
        self._launch_slice(mode)                    # the kernel turns CMD_INIT into CMD_RUN as it admits
        p = self.parity
        self.status_host[p].copy_(self.status_dev, non_blocking=True)
        self.status_event[p].record()
        self.pending_slices.append((p, self.slices))
        self.parity ^= 1
        self.slices += 1

    def _light(self) -> bool:
        n = sum(x is not None for x in self.slots)
        return 0 < n <= self.cfg.light_load_frames and not self._admissible()

    def step(self) -> int:
        """Admit what fits, queue one engine slice, harvest the previous one; returns frames finished.

        Under load, short slices are queued back to back and each is harvested while the next one
        runs.  Under light load one long slice runs at a time: it ends when a frame finishes (its
        result is harvested at once) or when the host raises the irq word because a new request can
        be admitted, so neither a finished frame nor a new arrival waits for a fixed slice length."""
        done = 0
        t0 = time.perf_counter()
        if self.long_running:
            if not self.status_event[self.pending_slices[0][0]].query():
                if not self.irq_sent and self._admissible():
                    with torch.cuda.stream(self.irq_stream):
                        self.irq_dev.copy_(self.irq_one, non_blocking=True)
                    self.irq_sent = True
                self._complete()
                self.busy_time += time.perf_counter() - t0
                return 0
            self.long_running = False
            done += self._harvest(*self.pending_slices.popleft())
        self._admit()
        light = self._light()
        if light and self.pending_slices:
            # switching to a long slice: let the queued short slices finish first (without blocking)
            while self.pending_slices and self.status_event[self.pending_slices[0][0]].query():
                done += self._harvest(*self.pending_slices.popleft())
            if self.pending_slices:
                self._complete()
                self.busy_time += time.perf_counter() - t0
                return done
            self._admit()
            light = self._light()
        if self._occupied():
            if light:
                self._capture_long()
                self._queue_slice("long")
                self.long_running = True
                self.long_slices += 1
                self.irq_sent = False
            else:
                self._queue_slice("short")
        # harvest the older slice while the newer one runs (at most one slice left unharvested, so
        # the two pinned status buffers never overlap); with no newer slice, harvest the last one
        while not self.long_running and (len(self.pending_slices) > 1 or (self.pending_slices and (
                not self._occupied() or self.status_event[self.pending_slices[0][0]].query()))):
            done += self._harvest(*self.pending_slices.popleft())
        self._complete()
        self.busy_time += time.perf_counter() - t0
        return done

    def _occupied(self) -> bool:
        return any(x is not None for x in self.slots)

    def run_until_idle(self):
        while self.pending() or self.pending_slices:
            self.step()
        self._complete(wait=True)
        return self.completed

    def stats(self) -> dict:
        lat = np.array([r.latency for r in self.completed if r.latency is not None])
        out = {"frames": len(self.completed), "slices": self.slices, "long_slices": self.long_slices,
               "graphs": sorted(self.graphs)}
        if lat.size:
            out.update(latency_ms_p50=1000 * float(np.percentile(lat, 50)),
                       latency_ms_p99=1000 * float(np.percentile(lat, 99)))
        return out


def solve_batch(frames, device=None, grid_blocks: int = 0):
    """One batched persistent launch over independent frames.

    ``frames``: list of ``(layout, def_image, u0, MeshDICConfig)``.  Returns a
    list of ``(u (Nn,2) numpy, n_iters, status, history numpy)``.
    """
    device = torch.device(device if device is not None else "cuda")
    slots = []
    for L, img, u0, cfg in frames:
        s = FrameSlot(L, cfg.max_iters)
        s.set_params(cfg.tol, cfg.reg_strength)
        s.load_image(img)
        s.set_u0(u0)
        slots.append(s)
    kinds = {s.layout.kind for s in slots}
    if len(kinds) != 1:
        raise ValueError("one batched launch uses one interpolation kind")
    eng = Engine(device, len(slots))
    desc = descriptors_to_device([s.desc for s in slots], device)
    eng.solve(desc, len(slots), kinds.pop(), grid_blocks)
    torch.cuda.synchronize(device)
    out = []
    for s in slots:
        info = s.info.cpu().tolist()
        out.append((s.u_out.cpu().numpy(), info[0], _lib.STATUS_NAMES.get(info[1], str(info[1])),
                    s.hist.cpu().numpy()))
    return out
