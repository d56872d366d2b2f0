"""Device-resident sequence solve: every frame of a sequence without a host round trip.

The reference's frame loop (d2ic/batch_mesh_based.py:140-225) calls
``DICMeshBased.run`` per frame and forces a device->host sync per frame
(``int(n_iters)``, d2ic/solver_global_cg.py:197).  Here a whole sequence is
issued at once on one CUDA stream:

* host frames (ideally pinned torch tensors) are copied on a separate copy
  stream into a double buffer, overlapping the previous frame's solve;
* per frame: B-spline prefilter -> persistent CG launch -> strain kernel;
* the warm start of frame k+1 is formed on the device from frames k and k-1
  (previous-displacement or constant-velocity propagation);
* frame 0 can be initialised by ZNCC at element centres + IDW (both kernels).

Results stay on the device until the caller asks for them.  Per-frame results
are bitwise identical to solving the frames one by one through
``GlobalCGSolver.solve`` with the same warm starts.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from .dic_init_motion import project_centers_to_nodes_idw_device
from .solver_translation_zncc import match_centers_device
from .strain import strain_device


@dataclass
class SequenceResult:
    u: torch.Tensor          # (F, Nn, 2)
    strain: torch.Tensor     # (F, Nn, 3)
    hist: torch.Tensor       # (F, max_iter, 3)
    info: torch.Tensor       # (F, 3): n_iters, status, n_evals
    u_init: torch.Tensor     # (Nn, 2) initial guess of frame 0
    engine_events: list      # [(start, end)] CUDA events per CG launch (when timed)


class SequenceRunner:
    def __init__(self, solver, state, strain_tables=None):
        """``solver``: a prepared GlobalCGSolver; ``state``: its MeshDICState (after prepare())."""
        self.solver = solver
        self.state = state
        self.slot = solver._ensure(state)
        self.layout = solver._layout
        self.dev = self.layout.device
        a = state.assets
        T = lambda x, dt: torch.as_tensor(np.ascontiguousarray(np.asarray(x)), dtype=dt, device=self.dev)
        self.nodes = T(state.nodes_xy_device if state.nodes_xy_device is not None else a.mesh.nodes_xy, torch.float32)
        if strain_tables is None and a.node_neighbor_index is not None:
            strain_tables = (a.node_neighbor_index, a.node_neighbor_degree)
        self.strain_tables = None
        if strain_tables is not None:
            self.strain_tables = (T(strain_tables[0], torch.int32), T(strain_tables[1], torch.int32))
        self.centers = np.asarray(a.element_centers_xy, dtype=np.float32)
        self.copy_stream = torch.cuda.Stream(device=self.dev)
        H, W = self.layout.H, self.layout.W
        self.bufs = [torch.empty((H, W), dtype=torch.float32, device=self.dev) for _ in range(2)]
        self.ev_copied = [torch.cuda.Event() for _ in range(2)]
        self.ev_free = [torch.cuda.Event() for _ in range(2)]

    def init_motion(self, frame0, init_cfg) -> torch.Tensor:
        """ZNCC at element centres + IDW onto nodes (DICInitMotion.run on the device)."""
        c = self.centers if init_cfg.max_centers is None else self.centers[: int(init_cfg.max_centers)]
        u_c, s = match_centers_device(c, self.layout.ref_image, frame0, init_cfg.win, init_cfg.search, self.dev)
        if init_cfg.score_min is not None:
            ok = s >= float(init_cfg.score_min)
            u_c = torch.where(ok[:, None], u_c, torch.zeros_like(u_c))
        return project_centers_to_nodes_idw_device(self.nodes, c, u_c, 2.0, self.dev)

    def run(self, images, u0=None, init_cfg=None, propagation: str = "previous", with_strain: bool = True,
            time_engine: bool = False) -> SequenceResult:
        L, S = self.layout, self.slot
        nF = len(images)
        Nn = L.n_nodes
        cfg = self.state.config
        u_all = torch.empty((nF, Nn, 2), dtype=torch.float32, device=self.dev)
        st_all = torch.zeros((nF, Nn, 3), dtype=torch.float32, device=self.dev)
        h_all = torch.empty((nF,) + tuple(S.hist.shape), dtype=torch.float32, device=self.dev)
        i_all = torch.empty((nF, 3), dtype=torch.int32, device=self.dev)
        compute = torch.cuda.current_stream(self.dev)
        events = []
        used = [False, False]
        u_first = None
        for k, img in enumerate(images):
            b = k % 2
            if isinstance(img, torch.Tensor) and img.is_cuda:
                cur = img.to(torch.float32)
            else:
                src = img if isinstance(img, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(img, np.float32))
                with torch.cuda.stream(self.copy_stream):
                    if used[b]:
                        self.copy_stream.wait_event(self.ev_free[b])
                    self.bufs[b].copy_(src, non_blocking=True)
                    self.ev_copied[b].record(self.copy_stream)
                compute.wait_event(self.ev_copied[b])
                cur = self.bufs[b]
                used[b] = True
            # warm start
            if k == 0:
                if init_cfg is not None:
                    u_first = self.init_motion(cur, init_cfg)
                elif u0 is not None:
                    u_first = torch.as_tensor(np.asarray(u0, np.float32) if not isinstance(u0, torch.Tensor) else u0,
                                              device=self.dev, dtype=torch.float32).reshape(Nn, 2)
                else:
                    u_first = torch.zeros((Nn, 2), dtype=torch.float32, device=self.dev)
                S.u0.copy_(u_first)
            elif propagation == "constant_velocity" and k >= 2:
                torch.sub(u_all[k - 1] * 2.0, u_all[k - 2], out=S.u0)
            elif propagation in ("previous", "constant_velocity"):
                S.u0.copy_(u_all[k - 1])
            else:
                S.u0.zero_()
            S.load_image(cur)
            if not (isinstance(img, torch.Tensor) and img.is_cuda):
                self.ev_free[b].record(compute)
            if time_engine:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(compute)
            self.solver._engine.solve(self.solver._desc_dev, 1, self.solver._kind, self.solver._grid_blocks)
            if time_engine:
                e1.record(compute)
                events.append((e0, e1))
            u_all[k].copy_(S.u_out)
            h_all[k].copy_(S.hist)
            i_all[k].copy_(S.info)
            if with_strain and self.strain_tables is not None:
                v, _ = strain_device(S.u_out, self.nodes, self.strain_tables[0], self.strain_tables[1],
                                     cfg.strain_gauge_length, cfg.strain_eps, self.dev)
                st_all[k].copy_(v)
        return SequenceResult(u_all, st_all, h_all, i_all, u_first, events)
