"""Mesh-based DIC pipeline (reference: d2ic/dic_mesh_based.py:30-155).

``prepare`` completes the assets (strain neighbour tables, pixel assets),
compiles and warms up the solver; ``run`` solves one frame, computes nodal
Green-Lagrange strain on the GPU from the device-resident solution, and
returns host arrays.
"""
from __future__ import annotations

from dataclasses import dataclass, replace
from typing import Optional

import numpy as np

from .dataclasses import DICDiagnostics, DICResult, MeshDICConfig
from .dic_base import DICBase
from .mesh_assets import Mesh, MeshAssets, build_node_neighbor_tables, make_mesh_assets
from .pixel_assets import build_pixel_assets
from .solver_base import SolverBase
from .strain import strain_device
from .types import Array


@dataclass
class MeshDICState:
    ref_image: Array
    nodes_xy_device: Array
    assets: MeshAssets
    config: MeshDICConfig
    u0_nodal: Array | None = None


class _PendingFrame:
    """A frame queued by ``DICMeshBased.run_begin``."""

    def __init__(self):
        self.handle = None
        self.u_device = None
        self.strain = None
        self.strain_state = None
        self.strain_error = None
        self.disc_state = None
        self.disc_map = None
        self.disc_pending = None
        self.event = None


class DICMeshBased(DICBase):
    def __init__(self, mesh: Mesh, solver: SolverBase, config: MeshDICConfig) -> None:
        self.mesh = mesh
        self.solver = solver
        self.config = config
        self._state: MeshDICState | None = None
        self._strain_dev = None
        self._strain_pinned = [None, None]   # per pending frame (two in flight at most)
        self._strain_flip = 0
        self._map_layout = None

    def prepare(self, ref_image: Array, assets: Optional[MeshAssets] = None) -> None:
        if assets is None:
            assets = make_mesh_assets(self.mesh, with_neighbors=True)
        elif assets.node_neighbor_index is None or assets.node_neighbor_degree is None:
            idx, deg = build_node_neighbor_tables(assets.mesh)
            assets = replace(assets, node_neighbor_index=idx, node_neighbor_degree=deg)
        if assets.pixel_data is None:
            pixel_data = build_pixel_assets(mesh=assets.mesh, ref_image=ref_image, binning=1.0,
                                            roi_mask=getattr(assets, "roi_mask", None))
            assets = replace(assets, pixel_data=pixel_data)
        ref = np.asarray(ref_image, dtype=np.float32) if not hasattr(ref_image, "device") else ref_image
        self._state = MeshDICState(ref_image=ref, nodes_xy_device=np.asarray(assets.mesh.nodes_xy, dtype=np.float32),
                                   assets=assets, config=self.config, u0_nodal=None)
        self._strain_dev = None
        self._map_layout = None
        self.solver.compile(assets)
        if hasattr(self.solver, "warmup"):
            self.solver.warmup(self._state)

    @property
    def state(self) -> MeshDICState | None:
        return self._state

    def set_initial_guess(self, u0_nodal: Array) -> None:
        if self._state is None:
            raise RuntimeError("Call prepare() before set_initial_guess().")
        self._state.u0_nodal = u0_nodal

    def _strain(self, u):
        import torch
        assets = self._state.assets
        if self._strain_dev is None:
            dev = u.device if isinstance(u, torch.Tensor) else torch.device("cuda")
            T = lambda a, dt: torch.as_tensor(np.ascontiguousarray(np.asarray(a)), dtype=dt, device=dev)
            self._strain_dev = (T(self._state.nodes_xy_device, torch.float32),
                                T(assets.node_neighbor_index, torch.int32),
                                T(assets.node_neighbor_degree, torch.int32))
        X, idx, deg = self._strain_dev
        voigt, _ = strain_device(u, X, idx, deg, self.config.strain_gauge_length, self.config.strain_eps)
        return voigt

    def run(self, def_image: Array) -> DICResult:
        return self.run_end(self.run_begin(def_image))

    def run_begin(self, def_image: Array):
        """Queue one frame on the current stream -- the solve, the strain, the discrepancy map if
        configured, and the copies of their results to pinned host memory -- without waiting, and
        return the pending frame for :meth:`run_end`.  A sequence driver can queue frame k + 1
        before it collects frame k, so the host work of a frame overlaps the next solve.  Solvers
        without a split solve (``solve_begin``) run synchronously here."""
        import torch
        if self._state is None:
            raise RuntimeError("DICMeshBased.prepare() must be called before run().")
        begin = getattr(self.solver, "solve_begin", None)
        if begin is None:
            return self._run_sync(def_image)
        assets = self._state.assets
        pend = _PendingFrame()
        pend.handle = begin(self._state, def_image)
        u_dev = pend.handle.u_device
        pend.u_device = u_dev
        if assets.node_neighbor_index is not None and assets.node_neighbor_degree is not None:
            try:
                sd = self._strain(u_dev)
                i = self._strain_flip
                self._strain_flip ^= 1
                if self._strain_pinned[i] is None or self._strain_pinned[i].shape != sd.shape:
                    self._strain_pinned[i] = torch.empty(sd.shape, dtype=sd.dtype).pin_memory()
                self._strain_pinned[i].copy_(sd, non_blocking=True)
                pend.strain = self._strain_pinned[i]
                pend.strain_state = "green_lagrange"
            except Exception as exc:   # recorded, not raised (reference behaviour)
                pend.strain_state = "failed_green_lagrange"
                pend.strain_error = str(exc)
        else:
            pend.strain_state = "skipped_no_neighbors"
        if bool(getattr(self.config, "compute_discrepancy_map", False)):
            if assets.pixel_data is None:
                pend.disc_state = "skipped_no_pixel_assets"
            else:
                pend.disc_map, pend.disc_pending = self._discrepancy(def_image, u_dev, wait=False)
                pend.disc_state = "discrepancy_ref"
        pend.event = torch.cuda.Event()
        pend.event.record()
        return pend

    def run_end(self, pend) -> DICResult:
        """Wait for a frame queued by :meth:`run_begin` and return its result."""
        if isinstance(pend, DICResult):
            return pend
        from .pixel_maps import discrepancy_rms
        pend.event.synchronize()
        sol = self.solver.solve_end(self._state, pend.handle, wait=False)
        u_nodal = sol.u_nodal
        info = {"stage": "mesh_based"}
        if getattr(sol, "n_iters", None) is not None:
            info["n_iters"] = int(sol.n_iters)
        if getattr(sol, "status", None) is not None:
            info["status"] = sol.status
        if getattr(sol, "history", None) is not None:
            info["history"] = "attached"
        info["strain"] = pend.strain_state
        if pend.strain is not None:
            strain = pend.strain.numpy().copy()
        else:
            strain = np.zeros((np.asarray(u_nodal).shape[0], 3), dtype=np.float32)
            if pend.strain_error is not None:
                info["strain_error"] = pend.strain_error
        pixel_maps = {}
        if pend.disc_state is not None:
            info["discrepancy"] = pend.disc_state
            if pend.disc_map is not None:
                pixel_maps["discrepancy_ref"] = pend.disc_map   # kept on the device, as the reference keeps it
                info["discrepancy_rms"] = discrepancy_rms(pend.disc_pending)
        return DICResult(u_nodal=u_nodal, strain=strain, diagnostics=DICDiagnostics(info=info),
                         history=getattr(sol, "history", None), pixel_maps=pixel_maps)

    def _run_sync(self, def_image: Array) -> DICResult:
        """One frame through a solver without a split solve."""
        assets = self._state.assets
        sol = self.solver.solve(self._state, def_image)
        u_nodal = sol.u_nodal
        info = {"stage": "mesh_based"}
        if getattr(sol, "n_iters", None) is not None:
            info["n_iters"] = int(sol.n_iters)
        if getattr(sol, "status", None) is not None:
            info["status"] = sol.status
        if getattr(sol, "history", None) is not None:
            info["history"] = "attached"
        if assets.node_neighbor_index is not None and assets.node_neighbor_degree is not None:
            try:
                u_src = getattr(sol, "u_device", None)
                strain = self._strain(u_src if u_src is not None else u_nodal).cpu().numpy()
                info["strain"] = "green_lagrange"
            except Exception as exc:   # recorded, not raised (reference behaviour)
                strain = np.zeros((np.asarray(u_nodal).shape[0], 3), dtype=np.float32)
                info["strain"] = "failed_green_lagrange"
                info["strain_error"] = str(exc)
        else:
            strain = np.zeros((np.asarray(u_nodal).shape[0], 3), dtype=np.float32)
            info["strain"] = "skipped_no_neighbors"
        pixel_maps = {}
        if bool(getattr(self.config, "compute_discrepancy_map", False)):
            if assets.pixel_data is None:
                info["discrepancy"] = "skipped_no_pixel_assets"
            else:
                u_src = getattr(sol, "u_device", None)
                dmap, rms = self._discrepancy(def_image, u_src if u_src is not None else u_nodal)
                pixel_maps["discrepancy_ref"] = dmap        # kept on the device, as the reference keeps it
                info["discrepancy"] = "discrepancy_ref"
                info["discrepancy_rms"] = rms
        return DICResult(u_nodal=u_nodal, strain=strain, diagnostics=DICDiagnostics(info=info),
                         history=getattr(sol, "history", None), pixel_maps=pixel_maps)

    def _discrepancy(self, def_image, u, wait: bool = True):
        """Discrepancy map through the solver's device layout (or one built for the maps):
        ``(map, rms)``, or ``(map, pending sums)`` with ``wait=False``."""
        from .engine import FrameSlot, descriptors_to_device
        from .pixel_maps import discrepancy_map_queue, discrepancy_map_ref
        layout = getattr(self.solver, "_layout", None)
        desc = getattr(self.solver, "_desc_dev", None)
        if layout is None or desc is None:
            if self._map_layout is None:
                from .engine import FrameLayout
                n_nodes = int(np.asarray(self._state.assets.mesh.nodes_xy).shape[0])
                lay = FrameLayout(self._state.assets.pixel_data, n_nodes, self._state.ref_image, "linear")
                self._map_layout = (lay, descriptors_to_device([FrameSlot(lay, 1).desc], lay.device))
            layout, desc = self._map_layout
        if not wait:
            return discrepancy_map_queue(layout, desc, def_image, u)
        return discrepancy_map_ref(layout, desc, def_image, u)
