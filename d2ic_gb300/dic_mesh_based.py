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


class DICMeshBased(DICBase):
    def __init__(self, mesh: Mesh, solver: SolverBase, config: MeshDICConfig) -> None:
        self.mesh = mesh
        self.solver = solver
        self.config = config
        self._state: MeshDICState | None = None
        self._strain_dev = None
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
        if self._state is None:
            raise RuntimeError("DICMeshBased.prepare() must be called before run().")
        sol = self.solver.solve(self._state, def_image)
        u_nodal = sol.u_nodal
        assets = self._state.assets
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

    def _discrepancy(self, def_image, u):
        """Discrepancy map through the solver's device layout (or one built for the maps)."""
        from .engine import FrameSlot, descriptors_to_device
        from .pixel_maps import discrepancy_map_ref
        layout = getattr(self.solver, "_layout", None)
        desc = getattr(self.solver, "_desc_dev", None)
        if layout is None or desc is None:
            if self._map_layout is None:
                from .engine import FrameLayout
                n_nodes = int(np.asarray(self._state.assets.mesh.nodes_xy).shape[0])
                lay = FrameLayout(self._state.assets.pixel_data, n_nodes, self._state.ref_image, "linear")
                self._map_layout = (lay, descriptors_to_device([FrameSlot(lay, 1).desc], lay.device))
            layout, desc = self._map_layout
        return discrepancy_map_ref(layout, desc, def_image, u)
