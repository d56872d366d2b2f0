"""Coarse initial motion: ZNCC at element centres + IDW onto nodes (reference: d2ic/dic_init_motion.py:23-91)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import ptr
from .dataclasses import DICDiagnostics, DICResult, InitMotionConfig
from .dic_base import DICBase
from .mesh_assets import MeshAssets
from .solver_base import SolverBase
from .types import Array


@dataclass
class InitMotionState:
    ref_image: Array
    assets: MeshAssets


def project_centers_to_nodes_idw_device(nodes, centers, disp, power: float = 2.0, device=None):
    """IDW (power ``power``) of centre displacements onto nodes on the GPU; NaN centres dropped."""
    device = torch.device(device if device is not None else "cuda")
    T = lambda a: (a.to(device=device, dtype=torch.float32).contiguous() if isinstance(a, torch.Tensor)
                   else torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float32))).to(device))
    X = T(nodes).reshape(-1, 2)
    C = T(centers).reshape(-1, 2)
    D = T(disp).reshape(-1, 2)
    out = torch.empty_like(X)
    _lib.call("d2ic_idw_project", ptr(X), X.shape[0], ptr(C), ptr(D), C.shape[0], float(power), ptr(out),
              _lib.stream_handle())
    return out


def _project_centers_to_nodes_idw(assets: MeshAssets, centers_xy, disp_centers, power: float = 2.0):
    return project_centers_to_nodes_idw_device(assets.mesh.nodes_xy, centers_xy, disp_centers, power).cpu().numpy()


class DICInitMotion(DICBase):
    def __init__(self, config: InitMotionConfig, solver: SolverBase) -> None:
        self.config = config
        self.solver = solver
        self._state: InitMotionState | None = None

    def prepare(self, ref_image: Array, assets: MeshAssets) -> None:
        self._state = InitMotionState(ref_image=ref_image, assets=assets)
        self.solver.compile(assets)

    def run(self, def_image: Array) -> DICResult:
        if self._state is None:
            raise RuntimeError("DICInitMotion.prepare() must be called before run().")
        if hasattr(self.solver, "solve_device"):
            u_c, scores = self.solver.solve_device(self._state, def_image)
        else:
            sol = self.solver.solve(self._state, def_image)
            u_c, scores = sol.u_centers, torch.as_tensor(np.asarray(sol.scores))
        centers = np.asarray(self._state.assets.element_centers_xy, dtype=np.float32)[: u_c.shape[0]]
        u = project_centers_to_nodes_idw_device(self._state.assets.mesh.nodes_xy, centers, u_c).cpu().numpy()
        matches = int((~torch.isnan(torch.as_tensor(scores))).sum().item())
        diag = DICDiagnostics(info={"stage": "init_motion", "matches": matches, "note": "IDW projection"})
        return DICResult(u_nodal=u, strain=np.zeros_like(u), diagnostics=diag, history=None)
