"""Local Gauss-Newton refinement solver on the GB300 kernels.

Drop-in for ``LocalGaussNewtonSolver`` (d2ic/solver_local_gn.py:34-202): same
constructor (``lam``, ``max_step``, ``omega``, ``interpolation``,
``use_map_coordinates``), ``compile(assets)`` / ``solve(state, def_image)``,
``LocalGNResult(u_nodal, strain, history)``; ``state.config.max_iters`` sweeps
of the relaxed nodal Jacobi update, ``state.config.reg_strength`` as the spring
weight, history rows ``[rms residual, rms step]`` when ``save_history``.
Each sweep is two CUDA kernels (``d2ic_local_gn_sweep``); the gradient images
and their sampling arrays are built on the device once per frame.  In the
reference pipeline it runs after the global CG (``BatchMeshBased(dic_local=...)``).
"""
from __future__ import annotations

import warnings
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import ptr
from .engine import FrameLayout, FrameSlot, as_device_image, descriptors_to_device, prepare_coefficients
from .solver_base import SolverBase
from .solver_global_cg import _normalize_interpolation
from .types import Array


@dataclass(frozen=True)
class LocalGNResult:
    u_nodal: Array
    strain: Array
    history: Array | None = None
    u_device: object = None


class LocalGaussNewtonSolver(SolverBase):
    """Local (nodal) Gauss-Newton sweeps for mesh DIC; expects ``MeshAssets.pixel_data``."""

    def __init__(self, lam: float = 1e-3, max_step: float = 0.2, omega: float = 0.5, interpolation: str = "cubic",
                 use_map_coordinates: bool | None = None, device=None) -> None:
        self._compiled = False
        self._lam = float(lam)
        self._max_step = float(max_step)
        self._omega = float(omega)
        if use_map_coordinates is not None:
            warnings.warn("use_map_coordinates is kept for backward compatibility; use interpolation='cubic' or "
                          "'linear'.", DeprecationWarning, stacklevel=2)
            interpolation = "cubic" if use_map_coordinates else "linear"
        self._interpolation = _normalize_interpolation(interpolation)
        self._device = torch.device(device if device is not None else "cuda")
        self._key = None

    def compile(self, assets) -> None:
        if getattr(assets, "pixel_data", None) is None:
            raise ValueError("MeshAssets must provide pixel_data for LocalGaussNewtonSolver.")
        _lib.load()
        self._compiled = True

    def _ensure(self, state):
        pix = state.assets.pixel_data
        key = (id(pix), id(state.ref_image))
        if self._key == key:
            return
        dev = self._device
        nn = int(np.asarray(state.assets.mesh.nodes_xy).shape[0])
        L = FrameLayout(pix, nn, state.ref_image, self._interpolation, dev)
        self._layout = L
        self._slot = FrameSlot(L, 1)
        self._desc = descriptors_to_device([self._slot.desc], dev)
        T = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
        # raw spring table (the local step weights springs by alpha * rho_i, not (rho_i + rho_j) / 2)
        idx = np.asarray(pix.node_neighbor_index, dtype=np.int64).reshape(nn, -1)
        deg = np.asarray(pix.node_neighbor_degree, dtype=np.int64)
        md = idx.shape[1]
        valid = np.arange(md)[None, :] < deg[:, None]
        w = np.asarray(pix.node_neighbor_weight, dtype=np.float32).reshape(nn, -1)
        self._md = md
        self._nbr = T(np.where(valid, idx, -1).astype(np.int32).T.copy(), torch.int32) if md else None
        self._nbw = T(np.where(valid, w, 0).astype(np.float32).T.copy(), torch.float32) if md else None
        self._rho = T(np.asarray(pix.node_reg_weight, dtype=np.float32), torch.float32)
        has = np.zeros(nn, dtype=np.int32)
        has[np.asarray(pix.pixel_nodes).ravel()] = 1
        self._has_pix = T(has, torch.int32)
        self._slots = torch.zeros(_lib.load().d2ic_local_gn_slot_bytes(nn, L.node_chunk_k) // 4, dtype=torch.float32,
                                  device=dev)
        self._r2 = torch.zeros(max(L.n_chunks, 1), dtype=torch.float64, device=dev)
        self._st = torch.zeros((nn + 255) // 256, dtype=torch.float64, device=dev)
        self._cgx = torch.empty_like(self._slot.coeff)
        self._cgy = torch.empty_like(self._slot.coeff)
        self._gx = torch.empty((L.H, L.W), dtype=torch.float32, device=dev)
        self._gy = torch.empty_like(self._gx)
        self._key = key

    def solve(self, state, def_image: Array) -> LocalGNResult:
        if not self._compiled:
            raise RuntimeError("LocalGaussNewtonSolver.compile() must be called before solve().")
        if state.assets.pixel_data is None:
            raise ValueError("MeshAssets must provide pixel_data for LocalGaussNewtonSolver.")
        self._ensure(state)
        L, dev = self._layout, self._device
        img = as_device_image(def_image, dev)
        self._slot.load_image(img)
        _lib.call("d2ic_central_gradient", ptr(img), L.H, L.W, ptr(self._gx), ptr(self._gy), _lib.stream_handle())
        prepare_coefficients(self._gx, L.kind, self._cgx, self._slot.tmp)
        prepare_coefficients(self._gy, L.kind, self._cgy, self._slot.tmp)
        nn = L.n_nodes
        if state.u0_nodal is None:
            u = torch.zeros((nn, 2), dtype=torch.float32, device=dev)
        else:
            u = torch.as_tensor(np.asarray(state.u0_nodal, dtype=np.float32) if not isinstance(state.u0_nodal, torch.Tensor)
                                else state.u0_nodal, dtype=torch.float32, device=dev).reshape(nn, 2).clone()
        v = torch.empty_like(u)
        n_sweeps = int(state.config.max_iters)
        hist = torch.full((max(n_sweeps, 1), 2), float("nan"), dtype=torch.float64, device=dev)
        alpha = float(state.config.reg_strength)
        for k in range(n_sweeps):
            _lib.call("d2ic_local_gn_sweep", ptr(self._desc), L.n_chunks, nn, L.node_chunk_k, L.kind, ptr(self._cgx),
                      ptr(self._cgy), ptr(u), ptr(self._slots), ptr(self._r2), ptr(self._has_pix), ptr(self._nbr),
                      ptr(self._nbw), self._md, ptr(self._rho), self._lam, self._max_step, alpha, self._omega,
                      ptr(v), ptr(self._st), _lib.stream_handle())
            hist[k, 0] = torch.sqrt(self._r2[: max(L.n_chunks, 1)].sum() / max(L.n_pix, 1))
            hist[k, 1] = torch.sqrt(self._st.sum() / (2 * nn))
            u, v = v, u
        u_host = u.cpu().numpy()
        save_history = bool(getattr(state.config, "save_history", False))
        return LocalGNResult(u_nodal=u_host, strain=np.zeros((nn, 3), dtype=np.float32),
                             history=hist[:n_sweeps].cpu().numpy() if save_history else None, u_device=u)
