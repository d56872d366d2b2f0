"""Global nonlinear-CG mesh DIC solver on the GB300 engine.

Drop-in for ``GlobalCGSolver`` (d2ic/solver_global_cg.py:35-198): same
constructor flags, ``compile(assets)`` / ``warmup(state)`` /
``solve(state, def_image)`` and the same result fields.  The whole CG loop
(d2ic/solver_global_cg.py:326-469) runs in one persistent cooperative CUDA
launch (``d2ic_cg_solve_batched`` with one frame); there is no CPU path.
"""
from __future__ import annotations

import warnings
from dataclasses import dataclass
from typing import Any

import numpy as np
import torch

from . import _lib
from .engine import Engine, FrameLayout, FrameSlot, descriptors_to_device, interp_kind
from .solver_base import SolverBase
from .types import Array


@dataclass(frozen=True)
class GlobalCGResult:
    u_nodal: Array
    strain: Array
    history: Array | None = None
    n_iters: int | None = None
    status: str = "ok"
    u_device: Any = None         # the solution as a CUDA tensor (kept on the device for post-processing)


def _normalize_interpolation(interpolation: str) -> str:
    value = str(interpolation).lower()
    if value == "bilinear":
        value = "linear"
    if value not in ("cubic", "linear"):
        raise ValueError(f"Unsupported interpolation: {interpolation}")
    return value


class SolveHandle:
    """A frame queued by ``GlobalCGSolver.solve_begin``: its device displacement and the pinned
    buffers its results are copied into."""

    def __init__(self, u_device, bufs):
        self.u_device = u_device
        self.bufs = bufs


class GlobalCGSolver(SolverBase):
    """Global CG solver for mesh DIC; expects ``MeshAssets.pixel_data``."""

    def __init__(self, verbose: bool = False, interpolation: str = "cubic", use_map_coordinates: bool | None = None,
                 log_cg: bool = False, device=None, grid_blocks: int = 0, chunk_pixels: int = 256,
                 autotune: bool = False) -> None:
        self._compiled = False
        self._verbose = bool(verbose)
        self._log_cg = bool(log_cg)
        if use_map_coordinates is not None:
            warnings.warn("use_map_coordinates is kept for backward compatibility; use interpolation='cubic' or "
                          "'linear'.", DeprecationWarning, stacklevel=2)
            interpolation = "cubic" if use_map_coordinates else "linear"
        self._interpolation = _normalize_interpolation(interpolation)
        self._kind = interp_kind(self._interpolation)
        self._device = torch.device(device if device is not None else "cuda")
        self._grid_blocks = int(grid_blocks)
        self._chunk_pixels = int(chunk_pixels)
        self._autotune = bool(autotune)
        self.launch_shape = None          # the autotuner's choice, when autotune=True
        self._layout = None
        self._layout_key = None
        self._slot = None
        self._desc_dev = None
        self._desc_params = None
        self._engine = None
        self._pinned_sets = None
        self._pinned_flip = 0
        self._last_handle = None

    # -- plugin interface -------------------------------------------------------------
    def compile(self, assets: Any) -> None:
        if getattr(assets, "pixel_data", None) is None:
            raise ValueError("MeshAssets must provide pixel_data for GlobalCGSolver.")
        _lib.load()
        self._compiled = True

    def _ensure(self, state):
        assets = state.assets
        pix = assets.pixel_data
        key = (id(pix), id(state.ref_image), int(state.config.max_iters))
        if self._layout is None or self._layout_key != key:
            n_nodes = int(np.asarray(assets.mesh.nodes_xy).shape[0])
            if self._autotune:
                # probe frame: the reference shifted by one pixel (non-zero residuals, so rounds run)
                from .autotune import default_tuner
                from .engine import as_device_image
                ref = as_device_image(state.ref_image, self._device)
                shape = default_tuner(self._device).tune(pix, n_nodes, ref, torch.roll(ref, 1, dims=1),
                                                         self._interpolation)
                self._chunk_pixels, self._grid_blocks = shape.chunk_pixels, shape.grid_blocks
                self.launch_shape = shape
            self._layout = FrameLayout(pix, n_nodes, state.ref_image, self._interpolation, self._device,
                                       chunk_max=self._chunk_pixels)
            self._slot = FrameSlot(self._layout, int(state.config.max_iters))
            self._engine = Engine(self._device, 1)
            self._layout_key = key
            self._desc_params = None
            nn = n_nodes
            # two sets of pinned result buffers: a frame's copies may still be pending while the
            # next frame is queued (solve_begin / solve_end)
            self._pinned_sets = [{
                "u": torch.empty((nn, 2), dtype=torch.float32).pin_memory(),
                "hist": torch.empty(self._slot.hist.shape, dtype=torch.float32).pin_memory(),
                "info": torch.empty(3, dtype=torch.int32).pin_memory(),
            } for _ in range(2)]
            self._pinned_flip = 0
        params = (float(state.config.tol), float(state.config.reg_strength))
        if params != self._desc_params:
            self._slot.set_params(*params)
            self._desc_dev = descriptors_to_device([self._slot.desc], self._device)
            self._desc_params = params
        return self._slot

    def warmup(self, state: Any) -> None:
        """Build the device layout for the state's reference image and run one zero-iteration launch."""
        if not self._compiled:
            raise RuntimeError("GlobalCGSolver.compile() must be called before warmup().")
        if state.assets.pixel_data is None:
            raise ValueError("MeshAssets must provide pixel_data for GlobalCGSolver warmup.")
        slot = self._ensure(state)
        slot.load_image(self._layout.ref_image)
        slot.set_u0(None)
        self._engine.solve(self._desc_dev, 1, self._kind, self._grid_blocks)
        torch.cuda.synchronize(self._device)

    def solve(self, state: Any, def_image: Array) -> GlobalCGResult:
        self.solve_begin(state, def_image)
        return self.solve_end(state)

    def solve_begin(self, state: Any, def_image: Array) -> "SolveHandle":
        """Queue one frame's solve and the copies of its results on the current stream without
        waiting.  The handle's ``u_device`` is the displacement on the device, on which more work
        (the strain) can be queued; :meth:`solve_end` returns the result.  Two frames may be
        pending at once (the second one's solve overwrites ``u_device``)."""
        if not self._compiled:
            raise RuntimeError("GlobalCGSolver.compile() must be called before solve().")
        slot = self._ensure(state)
        slot.load_image(def_image)
        slot.set_u0(state.u0_nodal)
        self._engine.solve(self._desc_dev, 1, self._kind, self._grid_blocks)
        bufs = self._pinned_sets[self._pinned_flip]
        self._pinned_flip ^= 1
        bufs["u"].copy_(slot.u_out, non_blocking=True)
        bufs["hist"].copy_(slot.hist, non_blocking=True)
        bufs["info"].copy_(slot.info, non_blocking=True)
        self._last_handle = SolveHandle(slot.u_out, bufs)
        return self._last_handle

    def solve_end(self, state: Any, handle: "SolveHandle" = None, wait: bool = True) -> GlobalCGResult:
        """The result of a frame queued by :meth:`solve_begin` (the last one by default); with
        ``wait=False`` the caller has already waited for its copies (an event after them)."""
        handle = handle if handle is not None else self._last_handle
        slot = self._slot
        pu, ph, pi = handle.bufs["u"], handle.bufs["hist"], handle.bufs["info"]
        if wait:
            torch.cuda.current_stream(self._device).synchronize()
        n_iters, status = int(pi[0]), int(pi[1])
        if status in (_lib.WAIT_TIMEOUT, _lib.CUDA_ERROR, _lib.INTERNAL):
            raise _lib.D2ICError(status, "CG engine aborted")
        if self._verbose and self._log_cg:
            for k in range(min(n_iters + 1, ph.shape[0])):
                J, g, a = ph[k].tolist()
                if np.isfinite(J):
                    print(f"CG iter {k}: J={J:.3e}, |grad|={g:.3e}, alpha={a:.3e}")
        u = pu.numpy().copy()
        save_history = bool(getattr(state.config, "save_history", False))
        return GlobalCGResult(
            u_nodal=u,
            strain=np.zeros_like(u),
            history=ph.numpy()[: slot.max_iter].copy() if save_history else None,
            n_iters=n_iters,
            status=_lib.STATUS_NAMES.get(status, str(status)),
            u_device=handle.u_device,
        )

    # -- diagnostics ---------------------------------------------------------------------
    def objective_and_gradient(self, state: Any, def_image: Array, u) -> tuple[float, np.ndarray]:
        """``J_total`` and its gradient at ``u`` on the GPU (the reference's ``_J_TOTAL_VG``)."""
        slot = self._ensure(state)
        slot.load_image(def_image)
        ud = torch.as_tensor(np.asarray(u, dtype=np.float32), device=self._device).reshape(-1, 2).contiguous()
        J, g = self._engine.eval_objective(self._desc_dev, ud, self._kind)
        return float(J.item()), g.cpu().numpy()
