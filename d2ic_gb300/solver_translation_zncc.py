"""Integer-translation ZNCC search at element centres on the GPU.

Drop-in for ``TranslationZNCCSolver`` (d2ic/solver_translation_zncc.py:26-82):
one CUDA block per centre (``d2ic_zncc_match``) instead of a sequential
``lax.map``.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import numpy as np
import torch

from . import _lib
from ._lib import ptr
from .dataclasses import InitMotionConfig
from .engine import as_device_image
from .solver_base import SolverBase
from .types import Array


@dataclass(frozen=True)
class TranslationZNCCResult:
    u_centers: Array   # (Ne, 2)
    scores: Array      # (Ne,)


def match_centers_device(centers, ref_image, def_image, win: int, search: int, device=None):
    """``(u (Nc,2), scores (Nc,))`` CUDA tensors: best integer shift per centre."""
    device = torch.device(device if device is not None else "cuda")
    ref = as_device_image(ref_image, device)
    dfm = as_device_image(def_image, device)
    if isinstance(centers, torch.Tensor):
        c = centers.to(device=device, dtype=torch.float32).reshape(-1, 2).contiguous()
    else:
        c = torch.as_tensor(np.asarray(centers, dtype=np.float32).reshape(-1, 2), device=device).contiguous()
    n = c.shape[0]
    u = torch.empty((n, 2), dtype=torch.float32, device=device)
    s = torch.empty((n,), dtype=torch.float32, device=device)
    _lib.call("d2ic_zncc_match", ptr(ref), ref.shape[0], ref.shape[1], ptr(dfm), dfm.shape[0], dfm.shape[1], ptr(c),
              n, int(win), int(search), ptr(u), ptr(s), _lib.stream_handle())
    return u, s


def _match_centers(centers, ref_image, def_image, *, win: int, search: int):
    """Host-array form of the match (reference name ``_match_centers_jax``)."""
    u, s = match_centers_device(centers, ref_image, def_image, win, search)
    return u.cpu().numpy(), s.cpu().numpy()


class TranslationZNCCSolver(SolverBase):
    def __init__(self, config: InitMotionConfig, chunk_size: int = 128, device=None) -> None:
        if config.win % 2 == 0:
            raise ValueError("InitMotionConfig.win must be odd for ZNCC matching.")
        self.config = config
        self.chunk_size = max(1, int(chunk_size))
        self._compiled = False
        self._device = torch.device(device if device is not None else "cuda")

    def compile(self, assets: Any) -> None:
        _lib.load()
        self._compiled = True

    def solve_device(self, state: Any, def_image: Array):
        if not self._compiled:
            raise RuntimeError("TranslationZNCCSolver.compile() must be called before solve().")
        centers = np.asarray(state.assets.element_centers_xy, dtype=np.float32)
        if self.config.max_centers is not None:
            centers = centers[: int(self.config.max_centers)]
        u, s = match_centers_device(centers, state.ref_image, def_image, self.config.win, self.config.search,
                                    self._device)
        if self.config.score_min is not None:
            valid = s >= float(self.config.score_min)
            u = torch.where(valid[:, None], u, torch.zeros_like(u))
            s = torch.where(valid, s, torch.full_like(s, float("nan")))
        return u, s

    def solve(self, state: Any, def_image: Array) -> TranslationZNCCResult:
        u, s = self.solve_device(state, def_image)
        return TranslationZNCCResult(u_centers=u.cpu().numpy(), scores=s.cpu().numpy())
