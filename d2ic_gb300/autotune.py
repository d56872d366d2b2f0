"""Launch-shape autotuner for the CG engine.

The engine's cost per objective evaluation depends on two shapes the data does
not fix:

* the chunk size (pixels per chunk, at most 256): it sets the shared-memory
  coefficient tile of each chunk, the number of chunks per warp (load balance
  of the pixel pass) and the number of gradient slots per node;
* the grid size (resident blocks): the warps that share the pixel pass and
  the node groups.

:class:`Autotuner` measures candidate shapes on the actual frame -- a fixed
number of engine rounds from a fresh start, timed with CUDA events on the
launching stream after one untimed slice -- and keeps the fastest per frame
signature (image size, ROI pixels, element size, interpolation).  Results are
cached in memory and, when ``cache_path`` (or the ``D2IC_TUNE_CACHE``
environment variable) names a file, in JSON so that later processes reuse them.
Every candidate gives the same converged solution up to the order of FP32
partial sums (each is a valid layout of the same frame); the tuner only times.
"""
from __future__ import annotations

import json
import os
from dataclasses import asdict, dataclass

import numpy as np
import torch

from . import _lib
from .engine import Engine, FrameLayout, FrameSlot, descriptors_to_device

CHUNK_CANDIDATES = (64, 128, 256)


@dataclass(frozen=True)
class LaunchShape:
    chunk_pixels: int
    grid_blocks: int                    # 0 = every resident block (SMs x blocks per SM)
    us_per_round: float = float("nan")


def _element_pixels(pix):
    """Pixels per element of a frame's assets (zeros dropped)."""
    from .engine import _elements_of
    if hasattr(type(pix), "element_pixel_counts"):           # GridPixelData: counted on the device
        per_elem = np.asarray(pix.element_pixel_counts())
    else:
        if int(np.asarray(pix.pixel_coords_ref).shape[0]) == 0:
            return np.zeros(0, np.int64)
        per_elem = np.bincount(_elements_of(pix))
    return per_elem[per_elem > 0]


def frame_signature(pix, H: int, W: int, interpolation: str) -> str:
    """Key of frames that share a launch shape: size, element size, ROI pixels to within a factor
    of 2^(1/4) (ROI coverage moves the best shape little; finer keys re-tune nearly every frame)."""
    pe = _element_pixels(pix)
    n_pix = int(pe.sum())
    elem = 0
    if pe.size:
        # the most common pixels-per-element count (interior elements), as an element-size estimate
        elem = int(round(np.sqrt(int(np.argmax(np.bincount(pe))))))
    bucket = int(round(4 * np.log2(max(n_pix, 1))))
    return f"{H}x{W}:{interpolation}:e{elem}:p{bucket}"


def distinct_chunk_sizes(candidates, max_element_pixels: int):
    """Chunk sizes that give different layouts: a chunk holds pixels of one element, so every
    size at or above the largest element's pixel count gives the same chunks; keep the smallest."""
    out = sorted(c for c in candidates if c < max_element_pixels)
    big = [c for c in candidates if c >= max_element_pixels]
    if big:
        out.append(min(big))
    return tuple(out)


def device_blocks(device) -> int:
    import ctypes
    sms, bps = ctypes.c_int(), ctypes.c_int()
    with torch.cuda.device(torch.device(device)):
        _lib.call("d2ic_device_info", torch.device(device).index or 0, ctypes.byref(sms), ctypes.byref(bps))
    return sms.value * bps.value


class Autotuner:
    """Times candidate (chunk size, grid size) pairs on a frame and caches the fastest."""

    def __init__(self, device=None, chunk_candidates=CHUNK_CANDIDATES, grid_fractions=(1.0, 0.75, 0.5),
                 rounds: int = 24, cache_path: str | None = None):
        self.device = torch.device(device if device is not None else "cuda")
        self.chunk_candidates = tuple(int(c) for c in chunk_candidates)
        if not self.chunk_candidates or any(not 1 <= c <= _lib.CHUNK_MAX for c in self.chunk_candidates):
            raise ValueError(f"chunk candidates must lie in [1, {_lib.CHUNK_MAX}]")
        self.grid_fractions = tuple(float(f) for f in grid_fractions)
        self.rounds = int(rounds)
        self.cache_path = cache_path if cache_path is not None else os.environ.get("D2IC_TUNE_CACHE")
        self.cache: dict[str, LaunchShape] = {}
        self.trials: dict[str, list[LaunchShape]] = {}
        if self.cache_path and os.path.exists(self.cache_path):
            with open(self.cache_path) as fh:
                for k, v in json.load(fh).items():
                    self.cache[k] = LaunchShape(**v)

    def _save(self):
        if self.cache_path:
            tmp = self.cache_path + ".tmp"
            with open(tmp, "w") as fh:
                json.dump({k: asdict(v) for k, v in self.cache.items()}, fh, indent=1)
            os.replace(tmp, self.cache_path)

    def _time_rounds(self, eng: Engine, desc, kind: int, grid: int) -> float:
        cmd = eng.commands(1)
        cmd.zero_()                                            # fresh start (INIT) for the timed slice
        eng.run_slice(desc, 1, kind, self.rounds, grid)
        cmd.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        eng.run_slice(desc, 1, kind, self.rounds, grid)
        e1.record()
        torch.cuda.synchronize(self.device)
        return e0.elapsed_time(e1) * 1e3 / self.rounds

    def tune(self, pix, n_nodes: int, ref_image, def_image, interpolation: str = "cubic", u0=None,
             tol: float = 1e-12, alpha_reg: float = 0.1) -> LaunchShape:
        """Fastest launch shape for this frame's signature (measured once per signature)."""
        ref = ref_image if isinstance(ref_image, torch.Tensor) else torch.as_tensor(np.asarray(ref_image, np.float32))
        H, W = int(ref.shape[0]), int(ref.shape[1])
        key = frame_signature(pix, H, W, interpolation)
        if key in self.cache:
            return self.cache[key]
        full = device_blocks(self.device)
        grids = sorted({max(1, int(round(full * f))) for f in self.grid_fractions}, reverse=True)
        eng = Engine(self.device, 1)
        trials = []
        pe = _element_pixels(pix)
        for chunk in distinct_chunk_sizes(self.chunk_candidates, int(pe.max()) if pe.size else 1):
            layout = FrameLayout(pix, n_nodes, ref_image, interpolation, self.device, chunk_max=chunk)
            slot = FrameSlot(layout, max_iter=10 * self.rounds)
            slot.set_params(tol, alpha_reg)
            slot.load_image(def_image)
            slot.set_u0(u0)
            desc = descriptors_to_device([slot.desc], self.device)
            for g in grids:
                us = self._time_rounds(eng, desc, layout.kind, g)
                trials.append(LaunchShape(chunk, 0 if g == full else g, us))
            del layout, slot, desc
        best = min(trials, key=lambda s: s.us_per_round)
        self.cache[key] = best
        self.trials[key] = trials
        self._save()
        return best


_default: Autotuner | None = None


def default_tuner(device=None) -> Autotuner:
    """Process-wide tuner (in-memory cache shared by solvers and servers)."""
    global _default
    if _default is None or (device is not None and torch.device(device) != _default.device):
        _default = Autotuner(device)
    return _default
