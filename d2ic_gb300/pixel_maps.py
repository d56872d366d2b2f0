"""Per-pixel result maps on the device.

``discrepancy_map_ref`` is the reference's ``compute_discrepancy_map_ref``
(d2ic/discrepancy.py:86-127): the bilinear grey-level residual
``I_def(x + u(x)) - I_ref(x)`` at every ROI pixel, NaN outside the ROI and
where the bilinear stencil leaves the image, with the RMS of the valid
residuals.  It runs as one CUDA kernel over the frame's element-major pixel
records (``d2ic_discrepancy_map``).
"""
from __future__ import annotations

import torch

from . import _lib
from ._lib import ptr
from .engine import FrameLayout, as_device_image


def discrepancy_map_ref(layout: FrameLayout, desc_dev: torch.Tensor, def_image, u, stream=None):
    """(map (H, W) float32 CUDA tensor, rms) for displacement ``u`` (Nn, 2) and a deformed image."""
    out, pending = discrepancy_map_queue(layout, desc_dev, def_image, u, stream)
    return out, discrepancy_rms(pending)


def discrepancy_rms(pending) -> float:
    """The RMS of a map queued by :func:`discrepancy_map_queue` (waits for it)."""
    sums, cnts = pending
    n = int(cnts.sum())
    return float(torch.sqrt(sums.sum() / max(n, 1)))


def discrepancy_map_queue(layout: FrameLayout, desc_dev: torch.Tensor, def_image, u, stream=None):
    """Queue the map without waiting: (map tensor, pending partial sums for :func:`discrepancy_rms`)."""
    dev = layout.device
    ref = layout.ref_image
    dimg = as_device_image(def_image, dev)
    uu = torch.as_tensor(u, dtype=torch.float32, device=dev).reshape(-1, 2).contiguous()
    out = torch.empty((layout.H, layout.W), dtype=torch.float32, device=dev)
    nc = max(layout.n_chunks, 1)
    sums = torch.zeros(nc, dtype=torch.float64, device=dev)
    cnts = torch.zeros(nc, dtype=torch.int32, device=dev)
    _lib.call("d2ic_discrepancy_map", ptr(desc_dev), layout.n_chunks, ptr(ref), ptr(dimg), ptr(uu), layout.H,
              layout.W, ptr(out), ptr(sums), ptr(cnts), _lib.stream_handle(stream))
    return out, (sums, cnts)
