"""On-disk results in the reference's formats.

- per-frame ``frame_XXXX.npz`` with ``u_nodal``, ``strain`` and, when computed,
  ``discrepancy_ref`` (d2ic/batch_mesh_based.py:174-185);
- the sequence file ``fields_sequence.npz`` with ``nodes_xy``, stacked ``u_nodal``
  (F, Nn, 2), ``strain`` (F, Nn, 3), ``ref_path``, ``def_paths`` and, when every
  frame has one, ``discrepancy_ref`` (F, H, W) in float32
  (doc/03_0_tutorial_sequentialDIC.py:213-239).

Device tensors are copied to the host here; nothing on the solve path waits on
these writes.
"""
from __future__ import annotations

from pathlib import Path
from typing import Optional, Sequence

import numpy as np


def to_host(x) -> np.ndarray:
    """A numpy view/copy of ``x`` (numpy array, list or torch tensor on any device)."""
    if hasattr(x, "detach") and hasattr(x, "cpu"):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def frame_payload(result) -> dict:
    """The per-frame npz fields of one ``DICResult``."""
    payload = {"u_nodal": to_host(result.u_nodal), "strain": to_host(result.strain)}
    disc = (getattr(result, "pixel_maps", None) or {}).get("discrepancy_ref")
    if disc is not None:
        payload["discrepancy_ref"] = to_host(disc)
    return payload


def save_frame_npz(path, result) -> Path:
    """Write ``frame_payload(result)`` to ``path`` (compressed)."""
    path = Path(path)
    np.savez_compressed(path, **frame_payload(result))
    return path


def fields_sequence_payload(nodes_xy, results: Sequence, ref_path: Optional[str] = None,
                            def_paths: Optional[Sequence[str]] = None) -> dict:
    """The ``fields_sequence.npz`` fields for a list of per-frame results."""
    if len(results) == 0:
        raise ValueError("fields_sequence_payload: no frames")
    payload = {
        "nodes_xy": to_host(nodes_xy),
        "u_nodal": np.stack([to_host(r.u_nodal) for r in results], axis=0),
        "strain": np.stack([to_host(r.strain) for r in results], axis=0),
        "ref_path": str(ref_path) if ref_path is not None else "",
        "def_paths": [str(p) for p in (def_paths if def_paths is not None else [])],
    }
    maps = []
    for r in results:
        disc = (getattr(r, "pixel_maps", None) or {}).get("discrepancy_ref")
        if disc is None:
            maps = []
            break
        maps.append(to_host(disc).astype(np.float32, copy=False))
    if maps:
        payload["discrepancy_ref"] = np.stack(maps, axis=0)
    return payload


def save_fields_sequence(path, nodes_xy, results: Sequence, ref_path: Optional[str] = None,
                         def_paths: Optional[Sequence[str]] = None) -> Path:
    """Write ``fields_sequence.npz`` (``path`` may be the file or its directory)."""
    path = Path(path)
    if path.is_dir() or path.suffix != ".npz":
        path.mkdir(parents=True, exist_ok=True)
        path = path / "fields_sequence.npz"
    np.savez_compressed(path, **fields_sequence_payload(nodes_xy, results, ref_path, def_paths))
    return path
