"""Configuration and result containers (same fields and defaults as the reference).

Reference: d2ic/dataclasses.py:8-239.  Arrays in results are host numpy arrays
(float32) unless a docstring says otherwise.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Dict, Optional, Sequence

from .types import Array


@dataclass(frozen=True)
class InitMotionConfig:
    """Element-centre ZNCC matching: odd window ``win``, +/- ``search`` px, score threshold."""
    win: int = 41
    search: int = 24
    score_min: Optional[float] = 0.2
    max_centers: Optional[int] = None


@dataclass(frozen=True)
class MeshDICConfig:
    """Global mesh DIC: CG iteration cap, gradient-norm tolerance, spring weight, strain options."""
    max_iters: int = 50
    tol: float = 1e-6
    reg_strength: float = 0.0
    strain_gauge_length: float = 0.0
    strain_eps: float = 1e-8
    save_history: bool = True
    compute_discrepancy_map: bool = False


@dataclass(frozen=True)
class DICDiagnostics:
    info: Dict[str, Any] = field(default_factory=dict)


@dataclass(frozen=True)
class DICResult:
    """Nodal displacement (Nn,2), Voigt strain (Nn,3), diagnostics, optional CG history."""
    u_nodal: Array
    strain: Array
    diagnostics: DICDiagnostics
    history: Array | None = None
    fields: Dict[str, Array] = field(default_factory=dict)
    pixel_maps: Dict[str, Array] = field(default_factory=dict)


@dataclass(frozen=True)
class BatchConfig:
    """Sequence processing options (warm start, per-frame saving; plotting fields kept for API parity)."""
    use_init_motion: bool = True
    warm_start_from_previous: bool = True
    init_motion_first_frame_only: bool = False
    init_motion_every_frame: bool = False
    prefer_init_motion_over_propagation: bool = False
    verbose: bool = False
    progress: bool = False
    save_per_frame: bool = False
    per_frame_dir: Optional[str] = None
    export_png: bool = False
    export_frames: Sequence[int] | None = None
    png_dir: Optional[str] = None
    plot_fields: Sequence[str] = ("u1", "u2", "e11", "e22", "e12")
    plot_include_discrepancy: bool = False
    plot_cmap: str = "jet"
    plot_alpha: float = 0.6
    plot_mesh: bool = True
    plot_dpi: int = 200
    plot_binning: float = 1.0
    plot_projection: str | bool = "fast"


@dataclass(frozen=True)
class BatchDiagnostics:
    info: Dict[str, Any] = field(default_factory=dict)


@dataclass(frozen=True)
class BatchResult:
    results: list
    diagnostics: BatchDiagnostics
