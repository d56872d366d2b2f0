"""d2ic_gb300: GB300-native (sm_103a) global finite-element DIC hot path.

Keeps the public names of the reference package ``d2ic`` (d2ic/__init__.py:34-81)
for the hot path: the solver plugins run hand-written CUDA kernels through the
C ABI in include/d2ic_gb300.h; the host side is numpy/torch.
"""
from .types import Array
from .dataclasses import (
    InitMotionConfig,
    MeshDICConfig,
    DICResult,
    DICDiagnostics,
    BatchConfig,
    BatchResult,
    BatchDiagnostics,
)
from .mesh_assets import Mesh, MeshAssets, PixelAssets, compute_element_centers, make_mesh_assets
from .mask2mesh import downsample_mask, mask_to_mesh, mask_to_mesh_assets, mask_to_mesh_gmsh, mask_to_mesh_assets_gmsh
from .pixel_assets import build_pixel_assets
from .strain import compute_green_lagrange_strain_nodes_lsq, green_lagrange_to_voigt, small_strain_nodes_lsq
from .solver_base import SolverBase
from .dic_base import DICBase
from .dic_init_motion import DICInitMotion
from .dic_mesh_based import DICMeshBased
from .batch_mesh_based import BatchBase, BatchMeshBased
from .propagators import DisplacementPropagatorBase, PreviousDisplacementPropagator, ConstantVelocityPropagator
from .solver_translation_zncc import TranslationZNCCSolver
from .solver_global_cg import GlobalCGSolver
from .solver_local_gn import LocalGaussNewtonSolver, LocalGNResult
from .outputs import save_fields_sequence, save_frame_npz

__all__ = [
    "Array", "InitMotionConfig", "MeshDICConfig", "DICResult", "DICDiagnostics", "BatchConfig", "BatchResult",
    "BatchDiagnostics", "Mesh", "MeshAssets", "PixelAssets", "compute_element_centers", "make_mesh_assets",
    "downsample_mask", "mask_to_mesh", "mask_to_mesh_assets", "mask_to_mesh_gmsh", "mask_to_mesh_assets_gmsh",
    "build_pixel_assets", "compute_green_lagrange_strain_nodes_lsq", "green_lagrange_to_voigt",
    "small_strain_nodes_lsq", "SolverBase", "DICBase", "DICInitMotion", "DICMeshBased", "BatchBase",
    "BatchMeshBased", "DisplacementPropagatorBase", "PreviousDisplacementPropagator", "ConstantVelocityPropagator",
    "TranslationZNCCSolver", "GlobalCGSolver", "LocalGaussNewtonSolver", "LocalGNResult",
    "save_fields_sequence", "save_frame_npz",
]
