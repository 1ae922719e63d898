"""msplat_gb300: a GB300 (sm_103a) Gaussian-splatting rasteriser with the
Python API of pointrix-project/msplat.

Every op runs hand-written CUDA through the C ABI in
include/msplat_gb300.h; there is no CPU fallback.
"""
from .project_point import project_point
from .compute_cov3d import compute_cov3d
from .ewa_project import ewa_project
from .compute_sh import compute_sh
from .sort_gaussian import sort_gaussian
from .alpha_blending import alpha_blending
from .rasterize import preprocess, rasterization, rasterization_sh
from .batch import rasterization_batch, rasterization_sh_batch, rasterization_sh_scenes
from .density import DensityStats, prune_and_densify

__all__ = [
    "project_point",
    "compute_cov3d",
    "ewa_project",
    "sort_gaussian",
    "compute_sh",
    "alpha_blending",
    "rasterization",
    "rasterization_sh",
    "preprocess",
    "rasterization_batch",
    "rasterization_sh_batch",
    "rasterization_sh_scenes",
    "DensityStats",
    "prune_and_densify",
]

__version__ = "0.1.0"
