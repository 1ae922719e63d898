"""msplat_gb300: a GB300 (sm_103a) Gaussian-splatting rasteriser with the
Python API of pointrix-project/msplat.

Every op runs hand-written CUDA through the C ABI in
include/msplat_gb300.h; there is no CPU fallback.
"""
from torch import Tensor

from .project_point import project_point
from .compute_cov3d import compute_cov3d
from .ewa_project import ewa_project
from .compute_sh import compute_sh
from .sort_gaussian import sort_gaussian
from .alpha_blending import alpha_blending

__all__ = [
    "project_point",
    "compute_cov3d",
    "ewa_project",
    "sort_gaussian",
    "compute_sh",
    "alpha_blending",
    "rasterization",
]

__version__ = "0.1.0"


def rasterization(
    xyz: Tensor,
    scale: Tensor,
    rotate: Tensor,
    opacity: Tensor,
    feature: Tensor,
    intr: Tensor,
    extr: Tensor,
    W: int,
    H: int,
    bg: float,
    ndc: Tensor = None,
) -> Tensor:
    """3-D Gaussian splatting of `feature` (msplat/__init__.py:22-93).

    xyz [P,3], scale [P,3], rotate [P,4] unit quaternions (r,x,y,z),
    opacity [P,1], feature [P,C], intr [4] = (fx,fy,cx,cy), extr [3,4]
    world-to-camera, image W x H, scalar background `bg`; `ndc` [P,2]
    optionally receives dL/duv * (W/2, H/2).  Returns [C, H, W].
    """
    uv, depth = project_point(xyz, intr, extr, W, H)
    visible = depth != 0
    cov3d = compute_cov3d(scale, rotate, visible)
    conic, radius, tiles_touched = ewa_project(xyz, cov3d, intr, extr, uv, W, H, visible)
    idx_sorted, tile_range = sort_gaussian(uv, depth, W, H, radius, tiles_touched)
    return alpha_blending(uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, ndc)
