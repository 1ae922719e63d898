"""Pinhole projection of 3-D points (drop-in for msplat/project_point.py)."""
from __future__ import annotations

from typing import Tuple

import torch
from torch import Tensor

from . import _lib
from . import _tensors as tt


def project_point(
    xyz: Tensor,
    intr: Tensor,
    extr: Tensor,
    W: int,
    H: int,
    nearest: float = 0.0,
    extent: float = 1.3,
) -> Tuple[Tensor, Tensor]:
    """Projects points to pixel coordinates (msplat/project_point.py:8-44).

    Parameters
    ----------
    xyz : [P, 3] float32 CUDA tensor, world-space positions.
    intr : [4] (fx, fy, cx, cy) in pixels.
    extr : [3, 4] world-to-camera [R | t] (OpenCV); a [4, 4] also works.
    W, H : image size.
    nearest : near-plane cull threshold; culling is off when <= 0.
    extent : points whose uv falls outside the image box scaled by `extent`
        around its centre are culled; off when <= 0.

    Returns
    -------
    uv : [P, 2] pixel coordinates (pixel centres at integers), 0 if culled.
    depth : [P, 1] camera-space z, 0 if culled.
    """
    return _ProjectPoint.apply(xyz, intr, extr, W, H, nearest, extent)


class _ProjectPoint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, intr, extr, W, H, nearest, extent):
        xyz_c = tt.f32(xyz, "xyz", 3)
        intr_c, extr_c = tt.camera(intr, extr)
        P = xyz_c.shape[0]
        uv = torch.empty((P, 2), dtype=torch.float32, device=xyz.device)
        depth = torch.empty((P, 1), dtype=torch.float32, device=xyz.device)
        lib = _lib.load()
        with _lib.stage("project_point_forward"):
            _lib.check(lib.msplat_project_point_forward(
                P, _lib.ptr(xyz_c), _lib.ptr(intr_c), _lib.ptr(extr_c), int(W), int(H),
                float(nearest), float(extent), _lib.ptr(uv), _lib.ptr(depth),
                _lib.stream(xyz.device)), "project_point_forward")
        ctx.W, ctx.H = int(W), int(H)
        ctx.save_for_backward(xyz_c, intr_c, extr_c, uv, depth)
        ctx.extr_shape = extr.shape
        return uv, depth

    @staticmethod
    def backward(ctx, dL_duv, dL_ddepth):
        xyz, intr, extr, uv, depth = ctx.saved_tensors
        P = xyz.shape[0]
        dev = xyz.device
        dL_duv = (dL_duv if dL_duv is not None else torch.zeros_like(uv)).float().contiguous()
        dL_ddepth = (dL_ddepth if dL_ddepth is not None else torch.zeros_like(depth)).float().contiguous()
        want_i, want_e = ctx.needs_input_grad[1], ctx.needs_input_grad[2]
        dL_dxyz = torch.empty((P, 3), dtype=torch.float32, device=dev)
        dL_dintr = torch.zeros(4, dtype=torch.float32, device=dev) if want_i else None
        dL_dextr = torch.zeros(12, dtype=torch.float32, device=dev) if want_e else None
        lib = _lib.load()
        ws = _lib.workspace(lib.msplat_camera_grad_workspace_size(P), dev)
        with _lib.stage("project_point_backward"):
            _lib.check(lib.msplat_project_point_backward(
                P, _lib.ptr(xyz), _lib.ptr(intr), _lib.ptr(extr), ctx.W, ctx.H, _lib.ptr(uv),
                _lib.ptr(depth), _lib.ptr(dL_duv), _lib.ptr(dL_ddepth), _lib.ptr(dL_dxyz),
                _lib.ptr(dL_dintr), _lib.ptr(dL_dextr), _lib.ptr(ws), ws.numel(),
                _lib.stream(dev)), "project_point_backward")
        if dL_dintr is not None and intr.numel() != 4:
            g = torch.zeros(intr.numel(), dtype=torch.float32, device=dev)
            g[:4] = dL_dintr
            dL_dintr = g
        if dL_dintr is not None:
            dL_dintr = dL_dintr.view(intr.shape)
        if dL_dextr is not None:
            dL_dextr = tt.extr_grad_like(dL_dextr, extr).view(ctx.extr_shape)
        return dL_dxyz, dL_dintr, dL_dextr, None, None, None, None
