"""EWA splatting to screen-space conics (drop-in for msplat/ewa_project.py)."""
from __future__ import annotations

from typing import Tuple

import torch
from torch import Tensor

from . import _lib
from . import _tensors as tt


def ewa_project(
    xyz: Tensor,
    cov3d: Tensor,
    intr: Tensor,
    extr: Tensor,
    uv: Tensor,
    W: int,
    H: int,
    visible: Tensor | None = None,
) -> Tuple[Tensor, Tensor, Tensor]:
    """Projects 3-D Gaussians to 2-D conics (msplat/ewa_project.py:8-53).

    Returns
    -------
    conic : [P, 3] inverse 2-D covariance (a, b, c), 0 where invisible.
    radius : [P] int32 pixel radius (3 sigma of the major axis), 0 if invisible.
    tiles : [P] int32 number of 16x16 tiles the radius box touches.
    """
    if visible is None:
        visible = torch.ones_like(uv[:, 0], dtype=torch.bool)
    return _EWAProject.apply(xyz, cov3d, intr, extr, uv, W, H, visible)


class _EWAProject(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, cov3d, intr, extr, uv, W, H, visible):
        x = tt.f32(xyz, "xyz", 3)
        c = tt.f32(cov3d, "cov3d", 6)
        intr_c, extr_c = tt.camera(intr, extr)
        u = tt.f32(uv, "uv", 2)
        P = x.shape[0]
        vis = tt.mask(visible, "visible", P)
        dev = x.device
        conic = torch.empty((P, 3), dtype=torch.float32, device=dev)
        radius = torch.empty((P,), dtype=torch.int32, device=dev)
        tiles = torch.empty((P,), dtype=torch.int32, device=dev)
        lib = _lib.load()
        with _lib.stage("ewa_project_forward"):
            _lib.check(lib.msplat_ewa_project_forward(
                P, _lib.ptr(x), _lib.ptr(c), _lib.ptr(intr_c), _lib.ptr(extr_c), _lib.ptr(u), int(W),
                int(H), _lib.ptr(vis), _lib.ptr(conic), _lib.ptr(radius), _lib.ptr(tiles),
                _lib.stream(dev)), "ewa_project_forward")
        ctx.save_for_backward(x, c, intr_c, extr_c, radius)
        ctx.extr_shape = extr.shape
        ctx.mark_non_differentiable(radius, tiles)
        ctx.set_materialize_grads(False)  # no zero-filled gradients for radius and tiles
        return conic, radius, tiles

    @staticmethod
    def backward(ctx, dL_dconic, dL_dradius, dL_dtiles):
        x, c, intr, extr, radius = ctx.saved_tensors
        P = x.shape[0]
        dev = x.device
        if dL_dconic is None:
            dL_dconic = torch.zeros((P, 3), dtype=torch.float32, device=dev)
        g = dL_dconic.float().contiguous()
        want_i, want_e = ctx.needs_input_grad[2], ctx.needs_input_grad[3]
        dxyz = torch.empty((P, 3), dtype=torch.float32, device=dev)
        dcov = torch.empty((P, 6), dtype=torch.float32, device=dev)
        dintr = torch.zeros(4, dtype=torch.float32, device=dev) if want_i else None
        dextr = torch.zeros(12, dtype=torch.float32, device=dev) if want_e else None
        lib = _lib.load()
        ws = _lib.workspace(lib.msplat_camera_grad_workspace_size(P), dev)
        with _lib.stage("ewa_project_backward"):
            _lib.check(lib.msplat_ewa_project_backward(
                P, _lib.ptr(x), _lib.ptr(c), _lib.ptr(intr), _lib.ptr(extr), _lib.ptr(radius),
                _lib.ptr(g), _lib.ptr(dxyz), _lib.ptr(dcov), _lib.ptr(dintr), _lib.ptr(dextr),
                _lib.ptr(ws), ws.numel(), _lib.stream(dev)), "ewa_project_backward")
        if dintr is not None:
            if intr.numel() != 4:
                full = torch.zeros(intr.numel(), dtype=torch.float32, device=dev)
                full[:4] = dintr
                dintr = full
            dintr = dintr.view(intr.shape)
        if dextr is not None:
            dextr = tt.extr_grad_like(dextr, extr).view(ctx.extr_shape)
        return dxyz, dcov, dintr, dextr, None, None, None, None
