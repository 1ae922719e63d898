"""The rasterisation pipeline: fused preprocess, tile sort, alpha blend.

``rasterization`` is the drop-in for msplat/__init__.py:22-93 (same
arguments, same result); ``rasterization_sh`` additionally evaluates the
colour from SH coefficients on the view directions of the camera, the step
the reference's training loops run before calling ``rasterization``
(``compute_sh(shs, normalize(xyz - camera_centre))``).

Both run projection, covariance and EWA (and SH) in one forward kernel and
all their adjoints, camera gradients included, in one backward kernel
(msplat_rasterize_preprocess_forward / _backward); the forward outputs are
bit-identical to the stage-by-stage calls.
"""
from __future__ import annotations

import threading

import torch
from torch import Tensor

from . import _lib
from . import _tensors as tt
from .alpha_blending import alpha_blending
from .sort_gaussian import sort_gaussian, sort_gaussian_capacity


class _Preprocess(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, scale, rotate, shs, intr, extr, W, H, nearest, extent):
        xyz_c = tt.f32(xyz, "xyz", 3)
        P = xyz_c.shape[0]
        scale_c = tt.f32(scale, "scale", 3)
        rot_c = tt.f32_aligned16(rotate, "rotate", 4)
        intr_c, extr_c = tt.camera(intr, extr)
        if scale_c.shape[0] != P or rot_c.shape[0] != P:
            raise RuntimeError("xyz, scale and rotate must have the same number of Gaussians")
        dev = xyz.device
        if shs is not None:
            shs_c = tt.f32(shs, "shs")
            if shs_c.dim() != 3 or shs_c.shape[0] != P:
                raise RuntimeError(f"shs must be [P, C, D], got {tuple(shs.shape)}")
            C, D = int(shs_c.shape[1]), int(shs_c.shape[2])
        else:
            shs_c, C, D = None, 0, 0
        uv = torch.empty((P, 2), dtype=torch.float32, device=dev)
        depth = torch.empty((P, 1), dtype=torch.float32, device=dev)
        conic = torch.empty((P, 3), dtype=torch.float32, device=dev)
        radius = torch.empty((P,), dtype=torch.int32, device=dev)
        tiles = torch.empty((P,), dtype=torch.int32, device=dev)
        color = torch.empty((P, C), dtype=torch.float32, device=dev)
        lib = _lib.load()
        with _lib.stage("rasterize_preprocess_forward"):
            _lib.check(lib.msplat_rasterize_preprocess_forward(
                P, _lib.ptr(xyz_c), _lib.ptr(scale_c), _lib.ptr(rot_c), _lib.ptr(intr_c), _lib.ptr(extr_c),
                int(W), int(H), float(nearest), float(extent), C, D, _lib.ptr(shs_c), _lib.ptr(uv),
                _lib.ptr(depth), _lib.ptr(conic), _lib.ptr(radius), _lib.ptr(tiles),
                _lib.ptr(color) if C else None, _lib.stream(dev)), "rasterize_preprocess_forward")
        ctx.C, ctx.D = C, D
        ctx.intr_shape, ctx.extr_shape = intr.shape, extr.shape
        ctx.save_for_backward(xyz_c, scale_c, rot_c, shs_c, intr_c, extr_c, depth, radius)
        ctx.mark_non_differentiable(depth, radius, tiles)
        # outputs without a gradient arrive as None (no zero-filled tensors
        # for depth, radius and tiles); the backward fills what it needs
        ctx.set_materialize_grads(False)
        return uv, depth, conic, radius, tiles, color

    @staticmethod
    def backward(ctx, dL_duv, _dd, dL_dconic, _dr, _dt, dL_dcolor):
        xyz, scale, rot, shs, intr, extr, depth, radius = ctx.saved_tensors
        P, dev, C, D = xyz.shape[0], xyz.device, ctx.C, ctx.D
        dL_duv = (dL_duv if dL_duv is not None else torch.zeros((P, 2), device=dev)).float().contiguous()
        dL_dconic = (dL_dconic if dL_dconic is not None else torch.zeros((P, 3), device=dev)).float().contiguous()
        if C:
            dL_dcolor = (dL_dcolor if dL_dcolor is not None else torch.zeros((P, C), device=dev)).float().contiguous()
        want_i, want_e = ctx.needs_input_grad[4], ctx.needs_input_grad[5]
        dL_dxyz = torch.empty((P, 3), dtype=torch.float32, device=dev)
        dL_dscale = torch.empty((P, 3), dtype=torch.float32, device=dev)
        dL_drot = torch.empty((P, 4), dtype=torch.float32, device=dev)
        dL_dshs = torch.empty((P, C, D), dtype=torch.float32, device=dev) if C else None
        dL_dintr = torch.empty(4, dtype=torch.float32, device=dev) if want_i else None
        dL_dextr = torch.empty(12, dtype=torch.float32, device=dev) if want_e else None
        lib = _lib.load()
        ws = _lib.workspace(lib.msplat_rasterize_preprocess_workspace_size(P, C, D), dev)
        with _lib.stage("rasterize_preprocess_backward"):
            _lib.check(lib.msplat_rasterize_preprocess_backward(
                P, _lib.ptr(xyz), _lib.ptr(scale), _lib.ptr(rot), _lib.ptr(intr), _lib.ptr(extr), C, D,
                _lib.ptr(shs), _lib.ptr(depth), _lib.ptr(radius), _lib.ptr(dL_duv), _lib.ptr(dL_dconic),
                _lib.ptr(dL_dcolor) if C else None, _lib.ptr(dL_dxyz), _lib.ptr(dL_dscale),
                _lib.ptr(dL_drot), _lib.ptr(dL_dshs), _lib.ptr(dL_dintr), _lib.ptr(dL_dextr), _lib.ptr(ws),
                ws.numel(), _lib.stream(dev)), "rasterize_preprocess_backward")
        if dL_dintr is not None:
            if intr.numel() != 4:
                g = torch.zeros(intr.numel(), dtype=torch.float32, device=dev)
                g[:4] = dL_dintr
                dL_dintr = g
            dL_dintr = dL_dintr.view(ctx.intr_shape)
        if dL_dextr is not None:
            dL_dextr = tt.extr_grad_like(dL_dextr, extr).view(ctx.extr_shape)
        return dL_dxyz, dL_dscale, dL_drot, dL_dshs, dL_dintr, dL_dextr, None, None, None, None


def preprocess(xyz: Tensor, scale: Tensor, rotate: Tensor, intr: Tensor, extr: Tensor, W: int, H: int,
               shs: Tensor | None = None, nearest: float = 0.0, extent: float = 1.3):
    """Projection, covariance and EWA splat of every Gaussian (and its SH
    colour on the camera's view directions when `shs` [P, C, D] is given)
    in one kernel.  Returns uv [P,2], depth [P,1], conic [P,3], radius [P]
    int32, tiles_touched [P] int32 and colour [P, C] ([P, 0] without shs);
    uv, conic and colour are differentiable."""
    return _Preprocess.apply(xyz, scale, rotate, shs, intr, extr, W, H, nearest, extent)


# Eager fused calls keep the true intersection count of their last call per
# (device, Gaussians, image size), and sort the next call of that shape into
# a capacity above it without waiting for the count (see _sort_and_blend).
_CAP_LOCK = threading.Lock()
_CAP_CACHE: dict = {}
_CAP_MARGIN = 1.15


def _remember(key, count: int) -> None:
    with _CAP_LOCK:
        _CAP_CACHE[key] = min(int(count * _CAP_MARGIN) + 3072, 2**31 - 1)


def _sort_and_blend(uv, depth, conic, opacity, feature, radius, tiles, W, H, bg, ndc, capacity, status):
    """Sort and blend of the fused calls, which sort culled lists: only the
    image and gradients leave them, and those equal the reference lists'
    (see sort_gaussian's cull).  With a capacity (CUDA-graph capture) the
    caller's; eagerly, the first call of a shape reads the intersection
    count before it allocates the lists, later calls sort into the
    capacity their shape's last count suggests and check the true count
    only after the blend is enqueued -- the wait covers the sort's prepare
    alone, so the device never idles for it -- and redo the sort and blend
    exactly in the rare case that it did not fit (the result is the same
    either way)."""
    cull = (conic.detach(), opacity.detach())
    if capacity is not None:
        if status is None:
            raise RuntimeError("a capacity-bounded sort needs a status tensor to report overflow in")
        idx, tr = sort_gaussian_capacity(uv, depth, W, H, radius, tiles, capacity, status, cull=cull)
        return alpha_blending(uv, conic, opacity, feature, idx, tr, bg, W, H, ndc)
    key = (uv.device, uv.shape[0], int(W), int(H))
    with _CAP_LOCK:
        cap = _CAP_CACHE.get(key)
    if cap is not None and uv.is_cuda:
        flag = torch.empty(1, dtype=torch.int32, device=uv.device)
        idx, tr, pending = sort_gaussian_capacity(uv, depth, W, H, radius, tiles, cap, flag, cull=cull,
                                                  deferred=True)
        img = alpha_blending(uv, conic, opacity, feature, idx, tr, bg, W, H, ndc)
        count, mismatch = pending.result()
        _remember(key, count)
        if count <= cap and mismatch == 0:
            return img
    idx, tr = sort_gaussian(uv, depth, W, H, radius, tiles, cull=cull)
    _remember(key, idx.numel())
    return alpha_blending(uv, conic, opacity, feature, idx, tr, bg, W, H, ndc)


def rasterization(xyz: Tensor, scale: Tensor, rotate: Tensor, opacity: Tensor, feature: Tensor, intr: Tensor,
                  extr: Tensor, W: int, H: int, bg: float, ndc: Tensor = None, *, return_radius: bool = False,
                  capacity: int | None = None, status: Tensor | None = None):
    """3-D Gaussian splatting of `feature` (msplat/__init__.py:22-93).

    xyz [P,3], scale [P,3], rotate [P,4] unit quaternions (r,x,y,z),
    opacity [P,1], feature [P,C], intr [4] = (fx,fy,cx,cy), extr [3,4]
    world-to-camera, image W x H, scalar background `bg`; `ndc` [P,2]
    optionally receives dL/duv * (W/2, H/2).  Returns [C, H, W], and with
    return_radius=True also the screen radius [P] int32 (0 = not drawn),
    for density statistics.

    With `capacity` (intersections) and `status` ([1] int32 CUDA tensor) the
    frame makes no host read, so it can be captured in a CUDA graph; status
    becomes 1 on the device if the capacity was too small (or the sort
    needed the reference layout), and the frame must then be redone without
    a capacity.
    """
    uv, depth, conic, radius, tiles, _ = preprocess(xyz, scale, rotate, intr, extr, W, H)
    img = _sort_and_blend(uv, depth, conic, opacity, feature, radius, tiles, W, H, bg, ndc, capacity, status)
    return (img, radius) if return_radius else img


def rasterization_sh(xyz: Tensor, scale: Tensor, rotate: Tensor, opacity: Tensor, shs: Tensor, intr: Tensor,
                     extr: Tensor, W: int, H: int, bg: float, ndc: Tensor = None, *, return_radius: bool = False,
                     capacity: int | None = None, status: Tensor | None = None):
    """`rasterization` of the colour compute_sh(shs, view directions) with
    the view directions d = (xyz - c) / |xyz - c| of the camera centre
    c = -R^T t, evaluated inside the preprocess kernel; gradients flow into
    shs and, through d, into xyz and extr.  shs is [P, C, D] with
    D = (degree + 1)^2, degree <= 10.  Returns [C, H, W] (and the radius
    [P] with return_radius=True).  `capacity` / `status` as for
    `rasterization`."""
    uv, depth, conic, radius, tiles, color = preprocess(xyz, scale, rotate, intr, extr, W, H, shs=shs)
    img = _sort_and_blend(uv, depth, conic, opacity, color, radius, tiles, W, H, bg, ndc, capacity, status)
    return (img, radius) if return_radius else img
