"""Tile-based alpha blending of sorted 2-D Gaussians
(drop-in for msplat/alpha_blending.py)."""
from __future__ import annotations

import math

import torch
from torch import Tensor

from . import _lib
from . import _tensors as tt


def alpha_blending(
    uv: Tensor,
    conic: Tensor,
    opacity: Tensor,
    feature: Tensor,
    idx_sorted: Tensor,
    tile_range: Tensor,
    bg: float,
    W: int,
    H: int,
    ndc: Tensor | None = None,
) -> Tensor:
    """Blends C feature channels front to back per 16x16 tile
    (msplat/alpha_blending.py:7-52).

    Parameters
    ----------
    uv, conic, opacity : [P, 2], [P, 3], [P, 1] from the projection steps.
    feature : [P, C] any number of channels.
    idx_sorted, tile_range : output of sort_gaussian.
    bg : background value added as T_final * bg.
    ndc : optional [P, 2] tensor that only receives a gradient,
        dL/duv * (W/2, H/2), for density-control statistics.

    Returns
    -------
    feature_map : [C, H, W].
    """
    return _AlphaBlending.apply(uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, ndc)



def zeroed_views(dev, shapes):
    """Zero-filled float32 tensors of the given shapes, carved from one
    allocation (one fill instead of one per tensor), each contiguous and
    starting on a 16-byte boundary."""
    sizes = [math.prod(sh) for sh in shapes]
    offs, total = [], 0
    for n in sizes:
        offs.append(total)
        total += -(-n // 4) * 4
    buf = torch.zeros(max(total, 1), dtype=torch.float32, device=dev)
    return [buf[o:o + n].view(sh) for o, n, sh in zip(offs, sizes, shapes)]

class _AlphaBlending(torch.autograd.Function):
    @staticmethod
    def forward(ctx, uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, ndc):
        u = tt.f32(uv, "uv", 2)
        c = tt.f32(conic, "conic", 3)
        o = tt.f32(opacity, "opacity")
        f = tt.f32(feature, "feature")
        if f.dim() != 2:
            raise RuntimeError(f"feature must be [P, C], got {tuple(feature.shape)}")
        ids = tt.i32(idx_sorted, "idx_sorted")
        tr = tt.i32(tile_range, "tile_range")
        P, C = f.shape
        W, H = int(W), int(H)
        if tr.numel() != 2 * tt.ntiles(W, H):
            raise RuntimeError("tile_range does not match the image size")
        dev = f.device
        out = torch.empty((C, H, W), dtype=torch.float32, device=dev)
        final_T = torch.empty((H, W), dtype=torch.float32, device=dev)
        ncontrib = torch.empty((H, W), dtype=torch.int32, device=dev)
        # With a backward to come (C <= 4) the forward keeps every list
        # entry's warp-block mask for it (one byte per entry), so the
        # backward repeats no cull arithmetic.
        masks = None
        if C <= 4 and any(ctx.needs_input_grad[:4]):
            masks = torch.empty((max(ids.numel(), 1),), dtype=torch.uint8, device=dev)
        if C > 0:
            lib = _lib.load()
            with _lib.stage("alpha_blending_forward"):
                _lib.check(lib.msplat_alpha_blending_forward_masks(
                    P, C, _lib.ptr(u), _lib.ptr(c), _lib.ptr(o), _lib.ptr(f), _lib.ptr(ids),
                    _lib.ptr(tr), float(bg), W, H, _lib.ptr(out), _lib.ptr(final_T),
                    _lib.ptr(ncontrib), _lib.ptr(masks), _lib.stream(dev)), "alpha_blending_forward")
        ctx.W, ctx.H, ctx.bg = W, H, float(bg)
        ctx.has_ndc = ndc is not None
        ctx.masks = masks
        ctx.save_for_backward(u, c, o, f, ids, tr, final_T, ncontrib)
        ctx.opacity_shape = opacity.shape
        return out

    @staticmethod
    def backward(ctx, dL_drendered):
        u, c, o, f, ids, tr, final_T, ncontrib = ctx.saved_tensors
        P, C = f.shape
        dev = f.device
        g = dL_drendered.float().contiguous()
        dL_duv, dL_dconic, dL_dopacity, dL_dfeature = zeroed_views(
            dev, [(P, 2), (P, 3), tuple(ctx.opacity_shape), (P, C)])
        if C > 0 and P > 0:
            lib = _lib.load()
            with _lib.stage("alpha_blending_backward"):
                _lib.check(lib.msplat_alpha_blending_backward_masks(
                    P, C, _lib.ptr(u), _lib.ptr(c), _lib.ptr(o), _lib.ptr(f), _lib.ptr(ids),
                    _lib.ptr(tr), ctx.bg, ctx.W, ctx.H, _lib.ptr(final_T), _lib.ptr(ncontrib),
                    _lib.ptr(g), _lib.ptr(dL_duv), _lib.ptr(dL_dconic), _lib.ptr(dL_dopacity),
                    _lib.ptr(dL_dfeature), _lib.ptr(ctx.masks), _lib.stream(dev)), "alpha_blending_backward")
        dL_dndc = None
        if ctx.has_ndc:
            scale = torch.tensor([0.5 * ctx.W, 0.5 * ctx.H], dtype=u.dtype, device=dev)
            dL_dndc = dL_duv * scale[None, :]
        return dL_duv, dL_dconic, dL_dopacity, dL_dfeature, None, None, None, None, None, dL_dndc
