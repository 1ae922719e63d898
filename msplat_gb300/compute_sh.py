"""Spherical-harmonics colour, degrees 0-10 (drop-in for msplat/compute_sh.py)."""
from __future__ import annotations

import torch
from torch import Tensor

from . import _lib
from . import _tensors as tt


def compute_sh(shs: Tensor, view_dirs: Tensor, visible: Tensor | None = None) -> Tensor:
    """Evaluates real SH with coefficients `shs` along `view_dirs`
    (msplat/compute_sh.py:8-33).

    Parameters
    ----------
    shs : [P, C, D] coefficients, channel-major, D = (deg + 1)^2 <= 121.
    view_dirs : [P, 3] unit directions.
    visible : optional bool [P]; invisible points get zeros.

    Returns
    -------
    value : [P, C].
    """
    if visible is None:
        visible = torch.ones_like(shs[:, 0, 0], dtype=torch.bool)
    return _ComputeSH.apply(shs, view_dirs, visible)


class _ComputeSH(torch.autograd.Function):
    @staticmethod
    def forward(ctx, shs, view_dirs, visible):
        sh = tt.f32(shs, "shs")
        if sh.dim() != 3:
            raise RuntimeError(f"shs must be [P, C, D], got {tuple(shs.shape)}")
        d = tt.f32(view_dirs, "view_dirs", 3)
        P, C, D = sh.shape
        vis = tt.mask(visible, "visible", P)
        out = torch.empty((P, C), dtype=torch.float32, device=sh.device)
        lib = _lib.load()
        with _lib.stage("compute_sh_forward"):
            _lib.check(lib.msplat_compute_sh_forward(
                P, C, D, _lib.ptr(sh), _lib.ptr(d), _lib.ptr(vis), _lib.ptr(out),
                _lib.stream(sh.device)), "compute_sh_forward")
        ctx.save_for_backward(sh, d, vis)
        return out

    @staticmethod
    def backward(ctx, dL_dvalue):
        sh, d, vis = ctx.saved_tensors
        P, C, D = sh.shape
        g = dL_dvalue.float().contiguous()
        dsh = torch.empty_like(sh)
        ddir = torch.empty((P, 3), dtype=torch.float32, device=sh.device)
        lib = _lib.load()
        with _lib.stage("compute_sh_backward"):
            _lib.check(lib.msplat_compute_sh_backward(
                P, C, D, _lib.ptr(sh), _lib.ptr(d), _lib.ptr(vis), _lib.ptr(g), _lib.ptr(dsh),
                _lib.ptr(ddir), _lib.stream(sh.device)), "compute_sh_backward")
        return dsh, ddir, None
