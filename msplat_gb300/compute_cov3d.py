"""3-D covariance from scale and rotation (drop-in for msplat/compute_cov3d.py)."""
from __future__ import annotations

import torch
from torch import Tensor

from . import _lib
from . import _tensors as tt


def compute_cov3d(scales: Tensor, uquats: Tensor, visible: Tensor | None = None) -> Tensor:
    """Sigma = R S S R^T as its upper triangle (msplat/compute_cov3d.py:7-33).

    Parameters
    ----------
    scales : [P, 3] per-axis scales.
    uquats : [P, 4] unit quaternions (r, x, y, z).
    visible : optional bool [P] or [P, 1]; invisible points get zeros.

    Returns
    -------
    cov3d : [P, 6] = [s00, s01, s02, s11, s12, s22].
    """
    if visible is None:
        visible = torch.ones_like(scales[:, 0], dtype=torch.bool)
    return _ComputeCov3D.apply(scales, uquats, visible)


class _ComputeCov3D(torch.autograd.Function):
    @staticmethod
    def forward(ctx, scales, uquats, visible):
        s = tt.f32(scales, "scales", 3)
        q = tt.f32_aligned16(uquats, "uquats", 4)
        P = s.shape[0]
        vis = tt.mask(visible, "visible", P)
        out = torch.empty((P, 6), dtype=torch.float32, device=s.device)
        lib = _lib.load()
        with _lib.stage("compute_cov3d_forward"):
            _lib.check(lib.msplat_compute_cov3d_forward(
                P, _lib.ptr(s), _lib.ptr(q), _lib.ptr(vis), _lib.ptr(out), _lib.stream(s.device)),
                "compute_cov3d_forward")
        ctx.save_for_backward(s, q, vis)
        return out

    @staticmethod
    def backward(ctx, dL_dcov3d):
        s, q, vis = ctx.saved_tensors
        P = s.shape[0]
        g = dL_dcov3d.float().contiguous()
        ds = torch.empty((P, 3), dtype=torch.float32, device=s.device)
        dq = torch.empty((P, 4), dtype=torch.float32, device=s.device)
        lib = _lib.load()
        with _lib.stage("compute_cov3d_backward"):
            _lib.check(lib.msplat_compute_cov3d_backward(
                P, _lib.ptr(s), _lib.ptr(q), _lib.ptr(vis), _lib.ptr(g), _lib.ptr(ds), _lib.ptr(dq),
                _lib.stream(s.device)), "compute_cov3d_backward")
        return ds, dq, None
