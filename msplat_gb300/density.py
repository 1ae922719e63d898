"""Density control: statistics gathered after each backward pass, and the
fixed-count prune / densify step of the reference's training loop.

``DensityStats`` accumulates, per Gaussian visible in a frame, the 2-norm
of its screen-space (ndc) gradient, how often it was visible and its
largest screen radius (msplat_density_stats_update).  The ndc gradient is
what ``rasterization(..., ndc=ndc)`` leaves in ``ndc.grad``
(msplat/alpha_blending.py:107-110); the radius comes from
``rasterization(..., return_radius=True)``.

``prune_and_densify`` is tutorials/gs_3d.py:193-225 as a function: the
Gaussians whose activated opacity is below a threshold are replaced by
copies of the same number of Gaussians with the largest scales, so the
count stays fixed.
"""
from __future__ import annotations

import torch

from . import _lib
from . import _tensors as tt


class DensityStats:
    def __init__(self, P: int, device="cuda"):
        self.grad_accum = torch.zeros(P, dtype=torch.float32, device=device)
        self.count = torch.zeros(P, dtype=torch.int32, device=device)
        self.max_radius = torch.zeros(P, dtype=torch.int32, device=device)

    def update(self, dL_dndc: torch.Tensor, radius: torch.Tensor) -> None:
        """Adds one frame: dL_dndc [P, 2] (``ndc.grad``), radius [P] int32."""
        g = tt.f32(dL_dndc, "dL_dndc", 2)
        r = tt.i32(radius, "radius").view(-1)
        P = self.count.numel()
        if g.shape[0] != P or r.numel() != P:
            raise RuntimeError(f"density stats hold {P} Gaussians; got {g.shape[0]} gradients, {r.numel()} radii")
        lib = _lib.load()
        _lib.check(lib.msplat_density_stats_update(P, _lib.ptr(g), _lib.ptr(r), _lib.ptr(self.grad_accum),
                                                   _lib.ptr(self.count), _lib.ptr(self.max_radius),
                                                   _lib.stream(g.device)), "density_stats_update")

    def mean_grad(self) -> torch.Tensor:
        """Average screen-space gradient norm over the frames a Gaussian was
        visible in (0 where it never was)."""
        return self.grad_accum / self.count.clamp(min=1).float()

    def reset(self) -> None:
        self.grad_accum.zero_()
        self.count.zero_()
        self.max_radius.zero_()


@torch.no_grad()
def prune_and_densify(params: dict, opacity_act=torch.sigmoid, threshold: float = 0.01) -> int:
    """The reference's fixed-count step (tutorials/gs_3d.py:193-225): prune
    the Gaussians with opacity_act(opacity) < threshold and fill their slots
    with copies of the same number of Gaussians with the largest maximum
    scale (which keep their own slots, so each is duplicated).  `params`
    maps "xyzs", "opacity", "scales", "rot" and any other per-Gaussian
    tensors (e.g. "rgbs" / "shs") to [P, ...] tensors, changed in place.
    Returns the number of Gaussians replaced."""
    opacity = opacity_act(params["opacity"])
    prune = torch.nonzero(opacity[:, 0] < threshold).squeeze(-1)
    m = prune.numel()
    if m == 0:
        return 0
    densify = torch.argsort(params["scales"].amax(dim=1), descending=True)[:m]
    idx = torch.cat([prune, densify])
    for v in params.values():
        src = v[densify].repeat(2, *([1] * (v.dim() - 1)))
        v.data[idx] = src
    return m
