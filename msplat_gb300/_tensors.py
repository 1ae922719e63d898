"""Input checks and layout helpers shared by the step functions.

Errors mirror the reference's ``CHECK_INPUT`` (msplat/include/utils.h:9-10):
a non-CUDA tensor raises ``RuntimeError("<name> must be a CUDA tensor")``.
Dtype and shape problems, which the reference leaves to pybind/torch, raise
``RuntimeError`` too.
"""
from __future__ import annotations

import torch


def cuda(t: torch.Tensor, name: str) -> torch.Tensor:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    return t


def f32(t: torch.Tensor, name: str, last: int | None = None) -> torch.Tensor:
    cuda(t, name)
    if t.dtype != torch.float32:
        raise RuntimeError(f"{name} must be a float32 tensor, got {t.dtype}")
    if last is not None and (t.dim() == 0 or t.shape[-1] != last):
        raise RuntimeError(f"{name} must have trailing dimension {last}, got {tuple(t.shape)}")
    return t.contiguous()


def f32_aligned16(t: torch.Tensor, name: str, last: int | None = None) -> torch.Tensor:
    t = f32(t, name, last)
    if t.data_ptr() % 16 != 0:
        t = t.clone()
    return t


def i32(t: torch.Tensor, name: str) -> torch.Tensor:
    cuda(t, name)
    if t.dtype != torch.int32:
        raise RuntimeError(f"{name} must be an int32 tensor, got {t.dtype}")
    return t.contiguous()


def mask(t: torch.Tensor | None, name: str, P: int) -> torch.Tensor | None:
    if t is None:
        return None
    cuda(t, name)
    if t.dtype != torch.bool:
        raise RuntimeError(f"{name} must be a bool tensor, got {t.dtype}")
    if t.numel() != P:
        raise RuntimeError(f"{name} must have {P} elements, got {t.numel()}")
    return t.contiguous()


def camera(intr: torch.Tensor, extr: torch.Tensor):
    intr = f32(intr, "intr")
    extr = f32(extr, "extr")
    if intr.numel() < 4:
        raise RuntimeError("intr must hold [fx, fy, cx, cy]")
    if extr.numel() < 12:
        raise RuntimeError("extr must hold a [3, 4] (or [4, 4]) world-to-camera matrix")
    return intr, extr


def extr_grad_like(g12: torch.Tensor, extr: torch.Tensor) -> torch.Tensor:
    """The reference returns a [3, 4] extrinsic gradient; for a [4, 4] input
    the bottom row (unused by the projection) gets zero gradient."""
    if extr.numel() == 12:
        return g12.view_as(extr)
    out = torch.zeros_like(extr)
    out.view(-1)[:12] = g12.view(-1)
    return out


def ntiles(W: int, H: int) -> int:
    return ((W + 15) // 16) * ((H + 15) // 16)
