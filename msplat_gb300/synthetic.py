"""Seeded synthetic training scenes with the benchmark's distributions.

xyz ~ U[-1, 1]^3, scales = exp(U[-5, -3]) per axis, normalised N(0, 1)
quaternions, opacity = sigmoid(N(0, 1)), SH coefficients N(0, 0.3) laid out
[N, 3, D]; a look-at camera on a radius-4 sphere around the origin (OpenCV
convention: rows of R = right, down, forward), focal length f, principal
point at the image centre; loss weights W ~ N(0, 1) of the image's shape.
Used by the benchmark and the autotuner so both time the same frame.
"""
from __future__ import annotations

import numpy as np
import torch


def training_scene(n: int, width: int, height: int, focal: float, seed: int = 0, sh_degree: int = 3) -> dict:
    g = torch.Generator().manual_seed(seed)
    xyz = torch.rand(n, 3, generator=g) * 2 - 1
    scale = torch.exp(torch.rand(n, 3, generator=g) * 2 - 5)
    rot = torch.randn(n, 4, generator=g)
    rot = rot / rot.norm(dim=-1, keepdim=True)
    opacity = torch.sigmoid(torch.randn(n, 1, generator=g))
    shs = torch.randn(n, 3, (sh_degree + 1) ** 2, generator=g) * 0.3
    v = torch.randn(3, generator=g, dtype=torch.float64)
    eye = (v / v.norm() * 4.0).numpy()
    f = -eye / np.linalg.norm(eye)
    r = np.cross(f, [0.0, 1.0, 0.0])
    r /= np.linalg.norm(r)
    d = np.cross(f, r)
    R = np.stack([r, d, f])
    extr = torch.tensor(np.concatenate([R, (-R @ eye)[:, None]], 1), dtype=torch.float32)
    intr = torch.tensor([focal, focal, width / 2, height / 2], dtype=torch.float32)
    weights = torch.randn(3, height, width, generator=g)
    return dict(xyz=xyz, scale=scale, rot=rot, opacity=opacity, shs=shs, intr=intr, extr=extr, weights=weights)


def feature_scene(n: int, width: int, height: int, focal: float, seed: int = 1, sh_degree: int = 10,
                  n_features: int = 32) -> dict:
    """The extensible-features scene: `training_scene`'s distributions with SH
    coefficients N(0, 0.1) of degree `sh_degree`, plus `n_features` N(0, 1)
    features per Gaussian; the rendered channels are the SH colour (3), the
    features and the camera-space depth, so the loss weights are
    [3 + n_features + 1, H, W]."""
    s = training_scene(n, width, height, focal, seed=seed, sh_degree=sh_degree)
    g = torch.Generator().manual_seed(seed + 1000)
    s["shs"] = s["shs"] * (0.1 / 0.3)
    s["feats"] = torch.randn(n, n_features, generator=g)
    s["weights"] = torch.randn(3 + n_features + 1, height, width, generator=g)
    return s
