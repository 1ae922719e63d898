"""Seeded synthetic scenes with the distributions of the benchmark configs:
xyz ~ U[-1,1]^3, scales = exp(U[-5,-3]), normalised N(0,1) quaternions,
opacity = sigmoid(N(0,1)), features U[0,1], cameras on a radius-4 sphere
looking at the origin (OpenCV: rows of R = right, down, forward)."""
import math

import numpy as np
import torch


def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)):
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    if np.linalg.norm(r) < 1e-8:
        r = np.cross(f, np.array([1.0, 0.0, 0.0]))
    r /= np.linalg.norm(r)
    d = np.cross(f, r)
    R = np.stack([r, d, f])
    t = -R @ eye
    return np.concatenate([R, t[:, None]], axis=1).astype(np.float32)


def sphere_camera(rng, radius=4.0):
    v = rng.normal(size=3)
    v /= np.linalg.norm(v)
    return look_at(v * radius)


def scene(n, seed=0, C=3, sh_deg=None):
    g = torch.Generator().manual_seed(seed)
    xyz = torch.rand(n, 3, generator=g) * 2 - 1
    scale = torch.exp(torch.rand(n, 3, generator=g) * 2 - 5)
    rot = torch.randn(n, 4, generator=g)
    rot = rot / rot.norm(dim=-1, keepdim=True)
    opacity = torch.sigmoid(torch.randn(n, 1, generator=g))
    feat = torch.rand(n, C, generator=g)
    out = dict(xyz=xyz, scale=scale, rot=rot, opacity=opacity, feat=feat)
    if sh_deg is not None:
        out["shs"] = torch.randn(n, 3, (sh_deg + 1) ** 2, generator=g) * 0.3
    return out


def camera(W, H, f=None, seed=0, front=False):
    f = f if f is not None else 300.0 * W / 256
    intr = np.array([f, f, W / 2, H / 2], np.float32)
    if front:
        extr = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 4]], np.float32)
    else:
        extr = sphere_camera(np.random.default_rng(seed))
    return intr, extr


def to(d, device):
    return {k: (v.to(device) if isinstance(v, torch.Tensor) else v) for k, v in d.items()}
