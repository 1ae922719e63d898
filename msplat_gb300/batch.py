"""Multi-camera rendering of one scene in one call.

``rasterization_sh_batch`` / ``rasterization_batch`` render B cameras (any
mix of image sizes) of the same Gaussians and return B images; their
backward sums every parameter gradient over the cameras and gives each
camera its own intrinsic / extrinsic gradient.  Results are those of B
single-camera calls (``rasterization_sh`` / ``rasterization``).

What is shared across the cameras: one preprocess kernel reads each
Gaussian (and its SH rows) once and projects it into every camera
(msplat_batch_preprocess_forward); one adjoint kernel sums the per-camera
gradients per Gaussian (msplat_batch_preprocess_backward); the B tile
sorts read their intersection counts with one host synchronisation.  The
sort and blend of each camera run as in the single-camera path, spread over
four side streams so that small cameras overlap on the device.
"""
from __future__ import annotations

import threading
from typing import Sequence

import torch
from torch import Tensor

from . import _lib
from . import _tensors as tt
from .sort_gaussian import sort_gaussian_many


_TLS = threading.local()
N_SIDE_STREAMS = 4


def side_streams(dev: torch.device) -> list:
    """Streams on which the cameras' sorts and blends overlap (camera b on
    stream b % N_SIDE_STREAMS); one set per device and host thread, so
    concurrent callers (the server's workers) do not wait on each other."""
    key = dev.index if dev.index is not None else torch.cuda.current_device()
    cache = getattr(_TLS, "streams", None)
    if cache is None:
        cache = _TLS.streams = {}
    if key not in cache:
        cache[key] = [torch.cuda.Stream(device=dev) for _ in range(N_SIDE_STREAMS)]
    return cache[key]


def _fork(streams: list, dev) -> torch.cuda.Stream:
    """Makes every side stream wait for the work so far on the current one."""
    main = torch.cuda.current_stream(dev)
    ev = torch.cuda.Event()
    ev.record(main)
    for s in streams:
        s.wait_event(ev)
    return main


def _join(main: torch.cuda.Stream, streams: list) -> None:
    for s in streams:
        main.wait_stream(s)


_DIMS: dict = {}


def _dims(sizes, dev: torch.device) -> Tensor:
    """[B, 2] int32 (W, H) on the device, cached per size list so that a call
    under stream capture (after a warm-up call) makes no host-to-device
    copy."""
    key = (dev.index if dev.index is not None else torch.cuda.current_device(),
           tuple((int(w), int(h)) for w, h in sizes))
    if key not in _DIMS:
        if len(_DIMS) > 64:
            _DIMS.clear()
        _DIMS[key] = torch.tensor([list(k) for k in key[1]], dtype=torch.int32, device=dev)
    return _DIMS[key]


def _cameras(intrs: Tensor, extrs: Tensor, B: int):
    intrs = tt.f32(intrs, "intrs")
    extrs = tt.f32(extrs, "extrs")
    if intrs.numel() != 4 * B:
        raise RuntimeError(f"intrs must be [B, 4] with B = {B}, got {tuple(intrs.shape)}")
    e = extrs.reshape(B, -1)
    if e.shape[1] not in (12, 16):
        raise RuntimeError(f"extrs must be [B, 3, 4] or [B, 4, 4], got {tuple(extrs.shape)}")
    return torch.cat([intrs.reshape(B, 4), e[:, :12]], dim=1).contiguous()


class _RasterizeBatch(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, scale, rotate, opacity, shs, feature, intrs, extrs, sizes, bg, capacities=None,
                status=None):
        xyz_c = tt.f32(xyz, "xyz", 3)
        P = xyz_c.shape[0]
        scale_c = tt.f32(scale, "scale", 3)
        rot_c = tt.f32_aligned16(rotate, "rotate", 4)
        op_c = tt.f32(opacity, "opacity")
        if op_c.numel() != P or scale_c.shape[0] != P or rot_c.shape[0] != P:
            raise RuntimeError("xyz, scale, rotate and opacity must have the same number of Gaussians")
        B = len(sizes)
        dev = xyz.device
        cams = _cameras(intrs, extrs, B)
        dims = _dims(sizes, dev)
        if shs is not None:
            shs_c = tt.f32(shs, "shs")
            if shs_c.dim() != 3 or shs_c.shape[0] != P:
                raise RuntimeError(f"shs must be [P, C, D], got {tuple(shs.shape)}")
            C, D, feat_c = int(shs_c.shape[1]), int(shs_c.shape[2]), None
        else:
            feat_c = tt.f32(feature, "feature")
            if feat_c.dim() != 2 or feat_c.shape[0] != P:
                raise RuntimeError(f"feature must be [P, C], got {tuple(feature.shape)}")
            shs_c, C, D = None, int(feat_c.shape[1]), 0
        uv = torch.empty((B, P, 2), dtype=torch.float32, device=dev)
        depth = torch.empty((B, P, 1), dtype=torch.float32, device=dev)
        conic = torch.empty((B, P, 3), dtype=torch.float32, device=dev)
        radius = torch.empty((B, P), dtype=torch.int32, device=dev)
        tiles = torch.empty((B, P), dtype=torch.int32, device=dev)
        color = torch.empty((B, P, C), dtype=torch.float32, device=dev) if shs_c is not None else None
        lib = _lib.load()
        st = _lib.stream(dev)
        with _lib.stage("batch_preprocess_forward"):
            _lib.check(lib.msplat_batch_preprocess_forward(
                P, B, _lib.ptr(xyz_c), _lib.ptr(scale_c), _lib.ptr(rot_c), _lib.ptr(cams), _lib.ptr(dims),
                0.0, 1.3, C if shs_c is not None else 0, D, _lib.ptr(shs_c), _lib.ptr(uv), _lib.ptr(depth),
                _lib.ptr(conic), _lib.ptr(radius), _lib.ptr(tiles), _lib.ptr(color), st),
                "batch_preprocess_forward")
        streams = side_streams(dev)
        # culled lists, as the single-camera calls (same images and gradients)
        sorted_ = sort_gaussian_many([(uv[b], depth[b], int(w), int(h), radius[b], tiles[b], conic[b], op_c)
                                      for b, (w, h) in enumerate(sizes)], streams, capacities, status)
        outs, finals = [], []
        main = _fork(streams, dev)
        with _lib.stage("alpha_blending_forward"):
            for b, (w, h) in enumerate(sizes):
                w, h = int(w), int(h)
                feat_b = color[b] if color is not None else feat_c
                idx, tr = sorted_[b]
                with torch.cuda.stream(streams[b % len(streams)]):
                    out = torch.empty((C, h, w), dtype=torch.float32, device=dev)
                    final_T = torch.empty((h, w), dtype=torch.float32, device=dev)
                    ncontrib = torch.empty((h, w), dtype=torch.int32, device=dev)
                    if C > 0:
                        _lib.check(lib.msplat_alpha_blending_forward(
                            P, C, _lib.ptr(uv[b]), _lib.ptr(conic[b]), _lib.ptr(op_c), _lib.ptr(feat_b),
                            _lib.ptr(idx), _lib.ptr(tr), float(bg), w, h, _lib.ptr(out), _lib.ptr(final_T),
                            _lib.ptr(ncontrib), _lib.stream(dev)), "alpha_blending_forward")
                    for x in (out, final_T, ncontrib):
                        x.record_stream(main)
                outs.append(out)
                finals.append((final_T, ncontrib))
        _join(main, streams)
        ctx.sizes, ctx.bg, ctx.C, ctx.D = [(int(w), int(h)) for w, h in sizes], float(bg), C, D
        ctx.sorted, ctx.finals = sorted_, finals
        ctx.intr_shape, ctx.extr_shape, ctx.op_shape = intrs.shape, extrs.shape, opacity.shape
        ctx.save_for_backward(xyz_c, scale_c, rot_c, op_c, shs_c, feat_c, cams, uv, depth, conic, radius, color)
        return tuple(outs)

    @staticmethod
    def backward(ctx, *grads):
        xyz, scale, rot, op, shs, feat, cams, uv, depth, conic, radius, color = ctx.saved_tensors
        B, P, C, D = len(ctx.sizes), xyz.shape[0], ctx.C, ctx.D
        dev = xyz.device
        lib = _lib.load()
        st = _lib.stream(dev)
        dL_duv = torch.zeros((B, P, 2), dtype=torch.float32, device=dev)
        dL_dconic = torch.zeros((B, P, 3), dtype=torch.float32, device=dev)
        dL_dop = torch.zeros((B, P), dtype=torch.float32, device=dev)
        dL_dcol = torch.zeros((B, P, C), dtype=torch.float32, device=dev)
        streams = side_streams(dev)
        main = _fork(streams, dev)
        with _lib.stage("alpha_blending_backward"):
            for b, (w, h) in enumerate(ctx.sizes):
                g = grads[b]
                if g is None or C == 0:
                    continue
                idx, tr = ctx.sorted[b]
                final_T, ncontrib = ctx.finals[b]
                feat_b = color[b] if color is not None else feat
                with torch.cuda.stream(streams[b % len(streams)]):
                    g = g.float().contiguous()
                    _lib.check(lib.msplat_alpha_blending_backward(
                        P, C, _lib.ptr(uv[b]), _lib.ptr(conic[b]), _lib.ptr(op), _lib.ptr(feat_b), _lib.ptr(idx),
                        _lib.ptr(tr), ctx.bg, w, h, _lib.ptr(final_T), _lib.ptr(ncontrib), _lib.ptr(g),
                        _lib.ptr(dL_duv[b]), _lib.ptr(dL_dconic[b]), _lib.ptr(dL_dop[b]), _lib.ptr(dL_dcol[b]),
                        _lib.stream(dev)), "alpha_blending_backward")
        _join(main, streams)
        want_i, want_e = ctx.needs_input_grad[6], ctx.needs_input_grad[7]
        sh = shs is not None
        dL_dxyz = torch.empty((P, 3), dtype=torch.float32, device=dev)
        dL_dscale = torch.empty((P, 3), dtype=torch.float32, device=dev)
        dL_drot = torch.empty((P, 4), dtype=torch.float32, device=dev)
        dL_dopacity = torch.empty((P,), dtype=torch.float32, device=dev)
        dL_dshs = torch.empty((P, C, D), dtype=torch.float32, device=dev) if sh else None
        dL_dcams = torch.empty((B, 16), dtype=torch.float32, device=dev) if (want_i or want_e) else None
        ws = _lib.workspace(lib.msplat_batch_preprocess_workspace_size(P, B, C if sh else 0, D), dev)
        with _lib.stage("batch_preprocess_backward"):
            _lib.check(lib.msplat_batch_preprocess_backward(
                P, B, _lib.ptr(xyz), _lib.ptr(scale), _lib.ptr(rot), _lib.ptr(cams), C if sh else 0, D,
                _lib.ptr(shs), _lib.ptr(depth), _lib.ptr(radius), _lib.ptr(dL_duv), _lib.ptr(dL_dconic),
                _lib.ptr(dL_dcol) if sh else None, _lib.ptr(dL_dop), _lib.ptr(dL_dxyz), _lib.ptr(dL_dscale),
                _lib.ptr(dL_drot), _lib.ptr(dL_dshs), _lib.ptr(dL_dopacity), _lib.ptr(dL_dcams), _lib.ptr(ws),
                ws.numel(), st), "batch_preprocess_backward")
        dL_dfeature = dL_dcol.sum(0) if (not sh and ctx.needs_input_grad[5]) else None
        dL_dintrs = dL_dcams[:, :4].reshape(ctx.intr_shape) if want_i else None
        dL_dextrs = None
        if want_e:
            g = dL_dcams[:, 4:]
            if ctx.extr_shape[-2:] == (4, 4):
                g = torch.cat([g, torch.zeros((B, 4), dtype=g.dtype, device=dev)], dim=1)
            dL_dextrs = g.reshape(ctx.extr_shape)
        return (dL_dxyz, dL_dscale, dL_drot, dL_dopacity.view(ctx.op_shape), dL_dshs, dL_dfeature, dL_dintrs,
                dL_dextrs, None, None, None, None)


def rasterization_sh_batch(xyz: Tensor, scale: Tensor, rotate: Tensor, opacity: Tensor, shs: Tensor,
                           intrs: Tensor, extrs: Tensor, sizes: Sequence[tuple], bg: float = 0.0, *,
                           capacities: Sequence[int] | None = None, status: Tensor | None = None) -> list:
    """Renders B cameras of one scene with colour from SH coefficients on
    each camera's view directions (``rasterization_sh`` per camera).
    intrs [B, 4], extrs [B, 3, 4], sizes [(W, H)] * B.  Returns B images
    [C, H_b, W_b].  With per-camera intersection `capacities` and a [B]
    int32 `status` the call makes no host read (CUDA-graph capturable);
    status[b] = 1 marks a camera whose capacity was too small."""
    return list(_RasterizeBatch.apply(xyz, scale, rotate, opacity, shs, None, intrs, extrs, tuple(sizes), bg,
                                      capacities, status))


def rasterization_batch(xyz: Tensor, scale: Tensor, rotate: Tensor, opacity: Tensor, feature: Tensor,
                        intrs: Tensor, extrs: Tensor, sizes: Sequence[tuple], bg: float = 0.0, *,
                        capacities: Sequence[int] | None = None, status: Tensor | None = None) -> list:
    """Renders B cameras of one scene with the same per-Gaussian features
    (``rasterization`` per camera).  Returns B images [C, H_b, W_b];
    `capacities` / `status` as for ``rasterization_sh_batch``."""
    return list(_RasterizeBatch.apply(xyz, scale, rotate, opacity, None, feature, intrs, extrs, tuple(sizes), bg,
                                      capacities, status))
