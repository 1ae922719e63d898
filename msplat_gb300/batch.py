"""Multi-camera rendering in one key space.

``rasterization_sh_batch`` / ``rasterization_batch`` render B cameras (any
mix of image sizes) of one scene, ``rasterization_sh_scenes`` B cameras of
several scenes; each returns B images.  The backward sums every parameter
gradient over a scene's cameras and gives each camera its own intrinsic /
extrinsic gradient.  Results are those of B single-camera calls
(``rasterization_sh`` / ``rasterization``): images bit for bit, gradients up
to the order of float atomics.

The whole batch is a handful of launches, whatever B is:
  * one preprocess kernel per scene reads each Gaussian (and its SH rows)
    once and projects it into every camera of that scene
    (msplat_batch_preprocess_forward);
  * one sort orders every camera's intersections by (camera, tile, depth):
    a segmented depth sort of all cameras' Gaussians, then a segmented sort
    by tile of all cameras' lists (msplat_batch_sort_prepare / _finish);
  * one blend grid covers every camera's tiles, forward and backward
    (msplat_batch_alpha_blending_forward / _backward);
  * one adjoint kernel per scene sums the per-camera gradients per Gaussian
    (msplat_batch_preprocess_backward).
With a `capacity` (the padded intersection count the sort may use) and a
`status` tensor the call makes no host read, so a whole batched forward +
backward can be captured in one CUDA graph.
"""
from __future__ import annotations

import threading
from typing import Sequence

import numpy as np
import torch
from torch import Tensor

from . import _lib
from . import _tensors as tt
from .alpha_blending import zeroed_views

SORT_TILE = 3072  # items per sort tile: capacities are multiples of it

_PLANS: dict = {}
_TLS = threading.local()


def last_capacity() -> int | None:
    """The padded intersection count the last eager batched call on this
    thread sorted (a capacity that fits the same batch under capture)."""
    return getattr(_TLS, "last_capacity", None)


class _Plan:
    """A batch's layout (msplat_batch_plan) on the host and on the device.
    Cached per (device, sizes, scene sizes, opacity offsets), so a call under
    stream capture (after a warm-up call) makes no host-to-device copy."""

    def __init__(self, dev, dims, npoints, op_off):
        lib = _lib.load()
        B = len(dims)
        nbytes = int(lib.msplat_batch_plan_bytes(B))
        host = np.zeros(nbytes, np.uint8)
        sizes = np.zeros(5, np.int64)
        d = np.ascontiguousarray(np.asarray(dims, np.int32).reshape(B, 2))
        n = np.ascontiguousarray(np.asarray(npoints, np.int32))
        o = np.ascontiguousarray(np.asarray(op_off, np.int64))
        _lib.check(lib.msplat_batch_plan(B, d.ctypes.data, n.ctypes.data, o.ctypes.data, host.ctypes.data, nbytes,
                                         sizes.ctypes.data), "batch_plan")
        self.B = B
        self.dims = [(int(w), int(h)) for w, h in d]
        self.tiles, self.rows, self.pixels, self.depth_items, self.passes = (int(x) for x in sizes)
        # digit bits of the last tile-key pass: local keys span [1, largest camera's tile count]
        max_tiles = max((-(-w // 16)) * (-(-h // 16)) for w, h in self.dims)
        self.last_pass_bits = max(1, int(max_tiles).bit_length() - 8 * (self.passes - 1))
        self.row_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))]).tolist()
        self.pix_off = np.concatenate([[0], np.cumsum(d[:, 0].astype(np.int64) * d[:, 1])]).tolist()
        self.device = torch.from_numpy(host).to(dev)


def _plan(dev, dims, npoints, op_off) -> _Plan:
    key = (dev.index if dev.index is not None else torch.cuda.current_device(), tuple(dims), tuple(npoints),
           tuple(op_off))
    p = _PLANS.get(key)
    if p is None:
        if len(_PLANS) > 64:
            _PLANS.clear()
        p = _PLANS[key] = _Plan(dev, dims, npoints, op_off)
    return p


_DIMS: dict = {}


def _dims(sizes, dev: torch.device) -> Tensor:
    """[B, 2] int32 (W, H) on the device, cached per size list."""
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


def padded_capacity(n: int) -> int:
    """A capacity of at least n intersections, as the batched sort needs it
    (a multiple of its sort tile)."""
    return -(-int(n) // SORT_TILE) * SORT_TILE


def _sort(lib, plan, uv, depth, radius, conic, opacity, capacity, status, dev, st):
    """The one-key-space sort; returns (idx_sorted, tile_range)."""
    B = plan.B
    counts = torch.empty(2 + B, dtype=torch.int64, device=dev)
    ws_prep = _lib.workspace(lib.msplat_batch_sort_prepare_workspace_size(B, plan.depth_items), dev)
    with _lib.stage("sort_gaussian_prepare"):
        _lib.check(lib.msplat_batch_sort_prepare(
            _lib.ptr(plan.device), B, plan.depth_items, _lib.ptr(uv), _lib.ptr(depth), _lib.ptr(radius),
            _lib.ptr(conic), _lib.ptr(opacity), _lib.ptr(counts), _lib.ptr(ws_prep), ws_prep.numel(), st),
            "batch_sort_prepare")
    if capacity is None:
        cap = int(counts[1].item())  # the one host read of an eager batch
        _TLS.last_capacity = cap
        if cap > 2**31 - 1:
            raise RuntimeError(f"batched sort: {cap} intersections exceed the int32 range")
        status = None
    else:
        cap = padded_capacity(capacity)
        if status is None:
            raise RuntimeError("a capacity-bounded batched sort needs a status tensor to report overflow in")
        status = tt.i32(status, "status")
    idx = torch.empty((max(cap, 1),), dtype=torch.int32, device=dev)
    tr = torch.empty((plan.tiles, 2), dtype=torch.int32, device=dev)
    ws = _lib.workspace(lib.msplat_batch_sort_finish_workspace_size(B, cap, plan.passes), dev)
    with _lib.stage("sort_gaussian_finish"):
        _lib.check(lib.msplat_batch_sort_finish_bits(
            _lib.ptr(plan.device), B, plan.depth_items, plan.tiles, plan.passes, plan.last_pass_bits, cap,
            _lib.ptr(ws_prep), _lib.ptr(idx), _lib.ptr(tr), _lib.ptr(status), _lib.ptr(ws), ws.numel(), st),
            "batch_sort_finish")
    return idx, tr


class _RasterizeScenes(torch.autograd.Function):
    """Cameras grouped by scene.  meta = (scene sizes per camera group,
    image sizes, bg, SH or feature mode, capacity, status); tensors = per
    scene (xyz, scale, rotate, opacity, shs-or-feature), then intrs, extrs."""

    @staticmethod
    def forward(ctx, meta, *tensors):
        groups, sizes, bg, use_sh, capacity, status = meta
        S = len(groups)
        scene_t = [tensors[5 * s:5 * s + 5] for s in range(S)]
        intrs, extrs = tensors[5 * S], tensors[5 * S + 1]
        B = len(sizes)
        dev = intrs.device
        cams = _cameras(intrs, extrs, B)
        dims = _dims(sizes, dev)
        lib = _lib.load()
        st = _lib.stream(dev)
        prep, P_cam, op_off, ops = [], [], [], []
        off = 0
        for s, (xyz, scale, rot, op, sf) in enumerate(scene_t):
            xyz_c = tt.f32(xyz, "xyz", 3)
            P = xyz_c.shape[0]
            scale_c = tt.f32(scale, "scale", 3)
            rot_c = tt.f32_aligned16(rot, "rotate", 4)
            op_c = tt.f32(op, "opacity").view(-1)
            if op_c.numel() != P or scale_c.shape[0] != P or rot_c.shape[0] != P:
                raise RuntimeError("xyz, scale, rotate and opacity must have the same number of Gaussians")
            sf_c = tt.f32(sf, "shs" if use_sh else "feature")
            if sf_c.shape[0] != P or sf_c.dim() != (3 if use_sh else 2):
                raise RuntimeError(f"{'shs must be [P, C, D]' if use_sh else 'feature must be [P, C]'}, got "
                                   f"{tuple(sf.shape)}")
            prep.append((xyz_c, scale_c, rot_c, op_c, sf_c))
            ops.append(op_c)
            for _ in range(groups[s]):
                P_cam.append(P)
                op_off.append(off)
            off += P
        C = int(prep[0][4].shape[1])
        D = int(prep[0][4].shape[2]) if use_sh else 0
        if any(int(p[4].shape[1]) != C or (use_sh and int(p[4].shape[2]) != D) for p in prep):
            raise RuntimeError("every scene of a batch must have the same channel count (and SH degree)")
        plan = _plan(dev, [(int(w), int(h)) for w, h in sizes], P_cam, op_off)
        op_all = ops[0] if S == 1 else torch.cat(ops)
        R = plan.rows
        uv = torch.empty((R, 2), dtype=torch.float32, device=dev)
        depth = torch.empty((R, 1), dtype=torch.float32, device=dev)
        conic = torch.empty((R, 3), dtype=torch.float32, device=dev)
        radius = torch.empty((R,), dtype=torch.int32, device=dev)
        tiles = torch.empty((R,), dtype=torch.int32, device=dev)
        color = torch.empty((R, C), dtype=torch.float32, device=dev) if use_sh else None
        b0 = 0
        with _lib.stage("batch_preprocess_forward"):
            for s, (xyz_c, scale_c, rot_c, op_c, sf_c) in enumerate(prep):
                Bs, P = groups[s], xyz_c.shape[0]
                if Bs == 0:
                    continue
                r0 = plan.row_off[b0]
                _lib.check(lib.msplat_batch_preprocess_forward(
                    P, Bs, _lib.ptr(xyz_c), _lib.ptr(scale_c), _lib.ptr(rot_c), _lib.ptr(cams[b0:b0 + Bs]),
                    _lib.ptr(dims[b0:b0 + Bs]), 0.0, 1.3, C if use_sh else 0, D, _lib.ptr(sf_c) if use_sh else None,
                    _lib.ptr(uv[r0:]), _lib.ptr(depth[r0:]), _lib.ptr(conic[r0:]), _lib.ptr(radius[r0:]),
                    _lib.ptr(tiles[r0:]), _lib.ptr(color[r0:]) if use_sh else None, st), "batch_preprocess_forward")
                b0 += Bs
        # features: per camera (SH colour, stacked like uv) or per scene
        feat = color if use_sh else (prep[0][4] if S == 1 else torch.cat([p[4] for p in prep]))
        idx, tr = _sort(lib, plan, uv, depth, radius, conic, op_all, capacity, status, dev, st)
        out = torch.empty((C * plan.pixels,), dtype=torch.float32, device=dev)
        final_T = torch.empty((plan.pixels,), dtype=torch.float32, device=dev)
        ncontrib = torch.empty((plan.pixels,), dtype=torch.int32, device=dev)
        # the forward keeps each list entry's warp-block mask for the backward
        masks = None
        if C <= 4 and any(ctx.needs_input_grad[1:]):
            masks = torch.empty((max(idx.numel(), 1),), dtype=torch.uint8, device=dev)
        with _lib.stage("alpha_blending_forward"):
            _lib.check(lib.msplat_batch_alpha_blending_forward_masks(
                _lib.ptr(plan.device), B, plan.tiles, C, 1 if use_sh else 0, _lib.ptr(uv), _lib.ptr(conic),
                _lib.ptr(op_all), _lib.ptr(feat), _lib.ptr(idx), _lib.ptr(tr), float(bg), _lib.ptr(out),
                _lib.ptr(final_T), _lib.ptr(ncontrib), _lib.ptr(masks), st), "batch_alpha_blending_forward")
        ctx.masks = masks
        imgs = tuple(out[C * plan.pix_off[b]:C * plan.pix_off[b + 1]].view(C, h, w)
                     for b, (w, h) in enumerate(plan.dims))
        ctx.meta = (groups, plan, bg, use_sh, C, D)
        ctx.intr_shape, ctx.extr_shape = intrs.shape, extrs.shape
        ctx.op_shapes = [t[3].shape for t in scene_t]
        flat = [x for p in prep for x in p]
        ctx.save_for_backward(*flat, cams, uv, depth, conic, radius, color, feat, op_all, idx, tr, final_T, ncontrib)
        return imgs

    @staticmethod
    def backward(ctx, *grads):
        groups, plan, bg, use_sh, C, D = ctx.meta
        S = len(groups)
        saved = ctx.saved_tensors
        prep = [saved[5 * s:5 * s + 5] for s in range(S)]
        cams, uv, depth, conic, radius, color, feat, op_all, idx, tr, final_T, ncontrib = saved[5 * S:]
        B, R = plan.B, plan.rows
        dev = cams.device
        lib = _lib.load()
        st = _lib.stream(dev)
        gout = torch.empty((C * plan.pixels,), dtype=torch.float32, device=dev)
        for b, g in enumerate(grads):
            seg = gout[C * plan.pix_off[b]:C * plan.pix_off[b + 1]]
            if g is None:
                seg.zero_()
            else:
                seg.copy_(g.reshape(-1))
        dL_duv, dL_dconic, dL_dop, dL_dfeat = zeroed_views(dev, [(R, 2), (R, 3), (R,), (R, C)])
        with _lib.stage("alpha_blending_backward"):
            _lib.check(lib.msplat_batch_alpha_blending_backward_masks(
                _lib.ptr(plan.device), B, plan.tiles, R, C, 1 if use_sh else 0, _lib.ptr(uv), _lib.ptr(conic),
                _lib.ptr(op_all), _lib.ptr(feat), _lib.ptr(idx), _lib.ptr(tr), float(bg), _lib.ptr(final_T),
                _lib.ptr(ncontrib), _lib.ptr(gout), _lib.ptr(dL_duv), _lib.ptr(dL_dconic), _lib.ptr(dL_dop),
                _lib.ptr(dL_dfeat), _lib.ptr(ctx.masks), st), "batch_alpha_blending_backward")
        n_in = 5 * S + 2
        want_i, want_e = ctx.needs_input_grad[1 + 5 * S], ctx.needs_input_grad[2 + 5 * S]
        dL_dcams = torch.empty((B, 16), dtype=torch.float32, device=dev) if (want_i or want_e) else None
        out = [None] * n_in
        b0 = 0
        with _lib.stage("batch_preprocess_backward"):
            for s, (xyz, scale, rot, op, sf) in enumerate(prep):
                Bs, P = groups[s], xyz.shape[0]
                gx, gs, gr, go, gsh = zeroed_views(dev, [(P, 3), (P, 3), (P, 4), (P,), (P, C, D) if use_sh else (0,)])
                gsh = gsh if use_sh else None
                gf = None
                if Bs > 0:
                    r0, r1 = plan.row_off[b0], plan.row_off[b0 + Bs]
                    ws = _lib.workspace(lib.msplat_batch_preprocess_workspace_size(P, Bs, C if use_sh else 0, D), dev)
                    _lib.check(lib.msplat_batch_preprocess_backward(
                        P, Bs, _lib.ptr(xyz), _lib.ptr(scale), _lib.ptr(rot), _lib.ptr(cams[b0:b0 + Bs]),
                        C if use_sh else 0, D, _lib.ptr(sf) if use_sh else None, _lib.ptr(depth[r0:r1]),
                        _lib.ptr(radius[r0:r1]), _lib.ptr(dL_duv[r0:r1]), _lib.ptr(dL_dconic[r0:r1]),
                        _lib.ptr(dL_dfeat[r0:r1]) if use_sh else None, _lib.ptr(dL_dop[r0:r1]), _lib.ptr(gx),
                        _lib.ptr(gs), _lib.ptr(gr), _lib.ptr(gsh), _lib.ptr(go),
                        _lib.ptr(dL_dcams[b0:b0 + Bs]) if dL_dcams is not None else None, _lib.ptr(ws), ws.numel(),
                        st), "batch_preprocess_backward")
                    if not use_sh and ctx.needs_input_grad[1 + 5 * s + 4]:
                        gf = dL_dfeat[r0:r1].view(Bs, P, C).sum(0)
                elif not use_sh:
                    gf = torch.zeros_like(sf)
                out[5 * s:5 * s + 5] = [gx, gs, gr, go.view(ctx.op_shapes[s]), gsh if use_sh else gf]
                b0 += Bs
        if want_i:
            out[5 * S] = dL_dcams[:, :4].reshape(ctx.intr_shape)
        if want_e:
            g = dL_dcams[:, 4:]
            if tuple(ctx.extr_shape[-2:]) == (4, 4):
                g = torch.cat([g, torch.zeros((B, 4), dtype=g.dtype, device=dev)], dim=1)
            out[5 * S + 1] = g.reshape(ctx.extr_shape)
        return (None, *out)


def _apply(scenes, scene_of, intrs, extrs, sizes, bg, use_sh, capacity, status):
    B = len(sizes)
    if len(scene_of) != B:
        raise RuntimeError("scene_of must name a scene for every camera")
    if B == 0:
        return []
    order = sorted(range(B), key=lambda b: int(scene_of[b]))  # cameras grouped by scene (stable)
    groups = [0] * len(scenes)
    for b in order:
        groups[int(scene_of[b])] += 1
    inv = list(order) != list(range(B))
    if inv:
        perm = torch.as_tensor(order, device=intrs.device)
        intrs, extrs = intrs.reshape(B, -1)[perm], extrs.reshape(B, *extrs.shape[-2:])[perm]
        sizes = [sizes[b] for b in order]
    flat = [t for sc in scenes for t in sc]
    meta = (groups, tuple((int(w), int(h)) for w, h in sizes), float(bg), use_sh, capacity, status)
    imgs = _RasterizeScenes.apply(meta, *flat, intrs, extrs)
    if not inv:
        return list(imgs)
    out = [None] * B
    for k, b in enumerate(order):
        out[b] = imgs[k]
    return out


def rasterization_sh_batch(xyz: Tensor, scale: Tensor, rotate: Tensor, opacity: Tensor, shs: Tensor,
                           intrs: Tensor, extrs: Tensor, sizes: Sequence[tuple], bg: float = 0.0, *,
                           capacity: int | None = None, status: Tensor | None = None) -> list:
    """Renders B cameras of one scene with colour from SH coefficients on
    each camera's view directions (``rasterization_sh`` per camera).
    intrs [B, 4], extrs [B, 3, 4], sizes [(W, H)] * B.  Returns B images
    [C, H_b, W_b].  With a `capacity` (intersections the sort may hold over
    all cameras, padded) and a [1] int32 `status` the call makes no host
    read (CUDA-graph capturable); status = 1 marks a capacity that was too
    small (the images are then not valid)."""
    return _apply([(xyz, scale, rotate, opacity, shs)], [0] * len(sizes), intrs, extrs, sizes, bg, True, capacity,
                  status)


def rasterization_batch(xyz: Tensor, scale: Tensor, rotate: Tensor, opacity: Tensor, feature: Tensor,
                        intrs: Tensor, extrs: Tensor, sizes: Sequence[tuple], bg: float = 0.0, *,
                        capacity: int | None = None, status: Tensor | None = None) -> list:
    """Renders B cameras of one scene with the same per-Gaussian features
    (``rasterization`` per camera).  Returns B images [C, H_b, W_b];
    `capacity` / `status` as for ``rasterization_sh_batch``."""
    return _apply([(xyz, scale, rotate, opacity, feature)], [0] * len(sizes), intrs, extrs, sizes, bg, False,
                  capacity, status)


def rasterization_sh_scenes(scenes: Sequence[tuple], scene_of: Sequence[int], intrs: Tensor, extrs: Tensor,
                            sizes: Sequence[tuple], bg: float = 0.0, *, capacity: int | None = None,
                            status: Tensor | None = None) -> list:
    """Renders B cameras of several scenes in one batch: scenes is a list of
    (xyz, scale, rotate, opacity, shs), scene_of[b] the scene of camera b
    (any order).  Returns B images; each scene's parameters get the
    gradients summed over its cameras.  `capacity` / `status` as for
    ``rasterization_sh_batch``."""
    return _apply(list(scenes), list(scene_of), intrs, extrs, sizes, bg, True, capacity, status)
