"""Tile/depth ordering of Gaussian-tile intersections
(drop-in for msplat/sort_gaussian.py)."""
from __future__ import annotations

from typing import Tuple

import torch
from torch import Tensor

from . import _lib
from . import _tensors as tt


def _prepare(lib, P, d, r, t, u, W, H, counts, ws_prep, st, cull):
    """The sort's prepare step; with cull = (conic [P,3], opacity [P,1]) the
    culled one (tile rectangles shrunk to what the Gaussians reach)."""
    if cull is None:
        _lib.check(lib.msplat_sort_gaussian_prepare(
            P, _lib.ptr(d), _lib.ptr(r), _lib.ptr(t), _lib.ptr(u), W, H, _lib.ptr(counts),
            _lib.ptr(ws_prep), ws_prep.numel(), st), "sort_gaussian_prepare")
        return
    conic = tt.f32(cull[0], "conic", 3)
    opacity = tt.f32(cull[1], "opacity")
    if conic.shape[0] != P or opacity.numel() != P:
        raise RuntimeError("conic and opacity must describe the same number of points as uv")
    _lib.check(lib.msplat_sort_gaussian_prepare_culled(
        P, _lib.ptr(d), _lib.ptr(r), _lib.ptr(t), _lib.ptr(u), _lib.ptr(conic), _lib.ptr(opacity), W, H,
        _lib.ptr(counts), _lib.ptr(ws_prep), ws_prep.numel(), st), "sort_gaussian_prepare_culled")


def sort_gaussian(
    uv: Tensor,
    depth: Tensor,
    W: int,
    H: int,
    radius: Tensor,
    tiles: Tensor,
    *,
    cull: Tuple[Tensor, Tensor] | None = None,
) -> Tuple[Tensor, Tensor]:
    """Sorts the intersections by [tile | depth] (msplat/sort_gaussian.py:8-54).

    Returns
    -------
    idx_sorted : [I] int32 Gaussian ids, I = sum(tiles), ordered by tile then
        depth (ties by Gaussian id, as the reference's stable sort).
    tile_range : [ntiles, 2] int32 [start, end) of each tile in idx_sorted.

    One device-to-host read (the intersection count) happens here, as in the
    reference (which reads it twice).

    With cull = (conic [P,3], opacity [P,1]) the lists leave out the tiles a
    Gaussian cannot reach (alpha < 1/255 at every pixel of them) and the
    negative-depth Gaussians: alpha_blending over them gives the same images
    and gradients, with fewer intersections to sort and blend, but the
    lists are not the reference's.
    """
    u = tt.f32(uv, "uv", 2)
    d = tt.f32(depth, "depth")
    r = tt.i32(radius, "radius").view(-1)
    t = tt.cuda(tiles, "tiles")
    if t.dtype != torch.int32:
        t = t.to(torch.int32)
    t = t.contiguous().view(-1)
    P = u.shape[0]
    if d.numel() != P or r.numel() != P or t.numel() != P:
        raise RuntimeError("uv, depth, radius and tiles must describe the same number of points")
    W, H = int(W), int(H)
    dev = u.device
    nt = tt.ntiles(W, H)
    lib = _lib.load()
    st = _lib.stream(dev)
    counts = torch.empty(2, dtype=torch.int64, device=dev)
    ws_prep = _lib.workspace(lib.msplat_sort_prepare_workspace_size(P, W, H), dev)
    with _lib.stage("sort_gaussian_prepare"):
        _prepare(lib, P, d, r, t, u, W, H, counts, ws_prep, st, cull)
    I, n_mismatch = (int(v) for v in counts.tolist())
    if n_mismatch:
        return _sort_reference_layout(u, d, W, H, r, t)
    if I > 2**31 - 1:
        raise RuntimeError(f"sort_gaussian: {I} intersections exceed the int32 range")
    idx_sorted = torch.empty((I,), dtype=torch.int32, device=dev)
    tile_range = torch.empty((nt, 2), dtype=torch.int32, device=dev)
    ws = _lib.workspace(lib.msplat_sort_finish_workspace_size(P, I, W, H), dev)
    with _lib.stage("sort_gaussian_finish"):
        _lib.check(lib.msplat_sort_gaussian_finish(
            P, _lib.ptr(u), _lib.ptr(d), _lib.ptr(r), W, H, I, _lib.ptr(ws_prep),
            _lib.ptr(idx_sorted), _lib.ptr(tile_range), _lib.ptr(ws), ws.numel(), st),
            "sort_gaussian_finish")
    return idx_sorted, tile_range


def _sort_reference_layout(u, d, W, H, r, t):
    """The reference's own sequence for inputs whose tiles[] disagree with
    the rectangles: int32 inclusive scan, key/index emission into zeroed
    buffers, stable signed-int64 sort, tile boundaries."""
    lib = _lib.load()
    dev = u.device
    st = _lib.stream(dev)
    P = u.shape[0]
    cums = torch.empty((P,), dtype=torch.int32, device=dev)
    total = torch.empty(1, dtype=torch.int64, device=dev)
    ws = _lib.workspace(lib.msplat_scan_workspace_size(P), dev)
    _lib.check(lib.msplat_inclusive_scan_i32(P, _lib.ptr(t), _lib.ptr(cums), _lib.ptr(total),
                                             _lib.ptr(ws), ws.numel(), st), "inclusive_scan_i32")
    I = int(cums[-1].item()) if P > 0 else 0  # int32 wrap, as torch.cumsum(dtype=int32)
    I = max(I, 0)
    nt = tt.ntiles(W, H)
    keys = torch.empty((I,), dtype=torch.int64, device=dev)
    idx = torch.empty((I,), dtype=torch.int32, device=dev)
    _lib.check(lib.msplat_compute_gaussian_key(
        P, _lib.ptr(u), _lib.ptr(d), W, H, _lib.ptr(r), _lib.ptr(cums), I, _lib.ptr(keys),
        _lib.ptr(idx), st), "compute_gaussian_key")
    keys_sorted = torch.empty_like(keys)
    idx_sorted = torch.empty_like(idx)
    if I > 0:
        ws = _lib.workspace(lib.msplat_radix_sort_i64_workspace_size(I), dev)
        _lib.check(lib.msplat_radix_sort_i64_pairs(
            I, _lib.ptr(keys), _lib.ptr(idx), _lib.ptr(keys_sorted), _lib.ptr(idx_sorted), 0, 64,
            _lib.ptr(ws), ws.numel(), st), "radix_sort_i64_pairs")
    tile_range = torch.empty((nt, 2), dtype=torch.int32, device=dev)
    _lib.check(lib.msplat_compute_tile_gaussian_range(W, H, I, _lib.ptr(keys_sorted),
                                                      _lib.ptr(tile_range), st),
               "compute_tile_gaussian_range")
    return idx_sorted, tile_range


class DeferredCounts:
    """The prepare's counts (intersections, rectangle mismatches) of a
    capacity-bounded sort, copied to pinned host memory behind an event
    recorded right after the prepare: result() waits for the prepare only,
    not for the work enqueued after it."""

    def __init__(self, counts: Tensor, stream):
        self._host = torch.empty(2, dtype=torch.int64, pin_memory=True)
        self._host.copy_(counts, non_blocking=True)
        self._event = torch.cuda.Event()
        self._event.record(stream)

    def result(self) -> Tuple[int, int]:
        self._event.synchronize()
        return int(self._host[0]), int(self._host[1])


def sort_gaussian_capacity(uv: Tensor, depth: Tensor, W: int, H: int, radius: Tensor, tiles: Tensor,
                           capacity: int, status: Tensor, *,
                           cull: Tuple[Tensor, Tensor] | None = None,
                           deferred: bool = False):
    """`sort_gaussian` without a host read, for stream capture: idx_sorted has
    `capacity` entries (those past the true count are unused; the tile
    ranges index the valid ones) and status (a [1] int32 CUDA tensor) is set
    to 1 on the device when the result is not valid (more intersections than
    the capacity, or tiles[] disagreeing with the rectangles), else 0.
    `cull` as for `sort_gaussian`.  With deferred=True a DeferredCounts is
    returned as a third value (the true counts, readable once the prepare
    has run, for a caller that checks the capacity after enqueueing the
    work that uses the lists)."""
    u = tt.f32(uv, "uv", 2)
    d = tt.f32(depth, "depth")
    r = tt.i32(radius, "radius").view(-1)
    t = tt.cuda(tiles, "tiles")
    if t.dtype != torch.int32:
        t = t.to(torch.int32)
    t = t.contiguous().view(-1)
    st_t = tt.i32(status, "status")
    P = u.shape[0]
    W, H, capacity = int(W), int(H), int(capacity)
    dev = u.device
    lib = _lib.load()
    st = _lib.stream(dev)
    counts = torch.empty(2, dtype=torch.int64, device=dev)
    ws_prep = _lib.workspace(lib.msplat_sort_prepare_workspace_size(P, W, H), dev)
    with _lib.stage("sort_gaussian_prepare"):
        _prepare(lib, P, d, r, t, u, W, H, counts, ws_prep, st, cull)
    pending = DeferredCounts(counts, torch.cuda.current_stream(dev)) if deferred else None
    idx_sorted = torch.empty((capacity,), dtype=torch.int32, device=dev)
    tile_range = torch.empty((tt.ntiles(W, H), 2), dtype=torch.int32, device=dev)
    ws = _lib.workspace(lib.msplat_sort_finish_workspace_size(P, capacity, W, H), dev)
    with _lib.stage("sort_gaussian_finish"):
        _lib.check(lib.msplat_sort_gaussian_finish_capacity(
            P, _lib.ptr(u), _lib.ptr(d), _lib.ptr(r), W, H, capacity, _lib.ptr(counts), _lib.ptr(ws_prep),
            _lib.ptr(idx_sorted), _lib.ptr(tile_range), _lib.ptr(st_t), _lib.ptr(ws), ws.numel(), st),
            "sort_gaussian_finish_capacity")
    if deferred:
        return idx_sorted, tile_range, pending
    return idx_sorted, tile_range

