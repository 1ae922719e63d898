"""CPU oracle of the reference rasteriser (numpy in/out over oracle.c).

TEST INFRASTRUCTURE ONLY.  Used by tests/, __graft_entry__.smoke() (as the
checker) and bench.py's CPU baseline / reference arm.  The product
(msplat_gb300) never imports it.  Each function restates a reference stage;
see the citations in oracle.c.  The oracle is pinned against golden vectors
generated from the reference's own PyTorch test implementations
(tests/golden/make_golden.py) and the reference's known-answer sort test.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from .build import LIB, build

_lib = None
_P = ctypes.c_void_p

# FMA contraction pattern of the GPU build (see oracle.c); pinned by
# tests/test_gpu_parity.py::test_fma_mode_is_the_compilers.
FMA_MODE = 0
# Pairing choices inside the covariance code (see oracle.c).
COV_VARIANT = 0


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        i, i64, f = ctypes.c_int, ctypes.c_int64, ctypes.c_float
        sig = {
            "oracle_set_fma_mode": (None, [i]),
            "oracle_get_fma_mode": (i, []),
            "oracle_set_cov_variant": (None, [i]),
            "oracle_set_threads": (None, [i]),
            "oracle_get_threads": (i, []),
            "oracle_project_point_forward": (None, [i, _P, _P, _P, i, i, f, f, _P, _P]),
            "oracle_project_point_backward": (None, [i, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_compute_cov3d_forward": (None, [i, _P, _P, _P, _P]),
            "oracle_compute_cov3d_backward": (None, [i, _P, _P, _P, _P, _P, _P]),
            "oracle_ewa_project_forward": (None, [i, _P, _P, _P, _P, _P, i, i, _P, _P, _P, _P, _P]),
            "oracle_ewa_project_forward_alt": (
                None, [i, _P, _P, _P, _P, _P, i, i, _P, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_ewa_project_backward": (None, [i, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_sh_basis": (None, [i, i, _P, _P, _P]),
            "oracle_compute_sh_forward": (i, [i, i, i, _P, _P, _P, _P]),
            "oracle_compute_sh_backward": (i, [i, i, i, _P, _P, _P, _P, _P, _P]),
            "oracle_num_intersects": (i64, [i, _P]),
            "oracle_sort_gaussian": (i64, [i, _P, _P, i, i, _P, _P, _P, _P, _P]),
            "oracle_alpha_blending_forward": (
                None, [i, i, _P, _P, _P, _P, _P, _P, f, i, i, _P, _P, _P, _P]),
            "oracle_alpha_blending_backward": (
                None, [i, i, _P, _P, _P, _P, _P, _P, f, i, i, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_alpha_blending_forward_guided": (
                i64, [i, i, _P, _P, _P, _P, _P, _P, f, i, i, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_alpha_blending_backward_guided": (
                None, [i, i, _P, _P, _P, _P, _P, _P, f, i, i, _P, _P, _P, _P, _P, _P, _P, _P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib.oracle_set_fma_mode(FMA_MODE)
        lib.oracle_set_cov_variant(COV_VARIANT)
        _lib = lib
    return _lib


def _a(x, dtype):
    return np.ascontiguousarray(np.asarray(x), dtype=dtype)


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _mask(v, P):
    if v is None:
        return None
    return _a(np.asarray(v).reshape(-1), np.uint8)


def set_fma_mode(mode: int) -> None:
    """0: a*b + c*d -> fma(a, b, c*d); 1: fma(c, d, a*b); 2: no FMAs."""
    _load().oracle_set_fma_mode(int(mode))


def set_cov_variant(v: int) -> None:
    _load().oracle_set_cov_variant(int(v))


def set_threads(n: int) -> None:
    """Host threads for the oracle's loops (1, the default, is what every
    parity check uses)."""
    _load().oracle_set_threads(int(n))


def get_threads() -> int:
    """Threads the oracle actually uses (1 when it was built without OpenMP)."""
    return int(_load().oracle_get_threads())


def get_fma_mode() -> int:
    return int(_load().oracle_get_fma_mode())


def ntiles(W, H):
    return ((W + 15) // 16) * ((H + 15) // 16)


# ------------------------------------------------------------ projection
def project_point_forward(xyz, intr, extr, W, H, nearest=0.0, extent=1.3):
    xyz, intr, extr = _a(xyz, np.float32), _a(intr, np.float32), _a(extr, np.float32)
    P = xyz.shape[0]
    uv = np.zeros((P, 2), np.float32)
    depth = np.zeros((P, 1), np.float32)
    _load().oracle_project_point_forward(P, _p(xyz), _p(intr), _p(extr), int(W), int(H), float(nearest),
                                         float(extent), _p(uv), _p(depth))
    return uv, depth


def project_point_backward(xyz, intr, extr, depth, dL_duv, dL_ddepth):
    xyz, intr, extr = _a(xyz, np.float32), _a(intr, np.float32), _a(extr, np.float32)
    depth, gu, gd = _a(depth, np.float32), _a(dL_duv, np.float32), _a(dL_ddepth, np.float32)
    P = xyz.shape[0]
    dxyz = np.zeros((P, 3))
    di = np.zeros(4)
    de = np.zeros(12)
    _load().oracle_project_point_backward(P, _p(xyz), _p(intr), _p(extr), _p(depth), _p(gu), _p(gd),
                                          _p(dxyz), _p(di), _p(de))
    return dxyz, di, de.reshape(3, 4)


# ----------------------------------------------------------------- cov3d
def compute_cov3d_forward(scales, quats, visible=None):
    s, q = _a(scales, np.float32), _a(quats, np.float32)
    P = s.shape[0]
    vis = _mask(visible, P)
    out = np.zeros((P, 6), np.float32)
    _load().oracle_compute_cov3d_forward(P, _p(s), _p(q), _p(vis), _p(out))
    return out


def compute_cov3d_backward(scales, quats, visible, dL_dcov):
    s, q, g = _a(scales, np.float32), _a(quats, np.float32), _a(dL_dcov, np.float32)
    P = s.shape[0]
    vis = _mask(visible, P)
    ds = np.zeros((P, 3))
    dq = np.zeros((P, 4))
    _load().oracle_compute_cov3d_backward(P, _p(s), _p(q), _p(vis), _p(g), _p(ds), _p(dq))
    return ds, dq


# ------------------------------------------------------------------- EWA
def ewa_project_forward(xyz, cov3d, intr, extr, uv, W, H, visible=None):
    xyz, cov = _a(xyz, np.float32), _a(cov3d, np.float32)
    intr, extr, uv = _a(intr, np.float32), _a(extr, np.float32), _a(uv, np.float32)
    P = xyz.shape[0]
    vis = _mask(visible, P)
    conic = np.zeros((P, 3), np.float32)
    radius = np.zeros(P, np.int32)
    tiles = np.zeros(P, np.int32)
    amb = np.zeros(P, np.uint8)
    _load().oracle_ewa_project_forward(P, _p(xyz), _p(cov), _p(intr), _p(extr), _p(uv), int(W), int(H), _p(vis),
                                       _p(conic), _p(radius), _p(tiles), _p(amb))
    return conic, radius, tiles, amb.astype(bool)


def ewa_project_alternatives(xyz, cov3d, intr, extr, uv, W, H, visible=None):
    """Two-branch EWA: the oracle's outcome (conic, radius, tiles) and, where
    the radius is within rounding reach of another integer (or det of 0),
    the other outcome a correct implementation can reach: radius_alt /
    tiles_alt (-1: no alternative; radius_alt 0: invisible) and conic_alt
    (the conic of a visible alternative)."""
    xyz, cov = _a(xyz, np.float32), _a(cov3d, np.float32)
    intr, extr, uv = _a(intr, np.float32), _a(extr, np.float32), _a(uv, np.float32)
    P = xyz.shape[0]
    vis = _mask(visible, P)
    conic = np.zeros((P, 3), np.float32)
    radius = np.zeros(P, np.int32)
    tiles = np.zeros(P, np.int32)
    amb = np.zeros(P, np.uint8)
    ralt = np.zeros(P, np.int32)
    talt = np.zeros(P, np.int32)
    calt = np.zeros((P, 3), np.float32)
    _load().oracle_ewa_project_forward_alt(P, _p(xyz), _p(cov), _p(intr), _p(extr), _p(uv), int(W), int(H),
                                           _p(vis), _p(conic), _p(radius), _p(tiles), _p(amb), _p(ralt), _p(talt),
                                           _p(calt))
    return conic, radius, tiles, ralt, talt, calt


def ewa_check_against(gpu_conic, gpu_radius, gpu_tiles, xyz, cov3d, intr, extr, uv, W, H, visible=None,
                      conic_rtol=2e-5, conic_atol=1e-7):
    """Holds a GPU EWA result to the two-branch oracle: every radius equals
    the oracle's or its alternative rounding, tiles equal the rectangle of
    the radius taken, and conics agree within the tolerances (exactly 0 for
    invisible entries).  Returns (n_alternate, max conic error, the
    oracle's radius / tiles / conic along the GPU's choices); raises
    AssertionError on any other outcome."""
    conic, radius, tiles, ralt, talt, calt = ewa_project_alternatives(xyz, cov3d, intr, extr, uv, W, H, visible)
    gr = np.asarray(gpu_radius).reshape(-1).astype(np.int32)
    gt = np.asarray(gpu_tiles).reshape(-1).astype(np.int32)
    gc = np.asarray(gpu_conic, np.float32).reshape(-1, 3)
    prim = (gr == radius) & (gt == tiles)
    alt = ~prim & (ralt >= 0) & (gr == ralt) & (gt == talt)
    bad = ~(prim | alt)
    assert not bad.any(), (f"{int(bad.sum())} radius/tiles outcomes are neither the oracle's nor its alternative "
                           f"rounding (first at {np.flatnonzero(bad)[:5].tolist()})")
    sel_r = np.where(alt, ralt, radius).astype(np.int32)
    sel_t = np.where(alt, talt, tiles).astype(np.int32)
    sel_c = np.where(alt[:, None], calt, conic).astype(np.float32)
    vis_sel = sel_r > 0
    assert not gc[~vis_sel].any(), "conic of an invisible entry is not 0"
    err = np.abs(gc[vis_sel].astype(np.float64) - sel_c[vis_sel])
    lim = conic_rtol * np.abs(sel_c[vis_sel]).astype(np.float64) + conic_atol
    assert (err <= lim).all(), f"conic beyond {conic_rtol} relative: max err {err.max():.3e}"
    return int(alt.sum()), float(err.max()) if err.size else 0.0, (sel_r, sel_t, sel_c)


def ewa_project_backward(xyz, cov3d, intr, extr, radius, dL_dconic):
    xyz, cov = _a(xyz, np.float32), _a(cov3d, np.float32)
    intr, extr = _a(intr, np.float32), _a(extr, np.float32)
    radius, g = _a(radius, np.int32), _a(dL_dconic, np.float32)
    P = xyz.shape[0]
    dxyz = np.zeros((P, 3))
    dcov = np.zeros((P, 6))
    di = np.zeros(4)
    de = np.zeros(12)
    _load().oracle_ewa_project_backward(P, _p(xyz), _p(cov), _p(intr), _p(extr), _p(radius), _p(g),
                                        _p(dxyz), _p(dcov), _p(di), _p(de))
    return dxyz, dcov, di, de.reshape(3, 4)


# -------------------------------------------------------------------- SH
def sh_basis(dirs, deg):
    """Basis values [n, D] and gradients [n, D, 3] (float64)."""
    d = _a(dirs, np.float64).reshape(-1, 3)
    n = d.shape[0]
    D = (deg + 1) ** 2
    Y = np.zeros((n, D))
    G = np.zeros((n, D, 3))
    _load().oracle_sh_basis(n, int(deg), _p(d), _p(Y), _p(G))
    return Y, G


def compute_sh_forward(shs, dirs, visible=None):
    sh, d = _a(shs, np.float32), _a(dirs, np.float32)
    P, C, D = sh.shape
    vis = _mask(visible, P)
    out = np.zeros((P, C))
    if _load().oracle_compute_sh_forward(P, C, D, _p(sh), _p(d), _p(vis), _p(out)):
        raise ValueError(f"D = {D} is not (deg + 1)^2 for deg <= 10")
    return out


def compute_sh_backward(shs, dirs, visible, dL_dval):
    sh, d, g = _a(shs, np.float32), _a(dirs, np.float32), _a(dL_dval, np.float32)
    P, C, D = sh.shape
    vis = _mask(visible, P)
    dsh = np.zeros((P, C, D))
    dd = np.zeros((P, 3))
    if _load().oracle_compute_sh_backward(P, C, D, _p(sh), _p(d), _p(vis), _p(g), _p(dsh), _p(dd)):
        raise ValueError(f"D = {D} is not (deg + 1)^2 for deg <= 10")
    return dsh, dd


# ------------------------------------------------------------------ sort
def sort_gaussian(uv, depth, W, H, radius, tiles, return_keys=False):
    uv, depth = _a(uv, np.float32), _a(depth, np.float32).reshape(-1)
    radius, tiles = _a(radius, np.int32).reshape(-1), _a(tiles, np.int32).reshape(-1)
    P = uv.shape[0]
    lib = _load()
    I = max(int(lib.oracle_num_intersects(P, _p(tiles))), 0)
    idx = np.zeros(I, np.int32)
    keys = np.zeros(I, np.int64)
    tr = np.zeros((ntiles(W, H), 2), np.int32)
    lib.oracle_sort_gaussian(P, _p(uv), _p(depth), int(W), int(H), _p(radius), _p(tiles), _p(idx), _p(tr),
                             _p(keys))
    return (idx, tr, keys) if return_keys else (idx, tr)


# ----------------------------------------------------------------- blend
def alpha_blending_forward(uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H):
    uv, conic = _a(uv, np.float32), _a(conic, np.float32)
    op, feat = _a(opacity, np.float32).reshape(-1), _a(feature, np.float32)
    ids, tr = _a(idx_sorted, np.int32), _a(tile_range, np.int32)
    P, C = feat.shape
    out = np.zeros((C, H, W), np.float32)
    T = np.zeros((H, W), np.float32)
    nc = np.zeros((H, W), np.int32)
    amb = np.zeros((H, W), np.uint8)
    _load().oracle_alpha_blending_forward(P, C, _p(uv), _p(conic), _p(op), _p(feat), _p(ids), _p(tr), float(bg),
                                          int(W), int(H), _p(out), _p(T), _p(nc), _p(amb))
    return out, T, nc, amb.astype(bool)


def alpha_blending_forward_guided(uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, gpu_T,
                                  gpu_ncontrib):
    """Guided (two-branch) replay of the forward blend: per pixel the path
    whose decisions within rounding reach of a threshold (alpha vs 1/255,
    T (1 - alpha) vs 1e-4) take the fewest alternate branches and whose
    outcome matches the given (final T, ncontrib).  Returns the oracle's
    own out, final_T, ncontrib along those paths, nflips [H, W] (alternate
    branches taken per pixel; 255 = no such path within 3 flips), forces
    (the alternate alpha decisions, for alpha_blending_backward) and the
    number of unresolved pixels."""
    uv, conic = _a(uv, np.float32), _a(conic, np.float32)
    op, feat = _a(opacity, np.float32).reshape(-1), _a(feature, np.float32)
    ids, tr = _a(idx_sorted, np.int32), _a(tile_range, np.int32)
    gT, gnc = _a(gpu_T, np.float32).reshape(H, W), _a(gpu_ncontrib, np.int32).reshape(H, W)
    P, C = feat.shape
    out = np.zeros((C, H, W), np.float32)
    T = np.zeros((H, W), np.float32)
    nc = np.zeros((H, W), np.int32)
    nfl = np.zeros((H, W), np.uint8)
    forces = np.zeros((H, W, 3), np.int32)
    unresolved = _load().oracle_alpha_blending_forward_guided(
        P, C, _p(uv), _p(conic), _p(op), _p(feat), _p(ids), _p(tr), float(bg), int(W), int(H), _p(gT), _p(gnc),
        _p(out), _p(T), _p(nc), _p(nfl), _p(forces))
    return out, T, nc, nfl, forces, int(unresolved)


def alpha_blending_backward(uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, final_T, ncontrib,
                            dL_dout, forces=None):
    uv, conic = _a(uv, np.float32), _a(conic, np.float32)
    op, feat = _a(opacity, np.float32).reshape(-1), _a(feature, np.float32)
    ids, tr = _a(idx_sorted, np.int32), _a(tile_range, np.int32)
    T, nc, g = _a(final_T, np.float32), _a(ncontrib, np.int32), _a(dL_dout, np.float32)
    P, C = feat.shape
    duv = np.zeros((P, 2))
    dcon = np.zeros((P, 3))
    dop = np.zeros(P)
    dfeat = np.zeros((P, C))
    if forces is None:
        _load().oracle_alpha_blending_backward(P, C, _p(uv), _p(conic), _p(op), _p(feat), _p(ids), _p(tr),
                                               float(bg), int(W), int(H), _p(T), _p(nc), _p(g), _p(duv), _p(dcon),
                                               _p(dop), _p(dfeat))
    else:
        f = _a(forces, np.int32)
        _load().oracle_alpha_blending_backward_guided(P, C, _p(uv), _p(conic), _p(op), _p(feat), _p(ids), _p(tr),
                                                      float(bg), int(W), int(H), _p(T), _p(nc), _p(g), _p(f),
                                                      _p(duv), _p(dcon), _p(dop), _p(dfeat))
    return duv, dcon, dop, dfeat


# -------------------------------------------------------------- pipeline
def rasterization_forward(xyz, scale, rotate, opacity, feature, intr, extr, W, H, bg):
    """The reference's rasterization chain (msplat/__init__.py:70-93).
    Returns the image and every intermediate as a dict."""
    uv, depth = project_point_forward(xyz, intr, extr, W, H)
    visible = (depth != 0).reshape(-1)
    cov3d = compute_cov3d_forward(scale, rotate, visible)
    conic, radius, tiles, amb = ewa_project_forward(xyz, cov3d, intr, extr, uv, W, H, visible)
    idx, tr = sort_gaussian(uv, depth, W, H, radius, tiles)
    out, T, nc, bamb = alpha_blending_forward(uv, conic, opacity, feature, idx, tr, bg, W, H)
    return out, dict(uv=uv, depth=depth, visible=visible, cov3d=cov3d, conic=conic, radius=radius, tiles=tiles,
                     ewa_ambiguous=amb, idx_sorted=idx, tile_range=tr, final_T=T, ncontrib=nc,
                     blend_ambiguous=bamb)


__all__ = [n for n in dir() if not n.startswith("_") and n not in ("ctypes", "math", "os", "np")]
