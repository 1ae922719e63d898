"""GPU outcomes held to the two-branch (guided) oracle.

The GPU evaluates exp, division and square root with the fast
approximations (as the reference's fast-math build does); where a discrete
decision sits within rounding reach of its threshold, either side is a
correct result.  These helpers let the oracle follow the GPU's branch at
exactly those decisions (and nowhere else), then hold every entry --
every pixel, every radius -- to the bar with nothing left out.
"""
import numpy as np
import torch

import oracle

DEV = "cuda"


def _t(x, dtype=None):
    t = torch.as_tensor(np.asarray(x))
    if dtype is not None:
        t = t.to(dtype)
    return t.to(DEV).contiguous()


def gpu_blend_forward(uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H):
    """The library's blend forward through the C ABI: (out, final_T, ncontrib)
    as numpy arrays."""
    from msplat_gb300 import _lib
    lib = _lib.load()
    feature = np.asarray(feature, np.float32)
    P, C = feature.shape
    ins = [_t(uv, torch.float32), _t(conic, torch.float32), _t(np.asarray(opacity, np.float32).reshape(-1)),
           _t(feature), _t(idx_sorted, torch.int32), _t(tile_range, torch.int32)]
    out = torch.empty(C, H, W, device=DEV)
    fT = torch.empty(H, W, device=DEV)
    nc = torch.empty(H, W, dtype=torch.int32, device=DEV)
    _lib.check(lib.msplat_alpha_blending_forward(P, C, *[x.data_ptr() for x in ins], float(bg), W, H,
                                                 out.data_ptr(), fT.data_ptr(), nc.data_ptr(), _lib.stream()),
               "alpha_blending_forward")
    torch.cuda.synchronize()
    return out.cpu().numpy(), fT.cpu().numpy(), nc.cpu().numpy()


def check_blend(gpu_out, gpu_T, gpu_nc, uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H,
                atol=1e-5):
    """Holds a GPU blend outcome to the guided oracle on every pixel: ncontrib
    equal, final T and the image within `atol`.  Returns a dict with the
    number of pixels whose path took an alternate branch, the largest image
    and T errors, and the forces for the guided backward."""
    oout, oT, onc, nfl, forces, unresolved = oracle.alpha_blending_forward_guided(
        uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, gpu_T, gpu_nc)
    assert unresolved == 0, f"{unresolved} pixels: no path within rounding reach explains the GPU's outcome"
    np.testing.assert_array_equal(np.asarray(gpu_nc), onc)
    err = float(np.abs(np.asarray(gpu_out, np.float64) - oout).max()) if oout.size else 0.0
    terr = float(np.abs(np.asarray(gpu_T, np.float64) - oT).max()) if oT.size else 0.0
    assert err <= atol, f"image: max abs err {err:.3e} > {atol} (all pixels)"
    assert terr <= atol, f"final T: max abs err {terr:.3e} > {atol} (all pixels)"
    return {"alternate_pixels": int((nfl > 0).sum()), "pixels": int(nfl.size), "max_err": err, "max_T_err": terr,
            "forces": forces, "final_T": oT, "ncontrib": onc}
