"""ctypes binding of the native library (C ABI in include/msplat_gb300.h).

The library is the only compute path: if it is missing, every op raises.
Tensors cross the boundary as raw device pointers; each call is enqueued on
torch's current CUDA stream.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

from ._build import LIB_PATH

_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_F = ctypes.c_float
_SZ = ctypes.c_size_t

# name -> (restype, argtypes)
_SIGNATURES = {
    "msplat_status_string": (ctypes.c_char_p, [_I]),
    "msplat_last_error": (ctypes.c_char_p, []),
    "msplat_version": (ctypes.c_char_p, []),
    "msplat_kernel_launches": (ctypes.c_ulonglong, []),
    "msplat_project_point_forward": (_I, [_I, _P, _P, _P, _I, _I, _F, _F, _P, _P, _P]),
    "msplat_camera_grad_workspace_size": (_SZ, [_I]),
    "msplat_project_point_backward": (
        _I, [_I, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "msplat_compute_cov3d_forward": (_I, [_I, _P, _P, _P, _P, _P]),
    "msplat_compute_cov3d_backward": (_I, [_I, _P, _P, _P, _P, _P, _P, _P]),
    "msplat_ewa_project_forward": (_I, [_I, _P, _P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P]),
    "msplat_ewa_project_backward": (
        _I, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "msplat_compute_sh_forward": (_I, [_I, _I, _I, _P, _P, _P, _P, _P]),
    "msplat_compute_sh_backward": (_I, [_I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "msplat_compute_gaussian_key": (_I, [_I, _P, _P, _I, _I, _P, _P, _I64, _P, _P, _P]),
    "msplat_compute_tile_gaussian_range": (_I, [_I, _I, _I64, _P, _P, _P]),
    "msplat_scan_workspace_size": (_SZ, [_I]),
    "msplat_inclusive_scan_i32": (_I, [_I, _P, _P, _P, _P, _SZ, _P]),
    "msplat_inclusive_scan_i32_noalloc": (_I, [_I, _P, _P, _P, _P]),
    "msplat_radix_sort_i64_workspace_size": (_SZ, [_I64]),
    "msplat_radix_sort_i64_pairs": (_I, [_I64, _P, _P, _P, _P, _I, _I, _P, _SZ, _P]),
    "msplat_sort_prepare_workspace_size": (_SZ, [_I, _I, _I]),
    "msplat_sort_finish_workspace_size": (_SZ, [_I, _I64, _I, _I]),
    "msplat_sort_gaussian_prepare": (_I, [_I, _P, _P, _P, _P, _I, _I, _P, _P, _SZ, _P]),
    "msplat_sort_gaussian_prepare_culled": (_I, [_I, _P, _P, _P, _P, _P, _P, _I, _I, _P, _P, _SZ, _P]),
    "msplat_sort_gaussian_finish": (
        _I, [_I, _P, _P, _P, _I, _I, _I64, _P, _P, _P, _P, _SZ, _P]),
    "msplat_sort_gaussian_finish_capacity": (
        _I, [_I, _P, _P, _P, _I, _I, _I64, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "msplat_alpha_blending_forward": (
        _I, [_I, _I, _P, _P, _P, _P, _P, _P, _F, _I, _I, _P, _P, _P, _P]),
    "msplat_alpha_blending_backward": (
        _I, [_I, _I, _P, _P, _P, _P, _P, _P, _F, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "msplat_alpha_blending_forward_masks": (
        _I, [_I, _I, _P, _P, _P, _P, _P, _P, _F, _I, _I, _P, _P, _P, _P, _P]),
    "msplat_alpha_blending_backward_masks": (
        _I, [_I, _I, _P, _P, _P, _P, _P, _P, _F, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "msplat_rasterize_preprocess_forward": (
        _I, [_I, _P, _P, _P, _P, _P, _I, _I, _F, _F, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "msplat_rasterize_preprocess_workspace_size": (_SZ, [_I, _I, _I]),
    "msplat_density_stats_update": (_I, [_I, _P, _P, _P, _P, _P, _P]),
    "msplat_batch_preprocess_workspace_size": (_SZ, [_I, _I, _I, _I]),
    "msplat_batch_preprocess_forward": (
        _I, [_I, _I, _P, _P, _P, _P, _P, _F, _F, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "msplat_batch_preprocess_backward": (
        _I, [_I, _I, _P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "msplat_set_blend_ring": (_I, [_I, _I]),
    "msplat_set_blend_ring_bwd": (_I, [_I, _I]),
    "msplat_set_wait_limit": (_I, [_I]),
    "msplat_set_sort_onesweep": (_I, [_I]),
    "msplat_wait_error": (_I, [_I, _P, _P]),
    "msplat_batch_plan_bytes": (_SZ, [_I]),
    "msplat_batch_plan": (_I, [_I, _P, _P, _P, _P, _SZ, _P]),
    "msplat_batch_sort_prepare_workspace_size": (_SZ, [_I, _I64]),
    "msplat_batch_sort_prepare": (_I, [_P, _I, _I64, _P, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "msplat_batch_sort_finish_workspace_size": (_SZ, [_I, _I64, _I]),
    "msplat_batch_sort_finish": (_I, [_P, _I, _I64, _I, _I, _I64, _P, _P, _P, _P, _P, _SZ, _P]),
    "msplat_batch_sort_finish_bits": (_I, [_P, _I, _I64, _I, _I, _I, _I64, _P, _P, _P, _P, _P, _SZ, _P]),
    "msplat_batch_alpha_blending_forward": (
        _I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _F, _P, _P, _P, _P]),
    "msplat_batch_alpha_blending_backward": (
        _I, [_P, _I, _I, _I64, _I, _I, _P, _P, _P, _P, _P, _P, _F, _P, _P, _P, _P, _P, _P, _P, _P]),
    "msplat_batch_alpha_blending_forward_masks": (
        _I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _F, _P, _P, _P, _P, _P]),
    "msplat_batch_alpha_blending_backward_masks": (
        _I, [_P, _I, _I, _I64, _I, _I, _P, _P, _P, _P, _P, _P, _F, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "msplat_rasterize_preprocess_backward": (
        _I, [_I, _P, _P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _SZ, _P]),
}

_lock = threading.Lock()
_lib = None


def exported_names() -> list[str]:
    return list(_SIGNATURES)


def load(path: str | None = None):
    """Loads (once) and returns the native library; raises if it is absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or os.environ.get("MSPLAT_GB300_LIB") or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                f"msplat_gb300 native library not found at {p}; build it with "
                "`python -m msplat_gb300._build` (there is no CPU fallback)")
        lib = ctypes.CDLL(p)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def kernel_launches() -> int:
    """Kernels the native library has launched in this process so far."""
    return int(load().msplat_kernel_launches())


def check(status: int, what: str) -> None:
    if status != 0:
        lib = load()
        detail = lib.msplat_last_error().decode(errors="replace")
        kind = lib.msplat_status_string(status).decode(errors="replace")
        raise RuntimeError(f"{what} failed ({kind}): {detail}")


def ptr(t: torch.Tensor | None):
    return None if t is None else t.data_ptr()


def stream(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def workspace(nbytes: int, device: torch.device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


# ------------------------------------------------------------ stage timing
# Optional per-stage CUDA-event timing of the native calls (off by default;
# bench.py turns it on around its timed region).
_prof: list | None = None


class _Stage:
    __slots__ = ("name", "start")

    def __init__(self, name: str):
        self.name = name
        self.start = None

    def __enter__(self):
        if _prof is not None:
            self.start = torch.cuda.Event(enable_timing=True)
            self.start.record()
        return self

    def __exit__(self, *exc):
        if _prof is not None and self.start is not None:
            end = torch.cuda.Event(enable_timing=True)
            end.record()
            _prof.append((self.name, self.start, end))
        return False


def stage(name: str) -> _Stage:
    return _Stage(name)


def profile_start() -> None:
    global _prof
    _prof = []


def profile_stop() -> dict:
    """Returns {stage: (calls, total_ms)} for the calls since profile_start()."""
    global _prof
    recs, _prof = _prof or [], None
    torch.cuda.synchronize()
    out: dict = {}
    for name, s, e in recs:
        n, ms = out.get(name, (0, 0.0))
        out[name] = (n + 1, ms + s.elapsed_time(e))
    return out
