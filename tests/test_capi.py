"""The C-ABI library loads and exports every entry point include/msplat_gb300.h
declares, with the host-only queries working without a GPU."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "msplat_gb300.h")


def declared_names():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"MSPLAT_API\s+(?:const\s+char\s*\*|int|size_t|unsigned\s+long\s+long)\s*(msplat_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from msplat_gb300 import _build, _lib
    _build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_names()
    assert "msplat_alpha_blending_forward" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    from msplat_gb300._build import LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(msplat_\w+)", out))
    missing = [n for n in declared_names() if n not in exported]
    assert not missing, missing
    # ... and nothing else leaks out of the C ABI.
    others = set(re.findall(r"\sT\s(\w+)", out)) - exported
    assert not [o for o in others if not o.startswith("_")], others


def test_python_binding_covers_the_header(lib):
    from msplat_gb300 import _lib
    assert sorted(_lib.exported_names()) == declared_names()
    for n in declared_names():
        assert getattr(lib, n) is not None


def test_host_queries(lib):
    assert lib.msplat_version().decode() == "0.1.0"
    assert lib.msplat_status_string(0).decode() == "ok"
    assert lib.msplat_status_string(2).decode() == "workspace too small"
    assert lib.msplat_camera_grad_workspace_size(10) >= 16 * 4
    # Workspace sizes grow with the problem and are 256-byte granular.
    a = lib.msplat_sort_prepare_workspace_size(1000, 1920, 1080)
    b = lib.msplat_sort_prepare_workspace_size(1_000_000, 1920, 1080)
    assert 0 < a < b
    f = lib.msplat_sort_finish_workspace_size(1000, 29_000_000, 1920, 1080)
    assert f >= 2 * 4 * 29_000_000
    assert lib.msplat_radix_sort_i64_workspace_size(1 << 20) >= 12 * (1 << 20)
    assert lib.msplat_scan_workspace_size(0) >= 8


def test_argument_errors_are_reported_without_touching_the_device(lib):
    # Negative sizes are rejected before any CUDA call.
    st = lib.msplat_project_point_forward(-1, None, None, None, 10, 10, 0.0, 1.3, None, None, None)
    assert st == 1
    assert "bad sizes" in lib.msplat_last_error().decode()
    st = lib.msplat_compute_sh_forward(-1, 3, 16, None, None, None, None, None)
    assert st == 1


def test_missing_library_fails_loudly(tmp_path):
    from msplat_gb300 import _lib
    with pytest.raises(RuntimeError, match="not found"):
        _lib.load(str(tmp_path / "nope.so"))


def test_ops_require_cuda_tensors():
    import torch
    import msplat_gb300 as ms
    with pytest.raises(RuntimeError, match="must be a CUDA tensor"):
        ms.project_point(torch.zeros(4, 3), torch.ones(4), torch.eye(4)[:3], 8, 8)
    with pytest.raises(RuntimeError, match="must be a CUDA tensor"):
        ms.compute_cov3d(torch.zeros(4, 3), torch.zeros(4, 4))


def test_launch_counter_starts_at_zero_without_gpu_work(lib):
    assert lib.msplat_kernel_launches() == 0


def test_batch_plan_layout_on_the_host(lib):
    """msplat_batch_plan is host-only: tile, row, pixel and padded depth-key
    offsets of a three-camera batch over two scenes."""
    import numpy as np
    B = 3
    dims = np.array([[100, 50], [1920, 1080], [16, 16]], np.int32)
    npts = np.array([5000, 7000, 5000], np.int32)
    opoff = np.array([0, 5000, 0], np.int64)
    nbytes = int(lib.msplat_batch_plan_bytes(B))
    blob = np.zeros(nbytes, np.uint8)
    sizes = np.zeros(5, np.int64)
    st = lib.msplat_batch_plan(B, dims.ctypes.data, npts.ctypes.data, opoff.ctypes.data, blob.ctypes.data, nbytes,
                               sizes.ctypes.data)
    assert st == 0
    tiles = [7 * 4, 120 * 68, 1]
    assert sizes[0] == sum(tiles)
    assert sizes[1] == npts.sum()
    assert sizes[2] == (dims[:, 0].astype(np.int64) * dims[:, 1]).sum()
    assert sizes[3] == 3072 * (2 + 3 + 2)  # each camera's depth keys padded to 3072
    assert sizes[4] == 2  # 8160 tiles: two 8-bit passes
    cams = np.frombuffer(blob[:64 * B].tobytes(), dtype=np.dtype([("W", "i4"), ("H", "i4"), ("gx", "i4"),
                                                                     ("gy", "i4"), ("P", "i4"), ("tile_off", "i4"),
                                                                     ("dtile", "i4"), ("pad0", "i4"),
                                                                     ("row_off", "i8"), ("op_off", "i8"),
                                                                     ("pix_off", "i8"), ("pad1", "i8")]))
    assert list(cams["tile_off"]) == [0, 28, 28 + 8160]
    assert list(cams["row_off"]) == [0, 5000, 12000]
    assert list(cams["op_off"]) == [0, 5000, 0]
    assert list(cams["dtile"]) == [0, 2, 5]
    assert lib.msplat_batch_plan(B, dims.ctypes.data, npts.ctypes.data, None, blob.ctypes.data, nbytes - 1,
                                 sizes.ctypes.data) == 2  # buffer too small
    bad = dims.copy()
    bad[1, 0] = 0
    assert lib.msplat_batch_plan(B, bad.ctypes.data, npts.ctypes.data, None, blob.ctypes.data, nbytes,
                                 sizes.ctypes.data) == 1
