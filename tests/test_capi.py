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
