"""The allocation-free scan entry point against the workspace one.

msplat_inclusive_scan_i32_noalloc exists for callers that cannot allocate
device memory where they call the scan (inside a stream capture, under a
host framework that owns all device allocations, in a real-time loop that
may not call an allocator): it keeps its scratch in a fixed array inside the
library instead of taking a workspace.  This file is collected last so that
a failure here leaves every other test already run.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from msplat_gb300 import _build, _lib
    _build.build()
    return _lib.load()


def _scan_with_workspace(lib, x):
    from msplat_gb300 import _lib
    n = x.numel()
    out = torch.empty_like(x)
    total = torch.empty(1, dtype=torch.int64, device=x.device)
    ws = _lib.workspace(lib.msplat_scan_workspace_size(n), x.device)
    _lib.check(lib.msplat_inclusive_scan_i32(n, x.data_ptr(), out.data_ptr(), total.data_ptr(), ws.data_ptr(),
                                             ws.numel(), _lib.stream()), "inclusive_scan_i32")
    return out, total


def _scan_no_alloc(lib, x):
    from msplat_gb300 import _lib
    n = x.numel()
    out = torch.empty_like(x)
    total = torch.empty(1, dtype=torch.int64, device=x.device)
    _lib.check(lib.msplat_inclusive_scan_i32_noalloc(n, x.data_ptr(), out.data_ptr(), total.data_ptr(),
                                                     _lib.stream()), "inclusive_scan_i32_noalloc")
    return out, total


def test_no_alloc_scan_matches_workspace_scan_on_consecutive_calls(lib):
    rng = np.random.default_rng(7)
    # Two calls in a row on the shared scratch, the second smaller than the
    # first so stale partial sums from the first call would show up.
    for n in (3_000_017, 40_961):
        x = torch.from_numpy(rng.integers(0, 300, size=n, dtype=np.int32)).cuda()
        ref, ref_total = _scan_with_workspace(lib, x)
        got, got_total = _scan_no_alloc(lib, x)
        torch.cuda.synchronize()
        assert torch.equal(got, ref)
        assert int(got_total.item()) == int(ref_total.item()) == int(x.long().sum().item())


def test_no_alloc_scan_rejects_sizes_beyond_its_scratch(lib):
    limit = 64 * 1024 * 1024
    st = lib.msplat_inclusive_scan_i32_noalloc(limit + 1, None, None, None, None)
    assert st == 4  # MSPLAT_ERR_CAPACITY, before any device work
    assert "exceeds the maximum" in lib.msplat_last_error().decode()


def test_no_alloc_scan_at_tile_edges_and_at_its_maximum_size(lib):
    """n = 0 (only the total is written), one full 4096-element tile, one
    element past it, and MSPLAT_SCAN_NOALLOC_MAX_N, which fills every
    partial-sum slot of the fixed array (a 256 MB input)."""
    rng = np.random.default_rng(11)
    limit = 64 * 1024 * 1024
    for n in (0, 4096, 4097, limit):
        x = torch.from_numpy(rng.integers(0, 4, size=n, dtype=np.int32)).cuda()
        ref, ref_total = _scan_with_workspace(lib, x)
        got, got_total = _scan_no_alloc(lib, x)
        torch.cuda.synchronize()
        assert torch.equal(got, ref), n
        assert int(got_total.item()) == int(ref_total.item()) == int(x.long().sum().item()), n
        del x, ref, got
