"""Radix passes as one kernel each (histogram + onesweep with decoupled
look-back) against the three-launch passes (upsweep, row scan,
downsweep): identical outputs for every sort of the library -- the
single-camera tile lists (exact and culled, one sort tile up to ~9,000),
the depth sort inside them, the reference-layout int64 sort (signed keys,
constant digits, bit ranges) and the multi-camera one-key-space sort (one
segment per camera, cameras that see nothing); and the look-back's bounded
waits: with a wait limit of zero polls every look-back gives up at once,
the kernel still finishes and the device error word reports
MSPLAT_ERR_TIMEOUT, after which the context is healthy.  Also: sorted ids
outside their rows (what a look-back that gave up could leave) are
skipped by every kernel that gathers with them."""
import ctypes

import numpy as np
import pytest
import torch

from _scenes import scene, sphere_camera

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def lib():
    from msplat_gb300 import _build, _lib
    _build.build()
    lib = _lib.load()
    yield lib
    lib.msplat_set_sort_onesweep(0)  # the default
    lib.msplat_set_wait_limit(1 << 21)


def both(lib, fn):
    """fn() with the one-kernel passes, then with the three-launch passes."""
    out = []
    for on in (1, 0):
        assert lib.msplat_set_sort_onesweep(on) == 0
        out.append(fn())
        torch.cuda.synchronize()
    lib.msplat_set_sort_onesweep(0)  # the default
    return out


def projected(n, W, H, seed):
    import msplat_gb300 as ms
    s = scene(n, seed, C=3)
    f = 300.0 * W / 256
    intr = torch.tensor([f, f, W / 2, H / 2], device=DEV)
    extr = torch.tensor(sphere_camera(np.random.default_rng(seed)), device=DEV)
    xyz, scale, rot = (s[k].to(DEV).contiguous() for k in ("xyz", "scale", "rot"))
    uv, depth, conic, radius, tiles, _ = ms.preprocess(xyz, scale, rot, intr, extr, W, H)
    return uv, depth, conic, radius, tiles, s["opacity"].to(DEV).contiguous()


@pytest.mark.parametrize("n,W,H", [(40, 64, 48), (5000, 256, 192), (200000, 960, 540)])
def test_tile_lists_equal(lib, n, W, H):
    import msplat_gb300 as ms
    uv, depth, conic, radius, tiles, op = projected(n, W, H, 3)
    for cull in (None, (conic, op)):
        (i1, t1), (i0, t0) = both(lib, lambda: ms.sort_gaussian(uv, depth, W, H, radius, tiles, cull=cull))
        assert torch.equal(t1, t0) and torch.equal(i1, i0)
    if n == 200000:
        assert i1.numel() > 10 * 3072  # many sort tiles, so the look-back walks


@pytest.mark.parametrize("case", ["signed", "constant_digits", "bit_range"])
def test_int64_sort_equal(lib, case):
    from msplat_gb300 import _lib
    rng = np.random.default_rng(7)
    n, lo, hi = 150_001, 0, 64
    if case == "signed":
        keys = rng.integers(-2**40, 2**40, size=n, dtype=np.int64)
    elif case == "constant_digits":
        keys = rng.integers(0, 2**20, size=n, dtype=np.int64)
    else:
        keys = rng.integers(0, 2**44, size=n, dtype=np.int64) << 8
        lo, hi = 8, 52
    m = len(keys[2::5])
    keys[0:5 * m:5] = keys[2::5]  # duplicates
    tk = torch.from_numpy(keys).to(DEV)
    tv = torch.arange(n, dtype=torch.int32, device=DEV)

    def run():
        ko, vo = torch.empty_like(tk), torch.empty_like(tv)
        ws = _lib.workspace(lib.msplat_radix_sort_i64_workspace_size(n), tk.device)
        _lib.check(lib.msplat_radix_sort_i64_pairs(n, tk.data_ptr(), tv.data_ptr(), ko.data_ptr(), vo.data_ptr(), lo,
                                                   hi, ws.data_ptr(), ws.numel(), _lib.stream()), "sort")
        return ko, vo

    (k1, v1), (k0, v0) = both(lib, run)
    assert torch.equal(k1, k0) and torch.equal(v1, v0)
    order = np.argsort(keys if case != "bit_range" else (keys >> 8), kind="stable")
    np.testing.assert_array_equal(v1.cpu().numpy(), order.astype(np.int32))


def covered(tr, n):
    """Mask of the list positions some tile range covers."""
    m = torch.zeros(n + 1, dtype=torch.int32, device=tr.device)
    nz = tr[:, 1] > tr[:, 0]
    m.index_add_(0, tr[nz, 0].long(), torch.ones_like(tr[nz, 0]))
    m.index_add_(0, tr[nz, 1].long(), -torch.ones_like(tr[nz, 1]))
    return torch.cumsum(m, 0)[:n] > 0


def test_batch_sort_equal(lib, monkeypatch):
    """One segment per camera, including a camera that sees no Gaussian
    (an empty segment) and cameras whose keys need one pass and two."""
    import msplat_gb300 as ms
    import msplat_gb300.batch as mb
    s = scene(60000, 5, C=3, sh_deg=1)
    sizes = [(960, 540), (128, 128), (320, 240), (256, 256)]
    rng = np.random.default_rng(2)
    intrs, extrs = [], []
    for w, h in sizes:
        f = 300.0 * w / 256
        intrs.append([f, f, w / 2, h / 2])
        extrs.append(sphere_camera(rng))
    extrs[1] = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, -50.0]])  # looks away from the scene
    intrs = torch.tensor(intrs, dtype=torch.float32, device=DEV)
    extrs = torch.tensor(np.stack(extrs), dtype=torch.float32, device=DEV)
    p = {k: s[k].to(DEV).contiguous() for k in ("xyz", "scale", "rot", "opacity", "shs")}
    rec = []
    orig = mb._sort

    def spy(*a, **k):
        idx, tr = orig(*a, **k)
        rec.append((idx.clone(), tr.clone()))
        return idx, tr

    monkeypatch.setattr(mb, "_sort", spy)

    def run():
        with torch.no_grad():
            return ms.rasterization_sh_batch(p["xyz"], p["scale"], p["rot"], p["opacity"], p["shs"], intrs, extrs,
                                             sizes, 0.0)

    img1, img0 = both(lib, run)
    (i1, t1), (i0, t0) = rec
    assert torch.equal(t1, t0)
    m = covered(t1, i1.numel())
    assert int(m.sum()) > 10 * 3072
    assert torch.equal(i1[m], i0[m])
    for a, b in zip(img1, img0):
        assert torch.equal(a, b)


def test_lookback_wait_that_runs_out_reports_timeout(lib):
    """The forced expiry runs on the standalone int64 sort, whose outputs no
    kernel gathers with (a look-back that gives up leaves its output
    positions wrong, though in bounds; the library's own consumers of
    sorted ids skip ids outside their rows all the same)."""
    from msplat_gb300 import _lib
    n = 300_000
    rng = np.random.default_rng(3)
    keys = rng.integers(-2**40, 2**40, size=n, dtype=np.int64)
    tk = torch.from_numpy(keys).to(DEV)
    tv = torch.arange(n, dtype=torch.int32, device=DEV)

    def run():
        ko, vo = torch.empty_like(tk), torch.empty_like(tv)
        ws = _lib.workspace(lib.msplat_radix_sort_i64_workspace_size(n), tk.device)
        _lib.check(lib.msplat_radix_sort_i64_pairs(n, tk.data_ptr(), tv.data_ptr(), ko.data_ptr(), vo.data_ptr(), 0,
                                                   64, ws.data_ptr(), ws.numel(), _lib.stream()), "sort")
        torch.cuda.synchronize()
        return ko, vo

    err = ctypes.c_int(0)
    assert lib.msplat_wait_error(1, ctypes.byref(err), _lib.stream()) == 0  # clear
    lib.msplat_set_sort_onesweep(1)
    lib.msplat_set_wait_limit(0)  # every look-back gives up before its first poll
    try:
        run()
    finally:
        lib.msplat_set_wait_limit(1 << 21)
        lib.msplat_set_sort_onesweep(0)  # the default
    assert lib.msplat_wait_error(1, ctypes.byref(err), _lib.stream()) == 6  # MSPLAT_ERR_TIMEOUT
    assert err.value == 1
    assert lib.msplat_wait_error(0, ctypes.byref(err), _lib.stream()) == 0 and err.value == 0
    # the context is healthy and the next sort is right again
    lib.msplat_set_sort_onesweep(1)
    ko, vo = run()
    lib.msplat_set_sort_onesweep(0)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(ko.cpu().numpy(), keys[order])
    np.testing.assert_array_equal(vo.cpu().numpy(), order.astype(np.int32))
    assert lib.msplat_wait_error(0, ctypes.byref(err), _lib.stream()) == 0


@pytest.mark.parametrize("C", [3, 6])
def test_blend_skips_ids_outside_the_rows(lib, C):
    """Tiles whose list holds only ids outside [0, P) render as empty tiles
    (the gathers test every id before reading with it), forward and
    backward, in the C <= 4 kernels and the general ones."""
    import msplat_gb300 as ms
    W, H = 320, 240
    uv, depth, conic, radius, tiles, op = projected(20000, W, H, 6)
    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles, cull=(conic, op))
    P = uv.shape[0]
    feat = torch.rand(P, C, device=DEV)
    hit = torch.nonzero(tr[:, 1] > tr[:, 0]).flatten()[::5]
    assert hit.numel() > 20
    bad, empty = idx.clone(), tr.clone()
    for k, t in enumerate(hit.tolist()):
        bad[tr[t, 0]:tr[t, 1]] = P + 1000 if k % 2 else -7
        empty[t] = 0
    w = torch.randn(C, H, W, generator=torch.Generator().manual_seed(1)).to(DEV)
    res = []
    for lists in ((bad, tr), (idx, empty)):
        p = [x.detach().clone().requires_grad_() for x in (uv, conic, op, feat)]
        img = ms.alpha_blending(*p, lists[0], lists[1], 0.25, W, H)
        (img * w).sum().backward()
        res.append((img.detach(), [x.grad for x in p]))
    assert torch.equal(res[0][0], res[1][0])
    for a, b in zip(res[0][1], res[1][1]):
        scale = max(b.abs().max().item(), 1e-30)
        assert (a - b).abs().max().item() <= 1e-5 * scale
