"""The forward blend as a producer / consumer ring (mbarrier hand-off of two
shared-memory slots) against the block-barrier kernel: identical final T,
contributor counts and colours for every variant (2 or 4 producer warps),
single-camera and in the multi-camera grid, on projected scenes and on
strongly elongated, faint 2-D Gaussians; and its bounded waits: with a wait
limit of zero polls every wait gives up at once, the kernel still finishes
and the device error word reports MSPLAT_ERR_TIMEOUT."""
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
    lib.msplat_set_blend_ring(0, 0)
    lib.msplat_set_wait_limit(1 << 21)


def blend(lib, uv, conic, op, feat, idx, tr, bg, W, H):
    from msplat_gb300 import _lib
    P, C = feat.shape
    out = torch.empty(C, H, W, device=DEV)
    T = torch.empty(H, W, device=DEV)
    nc = torch.empty(H, W, dtype=torch.int32, device=DEV)
    _lib.check(lib.msplat_alpha_blending_forward(P, C, uv.data_ptr(), conic.data_ptr(), op.data_ptr(),
                                                 feat.data_ptr(), idx.data_ptr(), tr.data_ptr(), bg, W, H,
                                                 out.data_ptr(), T.data_ptr(), nc.data_ptr(), _lib.stream()), "fwd")
    torch.cuda.synchronize()
    return out, T, nc


def projected(n, W, H, seed, C=3):
    import msplat_gb300 as ms
    s = scene(n, seed, C=C)
    f = 300.0 * W / 256
    intr = torch.tensor([f, f, W / 2, H / 2], device=DEV)
    extr = torch.tensor(sphere_camera(np.random.default_rng(seed)), device=DEV)
    xyz, scale, rot = (s[k].to(DEV).contiguous() for k in ("xyz", "scale", "rot"))
    uv, depth, conic, radius, tiles, _ = ms.preprocess(xyz, scale, rot, intr, extr, W, H)
    op = s["opacity"].to(DEV).contiguous()
    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles, cull=(conic, op))
    return uv, conic, op, s["feat"].to(DEV).contiguous(), idx, tr


@pytest.mark.parametrize("C", [1, 3, 4])
def test_ring_forward_equals_the_barrier_kernel(lib, C):
    W, H = 320, 240
    args = projected(30000, W, H, 11 + C, C=C)
    lib.msplat_set_blend_ring(0, 0)
    ref = blend(lib, *args, 0.3, W, H)
    for np_ in (2, 4):
        assert lib.msplat_set_blend_ring(np_, np_) == 0
        got = blend(lib, *args, 0.3, W, H)
        for a, b in zip(got, ref):
            assert torch.equal(a, b), np_
    lib.msplat_set_blend_ring(0, 0)


def test_ring_forward_on_elongated_faint_gaussians(lib):
    import test_gpu_parity as tgp
    W, H = 320, 240
    uv, conic, op, feat, idx, tr, _ = tgp.elongated_2d(5000, W, H, seed=9)
    t = [torch.as_tensor(x).to(DEV).contiguous() for x in (uv, conic, op.reshape(-1), feat, idx, tr)]
    lib.msplat_set_blend_ring(0, 0)
    ref = blend(lib, *t, 0.5, W, H)
    lib.msplat_set_blend_ring(4, 4)
    got = blend(lib, *t, 0.5, W, H)
    lib.msplat_set_blend_ring(0, 0)
    for a, b in zip(got, ref):
        assert torch.equal(a, b)


def test_ring_in_the_multi_camera_grid(lib):
    import msplat_gb300 as ms
    s = scene(15000, 3, C=3, sh_deg=1)
    sizes = [(160, 120), (96, 96), (200, 104)]
    rng = np.random.default_rng(3)
    intrs = torch.tensor([[300.0 * w / 256, 300.0 * w / 256, w / 2, h / 2] for w, h in sizes], device=DEV)
    extrs = torch.tensor(np.stack([sphere_camera(rng) for _ in sizes]), device=DEV)
    p = [s[k].to(DEV).contiguous() for k in ("xyz", "scale", "rot", "opacity", "shs")]
    with torch.no_grad():
        lib.msplat_set_blend_ring(0, 0)
        ref = ms.rasterization_sh_batch(*p, intrs, extrs, sizes, 0.1)
        lib.msplat_set_blend_ring(0, 2)
        got = ms.rasterization_sh_batch(*p, intrs, extrs, sizes, 0.1)
    lib.msplat_set_blend_ring(0, 0)
    for a, b in zip(got, ref):
        assert torch.equal(a, b)


def test_ring_wait_that_runs_out_reports_timeout(lib):
    import ctypes
    from msplat_gb300 import _lib
    W, H = 128, 96
    args = projected(8000, W, H, 5)
    err = ctypes.c_int(0)
    assert lib.msplat_wait_error(1, ctypes.byref(err), _lib.stream()) == 0  # clear
    lib.msplat_set_blend_ring(4, 4)
    lib.msplat_set_wait_limit(0)  # every wait gives up at once
    try:
        blend(lib, *args, 0.0, W, H)
    finally:
        lib.msplat_set_wait_limit(1 << 21)
    assert lib.msplat_wait_error(1, ctypes.byref(err), _lib.stream()) == 6  # MSPLAT_ERR_TIMEOUT
    assert err.value == 1
    assert lib.msplat_wait_error(0, ctypes.byref(err), _lib.stream()) == 0 and err.value == 0
    # the context is healthy and the next forward is right again
    lib.msplat_set_blend_ring(0, 0)
    ref = blend(lib, *args, 0.0, W, H)
    lib.msplat_set_blend_ring(4, 4)
    got = blend(lib, *args, 0.0, W, H)
    lib.msplat_set_blend_ring(0, 0)
    for a, b in zip(got, ref):
        assert torch.equal(a, b)
    assert lib.msplat_wait_error(0, ctypes.byref(err), _lib.stream()) == 0
