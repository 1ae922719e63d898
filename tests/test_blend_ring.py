"""The blends as producer / consumer rings (mbarrier hand-off of two
shared-memory slots) against the block-barrier kernels: for the forward,
identical final T, contributor counts and colours for every variant (2 or
4 producer warps); for the backward (1 or 2 producer warps), the same
images and gradients up to the order of float atomics, with and without a
background -- single-camera and in the multi-camera grid, on projected
scenes and on strongly elongated, faint 2-D Gaussians; and their bounded
waits: with a wait limit of zero polls every wait gives up at once, the
kernel still finishes and the device error word reports
MSPLAT_ERR_TIMEOUT."""
import numpy as np
import pytest
import torch

from _scenes import scene, sphere_camera

pytestmark = pytest.mark.gpu
DEV = "cuda"


def tuned_rings():
    """The build's default ring settings (forward, batch forward)."""
    from msplat_gb300 import _build
    d = _build.tuned_defines()
    fwd = d.get("MSPLAT_BLEND_RING_FWD", 0)
    return fwd, d.get("MSPLAT_BATCH_BLEND_RING_FWD", fwd)


def tuned_rings_bwd():
    from msplat_gb300 import _build
    d = _build.tuned_defines()
    bwd = d.get("MSPLAT_BLEND_RING_BWD", 0)
    return bwd, d.get("MSPLAT_BATCH_BLEND_RING_BWD", bwd)


@pytest.fixture(scope="module")
def lib():
    from msplat_gb300 import _build, _lib
    _build.build()
    lib = _lib.load()
    yield lib
    lib.msplat_set_blend_ring(*tuned_rings())
    lib.msplat_set_blend_ring_bwd(*tuned_rings_bwd())
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
    lib.msplat_set_blend_ring(*tuned_rings())


def test_ring_forward_on_a_large_image(lib):
    """1600 x 1200 (7,500 tiles): the ring takes the tuned pixels per thread
    there (one per thread below 6,000 tiles); results stay those of the
    barrier kernel."""
    W, H = 1600, 1200
    args = projected(200000, W, H, 21, C=3)
    lib.msplat_set_blend_ring(0, 0)
    ref = blend(lib, *args, 0.0, W, H)
    for np_ in (2, 4):
        assert lib.msplat_set_blend_ring(np_, np_) == 0
        got = blend(lib, *args, 0.0, W, H)
        for a, b in zip(got, ref):
            assert torch.equal(a, b), np_
    lib.msplat_set_blend_ring(*tuned_rings())


def test_ring_forward_on_elongated_faint_gaussians(lib):
    import test_gpu_parity as tgp
    W, H = 320, 240
    uv, conic, op, feat, idx, tr, _ = tgp.elongated_2d(5000, W, H, seed=9)
    t = [torch.as_tensor(x).to(DEV).contiguous() for x in (uv, conic, op.reshape(-1), feat, idx, tr)]
    lib.msplat_set_blend_ring(0, 0)
    ref = blend(lib, *t, 0.5, W, H)
    lib.msplat_set_blend_ring(4, 4)
    got = blend(lib, *t, 0.5, W, H)
    lib.msplat_set_blend_ring(*tuned_rings())
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
    lib.msplat_set_blend_ring(*tuned_rings())
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
    lib.msplat_set_blend_ring(*tuned_rings())
    for a, b in zip(got, ref):
        assert torch.equal(a, b)
    assert lib.msplat_wait_error(0, ctypes.byref(err), _lib.stream()) == 0


# ------------------------------------------------------------- backward ring
def blend_grads(uv, conic, op, feat, idx, tr, bg, W, H, seed=0):
    import msplat_gb300 as ms
    p = [x.detach().clone().requires_grad_() for x in (uv, conic, op, feat)]
    img = ms.alpha_blending(*p, idx, tr, bg, W, H)
    w = torch.randn(img.shape, generator=torch.Generator().manual_seed(seed)).to(DEV)
    (img * w).sum().backward()
    torch.cuda.synchronize()
    return img.detach(), [x.grad for x in p]


def grads_close(got, ref, rtol=1e-5):
    for a, b in zip(got, ref):
        scale = max(b.abs().max().item(), 1e-30)
        assert (a - b).abs().max().item() <= rtol * scale


@pytest.mark.parametrize("C,bg", [(1, 0.0), (3, 0.0), (3, 0.4), (4, 0.2)])
def test_ring_backward_equals_the_barrier_kernel(lib, C, bg):
    W, H = 640, 480  # the single-camera ring runs from 1,024 tiles
    uv, conic, op, feat, idx, tr = projected(30000, W, H, 21 + C, C=C)
    lib.msplat_set_blend_ring_bwd(0, 0)
    img0, ref = blend_grads(uv, conic, op, feat, idx, tr, bg, W, H)
    for np_ in (1, 2):
        assert lib.msplat_set_blend_ring_bwd(np_, np_) == 0
        img, got = blend_grads(uv, conic, op, feat, idx, tr, bg, W, H)
        assert torch.equal(img, img0)
        grads_close(got, ref)
    lib.msplat_set_blend_ring_bwd(*tuned_rings_bwd())


def test_ring_backward_on_elongated_faint_gaussians(lib):
    import test_gpu_parity as tgp
    W, H = 640, 480
    uv, conic, op, feat, idx, tr, _ = tgp.elongated_2d(5000, W, H, seed=10)
    t = [torch.as_tensor(x).to(DEV).contiguous() for x in (uv, conic, op.reshape(-1, 1), feat, idx, tr)]
    lib.msplat_set_blend_ring_bwd(0, 0)
    _, ref = blend_grads(*t, 0.5, W, H)
    lib.msplat_set_blend_ring_bwd(2, 2)
    _, got = blend_grads(*t, 0.5, W, H)
    lib.msplat_set_blend_ring_bwd(*tuned_rings_bwd())
    # the gradient bar of the culled-list checks: 1e-4 of the largest (the uv
    # gradients of these faint, elongated Gaussians are sums of opposite
    # moments, and the float atomics arrive in another order)
    grads_close(got, ref, rtol=1e-4)


def test_ring_backward_in_the_multi_camera_grid(lib):
    import msplat_gb300 as ms
    s = scene(15000, 4, C=3, sh_deg=1)
    sizes = [(160, 120), (96, 96), (200, 104)]
    rng = np.random.default_rng(4)
    intrs = torch.tensor([[300.0 * w / 256, 300.0 * w / 256, w / 2, h / 2] for w, h in sizes], device=DEV)
    extrs = torch.tensor(np.stack([sphere_camera(rng) for _ in sizes]), device=DEV)
    res = []
    for ring in (0, 1):
        lib.msplat_set_blend_ring_bwd(0, ring)
        p = [s[k].to(DEV).contiguous().requires_grad_() for k in ("xyz", "scale", "rot", "opacity", "shs")]
        imgs = ms.rasterization_sh_batch(*p, intrs, extrs, sizes, 0.1)
        sum((im * (k + 1)).sum() for k, im in enumerate(imgs)).backward()
        res.append(([im.detach() for im in imgs], [x.grad for x in p]))
    lib.msplat_set_blend_ring_bwd(*tuned_rings_bwd())
    for a, b in zip(res[1][0], res[0][0]):
        assert torch.equal(a, b)
    grads_close(res[1][1], res[0][1], rtol=1e-4)


def test_ring_backward_wait_that_runs_out_reports_timeout(lib):
    import ctypes
    from msplat_gb300 import _lib
    W, H = 640, 480
    uv, conic, op, feat, idx, tr = projected(8000, W, H, 6)
    err = ctypes.c_int(0)
    assert lib.msplat_wait_error(1, ctypes.byref(err), _lib.stream()) == 0  # clear
    lib.msplat_set_blend_ring(0, 0)  # only the backward's waits run out
    lib.msplat_set_blend_ring_bwd(2, 2)
    lib.msplat_set_wait_limit(0)  # every wait gives up at once
    try:
        blend_grads(uv, conic, op, feat, idx, tr, 0.0, W, H)
    finally:
        lib.msplat_set_wait_limit(1 << 21)
        lib.msplat_set_blend_ring(*tuned_rings())
    assert lib.msplat_wait_error(1, ctypes.byref(err), _lib.stream()) == 6  # MSPLAT_ERR_TIMEOUT
    assert err.value == 1
    # the context is healthy and the next backward is right again
    lib.msplat_set_blend_ring_bwd(0, 0)
    _, ref = blend_grads(uv, conic, op, feat, idx, tr, 0.0, W, H)
    lib.msplat_set_blend_ring_bwd(2, 2)
    _, got = blend_grads(uv, conic, op, feat, idx, tr, 0.0, W, H)
    lib.msplat_set_blend_ring_bwd(*tuned_rings_bwd())
    grads_close(got, ref)
    assert lib.msplat_wait_error(0, ctypes.byref(err), _lib.stream()) == 0
