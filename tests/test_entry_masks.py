"""The forward's entry masks carried to the backward
(msplat_alpha_blending_forward_masks / _backward_masks) against the plain
calls: the same images, final T and contributor counts, and the same
gradients up to the order of float atomics -- with the forward ring on
one and on two pixels per thread (the masks merged to the backward's warp
blocks or taken as they are), on the barrier kernels, with and without a
background, for 1, 3 and 4 channels."""
import numpy as np
import pytest
import torch

from _scenes import scene, sphere_camera

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def lib():
    from msplat_gb300 import _build, _lib
    from test_blend_ring import tuned_rings, tuned_rings_bwd
    _build.build()
    lib = _lib.load()
    yield lib
    lib.msplat_set_blend_ring(*tuned_rings())
    lib.msplat_set_blend_ring_bwd(*tuned_rings_bwd())


def projected(n, W, H, seed, C):
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


def run(lib, args, bg, W, H, masks):
    from msplat_gb300 import _lib
    uv, conic, op, feat, idx, tr = args
    P, C = feat.shape
    out = torch.empty(C, H, W, device=DEV)
    T = torch.empty(H, W, device=DEV)
    nc = torch.empty(H, W, dtype=torch.int32, device=DEV)
    em = torch.full((idx.numel(),), 0xAB, dtype=torch.uint8, device=DEV) if masks else None
    common = (P, C, uv.data_ptr(), conic.data_ptr(), op.data_ptr(), feat.data_ptr(), idx.data_ptr(), tr.data_ptr(),
              bg, W, H)
    if masks:
        _lib.check(lib.msplat_alpha_blending_forward_masks(*common, out.data_ptr(), T.data_ptr(), nc.data_ptr(),
                                                           em.data_ptr(), _lib.stream()), "fwd")
    else:
        _lib.check(lib.msplat_alpha_blending_forward(*common, out.data_ptr(), T.data_ptr(), nc.data_ptr(),
                                                     _lib.stream()), "fwd")
    dout = torch.randn(C, H, W, generator=torch.Generator().manual_seed(5)).to(DEV)
    g = [torch.zeros(P, 2, device=DEV), torch.zeros(P, 3, device=DEV), torch.zeros(P, device=DEV),
         torch.zeros(P, C, device=DEV)]
    gp = [x.data_ptr() for x in g]
    if masks:
        _lib.check(lib.msplat_alpha_blending_backward_masks(*common, T.data_ptr(), nc.data_ptr(), dout.data_ptr(),
                                                            *gp, em.data_ptr(), _lib.stream()), "bwd")
    else:
        _lib.check(lib.msplat_alpha_blending_backward(*common, T.data_ptr(), nc.data_ptr(), dout.data_ptr(), *gp,
                                                      _lib.stream()), "bwd")
    torch.cuda.synchronize()
    return (out, T, nc), g


def close(a, b, rtol):
    scale = max(b.abs().max().item(), 1e-30)
    return (a - b).abs().max().item() <= rtol * scale


@pytest.mark.parametrize("W,H", [(640, 480), (1600, 1200)])
@pytest.mark.parametrize("C", [1, 3, 4])
def test_masks_carry_over(lib, W, H, C):
    args = projected(30000 if W < 1000 else 200000, W, H, 31 + C, C)
    for fwd_ring, bwd_ring in ((4, 1), (2, 0), (0, 1), (0, 0)):
        lib.msplat_set_blend_ring(fwd_ring, fwd_ring)
        lib.msplat_set_blend_ring_bwd(bwd_ring, bwd_ring)
        for bg in (0.0, 0.4):
            (img0, g0) = run(lib, args, bg, W, H, False)
            (img1, g1) = run(lib, args, bg, W, H, True)
            for a, b in zip(img1, img0):
                assert torch.equal(a, b), (fwd_ring, bwd_ring, bg)
            for a, b in zip(g1, g0):
                assert close(a, b, 1e-5), (fwd_ring, bwd_ring, bg)


def test_autograd_path_uses_masks_and_matches(lib):
    """ms.alpha_blending (the autograd path, which carries the masks) gives
    the plain calls' results."""
    import msplat_gb300 as ms
    W, H = 640, 480
    args = projected(30000, W, H, 44, 3)
    (img0, g0) = run(lib, args, 0.2, W, H, False)
    uv, conic, op, feat, idx, tr = args
    p = [x.detach().clone().requires_grad_() for x in (uv, conic, op, feat)]
    img = ms.alpha_blending(*p, idx, tr, 0.2, W, H)
    dout = torch.randn(3, H, W, generator=torch.Generator().manual_seed(5)).to(DEV)
    (img * dout).sum().backward()
    assert torch.equal(img.detach(), img0[0])
    # dL/duv and dL/dconic of the autograd path are finished per Gaussian
    # exactly as the plain call's; opacity and features too
    for a, b in zip([x.grad for x in p], g0):
        assert close(a.reshape(b.shape), b, 1e-5)
