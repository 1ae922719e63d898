"""Parity at the benchmark sizes.

* 1M Gaussians at 1920x1080 (SH degree 3, random sphere camera, f = 1500):
  every stage of the GPU chain against the oracle on the same inputs, the
  oracle spread over the host's cores (its threaded mode is bit-identical to
  the serial one for everything but the order of float64 gradient sums).
  Projection, covariance, EWA, sort (29M intersections) and both blend
  passes over the full frame.
* 2M Gaussians at 1024x1024 (f = 800, keeping the 1080p field of view), SH
  degree 10 colours plus 32 N(0,1) features and a depth channel (C = 36):
  SH against the oracle on a sample of rows, and the size-independent
  properties of a multi-channel blend -- each channel block rendered alone
  is bit-identical to the same channels of the 36-channel render, its
  feature gradients equal up to the order of float atomics, and the uv /
  conic / opacity gradients are the sums of the blocks' gradients; and the
  36-channel blend, forward and backward, against the oracle on a band of 8
  tile rows.
"""
import os

import numpy as np
import pytest
import torch

import oracle
from _guided import check_blend, gpu_blend_forward
from _scenes import sphere_camera

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module", autouse=True)
def _built():
    from msplat_gb300 import _build, _lib
    _build.build()
    _lib.load()
    try:
        n = len(os.sched_getaffinity(0))
    except AttributeError:
        n = os.cpu_count() or 1
    oracle.set_threads(n)
    yield
    oracle.set_threads(1)


def N(x):
    return x.detach().cpu().numpy()


def rel_close(got, ref, rtol, what):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    scale = max(np.abs(ref).max(), 1e-30)
    err = np.abs(got - ref).max() if got.size else 0.0
    assert err <= rtol * scale, f"{what}: max abs err {err:.3e} > {rtol} * {scale:.3e}"


def big_scene(n, seed, sh_deg, sh_std):
    g = torch.Generator().manual_seed(seed)
    xyz = torch.rand(n, 3, generator=g) * 2 - 1
    scale = torch.exp(torch.rand(n, 3, generator=g) * 2 - 5)
    rot = torch.randn(n, 4, generator=g)
    rot = rot / rot.norm(dim=-1, keepdim=True)
    opacity = torch.sigmoid(torch.randn(n, 1, generator=g))
    shs = torch.randn(n, 3, (sh_deg + 1) ** 2, generator=g) * sh_std
    return dict(xyz=xyz, scale=scale, rot=rot, opacity=opacity, shs=shs)


def view_dirs(xyz, extr):
    R, t = extr[:, :3], extr[:, 3]
    d = xyz + R.transpose(0, 1) @ t
    return d / d.norm(dim=-1, keepdim=True)


def test_1m_gaussians_1080p_every_stage_against_the_oracle():
    import msplat_gb300 as ms
    W, H, f = 1920, 1080, 1500.0
    s = big_scene(1_000_000, 0, 3, 0.3)
    intr = np.array([f, f, W / 2, H / 2], np.float32)
    extr = sphere_camera(np.random.default_rng(0))
    t = {k: v.to(DEV) for k, v in s.items()}
    ti, te = torch.as_tensor(intr).to(DEV), torch.as_tensor(extr).to(DEV)
    xyz = s["xyz"].numpy()

    uv, depth = ms.project_point(t["xyz"], ti, te, W, H)
    ouv, od = oracle.project_point_forward(xyz, intr, extr, W, H)
    np.testing.assert_array_equal(N(uv), ouv)
    np.testing.assert_array_equal(N(depth), od)
    vis = depth.reshape(-1) != 0
    cov = ms.compute_cov3d(t["scale"], t["rot"], vis)
    ocov = oracle.compute_cov3d_forward(s["scale"].numpy(), s["rot"].numpy(), N(vis))
    assert np.abs(N(cov) - ocov).max() <= 1e-6 * np.abs(ocov).max()
    conic, radius, tiles = ms.ewa_project(t["xyz"], cov, ti, te, uv, W, H, vis)
    # EWA on the GPU's own covariances so the comparison isolates the stage.
    # Where 3 sqrt(lambda) is within rounding reach of an integer (about 0.7 %
    # of radii near 30 px) the GPU's approximate sqrt may round the other way,
    # as the reference's fast-math build does: every radius must be the
    # oracle's or that alternative, with its tiles.
    n_alt, cerr, _ = oracle.ewa_check_against(N(conic), N(radius), N(tiles), xyz, N(cov), intr, extr, N(uv), W, H,
                                              N(vis))
    print(f"EWA: {n_alt} of {int((N(radius) > 0).sum())} radii took the alternative rounding; "
          f"max conic err {cerr:.2e}")
    assert n_alt <= 100

    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles)
    oidx, otr = oracle.sort_gaussian(N(uv), N(depth), W, H, N(radius), N(tiles))
    assert oidx.size > 20_000_000
    np.testing.assert_array_equal(N(tr), otr)
    np.testing.assert_array_equal(N(idx), oidx)

    color = ms.compute_sh(t["shs"], view_dirs(t["xyz"], te))
    ocolor = oracle.compute_sh_forward(s["shs"].numpy(), N(view_dirs(t["xyz"], te)))
    rel_close(N(color), ocolor, 1e-5, "SH colour")

    ins = [uv.detach().clone(), conic.detach().clone(), t["opacity"].clone(), color.detach().clone()]
    for a in ins:
        a.requires_grad_()
    bg = 0.0
    img = ms.alpha_blending(*ins, idx, tr, bg, W, H)
    w = np.random.default_rng(1).normal(size=(3, H, W)).astype(np.float32)
    (img * torch.as_tensor(w).to(DEV)).sum().backward()
    a_uv, a_con, a_op, a_col = (N(a) for a in ins)
    # every pixel: ncontrib equal, image within 1e-5 of the guided oracle
    # (which follows the GPU only at skip / stop decisions within rounding
    # reach of their thresholds)
    gout, gT, gnc = gpu_blend_forward(a_uv, a_con, a_op, a_col, oidx, otr, bg, W, H)
    np.testing.assert_array_equal(N(img), gout)
    st = check_blend(gout, gT, gnc, a_uv, a_con, a_op, a_col, oidx, otr, bg, W, H)
    print(f"blend: {st['alternate_pixels']} of {st['pixels']} pixels took an alternate branch; "
          f"max image err {st['max_err']:.2e}, max T err {st['max_T_err']:.2e}")
    grads = oracle.alpha_blending_backward(a_uv, a_con, a_op, a_col, oidx, otr, bg, W, H, st["final_T"],
                                           st["ncontrib"], w, forces=st["forces"])
    for a, ref, name in zip(ins, grads, ["uv", "conic", "opacity", "colour"]):
        rel_close(N(a.grad).reshape(ref.shape), ref, 1e-4, f"dL/d{name}")


def test_2m_gaussians_1024px_deg10_sh_and_36_channel_blend_properties():
    import msplat_gb300 as ms
    W = H = 1024
    f = 800.0
    n = 2_000_000
    s = big_scene(n, 1, 10, 0.1)
    g = torch.Generator().manual_seed(2)
    feats = torch.randn(n, 32, generator=g)
    intr = torch.tensor([f, f, W / 2, H / 2]).to(DEV)
    extr = torch.as_tensor(sphere_camera(np.random.default_rng(1))).to(DEV)
    t = {k: v.to(DEV) for k, v in s.items()}

    dirs = view_dirs(t["xyz"], extr)
    color = ms.compute_sh(t["shs"], dirs)
    rows = np.random.default_rng(3).choice(n, 4000, replace=False)
    ocolor = oracle.compute_sh_forward(s["shs"].numpy()[rows], N(dirs)[rows])
    rel_close(N(color)[rows], ocolor, 1e-5, "SH degree 10")

    uv, depth = ms.project_point(t["xyz"], intr, extr, W, H)
    vis = depth.reshape(-1) != 0
    cov = ms.compute_cov3d(t["scale"], t["rot"], vis)
    conic, radius, tiles = ms.ewa_project(t["xyz"], cov, intr, extr, uv, W, H, vis)
    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles)
    assert idx.numel() > 10_000_000
    full = torch.cat([color, feats.to(DEV), depth], dim=1).contiguous()  # C = 36
    blocks = [(0, 3), (3, 35), (35, 36)]
    w = torch.randn(36, H, W, generator=g).to(DEV)
    bg = 0.1

    def run(feat, wt):
        ins = [uv.detach().clone(), conic.detach().clone(), t["opacity"].clone(), feat.detach().clone()]
        for a in ins:
            a.requires_grad_()
        img = ms.alpha_blending(*ins, idx, tr, bg, W, H)
        (img * wt).sum().backward()
        return img.detach(), [a.grad for a in ins]

    img, grads = run(full, w)
    sums = [torch.zeros_like(x) for x in grads[:3]]
    for a, b in blocks:
        bimg, bgr = run(full[:, a:b], w[a:b])
        assert torch.equal(bimg, img[a:b]), (a, b)
        # float atomics from many tiles: equal up to summation order
        rel_close(N(bgr[3]), N(grads[3][:, a:b]), 1e-5, f"dL/dfeature[{a}:{b}]")
        for acc, x in zip(sums, bgr[:3]):
            acc += x
    for got, ref, name in zip(grads[:3], sums, ["uv", "conic", "opacity"]):
        rel_close(N(got), N(ref), 1e-4, f"dL/d{name} (36 channels vs sum of blocks)")


def test_2m_gaussians_1024px_36_channel_band_against_the_oracle():
    """The 36-channel blend (SH degree 10 colour, 32 N(0,1) features, depth;
    bg 0.1) of 2M Gaussians at 1024x1024, forward and backward, against the
    oracle on a band of 8 tile rows across the middle: the multi-chunk path
    (32 + 4 channels forward, 4 x 10 backward).  Image within 1e-5 on every
    band pixel and ncontrib equal (guided oracle); gradients of a loss that
    weights only the band within 1e-4 of the oracle's adjoint."""
    import msplat_gb300 as ms
    W = H = 1024
    f = 800.0
    n = 2_000_000
    s = big_scene(n, 1, 10, 0.1)
    g = torch.Generator().manual_seed(2)
    feats = torch.randn(n, 32, generator=g)
    intr = torch.tensor([f, f, W / 2, H / 2]).to(DEV)
    extr = torch.as_tensor(sphere_camera(np.random.default_rng(1))).to(DEV)
    t = {k: v.to(DEV) for k, v in s.items()}
    with torch.no_grad():
        color = ms.compute_sh(t["shs"], view_dirs(t["xyz"], extr))
        uv, depth = ms.project_point(t["xyz"], intr, extr, W, H)
        vis = depth.reshape(-1) != 0
        cov = ms.compute_cov3d(t["scale"], t["rot"], vis)
        conic, radius, tiles = ms.ewa_project(t["xyz"], cov, intr, extr, uv, W, H, vis)
        idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles)
    full = torch.cat([color, feats.to(DEV), depth], dim=1).contiguous()
    C = full.shape[1]
    assert C == 36
    gx, gy = W // 16, H // 16
    r0, rows = gy // 2 - 4, 8
    y0, y1 = r0 * 16, (r0 + rows) * 16
    bg = 0.1
    w = torch.randn(C, H, W, generator=g)
    w_band = torch.zeros_like(w)
    w_band[:, y0:y1] = w[:, y0:y1]
    ins = [uv.clone(), conic.clone(), t["opacity"].clone(), full.clone()]
    for a in ins:
        a.requires_grad_()
    img = ms.alpha_blending(*ins, idx, tr, bg, W, H)
    (img * w_band.to(DEV)).sum().backward()

    trb = N(tr).reshape(gy, gx, 2)[r0:r0 + rows].reshape(-1, 2)
    uvb = N(uv).copy()
    uvb[:, 1] -= y0
    op, feat = N(t["opacity"]), N(full)
    gout, gT, gnc = gpu_blend_forward(uvb, N(conic), op, feat, N(idx), trb, bg, W, rows * 16)
    assert np.abs(N(img)[:, y0:y1] - gout).max() <= 1e-5  # the band rendered alone vs the full frame's band
    st = check_blend(gout, gT, gnc, uvb, N(conic), op, feat, N(idx), trb, bg, W, rows * 16)
    print(f"36 channels: {st['alternate_pixels']} of {st['pixels']} band pixels on an alternate branch, "
          f"max image err {st['max_err']:.2e}")
    grads = oracle.alpha_blending_backward(uvb, N(conic), op, feat, N(idx), trb, bg, W, rows * 16, st["final_T"],
                                           st["ncontrib"], w[:, y0:y1].numpy(), forces=st["forces"])
    for a, ref, name in zip(ins, grads, ["uv", "conic", "opacity", "feature"]):
        rel_close(N(a.grad).reshape(ref.shape), ref, 1e-4, f"dL/d{name} (36 channels, band)")


def test_ndc_receives_the_scaled_uv_gradient():
    import msplat_gb300 as ms
    W, H, f = 320, 240, 300.0
    s = big_scene(20000, 4, 0, 1.0)
    intr = torch.tensor([f, f, W / 2, H / 2]).to(DEV)
    extr = torch.tensor([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 4.0]]).to(DEV)
    t = {k: v.to(DEV) for k, v in s.items()}
    uv, depth = ms.project_point(t["xyz"], intr, extr, W, H)
    vis = depth.reshape(-1) != 0
    cov = ms.compute_cov3d(t["scale"], t["rot"], vis)
    conic, radius, tiles = ms.ewa_project(t["xyz"], cov, intr, extr, uv, W, H, vis)
    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles)
    feat = torch.rand(20000, 3).to(DEV)
    u = uv.detach().clone().requires_grad_()
    ndc = torch.zeros_like(uv).requires_grad_()
    img = ms.alpha_blending(u, conic, t["opacity"], feat, idx, tr, 0.0, W, H, ndc)
    img.square().sum().backward()
    assert u.grad.abs().max() > 0
    scale = torch.tensor([0.5 * W, 0.5 * H], device=DEV)
    assert torch.equal(ndc.grad, u.grad * scale[None, :])


def test_4k_frame_fits_and_a_band_matches_the_oracle():
    """3840x2160 forward + backward of 1M Gaussians: per pixel only final T
    and the contributor count are kept (8 B), the backward recomputes the
    rest, so the frame fits easily; a band of 8 tile rows across the middle
    is checked against the guided oracle (image 1e-5 on every pixel)."""
    import msplat_gb300 as ms
    W, H, f = 3840, 2160, 3000.0
    s = big_scene(1_000_000, 5, 3, 0.3)
    intr = np.array([f, f, W / 2, H / 2], np.float32)
    extr = sphere_camera(np.random.default_rng(5))
    t = {k: v.to(DEV).requires_grad_() for k, v in s.items()}
    ti, te = torch.as_tensor(intr).to(DEV), torch.as_tensor(extr).to(DEV)
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    img, radius = ms.rasterization_sh(t["xyz"], t["scale"], t["rot"], t["opacity"], t["shs"], ti, te, W, H, 0.0,
                                      return_radius=True)
    w = torch.randn(3, H, W, generator=torch.Generator().manual_seed(6)).to(DEV)
    (img * w).sum().backward()
    torch.cuda.synchronize()
    peak_gb = (torch.cuda.max_memory_allocated() - base) / 1e9
    assert peak_gb < 16, peak_gb
    for k in ("xyz", "scale", "rot", "opacity", "shs"):
        assert torch.isfinite(t[k].grad).all(), k
    # oracle on a band of tile rows, with the GPU's own projected inputs
    with torch.no_grad():
        uv, depth, conic, rad, tiles, color = ms.preprocess(t["xyz"], t["scale"], t["rot"], ti, te, W, H,
                                                            shs=t["shs"])
        idx, tr = ms.sort_gaussian(uv, depth, W, H, rad, tiles)
    gx, gy = W // 16, H // 16
    r0, rows = gy // 2 - 4, 8
    trb = N(tr).reshape(gy, gx, 2)[r0:r0 + rows].reshape(-1, 2)
    uvb = N(uv).copy()
    uvb[:, 1] -= r0 * 16
    op = N(t["opacity"])
    gout, gT, gnc = gpu_blend_forward(uvb, N(conic), op, N(color), N(idx), trb, 0.0, W, rows * 16)
    got = N(img)[:, r0 * 16:(r0 + rows) * 16]
    assert np.abs(got - gout).max() <= 1e-5  # the band rendered alone vs the full frame's band
    check_blend(gout, gT, gnc, uvb, N(conic), op, N(color), N(idx), trb, 0.0, W, rows * 16)
