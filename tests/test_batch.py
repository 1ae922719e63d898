"""Multi-camera rendering in one key space against one single-camera call
per camera.

Images must be bit-identical (the batched preprocess evaluates the same
device code per camera; the batched sort orders each camera's list exactly
as the single-camera culled sort; the blend grid over all cameras runs the
single-camera per-pixel arithmetic); gradients summed over the cameras
agree up to float summation order, and every camera gets its own intrinsic
/ extrinsic gradient.  Also: several scenes in one batch (cameras in any
order), more than four channels, and a capacity too small for the sort.
"""
import numpy as np
import pytest
import torch

from _scenes import scene, sphere_camera

pytestmark = pytest.mark.gpu
DEV = "cuda"
SIZES = [(128, 128), (256, 192), (320, 240), (96, 160), (200, 120)]


@pytest.fixture(scope="module", autouse=True)
def _built():
    from msplat_gb300 import _build, _lib
    _build.build()
    _lib.load()
    yield


def rel_close(got, ref, rtol, what):
    got, ref = got.detach().double().cpu().numpy(), ref.detach().double().cpu().numpy()
    scale = max(np.abs(ref).max(), 1e-30)
    err = np.abs(got - ref).max() if got.size else 0.0
    assert err <= rtol * scale, f"{what}: max abs err {err:.3e} > {rtol} * {scale:.3e}"


def cameras(sizes, seed):
    rng = np.random.default_rng(seed)
    intrs, extrs = [], []
    for w, h in sizes:
        f = 300.0 * w / 256
        intrs.append([f, f, w / 2, h / 2])
        extrs.append(sphere_camera(rng))
    return torch.tensor(intrs, dtype=torch.float32), torch.tensor(np.stack(extrs), dtype=torch.float32)


def leaves(d):
    return {k: v.detach().clone().to(DEV).contiguous().requires_grad_() for k, v in d.items()}


@pytest.mark.parametrize("sh_deg", [3, None])
def test_batch_matches_single_camera_calls(sh_deg):
    import msplat_gb300 as ms
    s = scene(20000, 4, C=3, sh_deg=sh_deg if sh_deg is not None else 0)
    intrs, extrs = cameras(SIZES, 9)
    base = {"xyz": s["xyz"], "scale": s["scale"], "rot": s["rot"], "opacity": s["opacity"],
            "col": s["shs"] if sh_deg is not None else s["feat"], "intrs": intrs, "extrs": extrs}
    a, r = leaves(base), leaves(base)
    bg = 0.2
    fn = ms.rasterization_sh_batch if sh_deg is not None else ms.rasterization_batch
    imgs = fn(a["xyz"], a["scale"], a["rot"], a["opacity"], a["col"], a["intrs"], a["extrs"], SIZES, bg)
    single = ms.rasterization_sh if sh_deg is not None else ms.rasterization
    refs = [single(r["xyz"], r["scale"], r["rot"], r["opacity"], r["col"], r["intrs"][b], r["extrs"][b], w, h, bg)
            for b, (w, h) in enumerate(SIZES)]
    gen = torch.Generator().manual_seed(3)
    ws = [torch.randn(img.shape, generator=gen).to(DEV) for img in refs]
    for b, (img, ref) in enumerate(zip(imgs, refs)):
        assert img.shape == ref.shape
        assert torch.equal(img, ref), f"camera {b}"
    sum((i * w).sum() for i, w in zip(imgs, ws)).backward()
    sum((i * w).sum() for i, w in zip(refs, ws)).backward()
    for k in base:
        rel_close(a[k].grad, r[k].grad, 1e-4, f"dL/d{k}")
    assert a["extrs"].grad.abs().sum(dim=(1, 2)).min() > 0  # every camera has its own gradient


def test_batch_with_one_camera_and_no_grad_cameras():
    import msplat_gb300 as ms
    s = scene(5000, 2, C=3, sh_deg=1)
    intrs, extrs = cameras([(64, 64)], 1)
    p = leaves({"xyz": s["xyz"], "scale": s["scale"], "rot": s["rot"], "opacity": s["opacity"], "shs": s["shs"]})
    imgs = ms.rasterization_sh_batch(p["xyz"], p["scale"], p["rot"], p["opacity"], p["shs"], intrs.to(DEV),
                                     extrs.to(DEV), [(64, 64)])
    ref = ms.rasterization_sh(p["xyz"], p["scale"], p["rot"], p["opacity"], p["shs"], intrs[0].to(DEV),
                              extrs[0].to(DEV), 64, 64, 0.0)
    assert torch.equal(imgs[0], ref)
    imgs[0].sum().backward()
    assert torch.isfinite(p["shs"].grad).all() and p["xyz"].grad.abs().sum() > 0


def test_batch_over_several_scenes_in_any_camera_order():
    import msplat_gb300 as ms
    s1 = scene(15000, 5, C=3, sh_deg=2)
    s2 = scene(7000, 6, C=3, sh_deg=2)
    sizes = [(160, 120), (128, 128), (96, 144), (200, 104), (64, 64)]
    scene_of = [1, 0, 1, 0, 0]
    intrs, extrs = cameras(sizes, 12)
    keys = ("xyz", "scale", "rot", "opacity", "shs")
    a = [leaves({k: sc[k] for k in keys}) for sc in (s1, s2)]
    r = [leaves({k: sc[k] for k in keys}) for sc in (s1, s2)]
    ci, ce = intrs.to(DEV).requires_grad_(), extrs.to(DEV).requires_grad_()
    ri, re = intrs.to(DEV).requires_grad_(), extrs.to(DEV).requires_grad_()
    imgs = ms.rasterization_sh_scenes([tuple(p[k] for k in keys) for p in a], scene_of, ci, ce, sizes, 0.1)
    refs = [ms.rasterization_sh(*(r[scene_of[b]][k] for k in keys), ri[b], re[b], w, h, 0.1)
            for b, (w, h) in enumerate(sizes)]
    gen = torch.Generator().manual_seed(5)
    ws = [torch.randn(img.shape, generator=gen).to(DEV) for img in refs]
    for b, (img, ref) in enumerate(zip(imgs, refs)):
        assert torch.equal(img, ref), f"camera {b}"
    sum((i * w).sum() for i, w in zip(imgs, ws)).backward()
    sum((i * w).sum() for i, w in zip(refs, ws)).backward()
    for sa, sr in zip(a, r):
        for k in keys:
            rel_close(sa[k].grad, sr[k].grad, 1e-4, f"dL/d{k}")
    rel_close(ci.grad, ri.grad, 1e-4, "dL/dintrs")
    rel_close(ce.grad, re.grad, 1e-4, "dL/dextrs")


def test_batch_with_more_than_four_channels():
    import msplat_gb300 as ms
    s = scene(12000, 7, C=6)
    sizes = [(128, 96), (80, 80), (144, 112)]
    intrs, extrs = cameras(sizes, 3)
    base = {"xyz": s["xyz"], "scale": s["scale"], "rot": s["rot"], "opacity": s["opacity"], "feat": s["feat"]}
    a, r = leaves(base), leaves(base)
    imgs = ms.rasterization_batch(a["xyz"], a["scale"], a["rot"], a["opacity"], a["feat"], intrs.to(DEV),
                                  extrs.to(DEV), sizes, 0.3)
    refs = [ms.rasterization(r["xyz"], r["scale"], r["rot"], r["opacity"], r["feat"], intrs[b].to(DEV),
                             extrs[b].to(DEV), w, h, 0.3) for b, (w, h) in enumerate(sizes)]
    for b, (img, ref) in enumerate(zip(imgs, refs)):
        assert torch.equal(img, ref), f"camera {b}"
    gen = torch.Generator().manual_seed(2)
    ws = [torch.randn(img.shape, generator=gen).to(DEV) for img in refs]
    sum((i * w).sum() for i, w in zip(imgs, ws)).backward()
    sum((i * w).sum() for i, w in zip(refs, ws)).backward()
    for k in base:
        rel_close(a[k].grad, r[k].grad, 1e-4, f"dL/d{k}")


def test_batch_capacity_too_small_reports_status():
    import msplat_gb300 as ms
    s = scene(20000, 8, C=3, sh_deg=1)
    sizes = [(160, 160), (128, 96)]
    intrs, extrs = cameras(sizes, 4)
    p = leaves({"xyz": s["xyz"], "scale": s["scale"], "rot": s["rot"], "opacity": s["opacity"], "shs": s["shs"]})
    status = torch.full((1,), 7, dtype=torch.int32, device=DEV)
    with torch.no_grad():
        ms.rasterization_sh_batch(p["xyz"], p["scale"], p["rot"], p["opacity"], p["shs"], intrs.to(DEV),
                                  extrs.to(DEV), sizes, capacity=3072, status=status)
    torch.cuda.synchronize()
    assert int(status.item()) == 1
    with torch.no_grad():
        imgs = ms.rasterization_sh_batch(p["xyz"], p["scale"], p["rot"], p["opacity"], p["shs"], intrs.to(DEV),
                                         extrs.to(DEV), sizes, capacity=4_000_000, status=status)
        ref = ms.rasterization_sh(p["xyz"], p["scale"], p["rot"], p["opacity"], p["shs"], intrs[1].to(DEV),
                                  extrs[1].to(DEV), 128, 96, 0.0)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.equal(imgs[1], ref)


def test_batch_rows_too_long_are_refused():
    """The batched preprocess stages each Gaussian's coefficient row in
    shared memory: rows longer than it takes (C * D beyond 1,599 floats
    forward) are refused with MSPLAT_ERR_UNSUPPORTED, not launched."""
    import msplat_gb300 as ms
    s = scene(500, 6, C=3)
    intrs, extrs = cameras([(64, 64)], 2)
    shs = torch.zeros(500, 16, 121, device=DEV)
    with pytest.raises(RuntimeError, match="too large"):
        ms.rasterization_sh_batch(s["xyz"].to(DEV), s["scale"].to(DEV), s["rot"].to(DEV), s["opacity"].to(DEV), shs,
                                  intrs.to(DEV), extrs.to(DEV), [(64, 64)])
