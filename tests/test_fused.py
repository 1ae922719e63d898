"""The fused rasterisation path against the stage-by-stage composite of the
step functions (the reference's rasterization, msplat/__init__.py:70-93).

* preprocess forward: uv, depth, conic, radius, tiles bit-identical;
* rasterization image bit-identical (same sort and blend downstream);
* gradients of every input, camera included, equal up to float summation
  order (the fused backward adds the projection, EWA and view-direction
  terms in registers instead of through separate tensors);
* rasterization_sh against compute_sh on torch view directions.
"""
import numpy as np
import pytest
import torch

from _scenes import camera, scene

pytestmark = pytest.mark.gpu
DEV = "cuda"


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


def view_dirs(xyz, extr):
    R, t = extr[:, :3], extr[:, 3]
    d = xyz + R.transpose(0, 1) @ t
    return d / d.norm(dim=-1, keepdim=True)


def composite(ms, p, W, H, bg, feat):
    uv, depth = ms.project_point(p["xyz"], p["intr"], p["extr"], W, H)
    vis = depth != 0
    cov = ms.compute_cov3d(p["scale"], p["rot"], vis)
    conic, radius, tiles = ms.ewa_project(p["xyz"], cov, p["intr"], p["extr"], uv, W, H, vis)
    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles)
    return ms.alpha_blending(uv, conic, p["opacity"], feat, idx, tr, bg, W, H), (uv, depth, conic, radius, tiles)


def make(n, W, H, seed, sh_deg=None, front=False):
    s = scene(n, seed, C=3, sh_deg=sh_deg)
    intr, extr = camera(W, H, seed=seed, front=front)
    p = {k: s[k] for k in ("xyz", "scale", "rot", "opacity", "feat")}
    if sh_deg is not None:
        p["shs"] = s["shs"]
    p["intr"], p["extr"] = torch.as_tensor(intr), torch.as_tensor(extr)
    return {k: v.to(DEV).contiguous().requires_grad_() for k, v in p.items()}


@pytest.mark.parametrize("seed,front", [(0, True), (1, False), (2, False)])
def test_preprocess_bit_identical_to_the_stage_functions(seed, front):
    import msplat_gb300 as ms
    W, H = 640, 480
    p = make(30000, W, H, seed, front=front)
    with torch.no_grad():
        got = ms.preprocess(p["xyz"], p["scale"], p["rot"], p["intr"], p["extr"], W, H)
        _, ref = composite(ms, p, W, H, 0.0, p["feat"])
    for g, r, name in zip(got[:5], ref, ["uv", "depth", "conic", "radius", "tiles"]):
        assert torch.equal(g, r.view_as(g)), name
    assert int(got[4].sum()) > 0


@pytest.mark.parametrize("bg", [0.0, 0.4])
def test_rasterization_fused_matches_composite(bg):
    import msplat_gb300 as ms
    W, H = 320, 240
    p = make(20000, W, H, 5)
    q = {k: v.detach().clone().requires_grad_() for k, v in p.items()}
    img = ms.rasterization(p["xyz"], p["scale"], p["rot"], p["opacity"], p["feat"], p["intr"], p["extr"], W, H, bg)
    ref, _ = composite(ms, q, W, H, bg, q["feat"])
    assert torch.equal(img, ref)
    w = torch.randn(img.shape, generator=torch.Generator().manual_seed(1)).to(DEV)
    (img * w).sum().backward()
    (ref * w).sum().backward()
    for k in p:
        rel_close(p[k].grad, q[k].grad, 1e-5, f"dL/d{k}")


def misaligned_copy(t):
    """A leaf copy of `t` whose data starts 4 bytes past a 16-byte boundary."""
    flat = torch.empty(t.numel() + 4, dtype=t.dtype, device=t.device)
    m = flat[1:1 + t.numel()].view(t.shape)
    m.copy_(t.detach())
    assert m.data_ptr() % 16 == 4
    return m.requires_grad_()


# degrees 1 and 3 with 3 channels take the register-row kernels
# (preprocess_sh3_*), 0 and 2 the staged ones, 6 the two-kernel path; a
# misaligned coefficient array takes the staged kernels at degree 3
@pytest.mark.parametrize("deg,misaligned", [(0, False), (1, False), (2, False), (3, False), (3, True), (6, False)])
def test_rasterization_sh_matches_compute_sh_on_view_directions(deg, misaligned):
    import msplat_gb300 as ms
    W, H = 320, 240
    p = make(20000, W, H, 7 + deg, sh_deg=deg)
    if misaligned:
        p["shs"] = misaligned_copy(p["shs"])
    q = {k: v.detach().clone().requires_grad_() for k, v in p.items()}
    img = ms.rasterization_sh(p["xyz"], p["scale"], p["rot"], p["opacity"], p["shs"], p["intr"], p["extr"], W, H,
                              0.1)
    color = ms.compute_sh(q["shs"], view_dirs(q["xyz"], q["extr"]))
    ref = ms.rasterization(q["xyz"], q["scale"], q["rot"], q["opacity"], color, q["intr"], q["extr"], W, H, 0.1)
    assert (img - ref).abs().max().item() <= 1e-5
    w = torch.randn(img.shape, generator=torch.Generator().manual_seed(2)).to(DEV)
    (img * w).sum().backward()
    (ref * w).sum().backward()
    for k in ("xyz", "scale", "rot", "opacity", "shs", "intr", "extr"):
        rel_close(p[k].grad, q[k].grad, 1e-4, f"dL/d{k}")
    assert p["feat"].grad is None


def test_preprocess_without_camera_grads_and_errors():
    import msplat_gb300 as ms
    W, H = 128, 96
    p = make(2000, W, H, 3, sh_deg=2)
    intr, extr = p["intr"].detach(), p["extr"].detach()
    img = ms.rasterization_sh(p["xyz"], p["scale"], p["rot"], p["opacity"], p["shs"], intr, extr, W, H, 0.0)
    img.sum().backward()
    assert p["xyz"].grad is not None and torch.isfinite(p["xyz"].grad).all()
    with pytest.raises(RuntimeError, match="CUDA tensor"):
        ms.preprocess(p["xyz"].detach().cpu(), p["scale"], p["rot"], intr, extr, W, H)
    with pytest.raises(RuntimeError, match="shs must be"):
        ms.preprocess(p["xyz"], p["scale"], p["rot"], intr, extr, W, H, shs=p["shs"].detach()[:, 0])
    with pytest.raises(RuntimeError, match="D = 5"):
        ms.preprocess(p["xyz"], p["scale"], p["rot"], intr, extr, W, H, shs=torch.zeros(2000, 3, 5, device=DEV))
