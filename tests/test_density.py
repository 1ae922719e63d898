"""Density control: the fixed-count prune / densify step of the reference's
training loop (tutorials/gs_3d.py:193-225), on CPU tensors, and the GPU
statistics accumulated from the ndc gradient of a real backward pass."""
import pytest
import torch

from _scenes import camera, scene


def test_prune_and_densify_follows_the_reference_loop():
    from msplat_gb300.density import prune_and_densify
    g = torch.Generator().manual_seed(0)
    P = 64
    params = {"xyzs": torch.randn(P, 3, generator=g), "rgbs": torch.rand(P, 3, generator=g),
              "opacity": torch.randn(P, 1, generator=g) * 3, "scales": torch.randn(P, 3, generator=g),
              "rot": torch.randn(P, 4, generator=g)}
    before = {k: v.clone() for k, v in params.items()}
    # the reference's own sequence, spelled out
    opacity = torch.sigmoid(before["opacity"])
    prune = torch.nonzero(opacity[:, 0] < 0.01).squeeze(-1)
    if prune.numel() == 0:
        before["opacity"][:5] = -10.0
        params["opacity"][:5] = -10.0
        prune = torch.nonzero(torch.sigmoid(before["opacity"])[:, 0] < 0.01).squeeze(-1)
    dens = torch.argsort(before["scales"].amax(dim=1), descending=True)[:prune.numel()]
    ref = {k: v.clone() for k, v in before.items()}
    for k in ref:
        ref[k][torch.cat([prune, dens])] = before[k][dens].repeat(2, 1)
    n = prune_and_densify(params)
    assert n == prune.numel() > 0
    for k in params:
        assert torch.equal(params[k], ref[k]), k
    assert prune_and_densify({k: v.clone() for k, v in ref.items()}, threshold=0.0) == 0


@pytest.mark.gpu
def test_density_stats_accumulate_ndc_gradient_norms():
    import msplat_gb300 as ms
    from msplat_gb300 import _build
    _build.build()
    W, H = 160, 120
    s = scene(5000, 3, C=3)
    intr, extr = camera(W, H, seed=2)
    t = {k: v.cuda().requires_grad_() for k, v in s.items()}
    stats = ms.DensityStats(5000)
    ref_acc, ref_cnt, ref_max = torch.zeros(5000), torch.zeros(5000, dtype=torch.int32), torch.zeros(5000, dtype=torch.int32)
    for frame in range(3):
        ndc = torch.zeros(5000, 2, device="cuda", requires_grad=True)
        img, radius = ms.rasterization(t["xyz"], t["scale"], t["rot"], t["opacity"], t["feat"],
                                       torch.as_tensor(intr).cuda(), torch.as_tensor(extr).cuda(), W, H, 0.0, ndc,
                                       return_radius=True)
        (img * (frame + 1)).square().sum().backward()
        stats.update(ndc.grad, radius)
        vis = (radius > 0).cpu()
        ref_acc += torch.where(vis, ndc.grad.norm(dim=1).cpu(), torch.zeros(()))
        ref_cnt += vis.int()
        ref_max = torch.maximum(ref_max, radius.cpu())
    assert ref_cnt.sum() > 0
    torch.testing.assert_close(stats.grad_accum.cpu(), ref_acc, rtol=1e-5, atol=1e-7)
    assert torch.equal(stats.count.cpu(), ref_cnt)
    assert torch.equal(stats.max_radius.cpu(), ref_max)
    m = stats.mean_grad()
    assert torch.isfinite(m).all()
    stats.reset()
    assert stats.count.sum().item() == 0
