"""The fused path's tile sort through tile-row segments (one radix pass)
against the culled two-pass sort: every tile's list identical (same ids in
the same order), on odd image sizes and the benchmark's 1080p frame; with a
capacity: status 0 and the same lists when it suffices, 1 when it does not;
no Gaussians; and grids wider than 256 tiles falling back to the two-pass
sort inside rasterization."""
import numpy as np
import pytest
import torch

from _scenes import scene, sphere_camera

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module", autouse=True)
def _built():
    from msplat_gb300 import _build, _lib
    _build.build()
    _lib.load()
    yield


def projected(n, W, H, seed, f=None):
    import msplat_gb300 as ms
    s = scene(n, seed, C=3)
    f = f if f is not None else 300.0 * W / 256
    intr = torch.tensor([f, f, W / 2, H / 2], device=DEV)
    extr = torch.tensor(sphere_camera(np.random.default_rng(seed)), device=DEV)
    xyz, scale, rot = (s[k].to(DEV).contiguous() for k in ("xyz", "scale", "rot"))
    uv, depth, conic, radius, tiles, _ = ms.preprocess(xyz, scale, rot, intr, extr, W, H)
    return uv, depth, radius, tiles, conic, s["opacity"].to(DEV).contiguous()


def tile_lists(idx, tr):
    idx, tr = idx.cpu().numpy(), tr.cpu().numpy()
    lens = tr[:, 1] - tr[:, 0]
    cat = np.concatenate([idx[a:b] for a, b in tr]) if len(tr) else np.zeros(0, np.int32)
    return lens, cat


@pytest.mark.parametrize("W,H,n,seed", [(320, 240, 30000, 1), (333, 197, 20000, 2), (1920, 1080, 400000, 3),
                                        (64, 48, 500, 4)])
def test_row_lists_equal_the_two_pass_lists(W, H, n, seed):
    import msplat_gb300 as ms
    from msplat_gb300.sort_gaussian import sort_gaussian_rows
    uv, depth, radius, tiles, conic, op = projected(n, W, H, seed)
    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles, cull=(conic, op))
    ridx, rtr = sort_gaussian_rows(uv, depth, W, H, radius, tiles, (conic, op))
    l1, c1 = tile_lists(idx, tr)
    l2, c2 = tile_lists(ridx, rtr)
    np.testing.assert_array_equal(l1, l2)
    np.testing.assert_array_equal(c1, c2)
    assert c1.size == idx.numel() > 0


def test_row_lists_with_a_capacity():
    import msplat_gb300 as ms
    from msplat_gb300.sort_gaussian import sort_gaussian_rows
    W, H = 320, 240
    uv, depth, radius, tiles, conic, op = projected(30000, W, H, 5)
    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles, cull=(conic, op))
    status = torch.full((1,), 7, dtype=torch.int32, device=DEV)
    ridx, rtr = sort_gaussian_rows(uv, depth, W, H, radius, tiles, (conic, op), capacity=idx.numel(), status=status)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    np.testing.assert_array_equal(tile_lists(idx, tr)[1], tile_lists(ridx, rtr)[1])
    sort_gaussian_rows(uv, depth, W, H, radius, tiles, (conic, op), capacity=0, status=status)
    torch.cuda.synchronize()
    assert int(status.item()) == 1


def test_row_lists_without_gaussians():
    from msplat_gb300.sort_gaussian import sort_gaussian_rows
    z2 = torch.zeros(0, 2, device=DEV)
    z1 = torch.zeros(0, 1, device=DEV)
    zi = torch.zeros(0, dtype=torch.int32, device=DEV)
    idx, tr = sort_gaussian_rows(z2, z1, 100, 60, zi, zi, (torch.zeros(0, 3, device=DEV), z1))
    assert int(tr.abs().sum().item()) == 0


def test_wide_images_fall_back_to_two_passes():
    import msplat_gb300 as ms
    W, H = 4128, 64  # 258 tile columns
    s = scene(20000, 6, C=3)
    f = 300.0 * W / 256
    p = [s[k].to(DEV).contiguous() for k in ("xyz", "scale", "rot", "opacity", "feat")]
    intr = torch.tensor([f, f, W / 2, H / 2], device=DEV)
    extr = torch.tensor([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 4.0]], device=DEV)
    img = ms.rasterization(*p, intr, extr, W, H, 0.0)
    uv, depth = ms.project_point(p[0], intr, extr, W, H)
    vis = depth.reshape(-1) != 0
    cov = ms.compute_cov3d(p[1], p[2], vis)
    conic, radius, tiles = ms.ewa_project(p[0], cov, intr, extr, uv, W, H, vis)
    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles)
    ref = ms.alpha_blending(uv, conic, p[3], p[4], idx, tr, 0.0, W, H)
    assert torch.equal(img, ref)
