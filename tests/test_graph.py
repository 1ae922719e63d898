"""The frame without host reads: a capacity-bounded tile sort whose count
stays on the device, and a forward + backward frame captured in a CUDA
graph and replayed.

* with enough capacity the sort's valid part and tile ranges equal the
  exact sort, and status is 0;
* with too little capacity status is 1 (and nothing is written out of
  bounds: the ranges stay inside the capacity);
* the captured frame, replayed on new parameter values copied into its
  static inputs, gives the eager frame's image bit for bit and its
  gradients up to the order of float atomics.
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


def projected(n, W, H, seed):
    import msplat_gb300 as ms
    s = scene(n, seed, C=3, sh_deg=2)
    intr, extr = camera(W, H, seed=seed)
    p = {k: s[k].to(DEV).contiguous() for k in ("xyz", "scale", "rot", "opacity", "shs")}
    p["intr"], p["extr"] = torch.as_tensor(intr).to(DEV), torch.as_tensor(extr).to(DEV)
    uv, depth, conic, radius, tiles, color = ms.preprocess(p["xyz"], p["scale"], p["rot"], p["intr"], p["extr"],
                                                           W, H, shs=p["shs"])
    return p, uv, depth, radius, tiles


def test_capacity_sort_equals_the_exact_sort_and_reports_overflow():
    import msplat_gb300 as ms
    from msplat_gb300.sort_gaussian import sort_gaussian_capacity
    W, H = 320, 240
    p, uv, depth, radius, tiles = projected(30000, W, H, 3)
    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles)
    I = idx.numel()
    assert I > 10000
    status = torch.full((1,), 7, dtype=torch.int32, device=DEV)
    cidx, ctr = sort_gaussian_capacity(uv, depth, W, H, radius, tiles, I + 1000, status)
    assert int(status.item()) == 0
    assert torch.equal(ctr, tr)
    assert torch.equal(cidx[:I], idx)
    small = I // 2
    cidx, ctr = sort_gaussian_capacity(uv, depth, W, H, radius, tiles, small, status)
    torch.cuda.synchronize()
    assert int(status.item()) == 1
    assert int(ctr.max().item()) <= small


def test_captured_frame_replays_the_eager_frame():
    import msplat_gb300 as ms
    W, H = 256, 192
    p, uv, depth, radius, tiles = projected(20000, W, H, 5)
    idx, _ = ms.sort_gaussian(uv, depth, W, H, radius, tiles)
    cap = int(idx.numel() * 1.25) + 1024
    w = torch.randn(3, H, W, generator=torch.Generator().manual_seed(1)).to(DEV)
    static = {k: v.clone().requires_grad_() for k, v in p.items()}
    status = torch.zeros(1, dtype=torch.int32, device=DEV)

    def step():
        img = ms.rasterization_sh(static["xyz"], static["scale"], static["rot"], static["opacity"], static["shs"],
                                  static["intr"], static["extr"], W, H, 0.0, capacity=cap, status=status)
        (img * w).sum().backward()
        return img

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(3):
            for t in static.values():
                t.grad = None
            step()
    torch.cuda.current_stream().wait_stream(side)
    for t in static.values():
        t.grad = None
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        img_static = step()

    # new parameter values, then replay
    g = torch.Generator().manual_seed(9)
    newp = {k: v.detach().clone() for k, v in p.items()}
    newp["xyz"] += torch.randn(newp["xyz"].shape, generator=g).to(DEV) * 0.01
    newp["opacity"] = torch.sigmoid(torch.randn(newp["opacity"].shape, generator=g)).to(DEV)
    with torch.no_grad():
        for k in static:
            static[k].copy_(newp[k])
    graph.replay()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    eager = {k: v.clone().requires_grad_() for k, v in newp.items()}
    img = ms.rasterization_sh(eager["xyz"], eager["scale"], eager["rot"], eager["opacity"], eager["shs"],
                              eager["intr"], eager["extr"], W, H, 0.0)
    (img * w).sum().backward()
    assert torch.equal(img_static, img)
    for k in static:
        got, ref = static[k].grad, eager[k].grad
        scale = ref.abs().max().item()
        assert (got - ref).abs().max().item() <= 1e-5 * max(scale, 1e-30), k


def test_captured_batch_replays_the_eager_batch():
    """Four cameras of one scene, forward + backward, captured in one CUDA
    graph (one sort over all cameras, one blend grid over all their tiles)."""
    import msplat_gb300 as ms
    from _scenes import sphere_camera
    sizes = [(128, 96), (160, 120), (96, 96), (200, 104)]
    s = scene(15000, 8, C=3, sh_deg=1)
    rng = np.random.default_rng(8)
    intrs = torch.tensor([[300.0 * w / 256, 300.0 * w / 256, w / 2, h / 2] for w, h in sizes], device=DEV)
    extrs = torch.tensor(np.stack([sphere_camera(rng) for _ in sizes]), device=DEV)
    base = {k: s[k].to(DEV).contiguous() for k in ("xyz", "scale", "rot", "opacity", "shs")}
    static = {k: v.clone().requires_grad_() for k, v in base.items()}
    ws = [torch.randn(3, h, w, generator=torch.Generator().manual_seed(i)).to(DEV) for i, (w, h) in enumerate(sizes)]
    status = torch.zeros(1, dtype=torch.int32, device=DEV)
    cap = 800_000

    def step():
        imgs = ms.rasterization_sh_batch(static["xyz"], static["scale"], static["rot"], static["opacity"],
                                         static["shs"], intrs, extrs, sizes, 0.1, capacity=cap, status=status)
        sum((i * w).sum() for i, w in zip(imgs, ws)).backward()
        return imgs

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(3):
            for t in static.values():
                t.grad = None
            step()
    torch.cuda.current_stream().wait_stream(side)
    for t in static.values():
        t.grad = None
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        imgs_static = step()
    graph.replay()
    torch.cuda.synchronize()
    assert int(status.sum().item()) == 0
    eager = {k: v.clone().requires_grad_() for k, v in base.items()}
    refs = ms.rasterization_sh_batch(eager["xyz"], eager["scale"], eager["rot"], eager["opacity"], eager["shs"],
                                     intrs, extrs, sizes, 0.1)
    sum((i * w).sum() for i, w in zip(refs, ws)).backward()
    for a, b in zip(imgs_static, refs):
        assert torch.equal(a, b)
    for k in static:
        got, ref = static[k].grad, eager[k].grad
        assert (got - ref).abs().max().item() <= 1e-5 * max(ref.abs().max().item(), 1e-30), k


def test_capacity_finish_past_int32_counts_writes_nothing_out_of_bounds():
    """600 Gaussians that each cover all 2048 x 2048 tiles of a 32768^2 image
    give 600 * 2^22 (> 2^31) intersections; the third block of 256 Gaussians
    starts exactly at 2^31.  With a capacity of 4096 the status is 1, only
    the first Gaussian in depth order is emitted (its first 4096 tiles), and
    the guard words around the output and the workspace stay untouched."""
    from msplat_gb300 import _lib
    lib = _lib.load()
    W = H = 32768
    P, cap, G = 600, 4096, 4096
    nt = (W // 16) * (H // 16)
    uv = torch.full((P, 2), 16384.0, device=DEV)
    depth = torch.linspace(1.0, 2.0, P, device=DEV).reshape(P, 1).flip(0).contiguous()  # last id nearest
    radius = torch.full((P,), 30000, dtype=torch.int32, device=DEV)
    tiles = torch.full((P,), nt, dtype=torch.int32, device=DEV)
    st = _lib.stream()
    counts = torch.empty(2, dtype=torch.int64, device=DEV)
    ws_prep = _lib.workspace(lib.msplat_sort_prepare_workspace_size(P, W, H), DEV)
    _lib.check(lib.msplat_sort_gaussian_prepare(P, _lib.ptr(depth), _lib.ptr(radius), _lib.ptr(tiles), _lib.ptr(uv),
                                                W, H, _lib.ptr(counts), _lib.ptr(ws_prep), ws_prep.numel(), st),
               "prepare")
    sentinel = -123456789
    idx = torch.full((cap + 2 * G,), sentinel, dtype=torch.int32, device=DEV)
    wsb = int(lib.msplat_sort_finish_workspace_size(P, cap, W, H))
    ws = torch.full((wsb + 2 * 4 * G,), 0x5A, dtype=torch.uint8, device=DEV)
    tr = torch.full((nt, 2), sentinel, dtype=torch.int32, device=DEV)
    status = torch.zeros(1, dtype=torch.int32, device=DEV)
    _lib.check(lib.msplat_sort_gaussian_finish_capacity(
        P, _lib.ptr(uv), _lib.ptr(depth), _lib.ptr(radius), W, H, cap, _lib.ptr(counts), _lib.ptr(ws_prep),
        idx.data_ptr() + 4 * G, _lib.ptr(tr), _lib.ptr(status), ws.data_ptr() + 4 * G, wsb, st), "finish_capacity")
    torch.cuda.synchronize()
    assert int(counts[0].item()) == P * nt > 2**31
    assert int(status.item()) == 1
    assert bool((idx[:G] == sentinel).all()) and bool((idx[G + cap:] == sentinel).all())
    assert bool((ws[:4 * G] == 0x5A).all()) and bool((ws[4 * G + wsb:] == 0x5A).all())
    assert bool((idx[G:G + cap] == P - 1).all())  # the nearest Gaussian's first 4096 tiles
    t = torch.arange(cap, dtype=torch.int32, device=DEV)
    assert torch.equal(tr[:cap], torch.stack([t, t + 1], 1))
    assert bool((tr[cap:] == 0).all())
