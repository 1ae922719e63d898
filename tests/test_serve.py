"""The render server: every result equals the request served alone (images
bit-identical, gradients equal up to the order of float atomics), in a mix
of scenes, image sizes and forward / forward+backward requests that is
batched and run on several streams; and a budget that admits one request
at a time still serves everything."""
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


def scenes():
    out = []
    for n, seed in ((20000, 1), (50000, 2)):
        s = scene(n, seed, C=3, sh_deg=1)
        out.append({"xyz": s["xyz"].to(DEV), "scale": s["scale"].to(DEV), "rot": s["rot"].to(DEV),
                    "opacity": s["opacity"].to(DEV), "shs": s["shs"].to(DEV).contiguous()})
    return out


def requests(n, seed, spread):
    from msplat_gb300.serve import Request
    rng = np.random.default_rng(seed)
    sizes = [(64, 64), (96, 80), (128, 96)]
    out = []
    for i in range(n):
        w, h = sizes[rng.integers(len(sizes))]
        f = 300.0 * w / 256
        bwd = bool(rng.random() < 0.25)
        out.append(Request(scene=int(rng.integers(2)), intr=torch.tensor([f, f, w / 2, h / 2], device=DEV),
                           extr=torch.tensor(sphere_camera(rng), device=DEV), W=w, H=h, backward=bwd,
                           weights=torch.randn(3, h, w, generator=torch.Generator().manual_seed(i)).to(DEV)
                           if bwd else None,
                           arrival=0.0 if i < n // 2 else float(rng.uniform(0, spread))))
    return out


def alone(sc, r):
    import msplat_gb300 as ms
    leaves = {k: v.detach().requires_grad_() for k, v in sc.items()}
    img = ms.rasterization_sh(leaves["xyz"], leaves["scale"], leaves["rot"], leaves["opacity"], leaves["shs"],
                              r.intr, r.extr, r.W, r.H, r.bg)
    if not r.backward:
        return img.detach(), None
    (img * r.weights).sum().backward()
    return img.detach(), {k: v.grad for k, v in leaves.items()}


def check(scs, served):
    for r in served:
        img, grads = alone(scs[r.scene], r)
        assert torch.equal(r.image, img)
        if r.backward:
            for k, g in grads.items():
                ref = g.abs().max().item()
                assert (r.grads[k] - g).abs().max().item() <= 1e-5 * max(ref, 1e-30), k


@pytest.mark.timeout(300)
def test_served_results_equal_requests_alone():
    from msplat_gb300.serve import Server
    scs = scenes()
    reqs = requests(32, 0, 0.05)
    srv = Server(scs, hbm_budget=8 << 30, streams=3, max_batch=8, max_backward=4)
    served = srv.serve(reqs, timeout=120)
    assert all(r.done is not None and r.done >= r.arrival for r in served)
    assert max(r.batch for r in served) > 1, "nothing was batched"
    assert max(r.batch for r in served if r.backward) > 1, "no backward requests were batched together"
    assert srv.peak_allocated <= 8 << 30
    check(scs, served)


@pytest.mark.timeout(300)
def test_budget_of_one_request_still_serves_everything():
    from msplat_gb300.serve import Server, request_bytes
    scs = scenes()
    reqs = requests(10, 1, 0.01)
    big = max(request_bytes(scs[r.scene]["shs"].shape[0], r.W, r.H, 3, 4, r.backward) for r in reqs)
    served = Server(scs, hbm_budget=big, streams=2).serve(reqs, timeout=120)
    check(scs, served)
    with pytest.raises(RuntimeError, match="budget"):
        Server(scs, hbm_budget=1000).serve(requests(2, 2, 0.0))
