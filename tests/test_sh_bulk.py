"""The SH kernels' two ways of staging coefficient rows: one bulk copy per
block (rows of an odd number of floats, 16-byte aligned arrays) and the
padded thread loop (everything else).  Both run the same arithmetic on the
same rows, so their results must agree bit for bit where both use the
same kernel code; a coefficient array that starts 4 bytes past a 16-byte
boundary takes the thread loop.  Three channels at degree >= 4 on the bulk
path run kernels with the channel count fixed at compile time, whose
multiply-adds the compiler may contract differently from the general
kernels' (the misaligned thread loop at even degree): those two agree to
1e-6 of the largest value.  The
point counts leave every remainder of the last block's row count modulo 4
(the floats the bulk copy cannot move), and the oracle checks the values.
The bounded wait for a bulk copy is made to run out (a poll limit of 0) and
must be reported by msplat_wait_error with the context left usable."""
import ctypes

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def lib():
    from msplat_gb300 import _build, _lib
    _build.build()
    return _lib.load()


def misaligned(a: np.ndarray) -> torch.Tensor:
    """A device copy of `a` whose data starts 4 bytes past a 16-byte boundary."""
    flat = torch.empty(a.size + 4, dtype=torch.float32, device=DEV)
    assert flat.data_ptr() % 16 == 0
    t = flat[1:1 + a.size].view(a.shape)
    t.copy_(torch.from_numpy(a))
    assert t.data_ptr() % 16 == 4
    return t


def sh_case(P, C, deg, seed):
    rng = np.random.default_rng(seed)
    D = (deg + 1) ** 2
    shs = rng.normal(scale=0.3, size=(P, C, D)).astype(np.float32)
    d = rng.normal(size=(P, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    vis = rng.random(P) > 0.1
    w = rng.normal(size=(P, C)).astype(np.float32)
    return shs, d, vis, w


def run_sh(sh_t, d, vis, w):
    import msplat_gb300 as ms
    sh_t = sh_t.detach().requires_grad_()
    td = torch.from_numpy(d).to(DEV).requires_grad_()
    val = ms.compute_sh(sh_t, td, torch.from_numpy(vis).to(DEV))
    (val * torch.from_numpy(w).to(DEV)).sum().backward()
    return val.detach(), sh_t.grad, td.grad


@pytest.mark.parametrize("deg,C", [(0, 1), (2, 3), (4, 1), (6, 5), (10, 1), (10, 3)])
@pytest.mark.parametrize("P", [1, 2, 3, 5, 63, 65, 130, 1001])
def test_bulk_equals_thread_loop(lib, deg, C, P):
    shs, d, vis, w = sh_case(P, C, deg, seed=P * 31 + deg * 7 + C)
    a = run_sh(torch.from_numpy(shs).to(DEV), d, vis, w)
    b = run_sh(misaligned(shs), d, vis, w)
    same_code = not (C == 3 and deg >= 4)
    for x, y in zip(a, b):
        if same_code:
            assert torch.equal(x, y)
        else:
            assert (x - y).abs().max().item() <= 1e-6 * max(y.abs().max().item(), 1e-30)
    oval = oracle.compute_sh_forward(shs, d, vis)
    scale = max(np.abs(oval).max(), 1e-30)
    assert np.abs(a[0].cpu().numpy() - oval).max() <= 1e-5 * scale
    dsh, _ = oracle.compute_sh_backward(shs, d, vis, w)
    scale = max(np.abs(dsh).max(), 1e-30)
    assert np.abs(a[1].cpu().numpy() - dsh).max() <= 1e-5 * scale


def test_bulk_camera_mode(lib):
    """The fused preprocess's SH (view directions from the centres, degree
    10, 3 colours) through both staging paths, forward and backward."""
    import msplat_gb300 as ms
    from _scenes import scene, sphere_camera
    P, W, H = 4099, 320, 240
    s = scene(P, 12, C=3)
    rng = np.random.default_rng(3)
    shs = rng.normal(scale=0.1, size=(P, 3, 121)).astype(np.float32)
    intr = torch.tensor([300.0, 300.0, W / 2, H / 2], device=DEV)
    extr = torch.tensor(sphere_camera(np.random.default_rng(5)), device=DEV)
    outs = []
    for sh_t in (torch.from_numpy(shs).to(DEV), misaligned(shs)):
        xyz = s["xyz"].to(DEV).contiguous().requires_grad_()
        sh_t = sh_t.detach().requires_grad_()
        uv, depth, conic, radius, tiles, color = ms.preprocess(
            xyz, s["scale"].to(DEV).contiguous(), s["rot"].to(DEV).contiguous(), intr, extr, W, H, shs=sh_t)
        g = torch.from_numpy(np.random.default_rng(9).normal(size=(P, 3)).astype(np.float32)).to(DEV)
        (color * g).sum().backward()
        outs.append((color.detach(), sh_t.grad, xyz.grad))
    for x, y in zip(*outs):  # fixed-C kernels (bulk) against the general ones (thread loop)
        assert (x - y).abs().max().item() <= 1e-6 * max(y.abs().max().item(), 1e-30)


def test_bulk_wait_that_runs_out_reports_timeout(lib):
    from msplat_gb300 import _lib
    shs, d, vis, w = sh_case(700, 3, 10, seed=4)
    err = ctypes.c_int(0)
    assert lib.msplat_wait_error(1, ctypes.byref(err), _lib.stream()) == 0  # clear
    lib.msplat_set_wait_limit(0)  # every wait for a bulk copy gives up at once
    try:
        run_sh(torch.from_numpy(shs).to(DEV), d, vis, w)
        torch.cuda.synchronize()
    finally:
        lib.msplat_set_wait_limit(1 << 21)
    assert lib.msplat_wait_error(1, ctypes.byref(err), _lib.stream()) == 6  # MSPLAT_ERR_TIMEOUT
    assert err.value == 1
    assert lib.msplat_wait_error(0, ctypes.byref(err), _lib.stream()) == 0 and err.value == 0
    # the context is healthy and the next evaluation is right again
    a = run_sh(torch.from_numpy(shs).to(DEV), d, vis, w)
    b = run_sh(misaligned(shs), d, vis, w)
    for x, y in zip(a, b):
        assert (x - y).abs().max().item() <= 1e-6 * max(y.abs().max().item(), 1e-30)
    assert lib.msplat_wait_error(0, ctypes.byref(err), _lib.stream()) == 0


# Rows longer than a block's shared memory holds: even C * D beyond 1,600
# floats take the channel-sliced kernels (16 channels at degree 10, 20 at
# degree 9, 120 at degree 3), odd ones the bulk path with blocks of 4
# Gaussians (17 channels at degree 10).  The reference evaluates any
# channel count (one thread per Gaussian looping over the channels).
@pytest.mark.parametrize("deg,C", [(10, 16), (9, 20), (3, 120), (10, 17)])
def test_many_channels_against_the_oracle(lib, deg, C):
    P = 301
    shs, d, vis, w = sh_case(P, C, deg, seed=deg * 100 + C)
    val, dsh, ddir = run_sh(torch.from_numpy(shs).to(DEV), d, vis, w)
    oval = oracle.compute_sh_forward(shs, d, vis)
    assert np.abs(val.cpu().numpy() - oval).max() <= 1e-5 * max(np.abs(oval).max(), 1e-30)
    odsh, oddir = oracle.compute_sh_backward(shs, d, vis, w)
    assert np.abs(dsh.cpu().numpy() - odsh).max() <= 1e-5 * max(np.abs(odsh).max(), 1e-30)
    assert np.abs(ddir.cpu().numpy() - oddir).max() <= 1e-4 * max(np.abs(oddir).max(), 1e-30)


def test_many_channels_camera_mode(lib):
    """The fused preprocess's view-direction SH with 16 channels at degree
    10 (sliced kernels in camera mode) against compute_sh on the same
    directions computed in PyTorch, forward and backward."""
    import msplat_gb300 as ms
    from _scenes import scene, sphere_camera
    P, W, H, C = 2003, 320, 240, 16
    s = scene(P, 21, C=3)
    shs = torch.from_numpy(np.random.default_rng(8).normal(scale=0.1, size=(P, C, 121)).astype(np.float32)).to(DEV)
    intr = torch.tensor([300.0, 300.0, W / 2, H / 2], device=DEV)
    extr = torch.tensor(sphere_camera(np.random.default_rng(6)), device=DEV)
    xyz = s["xyz"].to(DEV).contiguous()
    g = torch.from_numpy(np.random.default_rng(10).normal(size=(P, C)).astype(np.float32)).to(DEV)
    a = shs.clone().requires_grad_()
    _, depth, _, _, _, color = ms.preprocess(xyz, s["scale"].to(DEV).contiguous(), s["rot"].to(DEV).contiguous(),
                                             intr, extr, W, H, shs=a)
    (color * g).sum().backward()
    R, t = extr[:, :3], extr[:, 3]
    v = xyz + R.transpose(0, 1) @ t
    dirs = v / v.norm(dim=-1, keepdim=True)
    b = shs.clone().requires_grad_()
    ref = ms.compute_sh(b, dirs, (depth != 0).view(-1))
    (ref * g).sum().backward()
    scale = ref.abs().max().item()
    assert (color.detach() - ref.detach()).abs().max().item() <= 1e-5 * scale
    assert (a.grad - b.grad).abs().max().item() <= 1e-5 * b.grad.abs().max().item()
