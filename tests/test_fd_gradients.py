"""Gradients of the whole differentiable chain (view directions -> SH ->
rasterization -> loss) against float64 central finite differences.

The GPU computes the loss sum(W * image) and its gradients with respect to
xyz, scales, rotations, opacity, SH coefficients, intrinsics and extrinsics.
The finite differences come from a float64 restatement of the same forward
(SH basis from the oracle, projection, covariance, EWA conic, front-to-back
blend) evaluated with the blend's discrete decisions frozen at the
unperturbed point: which (pixel, Gaussian) pairs pass the 1/255 and T < 1e-4
tests and which alphas sit at the 0.99 clamp.  Those decisions make the
loss piecewise smooth; the adjoint kernels differentiate the smooth piece
that the forward selected, and so does the frozen float64 forward.

Cases: the benchmark scene's distributions at 2,000 Gaussians and 64x64 (focal
length scaled to keep the 1080p field of view), and a front-facing camera
with larger Gaussians so that many pairs overlap.
"""
import numpy as np
import pytest
import torch

import oracle
from _scenes import camera, scene

pytestmark = pytest.mark.gpu
DEV = "cuda"
SH_DEG = 3


@pytest.fixture(scope="module", autouse=True)
def _built():
    from msplat_gb300 import _build, _lib
    _build.build()
    _lib.load()
    yield


def view_dirs(xyz, extr):
    R, t = extr[:, :3], extr[:, 3]
    d = xyz + R.transpose(0, 1) @ t
    return d / d.norm(dim=-1, keepdim=True)


def gpu_grads(p, W, H, bg, weights):
    import msplat_gb300 as ms
    t = {k: torch.as_tensor(v, dtype=torch.float32).to(DEV).requires_grad_() for k, v in p.items()}
    color = ms.compute_sh(t["shs"], view_dirs(t["xyz"], t["extr"]))
    img = ms.rasterization(t["xyz"], t["scale"], t["rot"], t["opacity"], color, t["intr"], t["extr"], W, H, bg)
    loss = (img * torch.as_tensor(weights).to(DEV)).sum()
    loss.backward()
    uv, depth = ms.project_point(t["xyz"].detach(), t["intr"].detach(), t["extr"].detach(), W, H)
    vis = depth.reshape(-1) != 0
    cov = ms.compute_cov3d(t["scale"].detach(), t["rot"].detach(), vis)
    _, radius, tiles = ms.ewa_project(t["xyz"].detach(), cov, t["intr"].detach(), t["extr"].detach(), uv, W, H, vis)
    idx, tr = ms.sort_gaussian(uv, depth, W, H, radius, tiles)
    lists = (idx.cpu().numpy(), tr.cpu().numpy())
    return float(loss.item()), {k: v.grad.double().cpu().numpy() for k, v in t.items()}, lists


class Frozen64:
    """float64 forward of the chain with the blend decisions of the point it
    was built at."""

    def __init__(self, p, W, H, bg, weights, lists):
        self.W, self.H, self.bg, self.w = W, H, bg, np.asarray(weights, np.float64)
        idx, tr = lists
        gx = (W + 15) // 16
        py, px = np.mgrid[0:H, 0:W]
        tile = (py // 16) * gx + px // 16
        s, e = tr[tile.reshape(-1), 0], tr[tile.reshape(-1), 1]
        L = int((e - s).max()) if e.size else 0
        j = np.arange(L)[None, :]
        self.inlist = j < (e - s)[:, None]
        self.ids = np.where(self.inlist, idx[np.minimum(s[:, None] + j, max(idx.size - 1, 0))], 0)
        self.px, self.py = px.reshape(-1, 1).astype(np.float64), py.reshape(-1, 1).astype(np.float64)
        self.mask = self.clamp = None
        self._decide(p)

    def _terms(self, p):
        xyz, extr, intr = p["xyz"], p["extr"], p["intr"]
        R, t = extr[:, :3], extr[:, 3]
        d = xyz + R.T @ t
        d = d / np.linalg.norm(d, axis=1, keepdims=True)
        Y, _ = oracle.sh_basis(d, SH_DEG)
        color = np.einsum("pk,pck->pc", Y, p["shs"])
        tc = xyz @ R.T + t
        fx, fy, cx, cy = intr
        u = fx * tc[:, 0] / tc[:, 2] + cx - 0.5
        v = fy * tc[:, 1] / tc[:, 2] + cy - 0.5
        r, x, y, z = p["rot"].T
        Rq = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)], -1),
                       np.stack([2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)], -1),
                       np.stack([2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)], -1)], 1)
        A = Rq * p["scale"][:, None, :]
        Sig = A @ A.transpose(0, 2, 1)
        zz = tc[:, 2]
        J = np.zeros((len(xyz), 2, 3))
        J[:, 0, 0] = fx / zz
        J[:, 0, 2] = -fx * tc[:, 0] / zz ** 2
        J[:, 1, 1] = fy / zz
        J[:, 1, 2] = -fy * tc[:, 1] / zz ** 2
        Tm = J @ R
        c2 = Tm @ Sig @ Tm.transpose(0, 2, 1)
        a, b, c = c2[:, 0, 0] + 0.3, c2[:, 0, 1], c2[:, 1, 1] + 0.3
        det = a * c - b * b
        conic = np.stack([c / det, -b / det, a / det], 1)
        ids = self.ids
        dx, dy = u[ids] - self.px, v[ids] - self.py
        A_, B_, C_ = conic[ids, 0], conic[ids, 1], conic[ids, 2]
        power = -0.5 * (A_ * dx * dx + C_ * dy * dy) - B_ * dx * dy
        raw = p["opacity"].reshape(-1)[ids] * np.exp(power)
        return color, power, raw

    def _decide(self, p):
        _, power, raw = self._terms(p)
        alpha = np.minimum(0.99, raw)
        ok = self.inlist & (power <= 0) & (alpha >= 1.0 / 255.0)
        T = np.ones(ok.shape[0])
        live = np.ones(ok.shape[0], bool)
        for j in range(ok.shape[1]):
            use = ok[:, j] & live
            nT = T * (1 - alpha[:, j])
            stop = use & (nT < 1e-4)
            live &= ~stop
            use &= ~stop
            ok[:, j] = use
            T = np.where(use, nT, T)
        self.mask, self.clamp = ok, raw > 0.99

    def loss(self, p):
        color, _, raw = self._terms(p)
        alpha = np.where(self.clamp, 0.99, raw) * self.mask
        one_m = 1.0 - alpha
        Texcl = np.concatenate([np.ones((alpha.shape[0], 1)), np.cumprod(one_m, axis=1)[:, :-1]], 1)
        wsum = alpha * Texcl
        F = np.einsum("nj,njc->nc", wsum, color[self.ids])
        Tf = np.prod(one_m, axis=1)
        img = F + Tf[:, None] * self.bg
        return float((img.T.reshape(-1, self.H, self.W) * self.w).sum())


def make_case(kind):
    W = H = 64
    if kind == "bench_scene":
        s = scene(2000, seed=11, C=3, sh_deg=SH_DEG)
        f = 1500.0 * W / 1920.0
        intr, extr = camera(W, H, f=f, seed=4)
        intr[2], intr[3] = W / 2, H / 2
    else:
        s = scene(2000, seed=12, C=3, sh_deg=SH_DEG)
        s["scale"] = s["scale"] * 6.0
        intr, extr = camera(W, H, seed=0, front=True)
    shs = s["shs"].numpy().astype(np.float64)
    p = {"xyz": s["xyz"].numpy(), "scale": s["scale"].numpy(), "rot": s["rot"].numpy(),
         "opacity": s["opacity"].numpy(), "shs": shs, "intr": intr, "extr": extr}
    p = {k: np.asarray(v, np.float32) for k, v in p.items()}
    weights = np.random.default_rng(5).normal(size=(3, H, W)).astype(np.float32)
    return p, W, H, weights


@pytest.mark.parametrize("kind", ["bench_scene", "front_large"])
def test_gradients_match_fp64_central_differences(kind):
    p, W, H, weights = make_case(kind)
    bg = 0.25
    loss32, grads, lists = gpu_grads(p, W, H, bg, weights)
    p64 = {k: v.astype(np.float64) for k, v in p.items()}
    fz = Frozen64(p64, W, H, bg, weights, lists)
    assert fz.mask.sum() > 2000, "too few blended pairs for a meaningful check"
    loss64 = fz.loss(p64)
    assert abs(loss64 - loss32) <= 1e-4 * max(1.0, abs(loss64)), (loss64, loss32)

    rng = np.random.default_rng(7)
    report = {}
    for name, g in grads.items():
        # a random direction per parameter group, scaled to the group's values
        d = rng.normal(size=g.shape)
        mag = np.abs(p64[name]).mean() or 1.0
        h = 1e-6 * mag
        pp = dict(p64)
        pp[name] = p64[name] + h * d
        lp = fz.loss(pp)
        pp[name] = p64[name] - h * d
        lm = fz.loss(pp)
        fd = (lp - lm) / (2 * h)
        an = float((g * d).sum())
        scale = float(np.abs(g * d).sum())
        err = abs(fd - an) / max(scale, 1e-30)
        report[name] = err
        assert err <= 1e-4, f"{name}: directional derivative fd={fd:.6e} analytic={an:.6e} rel err {err:.2e}"

        # and single coordinates: the largest gradient entries of the group
        flat = np.argsort(-np.abs(g).reshape(-1))[:3]
        for fi in flat:
            e = np.zeros(g.size)
            e[fi] = 1.0
            e = e.reshape(g.shape)
            hh = 1e-6 * max(abs(float(p64[name].reshape(-1)[fi])), mag)
            pp[name] = p64[name] + hh * e
            lp = fz.loss(pp)
            pp[name] = p64[name] - hh * e
            lm = fz.loss(pp)
            fd1 = (lp - lm) / (2 * hh)
            gi = float(g.reshape(-1)[fi])
            assert abs(fd1 - gi) <= 1e-4 * abs(gi) + 1e-6 * np.abs(g).max(), (name, fi, fd1, gi)
    print(kind, {k: f"{v:.1e}" for k, v in report.items()})
