"""Generates the golden fixtures in this folder from the reference's own tests.

Each reference test script (``test/test_*.py`` of pointrix-project/msplat)
is executed as ``__main__`` with:

* ``msplat`` replaced by a stub backed by the CPU oracle, so the scripts can
  chain their steps (the stub's outputs only feed later steps; the values
  recorded below come from the reference's PyTorch implementations);
* ``.cuda()`` and ``device="cuda"`` mapped to the CPU;
* ``torch.testing.assert_close`` recording instead of raising;
* ``jaxtyping`` / ``matplotlib`` stubbed and ``scipy.special.sph_harm``
  provided through ``sph_harm_y`` (SciPy >= 1.15 renamed it: ``sph_harm(m,
  n, azimuth, polar) == sph_harm_y(n, m, polar, azimuth)``).

From the globals the scripts leave behind we save their inputs and the
outputs and autograd gradients of the reference's PyTorch implementations.
The known-answer sort test is saved with its hand-written targets.  SH basis
values and gradients in float64 come from the reference's ``eval_sh_bases``.

Usage (needs the reference checkout; the fixtures are committed):
    python tests/golden/make_golden.py /path/to/msplat
"""
from __future__ import annotations

import functools
import os
import runpy
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402


def _np(t):
    if t is None:
        return None
    if isinstance(t, torch.Tensor):
        return t.detach().cpu().numpy()
    return np.asarray(t)


def _t(a, like=None):
    return torch.from_numpy(np.ascontiguousarray(a))


# --------------------------------------------------------------- harness
class Harness:
    def __init__(self):
        self.records = []

    def install(self):
        self._saved = {}
        # CUDA -> CPU.
        self._saved["Tensor.cuda"] = torch.Tensor.cuda
        torch.Tensor.cuda = lambda self, *a, **k: self
        self._saved["cuda.synchronize"] = torch.cuda.synchronize
        torch.cuda.synchronize = lambda *a, **k: None

        def strip(fn):
            @functools.wraps(fn)
            def w(*a, **k):
                d = k.get("device")
                if d is not None and str(d).startswith("cuda"):
                    k["device"] = "cpu"
                return fn(*a, **k)
            return w

        for name in ["rand", "randn", "zeros", "ones", "empty", "tensor", "zeros_like", "ones_like",
                     "rand_like", "randn_like", "empty_like", "full", "arange", "eye"]:
            self._saved[name] = getattr(torch, name)
            setattr(torch, name, strip(getattr(torch, name)))
        # assert_close records (actual, expected).
        self._saved["assert_close"] = torch.testing.assert_close

        def rec(actual, expected, *a, **k):
            self.records.append((_np(actual), _np(expected), dict(k)))
        torch.testing.assert_close = rec
        # Module stubs.
        sys.modules["jaxtyping"] = types.SimpleNamespace(Float=None, Int=None, Int32=None, Bool=None)
        mpl = types.ModuleType("matplotlib")
        mpl.pyplot = types.ModuleType("matplotlib.pyplot")
        sys.modules["matplotlib"] = mpl
        sys.modules["matplotlib.pyplot"] = mpl.pyplot
        import scipy.special as sps
        if not hasattr(sps, "sph_harm"):
            sps.sph_harm = lambda m, n, az, pol: np.complex128(sps.sph_harm_y(n, m, pol, az))
        sys.modules["msplat"] = _oracle_msplat()

    def uninstall(self):
        torch.Tensor.cuda = self._saved.pop("Tensor.cuda")
        torch.cuda.synchronize = self._saved.pop("cuda.synchronize")
        torch.testing.assert_close = self._saved.pop("assert_close")
        for name, fn in self._saved.items():
            setattr(torch, name, fn)
        for m in ["msplat", "jaxtyping", "matplotlib", "matplotlib.pyplot"]:
            sys.modules.pop(m, None)


def _leaf(t):
    t = t.detach().clone()
    if t.is_floating_point():
        t.requires_grad_()
    return t


def _oracle_msplat():
    """msplat look-alike backed by the oracle (forward values only)."""
    ms = types.ModuleType("msplat")

    def project_point(xyz, intr, extr, W, H, nearest=0.0, extent=1.3):
        uv, d = oracle.project_point_forward(_np(xyz), _np(intr), _np(extr), W, H, nearest, extent)
        return _leaf(_t(uv)), _leaf(_t(d))

    def compute_cov3d(scales, uquats, visible=None):
        vis = None if visible is None else _np(visible).reshape(-1)
        return _leaf(_t(oracle.compute_cov3d_forward(_np(scales), _np(uquats), vis)))

    def ewa_project(xyz, cov3d, intr, extr, uv, W, H, visible=None):
        vis = None if visible is None else _np(visible).reshape(-1)
        c, r, t, _ = oracle.ewa_project_forward(_np(xyz), _np(cov3d), _np(intr), _np(extr), _np(uv), W, H, vis)
        return _leaf(_t(c)), _t(r), _t(t)

    def sort_gaussian(uv, depth, W, H, radius, tiles):
        idx, tr = oracle.sort_gaussian(_np(uv), _np(depth), W, H, _np(radius), _np(tiles))
        return _t(idx), _t(tr)

    def alpha_blending(uv, conic, opacity, feature, idx_sorted, tile_range, bg, W, H, ndc=None):
        out, _, _, _ = oracle.alpha_blending_forward(_np(uv), _np(conic), _np(opacity), _np(feature),
                                                     _np(idx_sorted), _np(tile_range), bg, W, H)
        return _leaf(_t(out))

    def compute_sh(shs, view_dirs, visible=None):
        vis = None if visible is None else _np(visible).reshape(-1)
        return _leaf(_t(oracle.compute_sh_forward(_np(shs), _np(view_dirs), vis).astype(np.float32)))

    for f in [project_point, compute_cov3d, ewa_project, sort_gaussian, alpha_blending, compute_sh]:
        setattr(ms, f.__name__, f)
    return ms


def run_script(ref_root, name, seed=0):
    h = Harness()
    h.install()
    try:
        torch.manual_seed(seed)
        g = runpy.run_path(os.path.join(ref_root, "test", name), run_name="__main__")
    finally:
        h.uninstall()
    return g, h.records


def grad(t):
    return None if t is None or t.grad is None else _np(t.grad)


# ------------------------------------------------------------- fixtures
def make(ref_root):
    out = {}

    g, _ = run_script(ref_root, "test_sort_gaussian.py")
    out["sort_known_answer"] = dict(
        uv=_np(g["uv"]), depth=_np(g["depth"]), radius=_np(g["radius"]), tiles=_np(g["tiles"]),
        W=g["w"], H=g["h"], idx_sorted=_np(g["target_idx_sorted"]), tile_range=_np(g["target_tile_range"]))

    g, _ = run_script(ref_root, "test_project_points.py")
    out["project_point"] = dict(
        xyz=_np(g["xyz"]), intr=_np(g["intr"]), extr=_np(g["extr"]), W=g["W"], H=g["H"],
        uv=_np(g["out_pytorch_uv"]), depth=_np(g["out_pytorch_depth"]), dL_dxyz=grad(g["xyz1"]))

    g, _ = run_script(ref_root, "test_compute_cov3d.py", seed=7)
    out["compute_cov3d"] = dict(
        scales=_np(g["rand_scale"]), uquats=_np(g["rand_uquats"]), cov3d=_np(g["out_pytorch"]),
        dL_dscales=grad(g["scales1"]), dL_duquats=grad(g["uquats1"]))

    g, _ = run_script(ref_root, "test_ewa_project.py")
    out["ewa_project"] = dict(
        xyz=_np(g["xyz"]), cov3d=_np(g["cov3d"]), intr=_np(g["intr"]), extr=_np(g["extr"]),
        uv=_np(g["uv"]), visible=_np(g["visible"]), W=g["W"], H=g["H"],
        conic=_np(g["out_conic_pytorch"]), radius=_np(g["out_radius_pytorch"]),
        tiles=_np(g["out_tiles_pytorch"]), dL_dxyz=grad(g["xyz1"]), dL_dcov3d=grad(g["cov3d1"]),
        dL_dintr=grad(g["intr1"]), dL_dextr=grad(g["extr1"]))

    g, _ = run_script(ref_root, "test_alpha_blending.py")
    out["alpha_blending"] = dict(
        uv=_np(g["uv"]), conic=_np(g["conic"]), opacity=_np(g["opacity"]), feature=_np(g["feature"]),
        depth=_np(g["depth"]), radius=_np(g["radius"]), tiles=_np(g["tiles"]),
        idx_sorted=_np(g["idx_sorted"]), tile_range=_np(g["tile_range"]), bg=g["bg"], W=g["w"], H=g["h"],
        out=_np(g["render_feature_torch"]), dL_duv=grad(g["uv1"]), dL_dconic=grad(g["conic1"]),
        dL_dopacity=grad(g["opacity1"]), dL_dfeature=grad(g["feature1"]))

    g, _ = run_script(ref_root, "test_compute_sh.py")
    out["compute_sh"] = dict(
        viewdirs=_np(g["viewdirs"]), sh_coeffs=_np(g["sh_coeffs"]), value=_np(g["out_pytorch"]),
        dL_dsh=grad(g["sh_coeffs1"]), dL_ddirs=grad(g["viewdirs1"]))
    # The reference's SciPy known-answer check (test_compute_sh.py:328-375),
    # re-run on stored inputs: 4 unit directions per degree, N = 1 each.
    eval_scipy = g["eval_scipy"]
    gen = torch.Generator().manual_seed(99)
    sc = {}
    for deg in range(11):
        D = (deg + 1) ** 2
        dirs, coefs, vals = [], [], []
        for _ in range(4):
            v = torch.randn(1, 3, generator=gen, dtype=torch.float64)
            v /= torch.linalg.norm(v, dim=-1, keepdim=True)
            c = torch.randn(1, 1, D, generator=gen, dtype=torch.float64)
            dirs.append(v.numpy()); coefs.append(c.numpy()); vals.append(_np(eval_scipy(v, c)))
        sc[f"scipy_dirs_deg{deg}"] = np.concatenate(dirs)
        sc[f"scipy_coefs_deg{deg}"] = np.concatenate(coefs)
        sc[f"scipy_value_deg{deg}"] = np.concatenate(vals)
    out["sh_scipy"] = sc
    # float64 basis values and gradients, on and off the unit sphere.
    eval_sh_bases = g["eval_sh_bases"]
    rng = np.random.default_rng(1234)
    d = rng.normal(size=(256, 3))
    d[:128] /= np.linalg.norm(d[:128], axis=1, keepdims=True)
    d[128:] *= rng.uniform(0.5, 1.5, size=(128, 1)) / np.linalg.norm(d[128:], axis=1, keepdims=True)
    dirs = torch.tensor(d, dtype=torch.float64, requires_grad=True)
    Y = eval_sh_bases(121, dirs)
    G = np.zeros((256, 121, 3))
    for k in range(121):
        (gk,) = torch.autograd.grad(Y[:, k].sum(), dirs, retain_graph=True)
        G[:, k] = gk.numpy()
    out["sh_basis"] = dict(dirs=d, Y=Y.detach().numpy(), G=G)
    return out


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MSPLAT_REF", "")
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "test")):
        raise SystemExit("usage: make_golden.py /path/to/msplat (reference checkout)")
    fixtures = make(ref_root)
    for name, arrs in fixtures.items():
        clean = {k: np.asarray(v) for k, v in arrs.items() if v is not None}
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **clean)
        print(f"{path}: " + ", ".join(f"{k}{tuple(np.shape(v))}" for k, v in clean.items()))


if __name__ == "__main__":
    main()
