"""Pins the CPU oracle against golden vectors from the reference's own tests.

The fixtures were produced by tests/golden/make_golden.py from the
reference's PyTorch test implementations (float32, as in its test/ folder)
and its known-answer sort test.  Tolerances are the reference tests' own
(torch.testing.assert_close defaults, atol 5e-4 for SH) unless stated.
"""
import numpy as np
import pytest

import oracle
from _golden import load


def close(a, b, rtol=1.3e-6, atol=1e-5):
    np.testing.assert_allclose(np.asarray(a, np.float64), np.asarray(b, np.float64), rtol=rtol, atol=atol)


def test_sort_known_answer():
    g = load("sort_known_answer")
    idx, tr = oracle.sort_gaussian(g["uv"], g["depth"], g["W"], g["H"], g["radius"], g["tiles"])
    np.testing.assert_array_equal(idx, g["idx_sorted"])
    np.testing.assert_array_equal(tr, g["tile_range"])


def test_project_point_forward_backward():
    g = load("project_point")
    uv, depth = oracle.project_point_forward(g["xyz"], g["intr"], g["extr"], g["W"], g["H"])
    close(uv, g["uv"])
    close(depth, g["depth"])
    P = g["xyz"].shape[0]
    dxyz, _, _ = oracle.project_point_backward(g["xyz"], g["intr"], g["extr"], depth, np.ones((P, 2)),
                                               np.ones((P, 1)))
    close(dxyz, g["dL_dxyz"], rtol=1e-4, atol=1e-6)


def test_compute_cov3d_forward_backward():
    g = load("compute_cov3d")
    cov = oracle.compute_cov3d_forward(g["scales"], g["uquats"])
    close(cov, g["cov3d"])
    P = cov.shape[0]
    ds, dq = oracle.compute_cov3d_backward(g["scales"], g["uquats"], None, np.ones((P, 6)))
    close(ds, g["dL_dscales"], rtol=1e-5, atol=1e-5)
    close(dq, g["dL_duquats"], rtol=1e-5, atol=1e-5)


def test_ewa_project_forward():
    g = load("ewa_project")
    conic, radius, tiles, amb = oracle.ewa_project_forward(g["xyz"], g["cov3d"], g["intr"], g["extr"], g["uv"],
                                                           g["W"], g["H"], g["visible"])
    # Radius and tiles are compared exactly, as the reference's own test does
    # (test/test_ewa_project.py:283-284); entries whose value sits within
    # rounding reach of an integer boundary may differ by one.
    mism = (radius != g["radius"]) | (tiles != g["tiles"])
    assert not np.any(mism & ~amb), np.nonzero(mism & ~amb)
    assert mism.sum() <= 2
    ok = ~mism
    close(conic[ok], g["conic"][ok], rtol=1e-5, atol=1e-5)


def test_ewa_project_backward():
    g = load("ewa_project")
    conic, radius, tiles, _ = oracle.ewa_project_forward(g["xyz"], g["cov3d"], g["intr"], g["extr"], g["uv"],
                                                         g["W"], g["H"], g["visible"])
    P = radius.shape[0]
    dxyz, dcov, di, de = oracle.ewa_project_backward(g["xyz"], g["cov3d"], g["intr"], g["extr"], radius,
                                                     np.ones((P, 3)))
    # The PyTorch restatement differentiates every visible point's conic
    # (masked afterwards), the oracle only points with radius > 0: equal.
    scale = np.abs(g["dL_dcov3d"]).max()
    close(dcov, g["dL_dcov3d"], rtol=1e-4, atol=1e-6 * scale)
    close(dxyz, g["dL_dxyz"], rtol=1e-4, atol=1e-6 * np.abs(g["dL_dxyz"]).max())
    close(di, g["dL_dintr"], rtol=2e-3, atol=1e-6 * np.abs(g["dL_dintr"]).max())
    close(de.reshape(-1), g["dL_dextr"].reshape(-1), rtol=2e-3, atol=1e-4 * np.abs(g["dL_dextr"]).max())


def test_alpha_blending_forward_backward():
    g = load("alpha_blending")
    idx, tr = oracle.sort_gaussian(g["uv"], g["depth"], g["W"], g["H"], g["radius"], g["tiles"])
    np.testing.assert_array_equal(idx, g["idx_sorted"])
    np.testing.assert_array_equal(tr, g["tile_range"])
    out, T, nc, amb = oracle.alpha_blending_forward(g["uv"], g["conic"], g["opacity"], g["feature"], idx, tr,
                                                    g["bg"], g["W"], g["H"])
    close(out, g["out"])
    grads = oracle.alpha_blending_backward(g["uv"], g["conic"], g["opacity"], g["feature"], idx, tr, g["bg"],
                                           g["W"], g["H"], T, nc, np.ones_like(out))
    for got, key in zip(grads, ["dL_duv", "dL_dconic", "dL_dopacity", "dL_dfeature"]):
        ref = g[key].reshape(got.shape)
        close(got, ref, rtol=1e-4, atol=1e-5 * max(1.0, np.abs(ref).max()))


def test_sh_basis_matches_reference_polynomials():
    g = load("sh_basis")
    Y, G = oracle.sh_basis(g["dirs"], 10)
    close(Y, g["Y"], rtol=1e-10, atol=1e-10)
    close(G, g["G"], rtol=1e-9, atol=1e-9 * np.abs(g["G"]).max())


@pytest.mark.parametrize("deg", range(11))
def test_sh_scipy_known_answer(deg):
    g = load("sh_scipy")
    d, c, v = g[f"scipy_dirs_deg{deg}"], g[f"scipy_coefs_deg{deg}"], g[f"scipy_value_deg{deg}"]
    Y, _ = oracle.sh_basis(d, deg)
    close((Y[:, None, :] * c).sum(-1), v, rtol=1e-9, atol=1e-9)


def test_compute_sh_forward_backward():
    g = load("compute_sh")
    P = g["viewdirs"].shape[0]
    val = oracle.compute_sh_forward(g["sh_coeffs"], g["viewdirs"])
    close(val, g["value"], rtol=1e-5, atol=5e-4)
    C = g["sh_coeffs"].shape[1]
    dsh, dd = oracle.compute_sh_backward(g["sh_coeffs"], g["viewdirs"], None, np.full((P, C), 1.0 / (P * C)))
    close(dsh, g["dL_dsh"], rtol=1e-5, atol=5e-4)
    close(dd, g["dL_ddirs"], rtol=1e-5, atol=5e-4)
