"""The two-branch (guided) oracle, on the CPU.

The GPU's exponential, division and square root are the fast approximations
(as in the reference's fast-math build), so a decision whose value lies
within rounding reach of its threshold -- alpha against 1/255, T (1 - alpha)
against 1e-4, ceil(3 sqrt(lambda)) -- may fall on either side.  The guided
oracle follows, at exactly those decisions, the branch that explains a given
outcome, and only there.  These tests pin that it:

* takes no alternate branch when the outcome is its own;
* explains every pixel and radius of an outcome computed with slightly
  perturbed inputs (a stand-in for a different rounding of exp / sqrt);
* rejects outcomes no rounding explains (planted mistakes).
"""
import numpy as np
import pytest

import oracle
from _scenes import camera, scene


def _frame(n=10000, W=256, H=256, seed=0):
    s = scene(n, seed)
    intr, extr = camera(W, H, front=True)
    out, it = oracle.rasterization_forward(s["xyz"].numpy(), s["scale"].numpy(), s["rot"].numpy(),
                                           s["opacity"].numpy(), s["feat"].numpy(), intr, extr, W, H, 0.0)
    return s, it, out, W, H


def test_guided_blend_of_its_own_outcome_takes_no_alternate_branch():
    s, it, out, W, H = _frame()
    g = oracle.alpha_blending_forward_guided(it["uv"], it["conic"], s["opacity"].numpy(), s["feat"].numpy(),
                                             it["idx_sorted"], it["tile_range"], 0.0, W, H, it["final_T"],
                                             it["ncontrib"])
    gout, gT, gnc, nfl, forces, unresolved = g
    assert unresolved == 0
    assert not nfl.any()
    assert (forces == -1).all()
    np.testing.assert_array_equal(gout, out)
    np.testing.assert_array_equal(gnc, it["ncontrib"])
    np.testing.assert_array_equal(gT, it["final_T"])


def test_guided_blend_explains_a_perturbed_exponential():
    """Opacities scaled by 1 + 1e-5 move every alpha by that factor, like a
    different rounding of exp: the guided replay on the unperturbed inputs
    must reach the perturbed outcome at every pixel, some through alternate
    branches."""
    s, it, out, W, H = _frame(n=20000, W=320, H=320, seed=3)
    op = s["opacity"].numpy()
    pout, pT, pnc, _ = oracle.alpha_blending_forward(it["uv"], it["conic"], op * np.float32(1 + 1e-5),
                                                     s["feat"].numpy(), it["idx_sorted"], it["tile_range"], 0.0,
                                                     W, H)
    gout, gT, gnc, nfl, forces, unresolved = oracle.alpha_blending_forward_guided(
        it["uv"], it["conic"], op, s["feat"].numpy(), it["idx_sorted"], it["tile_range"], 0.0, W, H, pT, pnc)
    assert unresolved == 0
    np.testing.assert_array_equal(gnc, pnc)
    assert np.abs(gT - pT).max() <= 1e-3 * np.abs(pT).max()
    assert (nfl > 0).sum() > 0, "the perturbation should move some decisions across a threshold"
    # the backward along those paths runs and differs from the IEEE path's
    w = np.random.default_rng(0).normal(size=gout.shape).astype(np.float32)
    g1 = oracle.alpha_blending_backward(it["uv"], it["conic"], op, s["feat"].numpy(), it["idx_sorted"],
                                        it["tile_range"], 0.0, W, H, gT, gnc, w, forces=forces)
    assert all(np.isfinite(x).all() for x in g1)


def test_guided_blend_rejects_an_outcome_no_rounding_explains():
    s, it, out, W, H = _frame(seed=5)
    nc = it["ncontrib"].copy()
    picks = np.argwhere(nc > 10)[:12]
    for y, x in picks:
        nc[y, x] -= 7  # a planted mistake: the last contributor seven entries early
    res = oracle.alpha_blending_forward_guided(it["uv"], it["conic"], s["opacity"].numpy(), s["feat"].numpy(),
                                               it["idx_sorted"], it["tile_range"], 0.0, W, H, it["final_T"], nc)
    nfl, unresolved = res[3], res[5]
    assert unresolved == len(picks)
    assert all(nfl[y, x] == 255 for y, x in picks)


def _ewa_case(n=30000, W=800, H=600, seed=0):
    s = scene(n, seed)
    intr, extr = camera(W, H, seed=seed)
    uv, d = oracle.project_point_forward(s["xyz"].numpy(), intr, extr, W, H)
    vis = (d != 0).reshape(-1)
    cov = oracle.compute_cov3d_forward(s["scale"].numpy(), s["rot"].numpy(), vis)
    return s["xyz"].numpy(), cov, intr, extr, uv, vis, W, H


def test_ewa_alternatives_explain_a_perturbed_square_root():
    """Covariances scaled by 1 + 5e-5 move 3 sqrt(lambda) by 2.5e-5
    relative, like a different rounding of the square roots: every radius
    of that outcome is the oracle's or its alternative rounding."""
    xyz, cov, intr, extr, uv, vis, W, H = _ewa_case()
    pc, pr, pt, _ = oracle.ewa_project_forward(xyz, cov * np.float32(1 + 5e-5), intr, extr, uv, W, H, vis)
    n_alt, err, _ = oracle.ewa_check_against(pc, pr, pt, xyz, cov, intr, extr, uv, W, H, vis, conic_rtol=2e-4)
    assert n_alt > 0
    _, r, _, _, _, _ = oracle.ewa_project_alternatives(xyz, cov, intr, extr, uv, W, H, vis)
    assert int((pr != r).sum()) == n_alt  # every changed radius is an alternative rounding


def test_ewa_alternatives_reject_an_unexplained_radius():
    xyz, cov, intr, extr, uv, vis, W, H = _ewa_case(seed=1)
    c, r, t, ralt, _, _ = oracle.ewa_project_alternatives(xyz, cov, intr, extr, uv, W, H, vis)
    bad = r.copy()
    i = int(np.flatnonzero((r > 3) & (ralt < 0))[0])
    bad[i] += 2  # a planted mistake: two pixels too large, far from any rounding boundary
    with pytest.raises(AssertionError):
        oracle.ewa_check_against(c, bad, t, xyz, cov, intr, extr, uv, W, H, vis)
    oracle.ewa_check_against(c, r, t, xyz, cov, intr, extr, uv, W, H, vis)
