"""The oracle's multi-threaded mode (used only to time the CPU baseline on
all host cores) against its serial mode, which every parity check uses.

Integer outputs (sort order, tile ranges, radii) and the float32 forward
must be bit-identical; double-precision gradient sums may differ only by
summation order.
"""
import numpy as np
import pytest

import oracle
from _scenes import camera, scene


@pytest.fixture
def threads():
    yield
    oracle.set_threads(1)


def _frame(s, intr, extr, W, H, dout):
    xyz, sc, rot = s["xyz"].numpy(), s["scale"].numpy(), s["rot"].numpy()
    op, feat, shs = s["opacity"].numpy(), s["feat"].numpy(), s["shs"].numpy()
    dirs = xyz / np.linalg.norm(xyz, axis=1, keepdims=True)
    out = {}
    out["sh"] = oracle.compute_sh_forward(shs, dirs)
    out["sh_bwd"] = oracle.compute_sh_backward(shs, dirs, None, np.ones((len(xyz), 3), np.float32))
    img, it = oracle.rasterization_forward(xyz, sc, rot, op, feat, intr, extr, W, H, 0.0)
    out.update(img=img, **{k: it[k] for k in ("uv", "depth", "cov3d", "conic", "radius", "tiles",
                                               "idx_sorted", "tile_range", "final_T", "ncontrib")})
    duv, dcon, dop, dfeat = oracle.alpha_blending_backward(it["uv"], it["conic"], op, feat, it["idx_sorted"],
                                                           it["tile_range"], 0.0, W, H, it["final_T"],
                                                           it["ncontrib"], dout)
    out.update(duv=duv, dcon=dcon, dop=dop, dfeat=dfeat)
    out["ewa_bwd"] = oracle.ewa_project_backward(xyz, it["cov3d"], intr, extr, it["radius"],
                                                 dcon.astype(np.float32))
    out["pp_bwd"] = oracle.project_point_backward(xyz, intr, extr, it["depth"], duv.astype(np.float32),
                                                  np.zeros_like(it["depth"]))
    out["cov_bwd"] = oracle.compute_cov3d_backward(sc, rot, it["visible"],
                                                   np.ones_like(it["cov3d"]))
    return out


def _flat(v):
    if isinstance(v, (tuple, list)):
        return [a for x in v for a in _flat(x)]
    return [np.asarray(v)]


def test_threaded_oracle_matches_serial(threads):
    W, H = 200, 136
    s = scene(20000, seed=3, C=3, sh_deg=3)
    intr, extr = camera(W, H, seed=5)
    dout = np.random.default_rng(1).random((3, H, W)).astype(np.float32)
    oracle.set_threads(1)
    ref = _frame(s, intr, extr, W, H, dout)
    oracle.set_threads(4)
    got = _frame(s, intr, extr, W, H, dout)
    assert ref["idx_sorted"].size > 10000
    for k in ref:
        for a, b in zip(_flat(ref[k]), _flat(got[k])):
            if a.dtype.kind in "iub" or a.dtype == np.float32:
                assert np.array_equal(a, b), k
            else:
                np.testing.assert_allclose(b, a, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(a).max()), err_msg=k)
