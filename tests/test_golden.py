"""The CPU restatement against its committed golden fixtures (tests/golden/,
made by tests/golden/make_golden.py): integer and key outputs bit-exact,
FP64 outputs to 1e-12 relative."""
import glob
import os

import numpy as np
import pytest

from f_vigs_slam_gb300 import synthetic as S

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _scene(g):
    return S.Scene(g["positions"], g["scales"], g["orientations"], g["colors"], g["opacities"])


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_matches_golden(oracle, path):
    g = np.load(path)
    W, H, K, quirks = int(g["W"]), int(g["H"]), tuple(g["K"]), int(g["quirks"])
    P = oracle.default_params(quirks)
    pose = (np.zeros(3, np.float32), S.IDENTITY_Q)
    sc = _scene(g)
    b = oracle.prepare(sc, pose, K, W, H, P)
    for name, v in (("uv", b.proj.uv), ("cov2d", b.proj.cov2d), ("inv2d", b.proj.inv2d), ("zdepth", b.proj.depth),
                    ("phat", b.proj.phat), ("visible", b.proj.visible), ("counts", b.cnt), ("keys", b.keys),
                    ("vals", b.vals), ("ranges", b.ranges)):
        np.testing.assert_array_equal(v, g[name], err_msg=name)
    frame = (g["rgb"], g["depth"], g["gx"], g["gy"])
    tr = oracle.track(b, frame, pose, K, W, H, P, images=True)
    for name, v in (("JtJ", tr.JtJ), ("Jtr", tr.Jtr), ("tiles", tr.tiles), ("img_color", tr.color),
                    ("img_depth", tr.depth), ("img_T", tr.final_T)):
        np.testing.assert_allclose(v, g[name], rtol=1e-12, atol=1e-300, err_msg=name)
    np.testing.assert_array_equal(tr.n_contrib, g["img_nc"])
    if "delta2d" in g:
        m = oracle.map_step(sc, b, g["rgb"], g["depth"], pose, K, W, H, P, 0.002)
        for name, v in (("delta2d", m.delta2d), ("delta3d", m.delta3d), ("new_pos", m.pos), ("new_rot", m.rot),
                        ("new_col", m.col), ("new_opa", m.opa), ("new_scl", m.scl)):
            np.testing.assert_allclose(v, g[name], rtol=1e-9, atol=1e-12, err_msg=name)


def test_golden_exercise_the_path():
    assert len(GOLDEN) >= 3
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "small_default.npz"))
    assert g["keys"].shape[0] > 100 and np.abs(g["JtJ"]).max() > 0 and (g["delta2d"][:, 12] > 0).sum() > 10
    # with the reference's culled slots the Jacobian's second pass divides by a
    # zero depth in tile 0: the Hessian is NaN, as the reference's would be
    c = np.load(os.path.join(os.path.dirname(__file__), "golden", "small_culled_slots.npz"))
    assert np.isnan(c["JtJ"]).any()
