"""GPU parity of the fused tracking kernel against the FP64 oracle.

Tolerances: rendered colour and depth within
1e-5 relative; JtJ and Jtr within 1e-5 relative (Frobenius / 2-norm) of the
FP64 oracle.  The GPU blends in FP32, so a pixel whose FP32 and FP64 values
fall on opposite sides of a discrete threshold (alpha < 1/255, T < 1e-4,
T crossing 0.5) is a "flip"; flips are counted and must stay rare.
"""
import numpy as np
import pytest

from conftest import make_frame, rel_err, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

IMG_RTOL = 1e-5
JAC_RTOL = 1e-5


def _setup(oracle, fv, n, scale, seed, quirks=0x4 | 0x8):
    W, H, K = scaled_camera(scale)
    scene = S.cam_box(n, seed=seed)
    P = oracle.default_params(quirks)
    rng = np.random.default_rng(seed + 100)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    frame = make_frame(oracle, scene, true_pose, K, W, H, P)
    s = fv.Session(n, W, H, fv.default_params(quirks))
    s.upload(scene)
    s.set_frame(0, *frame)
    return W, H, K, scene, P, frame, s


def _img_compare(g, o, rtol, floor=1e-3):
    """Per-pixel relative error |g-o| / max(|o|, floor), excluding pixels whose
    FP32/FP64 results differ by a threshold flip (abs error above 1e-3 of the
    value range).  Depth uses floor = 1 m: the median depth z + dx*phx + dy*phy
    cancels to values near zero where an FP32 result can only be accurate to
    ~1e-5 m absolute, not relative."""
    g = np.asarray(g, np.float64)
    o = np.asarray(o, np.float64)
    err = np.abs(g - o)
    scale = np.maximum(np.abs(o), floor)
    flips = err > 1e-3 * max(1.0, float(np.abs(o).max()))
    rel = (err / scale)[~flips]
    return (float(rel.max()) if rel.size else 0.0), int(flips.sum())


def test_render_parity(oracle, fvgs_lib):
    W, H, K, scene, P, frame, s = _setup(oracle, fvgs_lib, 20_000, 0.5, 7)
    pose = (np.zeros(3), S.IDENTITY_Q)
    col, dep, fT, nc = s.render(pose, K, W, H)
    b = oracle.prepare(scene, pose, K, W, H, P)
    oc, od, oT, onc = oracle.render(b, pose, K, W, H, P)
    for name, g, o, floor in (("colour", col, oc, 1e-3), ("depth", dep, od, 1.0), ("final_T", fT, oT, 1e-3)):
        rel, flips = _img_compare(g, o, IMG_RTOL, floor)
        assert rel <= IMG_RTOL, (name, rel, flips)
        assert flips <= 0.001 * W * H, (name, flips)
    assert np.mean(nc == onc) > 0.999
    s.close()


@pytest.mark.parametrize("quirks", [0x4 | 0x8, 0x8])
def test_track_jacobian_parity(oracle, fvgs_lib, quirks):
    W, H, K, scene, P, frame, s = _setup(oracle, fvgs_lib, 20_000, 0.5, 3, quirks)
    pose = (np.zeros(3), S.IDENTITY_Q)
    JtJ, Jtr = s.track_jacobian(pose, K, 0)
    b = oracle.prepare(scene, pose, K, W, H, P)
    r = oracle.track(b, frame, pose, K, W, H, P, images=False)
    e1, e2 = rel_err(JtJ, r.JtJ), rel_err(Jtr, r.Jtr)
    print("JtJ rel", e1, "Jtr rel", e2)
    assert np.allclose(JtJ, JtJ.T)
    assert e1 <= JAC_RTOL, e1
    assert e2 <= JAC_RTOL, e2
    s.close()


def test_track_deterministic(oracle, fvgs_lib):
    W, H, K, scene, P, frame, s = _setup(oracle, fvgs_lib, 10_000, 0.5, 5)
    pose = (np.array([0.01, 0, 0], np.float32), S.IDENTITY_Q)
    a = s.track_jacobian(pose, K, 0)
    b = s.track_jacobian(pose, K, 0)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    s.close()


def test_track_frame_matches_host_loop(oracle, fvgs_lib):
    """The on-device Gauss-Newton loop equals the host loop that uses the
    same Jacobians and the eigen-regularised pseudo-factor step."""
    W, H, K, scene, P, frame, s = _setup(oracle, fvgs_lib, 10_000, 0.5, 9)
    pose0 = (np.zeros(3), S.IDENTITY_Q.astype(np.float64))
    pose = pose0
    for _ in range(3):
        JtJ, Jtr = s.track_jacobian(pose, K, 0)
        pose = oracle.pose_plus(pose, oracle.gn_delta(JtJ, Jtr))
    dev_pose, _ = s.track_frame(pose0, K, iterations=3)
    ang, tr = S.pose_error(dev_pose, pose)
    assert ang < 1e-6 and tr < 1e-6, (ang, tr)
    s.close()
