"""Precision form: scale and rotation stored in BF16, colour and opacity in
FP16 (means FP32), blending and Hessian accumulation FP32, solve FP64.

The form is exactly the FP32 path applied to the rounded attributes: its
binning is bit-identical to the oracle's on the rounded scene, and its
JtJ / Jtr agree with the oracle on the rounded scene within the FP32 path's
1e-5.  Its error against the FP64 oracle on the unrounded scene is measured
and bounded here (the rounding moves each Gaussian's footprint by up to
2^-9 relative), and its pose after 20 Gauss-Newton iterations agrees with
the FP32 path's within 1e-4 rad / 1e-4 m.
"""
import numpy as np
import pytest

from conftest import make_frame, rel_err, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _case(oracle, n=30_000, seed=61, scale=0.5):
    W, H, K = scaled_camera(scale)
    scene = S.cam_box(n, seed=seed)
    P = oracle.default_params()
    rng = np.random.default_rng(seed + 1)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    start = S.perturb(true_pose, 1.0, 2.0, rng)
    frame = make_frame(oracle, scene, true_pose, K, W, H, P)
    return W, H, K, scene, P, true_pose, start, frame


def _binning(s, pose, K, W, H):
    n = s.project_bin(pose, K, W, H)
    return s.download_binning(W, H, n)


def test_reduced_binning_is_the_oracle_on_rounded_attributes(oracle, fvgs_lib):
    fv = fvgs_lib
    W, H, K, scene, P, true_pose, start, frame = _case(oracle)
    want = oracle.prepare(S.reduced(scene), start, K, W, H, P)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.set_precision(fv.PRECISION_REDUCED)
        keys, vals, ranges = _binning(s, start, K, W, H)
        # the FP32 master copy is untouched
        np.testing.assert_array_equal(s.download()[1], scene.scales)
    np.testing.assert_array_equal(keys, want.keys)
    np.testing.assert_array_equal(vals, want.vals)
    np.testing.assert_array_equal(ranges, want.ranges)


def test_reduced_jacobian_and_error_against_fp64(oracle, fvgs_lib):
    fv = fvgs_lib
    W, H, K, scene, P, true_pose, start, frame = _case(oracle)
    rs = S.reduced(scene)
    ref_r = oracle.track(oracle.prepare(rs, start, K, W, H, P), frame, start, K, W, H, P, images=False)
    ref_f = oracle.track(oracle.prepare(scene, start, K, W, H, P), frame, start, K, W, H, P, images=False)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.set_frame(0, *frame)
        s.set_precision(fv.PRECISION_REDUCED)
        JtJ, Jtr = s.track_jacobian(start, K, 0)
    # the FP32 path on the rounded attributes
    assert rel_err(JtJ, ref_r.JtJ) < 1e-5 and rel_err(Jtr, ref_r.Jtr) < 1e-5
    # stated error against the FP64 oracle on the FP32 attributes
    e_jtj, e_jtr = rel_err(JtJ, ref_f.JtJ), rel_err(Jtr, ref_f.Jtr)
    print("reduced vs FP64 oracle: JtJ %.2e  Jtr %.2e" % (e_jtj, e_jtr))
    assert e_jtj < 5e-2 and e_jtr < 1e-1


def test_reduced_pose_matches_fp32_pose(oracle, fvgs_lib):
    fv = fvgs_lib
    W, H, K, scene, P, true_pose, start, frame = _case(oracle, seed=63)
    poses = {}
    for prec in (fv.PRECISION_FP32, fv.PRECISION_REDUCED):
        with fv.Session(scene.n, W, H) as s:
            s.upload(scene)
            s.set_frame(0, *frame)
            s.set_precision(prec)
            poses[prec], _ = s.track_frame(start, K, iterations=20)
    rot, trans = S.pose_error(poses[fv.PRECISION_REDUCED], poses[fv.PRECISION_FP32])
    print("reduced vs FP32 pose after 20 GN: %.2e rad  %.2e m" % (rot, trans))
    assert rot <= 1e-4 and trans <= 1e-4


def test_reduced_copy_follows_map_edits(oracle, fvgs_lib):
    """Mapping (the fused Adam update), removal and seeding keep the reduced
    copy equal to the rounding of the FP32 master: a binning after each is
    the oracle's binning of the rounded master."""
    fv = fvgs_lib
    W, H, K, scene, P, true_pose, start, frame = _case(oracle, n=20_000, seed=65)
    with fv.Session(scene.n + 20_000, W, H) as s:
        s.upload(scene)
        s.set_frame(0, *frame)
        s.set_precision(fv.PRECISION_REDUCED)

        def check():
            master = S.Scene(*s.download())
            want = oracle.prepare(S.reduced(master), start, K, W, H, P)
            keys, vals, ranges = _binning(s, start, K, W, H)
            np.testing.assert_array_equal(keys, want.keys)
            np.testing.assert_array_equal(vals, want.vals)
            np.testing.assert_array_equal(ranges, want.ranges)

        s.map_step(true_pose, K, 0.002)
        check()
        assert s.prune(alpha_threshold=0.3) > 0
        check()
        color = np.clip(np.rint(np.clip(frame[0], 0, 1) * 255), 0, 255).astype(np.uint8)
        s.preprocess_frame(color, frame[1], levels=1)
        assert s.densify(true_pose, K, sample_px=8) > 0
        check()
