"""Launch autotuner of the Jacobian kernel: every launch variant (CTAs per
SM, TMA-gathered record batches, batches of 128 / 256 / 512 Gaussians)
computes the same values in the same order, so poses and systems are
bit-identical whichever variant the tuner keeps."""
import numpy as np
import pytest

from conftest import make_frame, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("analytic", [False, True], ids=["ref_jacobian", "analytic_jacobian"])
def test_variants_agree_bit_for_bit(oracle, fvgs_lib, analytic):
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(30_000, seed=71)
    quirks = fv.QUIRKS_INTENDED if analytic else fv.QUIRKS_DEFAULT
    P = oracle.default_params(quirks)
    rng = np.random.default_rng(72)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    start = S.perturb(true_pose, 1.0, 2.0, rng)
    frame = make_frame(oracle, scene, true_pose, K, W, H, P)
    with fv.Session(scene.n, W, H, fv.default_params(quirks)) as s:
        s.upload(scene)
        s.set_frame(0, *frame)
        v, ms = s.autotune(start, K, 0, reps=3)
        assert 0 <= v < fv.TRACK_VARIANTS and np.all(ms > 0)
        out = []
        for variant in range(fv.TRACK_VARIANTS):
            s.set_track_variant(0, variant)
            JtJ, Jtr = s.track_jacobian(start, K, 0)
            pose, _ = s.track_frame(start, K, iterations=8)
            s.frame_submit(start, K, iterations=8)
            pa, _ = s.frame_wait()
            s.frame_submit(start, K, iterations=8)  # replayed from a captured graph
            pg, _ = s.frame_wait()
            out.append((JtJ, Jtr, pose, pa, pg))
        assert s.frame_stats()["graphed"] >= 1
    a = out[0]
    for b in out[1:]:
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
        for x, y in zip(a[2:], b[2:]):
            np.testing.assert_array_equal(x[0], y[0])
            np.testing.assert_array_equal(x[1], y[1])
    for b in out:
        for x in b[2:]:
            np.testing.assert_array_equal(x[0], a[2][0])
            np.testing.assert_array_equal(x[1], a[2][1])


def test_first_frame_of_a_shape_is_tuned(oracle, fvgs_lib):
    fv = fvgs_lib
    W, H, K = scaled_camera(0.25)
    scene = S.cam_box(5_000, seed=73)
    P = oracle.default_params()
    pose = (np.zeros(3), S.IDENTITY_Q)
    frame = make_frame(oracle, scene, pose, K, W, H, P)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.set_frame(0, *frame)
        s.set_timing(["track"])
        s.track_frame(pose, K, iterations=2)
        t = s.get_timing(reset=True)["track"]["launches"]
        assert t == 2 + fv.TRACK_VARIANTS * 5  # two iterations + five timed launches per variant
        s.track_frame(pose, K, iterations=2)
        assert s.get_timing(reset=True)["track"]["launches"] == 2


@pytest.mark.parametrize("analytic", [False, True], ids=["ref_jacobian", "analytic_jacobian"])
def test_split_tiles_give_the_same_tile_partials(oracle, fvgs_lib, analytic):
    """Variants 5 and 6 run each 16 x 16 tile's list on 2 or 4 CTAs; the
    per-tile partials (their rows added in a whole tile's order) and the
    systems are the same bits as one CTA per tile."""
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(30_000, seed=75)
    quirks = fv.QUIRKS_INTENDED if analytic else fv.QUIRKS_DEFAULT
    P = oracle.default_params(quirks)
    rng = np.random.default_rng(76)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    start = S.perturb(true_pose, 0.5, 1.0, rng)
    frame = make_frame(oracle, scene, true_pose, K, W, H, P)
    T = ((W + 15) // 16) * ((H + 15) // 16)
    with fv.Session(scene.n, W, H, fv.default_params(quirks)) as s:
        s.upload(scene)
        s.set_frame(0, *frame)
        out = {}
        for variant in (0, 5, 6):
            s.set_track_variant(0, variant)
            JtJ, Jtr = s.track_jacobian(start, K, 0)
            out[variant] = (JtJ, Jtr, s.download_tile_partials(T))
    for v in (5, 6):
        for x, y in zip(out[0], out[v]):
            np.testing.assert_array_equal(x, y)
