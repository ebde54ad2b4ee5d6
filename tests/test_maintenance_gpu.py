"""Map maintenance on the GPU against the oracle: visibility and covisibility
(computeGaussiansVisibility_kernel / computeGaussiansCovisibility_kernel),
outlier scores and marks (computeOutliers_kernel / removeOutliers_kernel),
prune marks (pruneGaussians_kernel), and the stable compaction that removes
the marked Gaussians (GSSlam::removeOutliers / prune).

Tolerances.  Prune marks are FP32 comparisons done in the same order on both
sides: bit-exact.  Compaction moves data: bit-exact.  Visibility and outlier
marks come from thresholds on exp() of FP32 values (one ex2.approx of an
FP32 exponent on the GPU, FP64 in the oracle), so an evaluation within a few
ulp of a threshold may
fall either way; such flips are rare (about one per ten million evaluations)
and the tests require >= 99.9 % agreement, and exact agreement wherever the
oracle's decision has a margin.  Outlier scores are FP32 sums (per tile in a
fixed order, then float atomics across tiles) against FP64 sums: 1e-5
relative, except for the Gaussians touched by a threshold flip, whose score
moves by one contribution of about 1/255.
"""
import numpy as np
import pytest

from conftest import make_frame, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

SCORE_RTOL = 1e-5


def _case(oracle, n=20_000, seed=31, scale=0.5, quirks=None):
    W, H, K = scaled_camera(scale)
    scene = S.cam_box(n, seed=seed)
    P = oracle.default_params() if quirks is None else oracle.default_params(quirks)
    rng = np.random.default_rng(seed + 1)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    return W, H, K, scene, P, pose


def _session(fv, scene, W, H, quirks=None):
    s = fv.Session(scene.n, W, H, None if quirks is None else fv.default_params(quirks))
    s.upload(scene)
    return s


@pytest.mark.parametrize("cap", [True, False])
def test_visibility_matches_oracle(oracle, fvgs_lib, cap):
    fv = fvgs_lib
    q = fv.QUIRKS_DEFAULT if cap else fv.QUIRKS_DEFAULT & ~fv.Q_VIS_CAP256
    W, H, K, scene, P, pose = _case(oracle, n=60_000, quirks=q)
    b = oracle.prepare(scene, pose, K, W, H, P)
    want = oracle.visibility(b, W, H, P)
    with _session(fv, scene, W, H, q) as s:
        got, count = s.visibility(pose, K, W, H)
    assert count == int(got.sum())
    assert 0 < want.sum() < scene.n
    assert np.mean(got == want) > 0.999, (int((got != want).sum()), int(want.sum()))


@pytest.mark.parametrize("cap", [True, False])
def test_visibility_dim_scene(oracle, fvgs_lib, cap):
    """Faint Gaussians: pixels stay above T = 0.5 past the 256th Gaussian of
    their tile, so the reference's per-tile cap changes the result."""
    fv = fvgs_lib
    q = fv.QUIRKS_DEFAULT if cap else fv.QUIRKS_DEFAULT & ~fv.Q_VIS_CAP256
    W, H, K, scene, P, pose = _case(oracle, n=60_000, quirks=q)
    scene.opacities *= np.float32(0.03)
    b = oracle.prepare(scene, pose, K, W, H, P)
    want = oracle.visibility(b, W, H, P)
    other = oracle.visibility(b, W, H, P, cap=0 if cap else 256)
    differ = other != want
    assert differ.any()
    with _session(fv, scene, W, H, q) as s:
        got, count = s.visibility(pose, K, W, H)
    assert count == int(got.sum())
    assert np.mean(got == want) > 0.999, (int((got != want).sum()), int(want.sum()))
    np.testing.assert_array_equal(got[differ], want[differ])  # the Gaussians the cap decides


def test_covisibility_matches_oracle(oracle, fvgs_lib):
    fv = fvgs_lib
    W, H, K, scene, P, pose_a = _case(oracle, n=30_000, seed=33)
    rng = np.random.default_rng(5)
    pose_b = S.perturb(pose_a, 8.0, 20.0, rng)
    Wk, Hk, Kk = scaled_camera(0.25)  # the keyframe view may differ in size
    va = oracle.visibility(oracle.prepare(scene, pose_a, Kk, Wk, Hk, P), Wk, Hk, P)
    vb = oracle.visibility(oracle.prepare(scene, pose_b, K, W, H, P), W, H, P)
    inter, uni, ratio = oracle.covisibility(va, vb)
    with _session(fv, scene, W, H) as s:
        gi, gu, gr = s.covisibility(pose_a, Kk, Wk, Hk, pose_b, K, W, H)
        # the same views through fvgs_visibility
        ga, _ = s.visibility(pose_a, Kk, Wk, Hk)
        gb, _ = s.visibility(pose_b, K, W, H)
    assert 0 < inter < uni
    assert (gi, gu) == (int(np.sum((ga != 0) & (gb != 0))), int(np.sum((ga != 0) | (gb != 0))))
    assert abs(gi - inter) <= max(2, inter // 1000) and abs(gu - uni) <= max(2, uni // 1000)
    assert abs(gr - float(ratio)) < 2e-3
    assert np.float32(gr) == np.float32(gi) / np.float32(gu)


def test_covisibility_edge_cases(oracle, fvgs_lib):
    fv = fvgs_lib
    W, H, K, scene, P, pose = _case(oracle, n=2_000)
    with fv.Session(scene.n, W, H) as s:  # empty map: the reference returns 1
        assert s.covisibility(pose, K, W, H, pose, K, W, H) == (0, 0, 1.0)
        s.upload(scene)
        # the same view twice: every visible Gaussian is in both sets
        i, u, r = s.covisibility(pose, K, W, H, pose, K, W, H)
        assert i == u > 0 and r == 1.0
        # a view facing away from every Gaussian has no instances: ratio 0
        away = (np.zeros(3), np.array([0.0, 1.0, 0.0, 0.0], np.float32))  # 180 degrees about y
        assert s.covisibility(pose, K, W, H, away, K, W, H) == (0, 0, 0.0)


def _outlier_frame(oracle, scene, pose, K, W, H, P):
    rgb, d, gx, gy = make_frame(oracle, scene, pose, K, W, H, P)
    obs = d.copy()
    obs[:, : W // 2] *= 1.6  # the left half observed far behind the map: its Gaussians look like outliers
    obs[: H // 8] = 0.0      # and a band without depth
    return rgb, obs, gx, gy


def _close(g, o):
    """Per Gaussian: FP32 GPU score within SCORE_RTOL of the FP64 one (both
    rounded to FP32 first: an indefinite stored-layout form can overflow)."""
    with np.errstate(over="ignore"):
        g = g.astype(np.float32).astype(np.float64)
        o = o.astype(np.float32).astype(np.float64)
    both_inf = np.isinf(g) & np.isinf(o) & (np.sign(g) == np.sign(o))
    with np.errstate(invalid="ignore"):
        near = np.abs(g - o) <= SCORE_RTOL * np.maximum(1.0, np.abs(o))
    return both_inf | near


def _check_scores(gta, gop, ta, op):
    """Returns the mask of Gaussians whose two scores agree."""
    ok = _close(gta, ta) & _close(gop, op)
    assert np.mean(ok) > 0.999, int((~ok).sum())
    return ok


def _check_states(gst, ta, op, want, ok, thr=0.6):
    assert np.mean(gst == want) > 0.999
    with np.errstate(over="ignore"):
        t32, o32 = ta.astype(np.float32), op.astype(np.float32)
    with np.errstate(invalid="ignore", divide="ignore"):
        share = np.where(t32 > 0, o32 / t32, 0.0)
    clear = ok & (np.abs(t32 - 1.0) > 1e-3) & ~(np.abs(share - thr) <= 1e-3)
    np.testing.assert_array_equal(gst[clear], want[clear])


def test_outlier_scores_and_marks(oracle, fvgs_lib):
    fv = fvgs_lib
    W, H, K, scene, P, pose = _case(oracle, n=20_000, seed=35)
    frame = _outlier_frame(oracle, scene, pose, K, W, H, P)
    b = oracle.prepare(scene, pose, K, W, H, P)
    ta, op = oracle.outlier_scores(b, frame[1], W, H, P)
    want = oracle.outlier_states(ta, op, 0.6)
    assert 0 < int((want != 0).sum()) < scene.n // 2
    with _session(fv, scene, W, H) as s:
        s.set_frame(0, *frame)
        marked = s.remove_outliers(pose, K, level=0, threshold=0.6, remove=False)
        gst, gta, gop = s.download_marks(scene.n, scores=True)
        assert s.n == scene.n  # mark only
    assert marked == int((gst != 0).sum())
    ok = _check_scores(gta.astype(np.float64), gop.astype(np.float64), ta, op)
    _check_states(gst, ta, op, want, ok)


def _compacted(scene, order, n_keep):
    sel = order[:n_keep]
    return (scene.positions[sel], scene.scales[sel], scene.orientations[sel], scene.colors[sel],
            scene.opacities[sel])


def _assert_scene_equal(got, want):
    for x, y in zip(got, want):
        np.testing.assert_array_equal(np.asarray(x).reshape(y.shape), y)


def test_remove_outliers_compacts_in_order(oracle, fvgs_lib):
    fv = fvgs_lib
    W, H, K, scene, P, pose = _case(oracle, n=20_000, seed=37)
    frame = _outlier_frame(oracle, scene, pose, K, W, H, P)
    with _session(fv, scene, W, H) as s:
        s.set_frame(0, *frame)
        removed = s.remove_outliers(pose, K, level=0, threshold=0.6)
        gst = s.download_marks(scene.n)  # the marks this removal used
        assert removed == int((gst != 0).sum()) > 0
        assert s.n == scene.n - removed
        order = oracle.compact_order(gst)
        _assert_scene_equal(s.download(), _compacted(scene, order, s.n))
        # a second pass over the survivors at the same pose removes far fewer
        again = s.remove_outliers(pose, K, level=0, threshold=0.6, remove=False)
        assert again < removed


def _prunable(seed=41, n=20_000):
    scene = S.cam_box(n, seed=seed)
    scene.opacities[::7] = 0.01                                  # transparent
    scene.scales[3::11, 0] = scene.scales[3::11, 1] * 1e-2      # needle: middle / max scale tiny
    scene.scales[3::11, 2] = scene.scales[3::11, 1] * 1e-3
    scene.scales[5::13] = 0.001                                  # tiny
    scene.opacities[9::17] = np.float32(0.05)                    # exactly at the threshold: kept
    return scene


def test_prune_bit_exact_and_compacted(oracle, fvgs_lib):
    fv = fvgs_lib
    scene = _prunable()
    W, H, K = scaled_camera(0.5)
    want = oracle.prune_states(scene)
    with _session(fv, scene, W, H) as s:
        marked = s.prune(remove=False)
        np.testing.assert_array_equal(s.download_marks(scene.n), want)
        assert marked == int((want != 0).sum()) > scene.n // 10
        removed = s.prune()
        assert removed == marked and s.n == scene.n - removed
        _assert_scene_equal(s.download(), _compacted(scene, oracle.compact_order(want), s.n))
        assert s.prune() == 0 and s.n == scene.n - removed  # nothing left to prune


@pytest.mark.parametrize("stay", [True, False])
def test_optimiser_state_on_compaction(oracle, fvgs_lib, stay):
    """FVGS_Q_ADAM_STAY (reference): the moments stay at their index;
    cleared: they move with their Gaussian."""
    fv = fvgs_lib
    q = fv.QUIRKS_DEFAULT if stay else fv.QUIRKS_DEFAULT & ~fv.Q_ADAM_STAY
    W, H, K, _, P, pose = _case(oracle, n=8_000, seed=43)
    scene = _prunable(seed=43, n=8_000)
    frame = make_frame(oracle, scene, pose, K, W, H, P)
    with _session(fv, scene, W, H, q) as s:
        s.set_frame(0, *frame)
        for _ in range(2):
            s.map_step(pose, K, 0.002)
        before = s.download_adam_state()
        assert np.abs(before).sum() > 0
        s.prune()
        st = s.download_marks(scene.n)
        after = s.download_adam_state()
    order = oracle.compact_order(st)
    keep = int((st == 0).sum())
    want = before[:, :keep] if stay else before[:, order[:keep]]
    np.testing.assert_array_equal(after, want)


def test_tracking_after_removal_equals_fresh_map(oracle, fvgs_lib):
    """After a removal the session tracks exactly like a fresh session holding
    the survivors: the binning history and captured frame graphs of the old
    numbering are dropped."""
    fv = fvgs_lib
    W, H, K, scene, P, pose = _case(oracle, n=20_000, seed=45)
    frame = _outlier_frame(oracle, scene, pose, K, W, H, P)
    rng = np.random.default_rng(7)
    starts = [S.perturb(pose, 0.5, 1.0, rng) for _ in range(3)]
    with _session(fv, scene, W, H) as s:
        s.set_frame(0, *frame)
        for st in starts:  # warm the history and capture a frame graph
            s.frame_submit(st, K, iterations=4)
            s.frame_wait()
        assert s.remove_outliers(pose, K, level=0) > 0
        survivors = s.download()
        got = []
        for st in starts:
            s.frame_submit(st, K, iterations=4)
            got.append(s.frame_wait()[0])
    fresh = S.Scene(*survivors)
    with _session(fv, fresh, W, H) as f:
        f.set_frame(0, *frame)
        for st, g in zip(starts, got):
            f.frame_submit(st, K, iterations=4)
            p = f.frame_wait()[0]
            np.testing.assert_array_equal(p[0], g[0])
            np.testing.assert_array_equal(p[1], g[1])


def test_maintenance_on_empty_map_and_errors(fvgs_lib):
    fv = fvgs_lib
    W, H, K = scaled_camera(0.25)
    pose = (np.zeros(3), S.IDENTITY_Q)
    with fv.Session(100, W, H) as s:
        with pytest.raises(fv.FvgsError) as e:  # no frame at level 0 yet
            s.remove_outliers(pose, K)
        assert e.value.status == -6
        z = np.zeros((H, W), np.float32)
        z3 = np.zeros((H, W, 3), np.float32)
        s.set_frame(0, z3, z, z3, z3)
        assert s.remove_outliers(pose, K) == 0
        assert s.prune() == 0
        assert s.visibility(pose, K, W, H)[1] == 0
