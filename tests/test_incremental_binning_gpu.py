"""Incremental binning: a binning built from the one before it must equal a
binning built from scratch, bit for bit.

Consecutive binnings of a tracking frame (one per Gauss-Newton iteration)
differ by a small pose update, so the library keeps each tile's previous
sorted list, drops the members that left the tile, re-keys the rest for the
new pose, appends the instances that entered the tile and re-sorts adaptively.
Every case below compares the result with the CPU restatement of the
reference's full binning (keys, sorted indices and ranges: exact) and checks
which mode the library took (fvgs_session_binning_info).
"""
import numpy as np
import pytest

from conftest import scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _expect_equal(oracle, scene, pose, K, W, H, params, keys, vals, ranges):
    b = oracle.prepare(scene, pose, K, W, H, params)
    np.testing.assert_array_equal(keys, b.keys)
    np.testing.assert_array_equal(vals, b.vals)
    np.testing.assert_array_equal(ranges, b.ranges)
    return b


def _walk(pose, rng, trans_m, rot_deg):
    return S.perturb(pose, rot_deg, trans_m * 100.0, rng)  # perturb takes degrees, centimetres


@pytest.mark.parametrize("step", [(0.0, 0.0), (0.0005, 0.02), (0.003, 0.2), (0.05, 3.0)])
def test_incremental_matches_full(oracle, fvgs_lib, step):
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(20_000, seed=5)
    P = oracle.default_params()
    rng = np.random.default_rng(7)
    pose0 = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.project_bin(pose0, K, W, H)
        assert not s.binning_info()["incremental"]  # nothing to start from
        pose = pose0
        for _ in range(3):
            pose = _walk(pose, rng, *step)
            n = s.project_bin(pose, K, W, H)
            info = s.binning_info()
            keys, vals, ranges = s.download_binning(W, H)
            b = _expect_equal(oracle, scene, pose, K, W, H, P, keys, vals, ranges)
            assert n == b.keys.shape[0]
            assert info["incremental"]
            if step == (0.0, 0.0):
                assert info["n_entering"] == 0 and info["n_changed"] == 0


def test_incremental_after_mapping_step(oracle, fvgs_lib):
    """The mapping step moves the Gaussians; the next binning still starts from
    the mapping step's own binning and must match a full binning of the
    updated Gaussians."""
    from conftest import make_frame

    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(20_000, seed=9)
    P = oracle.default_params()
    rng = np.random.default_rng(3)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    rgb, d, gx, gy = make_frame(oracle, scene, true_pose, K, W, H, P)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.set_frame(0, rgb, d, gx, gy)
        s.project_bin(true_pose, K, W, H)
        s.map_step(true_pose, K, eta=0.01)
        pose = _walk(true_pose, rng, 0.001, 0.05)
        s.project_bin(pose, K, W, H)
        assert s.binning_info()["incremental"]
        keys, vals, ranges = s.download_binning(W, H)
        updated = S.Scene(*s.download())
    _expect_equal(oracle, updated, pose, K, W, H, P, keys, vals, ranges)


def test_incremental_large_tiles(oracle, fvgs_lib):
    """Tiles above 4096 instances are gathered into global memory and sorted
    by the multi-CTA path, in incremental mode too."""
    from test_binning_gpu import _full_frame_splats

    fv = fvgs_lib
    W, H, K = scaled_camera(0.25)
    scene = _full_frame_splats(9000, seed=4)
    P = oracle.default_params()
    rng = np.random.default_rng(5)
    pose = (np.zeros(3, np.float32), S.IDENTITY_Q)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.project_bin(pose, K, W, H)
        for _ in range(2):
            pose = _walk(pose, rng, 0.002, 0.1)
            s.project_bin(pose, K, W, H)
            assert s.binning_info()["incremental"]
            keys, vals, ranges = s.download_binning(W, H)
            r = ranges.reshape(-1, 2)
            assert (r[:, 1] - r[:, 0]).max() > 4096
            _expect_equal(oracle, scene, pose, K, W, H, P, keys, vals, ranges)


def test_history_per_grid_and_invalidated(oracle, fvgs_lib):
    """Every tile grid keeps its own binning history (up to four grids, the
    least recently used one rebound): a new grid's first binning is a full
    one, going back to a grid continues its history.  A re-upload or a
    literal reference quirk makes the next binning a full one."""
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    W2, H2, K2 = scaled_camera(0.25)
    scene = S.cam_box(5000, seed=2)
    P = oracle.default_params()
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(2))
    rng = np.random.default_rng(3)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.project_bin(pose, K, W, H)
        s.project_bin(pose, K2, W2, H2)          # another tile grid: full
        assert not s.binning_info()["incremental"]
        pose = _walk(pose, rng, 0.002, 0.1)
        s.project_bin(pose, K, W, H)             # back to the first grid: its history continues
        assert s.binning_info()["incremental"]
        keys, vals, ranges = s.download_binning(W, H)
        _expect_equal(oracle, scene, pose, K, W, H, P, keys, vals, ranges)
        for sc in (0.125, 0.375, 0.3):           # three more grids: the second grid is rebound
            Wx, Hx, Kx = scaled_camera(sc)
            s.project_bin(pose, Kx, Wx, Hx)
            assert not s.binning_info()["incremental"]
        s.project_bin(pose, K, W, H)
        assert s.binning_info()["incremental"]
        s.project_bin(pose, K2, W2, H2)
        assert not s.binning_info()["incremental"]
        keys, vals, ranges = s.download_binning(W2, H2)
        _expect_equal(oracle, scene, pose, K2, W2, H2, P, keys, vals, ranges)
        s.project_bin(pose, K, W, H)
        assert s.binning_info()["incremental"]
        s.upload(scene)                            # re-upload
        s.project_bin(pose, K, W, H)
        assert not s.binning_info()["incremental"]
        keys, vals, ranges = s.download_binning(W, H)
        _expect_equal(oracle, scene, pose, K, W, H, P, keys, vals, ranges)
    for quirks in (0x1 | 0x4, 0x2 | 0x4):
        Pq = oracle.default_params(quirks)
        with fv.Session(scene.n, W, H, fv.default_params(quirks)) as s:
            s.upload(scene)
            s.project_bin(pose, K, W, H)
            s.project_bin(pose, K, W, H)
            assert not s.binning_info()["incremental"]
            keys, vals, ranges = s.download_binning(W, H)
            _expect_equal(oracle, scene, pose, K, W, H, Pq, keys, vals, ranges)


def test_tracking_loop_uses_incremental_binning(oracle, fvgs_lib):
    """fvgs_track_frame runs its binnings incrementally and still equals the
    host loop whose every binning is a full one (history dropped by a
    re-upload before each Jacobian)."""
    from conftest import make_frame

    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(20_000, seed=13)
    P = oracle.default_params()
    rng = np.random.default_rng(14)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    rgb, d, gx, gy = make_frame(oracle, scene, true_pose, K, W, H, P)
    start = _walk(true_pose, rng, 0.01, 0.5)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.set_frame(0, rgb, d, gx, gy)
        pose = start
        for _ in range(4):
            s.upload(scene)
            JtJ, Jtr = s.track_jacobian(pose, K, 0)
            assert not s.binning_info()["incremental"]
            pose = oracle.pose_plus(pose, oracle.gn_delta(JtJ, Jtr))
        s.upload(scene)
        dev_pose, _ = s.track_frame(start, K, iterations=4)
        assert s.binning_info()["incremental"]
    ang, tr = S.pose_error(dev_pose, pose)
    assert ang < 1e-6 and tr < 1e-6, (ang, tr)


def test_frame_end_leaves_lists_that_later_binnings_continue(oracle, fvgs_lib):
    """A frame with an odd number of binnings at a level copies that grid's
    current lists back into the buffer the grid started the frame with (so
    captured frames keep matching); the next binning of each grid continues
    from the copy, incrementally, and still equals a full binning."""
    from test_track_gpu import _target_pyramid, INTENDED

    fv = fvgs_lib
    W, H, K0 = scaled_camera(0.5)
    scene = S.cam_box(20_000, seed=31)
    P = oracle.default_params(INTENDED)
    rng = np.random.default_rng(32)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    iters = (1, 3, 3)  # odd at every level
    frames = _target_pyramid(oracle, scene, true_pose, K0, W, H, P, len(iters), 33)
    with fv.Session(scene.n, W, H, fv.default_params(INTENDED)) as s:
        s.upload(scene)
        for lv, fr in enumerate(frames):
            s.set_frame(lv, *fr)
        start = S.perturb(true_pose, 0.2, 0.5, rng)
        for _ in range(3):  # captured (no history), captured (histories), replayed
            s.frame_submit_pyramid(start, K0, iters)
            pose, _ = s.frame_wait()
        assert s.frame_stats()["graphed"] >= 2
        for lv in (2, 1, 0):
            sc = 1.0 / (1 << lv)
            K = tuple(np.float32(k * sc) for k in K0)
            w, h = W >> lv, H >> lv
            p = _walk(pose, rng, 0.001, 0.05)
            s.project_bin(p, K, w, h)
            assert s.binning_info()["incremental"]
            keys, vals, ranges = s.download_binning(w, h)
            _expect_equal(oracle, scene, p, K, w, h, P, keys, vals, ranges)
