"""The projection's candidate list: binnings near the pose a list was built at
project only the Gaussians on it, and must still equal a full binning.

A projection that finds the pose within 2 degrees and 5 cm of the pose the
list was built at (and a view cone no wider) projects only the listed
Gaussians; any other projection projects all of them and rebuilds the list.
Every binning below is compared with the CPU restatement of the reference's
full binning (keys, sorted indices and ranges: exact), and
fvgs_session_candidates says which of the two happened (the pose a list
holds is the pose of the binning that built it).
"""
import numpy as np
import pytest

from conftest import scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

MAX_DEG, MAX_CM = 2.0, 5.0


def _expect_equal(oracle, scene, pose, K, W, H, params, s):
    keys, vals, ranges = s.download_binning(W, H)
    b = oracle.prepare(scene, pose, K, W, H, params)
    np.testing.assert_array_equal(keys, b.keys)
    np.testing.assert_array_equal(vals, b.vals)
    np.testing.assert_array_equal(ranges, b.ranges)
    return vals


def _angle_deg(q0, q1):
    q0 = np.asarray(q0, np.float64) / np.linalg.norm(q0)
    q1 = np.asarray(q1, np.float64) / np.linalg.norm(q1)
    return np.rad2deg(2.0 * np.arccos(min(1.0, abs(float(np.dot(q0, q1))))))


def _held_pose(s):
    valid, n, t, q, cone = s.candidates()
    return valid, n, np.asarray(t, np.float32), np.asarray(q, np.float32), cone


def _room(n, seed):
    """A room map and a pose near its centre (most of the map out of view)."""
    scene = S.room(n, seed=seed)
    pose0 = S.perturb((np.zeros(3), S.IDENTITY_Q), 10.0, 20.0, np.random.default_rng(seed))
    return scene, pose0


def test_list_built_then_reused_at_the_bounds(oracle, fvgs_lib):
    """Poses 1.9 degrees and 4.9 cm from the build pose, in random directions,
    reuse the list and bin exactly as a full binning does."""
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    P = oracle.default_params()
    scene, pose0 = _room(60_000, seed=11)
    rng = np.random.default_rng(4)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        assert not s.candidates()[0]
        s.project_bin(pose0, K, W, H)
        valid, n, t, q, cone = _held_pose(s)
        vals = _expect_equal(oracle, scene, pose0, K, W, H, P, s)
        assert valid
        np.testing.assert_array_equal(t, pose0[0])
        np.testing.assert_array_equal(q, pose0[1])
        # the list holds every Gaussian in view and far fewer than the map
        assert np.unique(vals).size <= n < scene.n // 2
        for _ in range(8):
            pose = S.perturb(pose0, 0.95 * MAX_DEG, 0.98 * MAX_CM, rng)
            s.project_bin(pose, K, W, H)
            _expect_equal(oracle, scene, pose, K, W, H, P, s)
            v2, n2, t2, q2, _ = _held_pose(s)
            assert v2 and n2 == n  # reused: still the list built at pose0
            np.testing.assert_array_equal(t2, pose0[0])
            np.testing.assert_array_equal(q2, pose0[1])


def test_walk_rebuilds_past_the_bounds(oracle, fvgs_lib):
    """A walk of small steps reuses the list until the pose leaves the bounds
    of the pose it was built at, then rebuilds it at the current pose; the
    binnings are incremental throughout."""
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    P = oracle.default_params()
    scene, pose = _room(40_000, seed=12)
    rng = np.random.default_rng(9)
    rebuilds = reuses = 0
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.project_bin(pose, K, W, H)
        built = pose
        for _ in range(12):
            pose = S.perturb(pose, 0.7, 1.2, rng)
            s.project_bin(pose, K, W, H)
            _expect_equal(oracle, scene, pose, K, W, H, P, s)
            assert s.binning_info()["incremental"]
            ang = _angle_deg(built[1], pose[1])
            shift = 100.0 * float(np.linalg.norm(np.asarray(pose[0], np.float64) - built[0]))
            valid, _, t, q, _ = _held_pose(s)
            assert valid
            if ang < 0.99 * MAX_DEG and shift < 0.99 * MAX_CM:
                np.testing.assert_array_equal(t, built[0])
                reuses += 1
            elif ang > 1.01 * MAX_DEG or shift > 1.01 * MAX_CM:
                np.testing.assert_array_equal(t, pose[0])
                np.testing.assert_array_equal(q, pose[1])
                rebuilds += 1
            built = (t, q)
    assert reuses > 0 and rebuilds > 0


def test_each_tile_grid_keeps_its_list(oracle, fvgs_lib):
    """Every tile grid (pyramid level) bins in its own context with its own
    list: a coarser level builds one at its first binning, the finer level's
    list is still reused afterwards, and a wider view cone on the same grid
    rebuilds it."""
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    W2, H2, K2 = scaled_camera(0.25)
    P = oracle.default_params()
    scene, pose0 = _room(40_000, seed=13)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.project_bin(pose0, K, W, H)
        _, n, _, _, cone = _held_pose(s)
        pose = S.perturb(pose0, 1.0, 2.0, np.random.default_rng(1))
        s.project_bin(pose, K2, W2, H2)          # another grid: its own list, built here
        _expect_equal(oracle, scene, pose, K2, W2, H2, P, s)
        v2, _, t2, _, _ = _held_pose(s)
        assert v2
        np.testing.assert_array_equal(t2, pose[0])
        s.project_bin(pose, K, W, H)             # back on the first grid: its list reused
        _expect_equal(oracle, scene, pose, K, W, H, P, s)
        v1, n1, t1, _, cone1 = _held_pose(s)
        assert v1 and n1 == n and cone1 == cone
        np.testing.assert_array_equal(t1, pose0[0])
        assert s.binning_info()["incremental"]    # and its history: the binning continued
        # half the focal length: a much wider view on the same grid
        Kw = (K[0] * 0.5, K[1] * 0.5, K[2], K[3])
        s.project_bin(pose, Kw, W, H)
        _expect_equal(oracle, scene, pose, Kw, W, H, P, s)
        v3, n3, t3, _, cone3 = _held_pose(s)
        assert v3 and cone3 > cone and n3 > n
        np.testing.assert_array_equal(t3, pose[0])


def test_list_dropped_when_the_map_changes(oracle, fvgs_lib):
    """A mapping step, a download (staged through the binning records), a
    re-upload, the debug projection outputs and the no-candidates debug
    switch each leave no list; the next binning is exact."""
    from conftest import make_frame

    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    P = oracle.default_params()
    scene, pose0 = _room(30_000, seed=14)
    rgb, d, gx, gy = make_frame(oracle, scene, pose0, K, W, H, P)
    rng = np.random.default_rng(2)
    with fv.Session(scene.n, W, H) as s:
        s.upload(scene)
        s.set_frame(0, rgb, d, gx, gy)
        s.project_bin(pose0, K, W, H)
        assert s.candidates()[0]
        s.map_step(pose0, K, eta=0.01)      # moves the Gaussians
        assert not s.candidates()[0]
        s.project_bin(pose0, K, W, H)
        assert s.candidates()[0]
        updated = S.Scene(*s.download())    # stages through the binning records
        assert not s.candidates()[0]
        pose = S.perturb(pose0, 0.5, 1.0, rng)
        s.project_bin(pose, K, W, H)
        _expect_equal(oracle, updated, pose, K, W, H, P, s)
        assert s.candidates()[0]

        s.upload(scene)                     # a new map
        assert not s.candidates()[0]
        s.project_bin(pose, K, W, H)
        _expect_equal(oracle, scene, pose, K, W, H, P, s)
        assert s.candidates()[0]

        for flags in (fv.DEBUG_NO_CANDIDATES, fv.DEBUG_PROJECTION):
            s.set_debug(flags)
            pose = S.perturb(pose, 0.3, 0.5, rng)
            s.project_bin(pose, K, W, H)
            _expect_equal(oracle, scene, pose, K, W, H, P, s)
            assert not s.candidates()[0]
            s.set_debug(0)
            pose = S.perturb(pose, 0.3, 0.5, rng)
            s.project_bin(pose, K, W, H)
            _expect_equal(oracle, scene, pose, K, W, H, P, s)
            valid, _, t, _, _ = _held_pose(s)
            assert valid
            np.testing.assert_array_equal(t, pose[0])


def test_results_identical_with_and_without_list(fvgs_lib):
    """Binnings through built and reused lists give the same keys, indices
    and ranges, bit for bit, as projecting every Gaussian."""
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    scene, pose0 = _room(40_000, seed=15)
    rng = np.random.default_rng(6)
    poses = [pose0] + [S.perturb(pose0, 1.5, 3.0, rng) for _ in range(4)]
    out = []
    for flags in (0, fv.DEBUG_NO_CANDIDATES):
        with fv.Session(scene.n, W, H) as s:
            s.upload(scene)
            s.set_debug(flags)
            res = []
            for p in poses:
                s.project_bin(p, K, W, H)
                keys, vals, ranges = s.download_binning(W, H)
                res.append((keys.copy(), vals.copy(), ranges.copy()))
            out.append(res)
    for a, b in zip(*out):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
