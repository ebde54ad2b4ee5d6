"""GPU parity of projection, tile counts, keys, sorted indices and ranges.

The CUDA path (fvgs_project_bin) must match the CPU restatement bit for bit
(tile keys, ranges and sorted indices: exact; projection outputs: exact, both
sides use the same FP32 operation order).
"""
import numpy as np
import pytest

from conftest import scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


SORT_PATHS = {"tile": 0, "radix": 0x8}


def _gpu_binning(fv, scene, pose, K, W, H, params, sort_path="tile"):
    s = fv.Session(max(scene.n, 1), W, H, params)
    s.set_debug(fv.DEBUG_PROJECTION | SORT_PATHS[sort_path])
    s.upload(scene)
    n_inst = s.project_bin(pose, K, W, H)
    proj = s.download_projection() if scene.n else None
    keys, vals, ranges = s.download_binning(W, H)
    s.close()
    return n_inst, proj, keys, vals, ranges


def _check(oracle, fv, scene, pose, K, W, H, quirks, sort_path="tile"):
    P = oracle.default_params(quirks)
    b = oracle.prepare(scene, pose, K, W, H, P)
    n_inst, proj, keys, vals, ranges = _gpu_binning(fv, scene, pose, K, W, H, fv.default_params(quirks), sort_path)
    assert n_inst == b.keys.shape[0]
    if scene.n:
        vis = b.proj.visible.astype(bool)
        np.testing.assert_array_equal(proj["visible"], b.proj.visible)
        for name in ("uv", "depth", "phat"):
            g = proj[name][vis]
            o = getattr(b.proj, name)[vis]
            np.testing.assert_array_equal(g.view(np.uint32), o.view(np.uint32), err_msg=name)
        np.testing.assert_array_equal(proj["cov2d"][vis].view(np.uint32), b.proj.cov2d[vis].view(np.uint32))
        np.testing.assert_array_equal(proj["inv2d"][vis].view(np.uint32), b.proj.inv2d[vis].view(np.uint32))
        np.testing.assert_array_equal(proj["counts"], b.cnt)
    np.testing.assert_array_equal(keys, b.keys)
    np.testing.assert_array_equal(vals, b.vals)
    np.testing.assert_array_equal(ranges, b.ranges)
    return b


@pytest.mark.parametrize("sort_path", ["tile", "radix"])
@pytest.mark.parametrize("quirks", [0x4 | 0x8, 0x0, 0x1 | 0x4, 0x2 | 0x4])
def test_binning_small(oracle, fvgs_lib, quirks, sort_path):
    W, H, K = scaled_camera(0.25)
    scene = S.cam_box(3000, seed=11)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(1))
    _check(oracle, fvgs_lib, scene, pose, K, W, H, quirks, sort_path)


@pytest.mark.parametrize("sort_path", ["tile", "radix"])
def test_binning_vga_50k(oracle, fvgs_lib, sort_path):
    """Full small plain-method workload: N=50k at 640x480 (bit-exact)."""
    W, H, K = scaled_camera(1.0)
    scene = S.cam_box(50_000, seed=0)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(0))
    b = _check(oracle, fvgs_lib, scene, pose, K, W, H, 0x4 | 0x8, sort_path)
    assert b.keys.shape[0] > 100_000  # several sort tiles and passes exercised


def _full_frame_splats(n, seed):
    rng = np.random.default_rng(seed)
    pos = np.stack([rng.uniform(-0.1, 0.1, n), rng.uniform(-0.1, 0.1, n), rng.uniform(1.0, 1.2, n)], 1)
    return S.Scene(pos.astype(np.float32), np.full((n, 3), 1.5, np.float32),
                   np.tile(S.IDENTITY_Q, (n, 1)).astype(np.float32),
                   rng.uniform(0, 1, (n, 3)).astype(np.float32), np.full(n, 0.5, np.float32))


def test_binning_large_tiles(oracle, fvgs_lib):
    """Every tile holds more than 4096 instances: the per-tile sort must hand
    them to the global merge path and still match bit for bit."""
    W, H, K = scaled_camera(0.25)
    scene = _full_frame_splats(9000, 5)
    b = _check(oracle, fvgs_lib, scene, (np.zeros(3), S.IDENTITY_Q), K, W, H, 0x4 | 0x8)
    assert (b.ranges[:, 1] - b.ranges[:, 0]).min() > 4096


def test_binning_culled_slots_pile_into_tile0(oracle, fvgs_lib):
    """With the reference's culled slots, 20k Gaussians behind the camera all
    land in tile 0 with key 0 (one huge bucket of equal depth bits)."""
    W, H, K = scaled_camera(0.25)
    sc = S.cam_box(22_000, seed=8)
    sc.positions[:20_000, 2] *= -1.0
    b = _check(oracle, fvgs_lib, sc, (np.zeros(3), S.IDENTITY_Q), K, W, H, 0x1 | 0x4)
    assert b.ranges[0, 1] - b.ranges[0, 0] >= 20_000


def test_binning_empty_and_culled(oracle, fvgs_lib):
    W, H, K = scaled_camera(0.25)
    scene = S.cam_box(500, seed=2)
    behind = S.Scene(scene.positions * np.array([1, 1, -1], np.float32), scene.scales, scene.orientations,
                     scene.colors, scene.opacities)
    pose = (np.zeros(3), S.IDENTITY_Q)
    # all culled: no instances (intended) / one instance per Gaussian in tile 0 (reference slots)
    _check(oracle, fvgs_lib, behind, pose, K, W, H, 0x4)
    b = _check(oracle, fvgs_lib, behind, pose, K, W, H, 0x1 | 0x4)
    assert b.keys.shape[0] == behind.n and np.all(b.keys == 0)
    empty = S.Scene(*(a[:0] for a in (scene.positions, scene.scales, scene.orientations, scene.colors)),
                    scene.opacities[:0])
    _check(oracle, fvgs_lib, empty, pose, K, W, H, 0x4)


def test_binning_capacity_growth(oracle, fvgs_lib):
    """Large splats (every Gaussian covers the frame) overflow the initial
    instance capacity; the library must grow and return the exact result."""
    W, H, K = scaled_camera(1.0)
    rng = np.random.default_rng(4)
    n = 1500
    pos = np.stack([rng.uniform(-0.1, 0.1, n), rng.uniform(-0.1, 0.1, n), rng.uniform(1.0, 1.2, n)], 1)
    scene = S.Scene(pos.astype(np.float32), np.full((n, 3), 1.5, np.float32),
                    np.tile(S.IDENTITY_Q, (n, 1)).astype(np.float32),
                    rng.uniform(0, 1, (n, 3)).astype(np.float32), np.full(n, 0.5, np.float32))
    b = _check(oracle, fvgs_lib, scene, (np.zeros(3), S.IDENTITY_Q), K, W, H, 0x4 | 0x8)
    assert b.keys.shape[0] > (1 << 20)
