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


def _gpu_binning(fv, scene, pose, K, W, H, params):
    s = fv.Session(max(scene.n, 1), W, H, params)
    s.set_debug(fv.DEBUG_PROJECTION)
    s.upload(scene)
    n_inst = s.project_bin(pose, K, W, H)
    proj = s.download_projection() if scene.n else None
    keys, vals, ranges = s.download_binning(W, H)
    s.close()
    return n_inst, proj, keys, vals, ranges


def _check(oracle, fv, scene, pose, K, W, H, quirks):
    P = oracle.default_params(quirks)
    b = oracle.prepare(scene, pose, K, W, H, P)
    n_inst, proj, keys, vals, ranges = _gpu_binning(fv, scene, pose, K, W, H, fv.default_params(quirks))
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


@pytest.mark.parametrize("quirks", [0x4 | 0x8, 0x0, 0x1 | 0x4, 0x2 | 0x4])
def test_binning_small(oracle, fvgs_lib, quirks):
    W, H, K = scaled_camera(0.25)
    scene = S.cam_box(3000, seed=11)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(1))
    _check(oracle, fvgs_lib, scene, pose, K, W, H, quirks)


def test_binning_vga_50k(oracle, fvgs_lib):
    """Full small plain-method workload: N=50k at 640x480 (bit-exact)."""
    W, H, K = scaled_camera(1.0)
    scene = S.cam_box(50_000, seed=0)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(0))
    b = _check(oracle, fvgs_lib, scene, pose, K, W, H, 0x4 | 0x8)
    assert b.keys.shape[0] > 100_000  # several sort tiles and passes exercised


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
