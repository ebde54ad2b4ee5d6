"""Seeding Gaussians from an RGB-D camera frame on the GPU against the oracle:
the first map (initializeGaussiansFromRgbd) and densification
(computeDensityMask_kernel + densifyGaussians_kernel).

Seeds are FP32 values computed in the reference's operation order with one
rounding per operation on both sides: bit-exact, including their order (row-
major over the sample cells) and the capacity cut.  The density mask comes
from blending (expf on the GPU, FP64 in the oracle): >= 99.9 % of its pixels
within 1e-5; the seeds are then checked bit-exactly against the oracle fed the
GPU's own mask.
"""
import numpy as np
import pytest

from conftest import scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _camera_frame(oracle, scene, pose, K, W, H, P):
    """An 8-bit (b, g, r) colour image and a metric depth map of `scene`
    (render-form median depth; no depth where the map leaves a pixel open)."""
    b = oracle.prepare(scene, pose, K, W, H, P)
    col, dep = oracle.render_view(scene, b, W, H, P)
    depth = np.where(dep < 1e9, dep, 0.0).astype(np.float32)
    bgr = np.clip(np.rint(col[..., ::-1] * 255.0), 0, 255).astype(np.uint8)
    return bgr, depth


def _raw_pose(rng):
    """A camera pose (t, raw float4): the seeding kernels read the float4 as
    (w, x, y, z), so take a unit quaternion in that order."""
    t, q = S.perturb((np.zeros(3), S.IDENTITY_Q), 3.0, 5.0, rng)
    return t.astype(np.float32), np.array([q[3], q[0], q[1], q[2]], np.float32)


def _subset(scene, keep):
    return S.Scene(scene.positions[keep].copy(), scene.scales[keep].copy(), scene.orientations[keep].copy(),
                   scene.colors[keep].copy(), scene.opacities[keep].copy())


def _assert_seeds(got, want, start=0):
    n = want[0].shape[0]
    for g, w in zip(got, want):
        np.testing.assert_array_equal(np.asarray(g)[start:start + n].reshape(w.shape), w)


@pytest.mark.parametrize("sample", [10, 4])
def test_init_from_rgbd_bit_exact(oracle, fvgs_lib, sample):
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    P = oracle.default_params()
    scene = S.cam_box(30_000, seed=51)
    rng = np.random.default_rng(52)
    view = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    bgr, depth = _camera_frame(oracle, scene, view, K, W, H, P)
    depth[40:60, 100:140] = np.nan  # invalid depth is skipped
    assert (depth > 0).mean() > 0.5
    t, q = _raw_pose(rng)
    want = oracle.seed("init", bgr, depth, K, t, q, sample, init_scale=0.02, init_opacity=0.8)
    with fv.Session(W * H, W, H) as s:
        s.preprocess_frame(bgr, depth, levels=1)
        n = s.init_gaussians((t, q), K, sample_px=sample, init_scale=0.02, init_opacity=0.8)
        assert n == want[0].shape[0] > 0
        _assert_seeds(s.download(), want)
        assert np.abs(s.download_adam_state()).sum() == 0
    # capacity below the seed count: the first seeds in cell order
    cap = want[0].shape[0] // 3
    with fv.Session(cap, W, H) as s:
        s.preprocess_frame(bgr, depth, levels=1)
        assert s.init_gaussians((t, q), K, sample_px=sample, init_scale=0.02, init_opacity=0.8) == cap
        _assert_seeds(s.download(), tuple(a[:cap] for a in want))


@pytest.mark.parametrize("sample", [10, 1])
def test_densify_mask_and_seeds(oracle, fvgs_lib, sample):
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    P = oracle.default_params()
    full = S.cam_box(30_000, seed=53)
    rng = np.random.default_rng(54)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    bgr, depth = _camera_frame(oracle, full, pose, K, W, H, P)
    # the map misses the left part of the scene: open pixels there, and
    # pixels whose median depth now lies on farther Gaussians (marked 1)
    part = _subset(full, full.positions[:, 0] > -0.5)
    b = oracle.prepare(part, pose, K, W, H, P)
    want_mask = oracle.density_mask(b, depth, W, H, P)
    assert (want_mask > 0).mean() > 0.1
    with fv.Session(part.n + W * H, W, H) as s:
        s.upload(part)
        s.preprocess_frame(bgr, depth, levels=1)
        added, mask = s.densify(pose, K, sample_px=sample, W=W, H=H)
        got = s.download()
        assert s.n == part.n + added
    close = np.abs(mask - want_mask) <= 1e-5 * np.maximum(1.0, np.abs(want_mask))
    assert close.mean() > 0.999, int((~close).sum())
    _assert_seeds(got, (part.positions, part.scales, part.orientations, part.colors, part.opacities))
    t, q = pose[0].astype(np.float32), np.asarray(pose[1], np.float32)  # the same raw float4, read (w, x, y, z)
    want = oracle.seed("densify", bgr, depth, K, t, q, sample, mask=mask)
    assert added == want[0].shape[0] > 0
    _assert_seeds(got, want, start=part.n)


@pytest.mark.parametrize("stay", [True, False])
def test_densify_optimiser_state_and_capacity(oracle, fvgs_lib, stay):
    """After a removal, densify refills the freed slots up to the capacity
    (seeds beyond it are dropped).  With FVGS_Q_ADAM_STAY the optimiser state
    stays at its slots through both (the reference never moves or shrinks
    adam_states_), so new Gaussians inherit the state found there; otherwise
    the state moves with its Gaussian and new Gaussians start from zero."""
    fv = fvgs_lib
    q_bits = fv.QUIRKS_DEFAULT if stay else fv.QUIRKS_DEFAULT & ~fv.Q_ADAM_STAY
    W, H, K = scaled_camera(0.5)
    P = oracle.default_params()
    full = S.cam_box(20_000, seed=55)
    rng = np.random.default_rng(56)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    bgr, depth = _camera_frame(oracle, full, pose, K, W, H, P)
    with fv.Session(full.n, W, H, fv.default_params(q_bits)) as s:
        s.upload(full)
        s.preprocess_frame(bgr, depth, levels=1)
        s.map_step(pose, K, 0.002)
        before = s.download_adam_state()
        removed = s.prune(alpha_threshold=0.5)
        states = s.download_marks(full.n)
        n1 = s.n
        assert removed > 1000 and n1 == full.n - removed
        added = s.densify(pose, K, sample_px=1)
        assert added == removed and s.n == full.n  # more seeds than free slots
        after = s.download_adam_state()
    assert np.abs(before).sum() > 0
    if stay:
        np.testing.assert_array_equal(after, before)
    else:
        order = oracle.compact_order(states)
        np.testing.assert_array_equal(after[:, :n1], before[:, order[:n1]])
        assert np.abs(after[:, n1:]).sum() == 0


def test_graphs_follow_the_map_size(oracle, fvgs_lib):
    """A captured frame graph belongs to one Gaussian count: after the map
    grows (densify) or is replaced by one of another size (upload), frames
    track exactly like a fresh session holding that map."""
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    P = oracle.default_params()
    full = S.cam_box(20_000, seed=57)
    rng = np.random.default_rng(58)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    bgr, depth = _camera_frame(oracle, full, pose, K, W, H, P)
    part = _subset(full, full.positions[:, 0] > -0.5)
    starts = [S.perturb(pose, 0.5, 1.0, rng) for _ in range(3)]

    def frames(s):
        out = []
        for st in starts:
            s.frame_submit(st, K, iterations=4)
            out.append(s.frame_wait()[0])
        return out

    def fresh(scene):
        with fv.Session(full.n + W * H, W, H) as f:
            f.upload(scene)
            f.preprocess_frame(bgr, depth, levels=1)
            return frames(f)

    with fv.Session(full.n + W * H, W, H) as s:
        s.upload(part)
        s.preprocess_frame(bgr, depth, levels=1)
        frames(s)  # captures a graph for this map size
        assert s.densify(pose, K, sample_px=10) > 0
        grown = S.Scene(*s.download())
        got = frames(s)
        s.upload(_subset(full, full.positions[:, 0] > 0.5))  # smaller map, same shapes otherwise
        got2 = frames(s)
    for a, b in zip(got, fresh(grown)):
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    for a, b in zip(got2, fresh(_subset(full, full.positions[:, 0] > 0.5))):
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


def test_seeding_needs_a_camera_frame(fvgs_lib):
    fv = fvgs_lib
    W, H, K = scaled_camera(0.25)
    pose = (np.zeros(3), S.IDENTITY_Q)
    with fv.Session(1000, W, H) as s:
        with pytest.raises(fv.FvgsError) as e:
            s.init_gaussians(pose, K)
        assert e.value.status == -6
        bgr = np.zeros((H, W, 3), np.uint8)
        s.preprocess_frame(bgr, np.full((H, W), 2.0, np.float32), levels=1)
        assert s.init_gaussians(pose, K, sample_px=8) == ((W + 7) // 8) * ((H + 7) // 8)
        z = np.zeros((H, W), np.float32)
        z3 = np.zeros((H, W, 3), np.float32)
        s.set_frame(0, z3, z, z3, z3)  # level 0 no longer holds the camera frame
        with pytest.raises(fv.FvgsError) as e:
            s.densify(pose, K)
        assert e.value.status == -6
