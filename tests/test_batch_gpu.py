"""The batching form: tracking on 8 x 8 and 32 x 8 tiles against the oracle
binned at the same shape, and the persistent multi-session launch
(fvgs_batch_*) against each session's plain frames.

Tolerances: keys, sorted indices and ranges exact; JtJ and Jtr within 1e-5
relative of the FP64 oracle; batched poses bit-identical to the plain
per-session frames with the same tile shapes, and within 1e-4 rad / 1e-4 m
of the true poses after the 20 coarse-to-fine iterations.
"""
import numpy as np
import pytest

from conftest import make_frame, rel_err, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

JAC_RTOL = 1e-5
POSE_TOL = 1e-4
REF = 0x4 | 0x8 | 0x100 | 0x200  # the reference's conic layout, mapping cap, Jacobian and depth weight
INTENDED = 0x0
PYR = (4, 4, 6, 6)


@pytest.mark.parametrize("shape", [(8, 8), (32, 8), (16, 16)], ids=["8x8", "32x8", "16x16"])
@pytest.mark.parametrize("quirks", [REF, INTENDED], ids=["ref", "analytic"])
def test_tile_shape_parity(oracle, fvgs_lib, shape, quirks):
    """Binning and Jacobian on a non-default tile shape equal the oracle's at
    the same shape (every launch variant)."""
    fv = fvgs_lib
    tw, th = shape
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(20_000, seed=41)
    P = oracle.default_params(quirks, tile=(tw, th))
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(42))
    frame = make_frame(oracle, scene, true_pose, K, W, H, P)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 0.3, 0.5, np.random.default_rng(43))
    b = oracle.prepare(scene, pose, K, W, H, P)
    r = oracle.track(b, frame, pose, K, W, H, P, images=False)
    with fv.Session(scene.n, W, H, fv.default_params(quirks)) as s:
        s.upload(scene)
        s.set_frame(0, *frame)
        s.set_track_tiles(0, tw, th)
        for variant in (0, 3, 4):
            s.set_track_variant(0, variant)
            JtJ, Jtr = s.track_jacobian(pose, K, 0)
            keys, vals, ranges = s.download_binning(W, H)
            np.testing.assert_array_equal(keys, b.keys)
            np.testing.assert_array_equal(vals, b.vals)
            np.testing.assert_array_equal(ranges, b.ranges)
            e1, e2 = rel_err(JtJ, r.JtJ), rel_err(Jtr, r.Jtr)
            print(shape, hex(quirks), variant, "JtJ rel %.2e Jtr rel %.2e" % (e1, e2))
            assert e1 <= JAC_RTOL and e2 <= JAC_RTOL, (variant, e1, e2)


def _level_frames(s, pose, K0, W, H, rng):
    """Observed frames of every level: the session's render at `pose` + noise."""
    for lv in range(len(PYR)):
        sc = np.float32(1.0 / (1 << lv))
        K = tuple(float(np.float32(k) * sc) for k in K0)
        w, h = (W + (1 << lv) - 1) >> lv, (H + (1 << lv) - 1) >> lv
        col, dep, _, _ = s.render(pose, K, w, h)
        rgb, d = S.add_noise(col, dep, rng)
        gx, gy = S.sobel3(rgb)
        s.set_frame(lv, rgb, d, gx, gy)


def _sessions(fv, quirks, specs, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i, (n, cam) in enumerate(specs):
        W, H, K0 = cam.width, cam.height, cam.intrinsics
        s = fv.Session(n, W, H, fv.default_params(quirks))
        s.upload(S.room(n, seed=seed + 10 * i))
        true = S.trajectory(2, seed=seed + 10 * i + 1)[1]
        _level_frames(s, true, K0, W, H, rng)
        start = S.perturb(true, 0.05, 0.1, rng)
        out.append({"s": s, "K0": K0, "true": true, "start": start})
    return out


@pytest.mark.parametrize("quirks", [INTENDED, REF], ids=["analytic", "ref"])
def test_batch_equals_plain_frames(fvgs_lib, quirks):
    """Sessions of uneven maps and frame sizes in one batch, with a different
    tile shape / staging batch per level: every batched frame (eager, then
    captured, then replayed) gives each session's plain frame bit for bit."""
    fv = fvgs_lib
    specs = [(60_000, S.CAM_VGA), (150_000, S.CAM_HD), (30_000, S.CAM_VGA), (250_000, S.CAM_HD),
             (90_000, S.CAM_VGA)]
    ws = _sessions(fv, quirks, specs, 50)
    try:
        with fv.Batch([w["s"] for w in ws]) as bt:
            bt.set_level(3, 8, 8, 128)
            bt.set_level(2, 32, 8, 256)
            bt.set_level(1, 16, 16, 512)
            bt.set_level(0, 16, 16, 256)
            runs = [bt.run_pyramid([w["start"] for w in ws], [w["K0"] for w in ws], PYR) for _ in range(3)]
            st = bt.stats()
        plain = [w["s"].track_frame_pyramid(w["start"], w["K0"], PYR)[0] for w in ws]
    finally:
        for w in ws:
            w["s"].close()
    print("batch stats", st)
    assert st["graphed"] >= 1 and st["batch_launches"] > 0
    for got in runs:
        for p, q in zip(got, plain):
            np.testing.assert_array_equal(p[0], q[0])
            np.testing.assert_array_equal(p[1], q[1])
    if quirks == INTENDED:
        for p, w in zip(runs[-1], ws):
            err = S.pose_error(p, w["true"])
            assert err[0] <= POSE_TOL and err[1] <= POSE_TOL, err


def test_batch_autotune(fvgs_lib):
    """The autotuner times every tile shape x staging batch on every level
    and keeps a valid choice; the tuned batch still equals plain frames."""
    fv = fvgs_lib
    specs = [(80_000, S.CAM_VGA), (200_000, S.CAM_HD), (40_000, S.CAM_VGA)]
    ws = _sessions(fv, INTENDED, specs, 70)
    try:
        with fv.Batch([w["s"] for w in ws]) as bt:
            cfg, ms = bt.autotune([w["start"] for w in ws], [w["K0"] for w in ws], PYR, reps=3)
            print("tuned", cfg)
            for l, m in ms.items():
                print("level", l, "ms (rows 16x16, 8x8, 32x8; cols 128, 256, 512)\n", m)
                assert np.all(np.isfinite(m)) and np.all(m > 0)
            for l, c in cfg.items():
                assert (c[0], c[1]) in fv.TILE_SHAPES and c[2] in fv.STAGE_BATCHES
            got = bt.run_pyramid([w["start"] for w in ws], [w["K0"] for w in ws], PYR)
        plain = [w["s"].track_frame_pyramid(w["start"], w["K0"], PYR)[0] for w in ws]
    finally:
        for w in ws:
            w["s"].close()
    for p, q, w in zip(got, plain, ws):
        np.testing.assert_array_equal(p[0], q[0])
        np.testing.assert_array_equal(p[1], q[1])
        err = S.pose_error(p, w["true"])
        assert err[0] <= POSE_TOL and err[1] <= POSE_TOL, err


def test_batch_instance_overflow_and_reduced_precision(fvgs_lib):
    """A session whose instance buffers overflow inside the batched frame is
    repeated alone after they grow, and the batch still equals the plain
    frames; a session in the precision form is refused (the persistent
    kernel has no compensated variant)."""
    fv = fvgs_lib
    specs = [(150_000, S.CAM_HD), (60_000, S.CAM_VGA)]
    ws = _sessions(fv, INTENDED, specs, 90)
    try:
        # splats three times larger: about ten times the instances, past the
        # initial capacity of max(1 M, 8 N) instances
        big = S.room(150_000, seed=90)
        big.scales *= 3.0
        ws[0]["s"].upload(big)
        _level_frames(ws[0]["s"], ws[0]["true"], ws[0]["K0"], S.CAM_HD.width, S.CAM_HD.height,
                      np.random.default_rng(91))
        with fv.Batch([w["s"] for w in ws]) as bt:
            got = [bt.run_pyramid([w["start"] for w in ws], [w["K0"] for w in ws], PYR) for _ in range(2)]
            ws[1]["s"].set_precision(fv.PRECISION_REDUCED)
            with pytest.raises(fv.FvgsError):
                bt.run_pyramid([w["start"] for w in ws], [w["K0"] for w in ws], PYR)
            ws[1]["s"].set_precision(fv.PRECISION_FP32)
        assert ws[0]["s"].binning_info()["n_instances"] > 1_200_000
        plain = [w["s"].track_frame_pyramid(w["start"], w["K0"], PYR)[0] for w in ws]
    finally:
        for w in ws:
            w["s"].close()
    for run in got:
        for p, q in zip(run, plain):
            np.testing.assert_array_equal(p[0], q[0])
            np.testing.assert_array_equal(p[1], q[1])
