"""The visual-inertial tracking loop on the GPU Jacobian (precision form's
15 / 30-dim FP64 solve): frames rendered at the true camera poses of a smooth
trajectory with 200 Hz IMU samples (noise densities of the precision
workload, constant sensor biases), tracked with FP32 and with reduced
(BF16 / FP16) attribute storage.

Checks: the poses follow the true trajectory, the velocity stays on it, and
the reduced-precision poses agree with FP32 within 1e-4 rad / 1e-4 m.  (The
cost need not fall at every step: the RGB-D factor is the reference's
approximate Jacobian, so a Gauss-Newton step is not a descent step of the
cost it is reported with.)
"""
import numpy as np
import pytest

from conftest import scaled_camera
from f_vigs_slam_gb300 import synthetic as S
from f_vigs_slam_gb300.vi import VisualInertialTracker

pytestmark = pytest.mark.gpu


def test_vi_tracking_follows_the_trajectory(fvgs_lib):
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(30_000, seed=71)
    ba, bg = np.array([0.05, -0.03, 0.04]), np.array([0.002, -0.001, 0.0015])
    tr = S.imu_trajectory(7, seed=72, acc_bias=ba, gyr_bias=bg)
    s = fv.Session(scene.n, W, H)
    s.upload(scene)
    rng = np.random.default_rng(73)
    frames = []
    for k in range(1, len(tr["frame_t"])):
        col, dep, _, _ = s.render(tr["cam_pose"][k], K, W, H)
        rgb, d = S.add_noise(col, dep, rng)
        gx, gy = S.sobel3(rgb)
        frames.append((rgb, d, gx, gy))
    M = tr["imu_per_frame"]
    results = {}
    for name, prec in (("fp32", fv.PRECISION_FP32), ("reduced", fv.PRECISION_REDUCED)):
        s.set_precision(prec)
        vt = VisualInertialTracker(lambda cp: s.track_jacobian(cp, K, 0), tr["t_imu_cam"], tr["q_imu_cam"],
                                   tr["acc_sd"], tr["gyr_sd"])
        vt.start(tr["imu_pose"][0], np.concatenate([tr["imu_vel"][0], np.zeros(6)]), tr["acc"][0], tr["gyr"][0])
        out = []
        for k in range(1, len(tr["frame_t"])):
            s.set_frame(0, *frames[k - 1])
            sl = slice((k - 1) * M + 1, k * M + 1)
            pose, sb, costs = vt.track(tr["dt"], tr["acc"][sl], tr["gyr"][sl])
            assert np.all(np.isfinite(pose)) and np.all(np.isfinite(sb)) and np.all(np.isfinite(costs))
            ang, dist = S.pose_error((pose[:3], pose[3:]), (tr["imu_pose"][k][:3], tr["imu_pose"][k][3:]))
            v_err = float(np.linalg.norm(sb[:3] - tr["imu_vel"][k]))
            out.append((pose, sb, ang, dist, v_err))
        results[name] = out
        print(name, [("%.1e rad %.1e m %.3f m/s" % (o[2], o[3], o[4])) for o in out])
        assert max(o[2] for o in out) < 5e-3 and max(o[3] for o in out) < 5e-3
        assert max(o[4] for o in out) < 0.05
    for a, b in zip(results["fp32"], results["reduced"]):
        ang, dist = S.pose_error((a[0][:3], a[0][3:]), (b[0][:3], b[0][3:]))
        assert ang < 1e-4 and dist < 1e-4, (ang, dist)
    s.close()
