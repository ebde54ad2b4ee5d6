"""Visual-inertial tracking loop around the GPU pose Jacobian.

The host side of the reference's visual-inertial tracking
(the IMU branch of GSSlam::compute, src/GSSlam.cu:880-975, with the Ceres
problem of src/GSSlam.cu:150-185 and optimizeWithCeres, 2246-2290): per
camera frame
  * the IMU samples since the previous frame are preintegrated
    (Preintegration, linearised at the previous frame's bias estimates);
  * the newest state is predicted from the previous one;
  * the problem { RGB-D pose factor on the newest pose, IMU factor between
    the two states, marginalization prior on the previous state } is solved
    by Gauss-Newton steps (fvgs_vi_step), each taking the GPU Jacobian at the
    current camera pose (P_cam = P + Q t_imu_cam, Q_cam = Q q_imu_cam), its
    IMU-frame transform (fvgs_jacobian_cam_to_imu) and the 15- or 30-dim FP64
    normal equations;
  * the previous state is marginalised into the prior of the next frame
    (fvgs_vi_marginalize), and the newest state becomes the previous one.

Everything above the Jacobian is host FP64 through include/fvgs_estimator.h.
Camera poses are passed to the Jacobian as the raw (x, y, z, w) quaternion of
the camera-to-world rotation (not the reference's make_float4(w, x, y, z)
reordering, which the GSSlam mirror reproduces).
"""
from __future__ import annotations

import numpy as np

from . import fvgs


class VisualInertialTracker:
    """visual(cam_pose) -> (JtJ_cam [6x6], Jtr_cam [6]) is the RGB-D system at a
    camera pose (t float32 [3], q float32 [4]), e.g. a session's
    track_jacobian at the frame's pyramid level."""

    def __init__(self, visual, t_imu_cam, q_imu_cam, acc_n, gyr_n, acc_w=1e-4, gyr_w=1e-5, iterations=20,
                 eps=1e-4, marginalize=True):
        self.visual = visual
        self.t_ic = np.asarray(t_imu_cam, np.float64)
        self.q_ic = np.asarray(q_imu_cam, np.float64)
        self.noise = (acc_n, gyr_n, acc_w, gyr_w)
        self.iterations = iterations
        self.eps = eps
        self.use_prior = marginalize
        self.state = None  # (pose [7], speedbias [9]) of the newest frame
        self.prior = None
        self.last_imu = None  # (acc, gyr) of the newest sample

    def camera_pose(self, pose):
        """(t, q) float32 of the camera for the IMU pose [p, q x y z w]."""
        from .synthetic import qmul, qrot

        P, Q = pose[:3], pose[3:]
        Pc = P + qrot(Q) @ self.t_ic
        Qc = qmul(Q, self.q_ic)
        return Pc.astype(np.float32), (Qc / np.linalg.norm(Qc)).astype(np.float32)

    def imu_system(self, pose):
        JtJ, Jtr = self.visual(self.camera_pose(pose))
        return fvgs.jacobian_cam_to_imu(JtJ, Jtr, self.q_ic, self.t_ic, pose[3:])

    def start(self, pose, speedbias, acc0, gyr0):
        self.state = (np.asarray(pose, np.float64).copy(), np.asarray(speedbias, np.float64).copy())
        self.prior = None
        self.last_imu = (np.asarray(acc0, np.float64), np.asarray(gyr0, np.float64))

    def track(self, dt, acc, gyr):
        """One camera frame: the IMU samples since the previous frame (dt
        seconds apart, acc / gyr [k x 3]), then the Gauss-Newton solve.
        Returns (pose [7], speedbias [9], costs before each step)."""
        pose_i, sb_i = self.state
        pre = fvgs.Preintegration(self.last_imu[0], self.last_imu[1], sb_i[3:6], sb_i[6:9], *self.noise)
        for a, g in zip(acc, gyr):
            pre.add(dt, a, g)
        pj, vj = pre.predict(pose_i, sb_i[:3])
        state_i = (pose_i, sb_i)
        state_j = (pj, np.concatenate([vj, sb_i[3:]]))
        prior = self.prior if self.use_prior else None
        costs = []
        for _ in range(self.iterations):
            JtJ, Jtr = self.imu_system(state_j[0])
            state_i, state_j, cost, _ = fvgs.vi_step(pre, JtJ, Jtr, state_i, state_j, prior, self.eps)
            costs.append(cost)
        if self.use_prior:
            JtJ, Jtr = self.imu_system(state_j[0])
            self.prior = fvgs.vi_marginalize(pre, JtJ, Jtr, state_i, state_j, prior, self.eps)
        pre.close()
        self.state = state_j
        self.last_imu = (np.asarray(acc[-1], np.float64), np.asarray(gyr[-1], np.float64))
        return state_j[0], state_j[1], costs
