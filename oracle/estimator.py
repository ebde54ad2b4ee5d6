"""NumPy restatement of the host FP64 estimator glue (test infrastructure).

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the library.

Follows the reference's formulas (jcevasco2003/f_vigs_slam):
  * J_cam_imu: src/GSSlam.cu:2233-2243;
  * midpoint IMU preintegration with first-order Jacobian / covariance
    propagation: src/Preintegration.cpp:72-147, residual 165-184, predict
    186-192, gravity (0, 0, 9.81);
  * marginalization Schur complement: src/MarginalizationFactor.cpp:318-360.
Quaternions are (x, y, z, w) arrays; products and rotations use the
reference's Eigen formulas (q v = v + w t + q_v x t, t = 2 q_v x v).
"""
from __future__ import annotations

import numpy as np

G_PREINT = np.array([0.0, 0.0, 9.81])
G_FACTOR = np.array([0.0, 0.0, 9.8])


def qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz])


def qinv(q):
    n2 = float(np.dot(q, q))
    return np.array([-q[0], -q[1], -q[2], q[3]]) / n2 if n2 > 0 else np.zeros(4)


def qrot(q, v):
    qv = np.asarray(q[:3], np.float64)
    t = 2.0 * np.cross(qv, v)
    return v + q[3] * t + np.cross(qv, t)


def qmat(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def skew(v):
    return np.array([[0.0, -v[2], v[1]], [v[2], 0.0, -v[0]], [-v[1], v[0], 0.0]])


def jacobian_cam_to_imu(JtJ, Jtr, q_imu_cam, t_imu_cam, q_imu):
    J = np.zeros((6, 6))
    J[:3, :3] = np.eye(3)
    J[:3, 3:] = -qmat(q_imu) @ skew(t_imu_cam)
    J[3:, 3:] = qmat(q_imu_cam).T
    return J.T @ JtJ @ J, J.T @ Jtr


class Preint:
    """Preintegration restated (the same midpoint scheme)."""

    def __init__(self, acc0, gyr0, ba, bg, acc_n, gyr_n, acc_w, gyr_w):
        self.acc0, self.gyr0 = np.array(acc0, float), np.array(gyr0, float)
        self.ba, self.bg = np.array(ba, float), np.array(bg, float)
        self.dp, self.dv = np.zeros(3), np.zeros(3)
        self.dq = np.array([0.0, 0.0, 0.0, 1.0])
        self.sum_dt = 0.0
        self.jac = np.eye(15)
        self.cov = np.zeros((15, 15))
        self.noise = np.diag(np.repeat([acc_n ** 2, gyr_n ** 2, acc_n ** 2, gyr_n ** 2, acc_w ** 2, gyr_w ** 2], 3))

    def add(self, dt, acc1, gyr1):
        acc1, gyr1 = np.asarray(acc1, float), np.asarray(gyr1, float)
        prev = self.dq.copy()
        a0 = self.acc0 - self.ba
        a1 = acc1 - self.ba
        w = 0.5 * (self.gyr0 + gyr1) - self.bg
        u0 = qrot(self.dq, a0)
        self.dq = qmul(self.dq, np.array([w[0] * dt * 0.5, w[1] * dt * 0.5, w[2] * dt * 0.5, 1.0]))
        u1 = qrot(self.dq, a1)
        ua = 0.5 * (u0 + u1)
        self.dp = self.dp + self.dv * dt + 0.5 * ua * dt * dt
        self.dv = self.dv + ua * dt
        Rp, Rk = qmat(prev), qmat(self.dq)
        Rw, Ra0, Ra1 = skew(w), skew(a0), skew(a1)
        I3 = np.eye(3)
        F = np.zeros((15, 15))
        F[0:3, 0:3] = I3
        F[0:3, 3:6] = -0.25 * Rk @ Ra0 * dt * dt - 0.25 * Rk @ Ra1 @ (I3 - Rw * dt) * dt * dt
        F[0:3, 6:9] = I3 * dt
        F[0:3, 9:12] = -0.25 * (Rp + Rk) * dt * dt
        F[0:3, 12:15] = -0.25 * Rk @ Ra1 * dt * dt * -dt
        F[3:6, 3:6] = I3 - Rw * dt
        F[3:6, 12:15] = -I3 * dt
        F[6:9, 3:6] = -0.5 * Rp @ Ra0 * dt - 0.5 * Rk @ Ra1 @ (I3 - Rw * dt) * dt
        F[6:9, 6:9] = I3
        F[6:9, 9:12] = -0.5 * (Rp + Rk) * dt
        F[6:9, 12:15] = -0.5 * Rk @ Ra1 * dt * -dt
        F[9:12, 9:12] = I3
        F[12:15, 12:15] = I3
        V = np.zeros((15, 18))
        V[0:3, 0:3] = 0.25 * Rp * dt * dt
        V[0:3, 3:6] = 0.25 * -Rk @ Ra1 * dt * dt * 0.5 * dt
        V[0:3, 6:9] = 0.25 * Rk * dt * dt
        V[0:3, 9:12] = V[0:3, 3:6]
        V[3:6, 3:6] = 0.5 * I3 * dt
        V[3:6, 9:12] = 0.5 * I3 * dt
        V[6:9, 0:3] = 0.5 * Rp * dt
        V[6:9, 3:6] = 0.5 * -Rk @ Ra1 * dt * 0.5 * dt
        V[6:9, 6:9] = 0.5 * Rk * dt
        V[6:9, 9:12] = V[6:9, 3:6]
        V[9:12, 12:15] = I3 * dt
        V[12:15, 15:18] = I3 * dt
        self.jac = F @ self.jac
        self.cov = F @ self.cov @ F.T + V @ self.noise @ V.T
        self.dq = self.dq / np.linalg.norm(self.dq)
        self.sum_dt += dt
        self.acc0, self.gyr0 = acc1, gyr1

    def residual(self, pose_i, sb_i, pose_j, sb_j):
        Pi, Qi, Pj, Qj = pose_i[:3], pose_i[3:], pose_j[:3], pose_j[3:]
        Vi, Bai, Bgi = sb_i[:3], sb_i[3:6], sb_i[6:]
        Vj, Baj, Bgj = sb_j[:3], sb_j[3:6], sb_j[6:]
        J = self.jac
        dba, dbg = Bai - self.ba, Bgi - self.bg
        th = J[3:6, 12:15] @ dbg
        cdq = qmul(self.dq, np.array([th[0] / 2, th[1] / 2, th[2] / 2, 1.0]))
        cdv = self.dv + J[6:9, 9:12] @ dba + J[6:9, 12:15] @ dbg
        cdp = self.dp + J[0:3, 9:12] @ dba + J[0:3, 12:15] @ dbg
        T, G = self.sum_dt, G_PREINT
        Qii = qinv(Qi)
        r = np.zeros(15)
        r[0:3] = qrot(Qii, 0.5 * G * T * T + Pj - Pi - Vi * T) - cdp
        r[3:6] = qmul(qinv(cdq), qmul(Qii, Qj))[:3]
        r[6:9] = qrot(Qii, G * T + Vj - Vi) - cdv
        r[9:12] = Baj - Bai
        r[12:15] = Bgj - Bgi
        return r

    def predict(self, pose_i, v_i):
        Pi, Qi = pose_i[:3], pose_i[3:]
        T, G = self.sum_dt, G_PREINT
        R = qmat(Qi)
        vj = v_i - G * T + R @ self.dv
        pj = Pi + v_i * T - 0.5 * G * T * T + R @ self.dp
        return np.concatenate([pj, qmul(Qi, self.dq)]), vj


def sqrt_information(cov):
    return np.linalg.cholesky(np.linalg.inv(cov)).T


def marginalize(A, b, m, eps=1e-8):
    """Schur complement with eigen-thresholded pseudo-inverses: (A*, b*)."""
    Amm = 0.5 * (A[:m, :m] + A[:m, :m].T)
    w, V = np.linalg.eigh(Amm)
    inv = np.where(w > eps, 1.0 / np.where(w > eps, w, 1.0), 0.0)
    Amm_inv = V @ np.diag(inv) @ V.T
    As = A[m:, m:] - A[m:, :m] @ Amm_inv @ A[:m, m:]
    bs = b[m:] - A[m:, :m] @ Amm_inv @ b[:m]
    return As, bs


def thresholded(A, eps):
    """A restricted to its eigenvalues above eps, and the projector onto them."""
    w, V = np.linalg.eigh(0.5 * (A + A.T))
    keep = w > eps
    Vk = V[:, keep]
    return Vk @ np.diag(w[keep]) @ Vk.T, Vk @ Vk.T
