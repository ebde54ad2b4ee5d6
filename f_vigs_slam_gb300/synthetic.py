"""Seeded synthetic scenes and frames for the tracking / mapping workloads.

The reference publishes no dataset; these generators produce inputs with the
shapes and value distributions of its workloads:

* ``cam_box``  -- N Gaussians with camera-frame means uniform in
  [-2,2]x[-1.5,1.5]x[1,5] m seen from the identity pose, 640x480,
  fx=fy=525, cx=319.5, cy=239.5 (the small plain-method workload).
* ``room``     -- N Gaussians with means uniform in a 10x10x4 m room, a camera
  trajectory that random-walks 1 cm / 0.5 deg per step, 1280x720
  (the large plain-method workload).

Distributions for every Gaussian: scales exp(N(-3, 0.5)) per axis,
orientation normalise(N(0, I4)) stored (x, y, z, w), opacity sigmoid(N(0,1)),
colour U[0,1].  Poses are returned as ``(t[3], q[4])`` float32 with q in the
(x, y, z, w) order the kernels read (src/GSCudaKernels.cu:319-334).
"""
from __future__ import annotations

import dataclasses

import numpy as np

IDENTITY_Q = np.array([0.0, 0.0, 0.0, 1.0], dtype=np.float32)


@dataclasses.dataclass
class Scene:
    positions: np.ndarray  # (N,3) float32
    scales: np.ndarray  # (N,3) float32
    orientations: np.ndarray  # (N,4) float32, (x,y,z,w)
    colors: np.ndarray  # (N,3) float32
    opacities: np.ndarray  # (N,) float32

    @property
    def n(self) -> int:
        return int(self.positions.shape[0])


@dataclasses.dataclass
class Camera:
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float

    @property
    def intrinsics(self):
        return (self.fx, self.fy, self.cx, self.cy)


CAM_VGA = Camera(640, 480, 525.0, 525.0, 319.5, 239.5)
CAM_HD = Camera(1280, 720, 1050.0, 1050.0, 639.5, 359.5)


def _attributes(rng: np.random.Generator, n: int):
    scales = np.exp(rng.normal(-3.0, 0.5, size=(n, 3))).astype(np.float32)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    opac = (1.0 / (1.0 + np.exp(-rng.normal(size=n)))).astype(np.float32)
    col = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
    return scales, q.astype(np.float32), col, opac


def cam_box(n: int = 50_000, seed: int = 0) -> Scene:
    """Means uniform in the camera-frame box [-2,2]x[-1.5,1.5]x[1,5] m."""
    rng = np.random.default_rng(seed)
    pos = np.stack(
        [rng.uniform(-2, 2, n), rng.uniform(-1.5, 1.5, n), rng.uniform(1, 5, n)], axis=1
    ).astype(np.float32)
    s, q, c, o = _attributes(rng, n)
    return Scene(pos, s, q, c, o)


def room(n: int = 1_000_000, seed: int = 0) -> Scene:
    """Means uniform in a 10 x 10 x 4 m room centred on the origin (y is the
    4 m vertical axis, camera convention y down, z forward)."""
    rng = np.random.default_rng(seed)
    pos = np.stack(
        [rng.uniform(-5, 5, n), rng.uniform(-2, 2, n), rng.uniform(-5, 5, n)], axis=1
    ).astype(np.float32)
    s, q, c, o = _attributes(rng, n)
    return Scene(pos, s, q, c, o)


# ----------------------------------------------------------------------------
# quaternion helpers, (x, y, z, w) layout, float64
# ----------------------------------------------------------------------------
def qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array(
        [
            aw * bx + bw * ax + ay * bz - az * by,
            aw * by + bw * ay + az * bx - ax * bz,
            aw * bz + bw * az + ax * by - ay * bx,
            aw * bw - ax * bx - ay * by - az * bz,
        ]
    )


def qexp(rotvec):
    th = float(np.linalg.norm(rotvec))
    if th < 1e-12:
        return np.array([0.5 * rotvec[0], 0.5 * rotvec[1], 0.5 * rotvec[2], 1.0])
    ax = np.asarray(rotvec) / th
    s = np.sin(0.5 * th)
    return np.array([ax[0] * s, ax[1] * s, ax[2] * s, np.cos(0.5 * th)])


def qrot(q):
    """Rotation matrix of quaternionToMatrix for q = (x, y, z, w)."""
    x, y, z, w = q
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
            [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
            [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
        ]
    )


def pose_error(pa, pb):
    """(rotation angle rad, translation m) between two poses (t, q)."""
    ta, qa = pa
    tb, qb = pb
    dq = qmul(np.array([-qa[0], -qa[1], -qa[2], qa[3]], dtype=np.float64), np.asarray(qb, np.float64))
    ang = 2.0 * np.arctan2(np.linalg.norm(dq[:3]), abs(dq[3]))
    return float(ang), float(np.linalg.norm(np.asarray(ta, np.float64) - np.asarray(tb, np.float64)))


def perturb(pose, deg: float, cm: float, rng: np.random.Generator):
    """Rotate by `deg` degrees about a random axis (right-multiplied, as the
    pose update PoseLocalParameterization::Plus does) and translate `cm` cm in
    a random direction."""
    t, q = pose
    ax = rng.normal(size=3)
    ax /= np.linalg.norm(ax)
    dq = qexp(ax * np.deg2rad(deg))
    q2 = qmul(np.asarray(q, np.float64), dq)
    q2 /= np.linalg.norm(q2)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    t2 = np.asarray(t, np.float64) + d * (cm / 100.0)
    return t2.astype(np.float32), q2.astype(np.float32)


def trajectory(n_poses: int, seed: int = 0, step_cm: float = 1.0, step_deg: float = 0.5):
    """Random walk from the room centre: each step rotates `step_deg` and
    translates `step_cm` in random directions."""
    rng = np.random.default_rng(seed + 7919)
    pose = (np.zeros(3, np.float32), IDENTITY_Q.copy())
    out = [pose]
    for _ in range(n_poses - 1):
        pose = perturb(pose, step_deg, step_cm, rng)
        out.append(pose)
    return out


def qlog(q):
    """Rotation vector of the unit quaternion q = (x, y, z, w)."""
    q = np.asarray(q, np.float64)
    if q[3] < 0:
        q = -q
    s = float(np.linalg.norm(q[:3]))
    if s < 1e-15:
        return 2.0 * q[:3]
    return q[:3] * (2.0 * np.arctan2(s, q[3]) / s)


GRAVITY = np.array([0.0, 0.0, 9.81])


def imu_trajectory(n_frames: int, seed: int = 0, imu_rate: float = 200.0, imu_per_frame: int = 6,
                   t_imu_cam=(0.02, -0.01, 0.005), q_imu_cam=(0.0, 0.0, 0.0, 1.0), acc_n: float = 2e-3,
                   gyr_n: float = 1.7e-4, noise: bool = True, camera0=None, acc_bias=(0.0, 0.0, 0.0),
                   gyr_bias=(0.0, 0.0, 0.0)):
    """A smooth visual-inertial trajectory with IMU samples.

    The IMU body moves as P(t) = P0 + a_p sin(2 pi f_p t + phi_p) and
    Q(t) = Q0 exp(a_r sin(2 pi f_r t + phi_r)) (per-axis amplitudes and
    frequencies drawn from the seed).  Samples come at `imu_rate` Hz: the
    gyroscope reads the body angular rate (central difference of Q), the
    accelerometer R(t)^T (P''(t) + g) with g = (0, 0, 9.81), the
    preintegration's convention, both plus constant biases; with `noise`,
    white noise of the given densities (std density * sqrt(rate)) is added.  Camera frames come every
    `imu_per_frame` samples; the camera pose is P + Q t_imu_cam,
    Q q_imu_cam, starting at `camera0` (t, q) (default: the origin, identity).

    Returns a dict: frame times, IMU poses (7 doubles: p, q x y z w) and
    velocities at the frames, camera poses (float32 t, q) at the frames, the
    IMU sample times, accelerometer and gyroscope arrays, and the discrete
    noise standard deviations."""
    rng = np.random.default_rng(seed + 4241)
    t_ic = np.asarray(t_imu_cam, np.float64)
    q_ic = np.asarray(q_imu_cam, np.float64)
    q_ic_inv = np.array([-q_ic[0], -q_ic[1], -q_ic[2], q_ic[3]])
    if camera0 is None:
        camera0 = (np.zeros(3), IDENTITY_Q)
    Qc0 = np.asarray(camera0[1], np.float64)
    Q0 = qmul(Qc0, q_ic_inv)
    P0 = np.asarray(camera0[0], np.float64) - qrot(Q0) @ t_ic
    a_p = rng.uniform(0.02, 0.06, 3)
    f_p = rng.uniform(0.3, 0.8, 3)
    ph_p = rng.uniform(0, 2 * np.pi, 3)
    a_r = rng.uniform(0.01, 0.04, 3)
    f_r = rng.uniform(0.3, 0.8, 3)
    ph_r = rng.uniform(0, 2 * np.pi, 3)

    def pos(t):
        return P0 + a_p * np.sin(2 * np.pi * f_p * t + ph_p)

    def vel(t):
        return a_p * 2 * np.pi * f_p * np.cos(2 * np.pi * f_p * t + ph_p)

    def accel(t):
        return -a_p * (2 * np.pi * f_p) ** 2 * np.sin(2 * np.pi * f_p * t + ph_p)

    def rot(t):
        q = qmul(Q0, qexp(a_r * np.sin(2 * np.pi * f_r * t + ph_r)))
        return q / np.linalg.norm(q)

    def omega(t, h=1e-5):
        qa, qb = rot(t - h), rot(t + h)
        return qlog(qmul(np.array([-qa[0], -qa[1], -qa[2], qa[3]]), qb)) / (2 * h)

    dt = 1.0 / imu_rate
    n_imu = (n_frames - 1) * imu_per_frame + 1
    imu_t = np.arange(n_imu) * dt
    acc = np.zeros((n_imu, 3))
    gyr = np.zeros((n_imu, 3))
    for k, t in enumerate(imu_t):
        acc[k] = qrot(rot(t)).T @ (accel(t) + GRAVITY)
        gyr[k] = omega(t)
    acc += np.asarray(acc_bias, np.float64)
    gyr += np.asarray(gyr_bias, np.float64)
    acc_sd, gyr_sd = acc_n * np.sqrt(imu_rate), gyr_n * np.sqrt(imu_rate)
    if noise:
        acc += rng.normal(0.0, acc_sd, acc.shape)
        gyr += rng.normal(0.0, gyr_sd, gyr.shape)
    frame_t = imu_t[::imu_per_frame]
    imu_pose, imu_vel, cam_pose = [], [], []
    for t in frame_t:
        P, Q = pos(t), rot(t)
        imu_pose.append(np.concatenate([P, Q]))
        imu_vel.append(vel(t))
        Pc = P + qrot(Q) @ t_ic
        Qc = qmul(Q, q_ic)
        cam_pose.append((Pc.astype(np.float32), (Qc / np.linalg.norm(Qc)).astype(np.float32)))
    return dict(frame_t=frame_t, imu_pose=imu_pose, imu_vel=imu_vel, cam_pose=cam_pose, imu_t=imu_t, acc=acc,
                gyr=gyr, imu_per_frame=imu_per_frame, dt=dt, acc_sd=acc_sd, gyr_sd=gyr_sd, t_imu_cam=t_ic,
                q_imu_cam=q_ic)


def sobel3(img: np.ndarray):
    """3x3 Sobel derivatives of an (H, W, C) float image with reflect-101
    borders, as cv::Sobel(src, dst, CV_32F, 1, 0, 3) / (0, 1, 3) computes them
    for the reference's gradient pyramid (src/GSSlam.cu:1960-1961)."""
    p = np.pad(img.astype(np.float32), ((1, 1), (1, 1), (0, 0)), mode="reflect")
    gx = (
        (p[:-2, 2:] - p[:-2, :-2])
        + 2.0 * (p[1:-1, 2:] - p[1:-1, :-2])
        + (p[2:, 2:] - p[2:, :-2])
    )
    gy = (
        (p[2:, :-2] - p[:-2, :-2])
        + 2.0 * (p[2:, 1:-1] - p[:-2, 1:-1])
        + (p[2:, 2:] - p[:-2, 2:])
    )
    return gx.astype(np.float32), gy.astype(np.float32)


def add_noise(rgb, depth, rng, color_sigma=0.01, depth_sigma=0.005):
    rgb_n = (rgb + rng.normal(0.0, color_sigma, size=rgb.shape)).astype(np.float32)
    depth_n = (depth + rng.normal(0.0, depth_sigma, size=depth.shape)).astype(np.float32)
    return rgb_n, depth_n


def round_bf16(a):
    """FP32 -> BF16 -> FP32, round to nearest even (the rounding of
    __float2bfloat16_rn): keep the top 16 bits after adding 0x7fff plus the
    lowest kept bit; NaN stays NaN."""
    x = np.ascontiguousarray(a, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    r = (((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16).astype(np.uint32)
    out = r.view(np.float32).copy()
    out[np.isnan(x)] = np.nan
    return out


def round_f16(a):
    """FP32 -> FP16 -> FP32, round to nearest even."""
    return np.asarray(a, np.float32).astype(np.float16).astype(np.float32)


def reduced(scene: Scene) -> Scene:
    """The attributes the precision form stores: means FP32, scales and
    rotations BF16, colours and opacities FP16."""
    return Scene(np.asarray(scene.positions, np.float32).copy(), round_bf16(scene.scales),
                 round_bf16(scene.orientations), round_f16(scene.colors), round_f16(scene.opacities))
