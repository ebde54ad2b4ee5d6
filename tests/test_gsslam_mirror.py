"""The C++ mirror of the reference's GSSlam / RgbdPoseCostFunction
(include/f_vigs_slam) driven as the reference's Ceres problem drives it: a
map, a camera frame, extrinsics, an IMU pose, Evaluate().

The expected values restate the reference's host path around the kernels
(src/GSSlam.cu:2103-2243, src/RgbdPoseCost.cu:29-108) with the oracle:
  * the camera pose P_cam = P_imu + Q_imu t_imu_cam, Q_cam = Q_imu q_imu_cam,
    cast to float and stored as make_float4(w, x, y, z) (FVGS_Q_POSE_WXYZ,
    the reference's order; the kernels read the float4 as x, y, z, w);
  * the pyramid level's frame with the second /255 of the colour
    (FVGS_Q_COLOR_RESCALE) and intrinsics scaled by 1 / 2^level;
  * the oracle's FP64 JtJ / Jtr on that binning, then J_cam_imu;
  * Evaluate's pseudo factor: J*^T J* and J*^T r* reproduce the IMU-frame
    system restricted to eigenvalues above 1e-4.
Tolerances: camera pose bit-exact (float casts of the same FP64 formulas up to
an ulp), systems 1e-5 relative as the tracking tests.
"""
import os
import subprocess

import numpy as np
import pytest

import estimator as E  # oracle/estimator.py
from conftest import ROOT, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

DRIVER = os.path.join(ROOT, "tests", "cpp", "gsslam_mirror.cpp")


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "vector_types.h")):
            return os.path.join(d, "include")
    pytest.skip("CUDA headers not found")


def _compile(fvgs_lib, out_dir):
    lib_dir = os.path.dirname(fvgs_lib.LIB_PATH)
    exe = os.path.join(out_dir, "gsslam_mirror")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", _cuda_include(), DRIVER, "-L", lib_dir, "-lfvgs", "-Wl,-rpath," + lib_dir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_mirror_headers_compile(fvgs_lib, tmp_path):
    """The C++ mirror (GSSlam.hpp, RgbdPoseCost.hpp, ceres_compat.hpp) builds
    against the C-ABI headers and links against libfvgs.so (no GPU needed)."""
    assert os.path.exists(_compile(fvgs_lib, str(tmp_path)))


def _imu_to_camera(P_imu, Q_imu, t_ic, q_ic):
    """src/GSSlam.cu:2113-2121 in FP64 with the quaternion-vector product and
    product the reference's Eigen calls evaluate; float cast; (w, x, y, z)."""
    p = np.asarray(P_imu, float) + E.qrot(np.asarray(Q_imu, float), np.asarray(t_ic, float))
    q = E.qmul(np.asarray(Q_imu, float), np.asarray(q_ic, float))
    return p.astype(np.float32), np.array([q[3], q[0], q[1], q[2]], np.float32)


@pytest.mark.gpu
def test_mirror_evaluate_matches_reference_host_path(oracle, fvgs_lib, tmp_path):
    exe = _compile(fvgs_lib, str(tmp_path))
    W, H, K = scaled_camera(0.5)
    P = oracle.default_params()
    scene = S.cam_box(20_000, seed=81)
    rng = np.random.default_rng(82)
    # extrinsics and an IMU pose whose camera pose looks into the scene once
    # the reference's (w, x, y, z) float4 is read as (x, y, z, w)
    t_ic = np.array([0.02, -0.01, 0.005])
    q_ic = np.array([0.0, 0.0, 0.0, 1.0])
    P_imu = np.array([0.01, -0.02, 0.0])
    # (x, y, z, w) = about (0, 0, 1, 0): the camera's (w, x, y, z) float4 is
    # then about (0, 0, 0, 1), which the kernels read as a near-identity
    Q_imu = np.array([0.0, 0.0, 1.0, 0.0]) + rng.normal(0, 0.005, 4)
    Q_imu = Q_imu / np.linalg.norm(Q_imu)
    cam_t, cam_q_raw = _imu_to_camera(P_imu, Q_imu, t_ic, q_ic)
    # the observed frame: rendered at a nearby raw pose, to 8-bit colour
    view = S.perturb((cam_t, cam_q_raw), 0.5, 1.0, rng)
    b = oracle.prepare(scene, view, K, W, H, P)
    col, dep, _, _ = oracle.render(b, view, K, W, H, P)
    bgr = np.clip(np.rint(np.clip(col, 0, 1) * 255.0), 0, 255).astype(np.uint8)
    depth = dep.astype(np.float32)
    level = 1
    with open(tmp_path / "in.bin", "wb") as f:
        np.array([scene.n, W, H, level], np.int32).tofile(f)
        for a in (scene.positions, scene.scales, scene.orientations, scene.colors, scene.opacities):
            np.ascontiguousarray(a, np.float32).tofile(f)
        bgr.tofile(f)
        depth.tofile(f)
        np.array(K, np.float32).tofile(f)
        t_ic.astype(np.float64).tofile(f)
        q_ic.astype(np.float64).tofile(f)
        np.concatenate([P_imu, Q_imu]).astype(np.float64).tofile(f)
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = open(tmp_path / "out.bin", "rb").read()
    off = 0

    def take(dtype, n):
        nonlocal off
        a = np.frombuffer(raw, dtype, n, off)
        off += a.nbytes
        return a

    status = take(np.int32, 1)[0]
    cam = take(np.float32, 7)
    JtJ = take(np.float64, 36).reshape(6, 6)
    Jtr = take(np.float64, 6)
    eval_ok = take(np.int32, 1)[0]
    res = take(np.float64, 6)
    jac = take(np.float64, 42).reshape(6, 7)
    count = take(np.uint32, 1)[0]
    assert status == 0 and eval_ok == 1 and count == scene.n
    np.testing.assert_allclose(cam[:3], cam_t, rtol=0, atol=1e-7)
    np.testing.assert_allclose(cam[3:], cam_q_raw, rtol=0, atol=1e-7)

    # expected: the oracle on the pyramid level at the camera pose as the kernels read it
    lv = oracle.preprocess(bgr, depth, levels=3, double_scale=True)[level]
    Hl, Wl = lv[1].shape
    s = 1.0 / (1 << level)
    Kl = tuple(float(np.float32(k) * np.float32(s)) for k in K)
    pose_raw = (cam[:3].astype(np.float32), cam[3:].astype(np.float32))
    bl = oracle.prepare(scene, pose_raw, Kl, Wl, Hl, P)
    tr = oracle.track(bl, lv, pose_raw, Kl, Wl, Hl, P, images=False)
    JtJ_w, Jtr_w = E.jacobian_cam_to_imu(tr.JtJ, tr.Jtr, q_ic, t_ic, Q_imu)
    assert bl.keys.shape[0] > 1000 and np.linalg.norm(JtJ_w) > 0 and np.linalg.norm(Jtr_w) > 0
    assert np.linalg.norm(JtJ - JtJ_w) <= 1e-5 * np.linalg.norm(JtJ_w)
    assert np.linalg.norm(Jtr - Jtr_w) <= 1e-5 * np.linalg.norm(Jtr_w)
    # Evaluate: the pseudo factor of the same system, in the first six columns
    Jstar = jac[:, :6]
    assert np.all(jac[:, 6] == 0.0)
    Hk, Pk = E.thresholded(JtJ, 1e-4)
    np.testing.assert_allclose(Jstar.T @ Jstar, Hk, rtol=0, atol=1e-9 * np.abs(Hk).max())
    np.testing.assert_allclose(Jstar.T @ res, Pk @ Jtr, rtol=0, atol=1e-6 * max(1.0, np.abs(Pk @ Jtr).max()))

    # map maintenance through the mirror (removeOutliers at the camera pose
    # on the level-0 depth, covisibility of a keyframe taken at that pose,
    # prune, densify against it, a keyframe mapping step, renderView)
    st = take(np.int32, 6)
    counts = take(np.uint32, 3)
    ratio = take(np.float32, 1)[0]
    assert np.all(st == 0), st
    b0 = oracle.prepare(scene, pose_raw, K, W, H, P)
    ta, op = oracle.outlier_scores(b0, depth, W, H, P)
    marked = int((oracle.outlier_states(ta, op, 0.6) != 0).sum())
    removed = scene.n - int(counts[0])
    assert abs(removed - marked) <= max(2, scene.n // 1000), (removed, marked)
    assert ratio == 1.0  # the keyframe was taken at the current pose
    assert counts[1] <= counts[0] and counts[2] >= counts[1]
