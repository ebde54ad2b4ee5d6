"""Host FP64 estimator glue (include/fvgs_estimator.h) against the NumPy
restatement (oracle/estimator.py), closed-form known answers and finite
differences.  CPU only: these calls never touch the GPU.

Tolerances: FP64 throughout, 1e-12 relative against the restatement of the
same formulas; closed-form motions to the midpoint rule's exactness;
analytic Jacobians against central differences to 1e-6.
"""
import numpy as np
import pytest

import estimator as E  # oracle/estimator.py


@pytest.fixture(scope="module")
def fv(fvgs_lib):
    return fvgs_lib


def _unit(q):
    q = np.asarray(q, float)
    return q / np.linalg.norm(q)


def _rand_q(rng):
    return _unit(rng.normal(size=4))


def _close(a, b, tol=1e-12):
    a, b = np.asarray(a, float), np.asarray(b, float)
    assert np.max(np.abs(a - b)) <= tol * max(1.0, np.max(np.abs(b))), np.max(np.abs(a - b))


def test_jacobian_cam_to_imu(fv):
    """src/GSSlam.cu:2233-2243."""
    rng = np.random.default_rng(1)
    M = rng.normal(size=(6, 6))
    JtJ, Jtr = M @ M.T * 1e6, rng.normal(size=6)
    qc, t, qi = _rand_q(rng), rng.normal(size=3) * 0.1, _rand_q(rng)
    H, g = fv.jacobian_cam_to_imu(JtJ, Jtr, qc, t, qi)
    Hw, gw = E.jacobian_cam_to_imu(JtJ, Jtr, qc, t, qi)
    _close(H, Hw)
    _close(g, gw)
    # identity extrinsics leave the translation block and rotate nothing
    H0, g0 = fv.jacobian_cam_to_imu(JtJ, Jtr, [0, 0, 0, 1], [0, 0, 0], qi)
    _close(H0, JtJ)
    _close(g0, Jtr)


@pytest.mark.parametrize("rank", [6, 4])
def test_pseudo_factor(fv, rank):
    """src/RgbdPoseCost.cu:57-106: J*^T J* is the part of JtJ with eigenvalues
    above eps, J*^T r* its projection of Jtr."""
    rng = np.random.default_rng(2 + rank)
    U = np.linalg.qr(rng.normal(size=(6, 6)))[0]
    lam = np.array([1e12, 3e9, 2e6, 5e3, 10.0, 1e-2])
    lam[rank:] = 1e-7  # below eps = 1e-4
    JtJ = U @ np.diag(lam) @ U.T
    Jtr = rng.normal(size=6) * 1e3
    r, J = fv.pseudo_factor(JtJ, Jtr, 1e-4)
    Hk, Pk = E.thresholded(JtJ, 1e-4)
    _close(J.T @ J, Hk, 1e-10)
    # the kept subspace is known to eps x (largest / smallest kept eigenvalue)
    _close(J.T @ r, Pk @ Jtr, 1e-16 * lam[0] / lam[rank - 1] * 100)
    assert np.sum(np.any(J != 0.0, axis=1)) == rank
    # eigenvalues ascend down the rows, as the reference's solver orders them
    norms = np.linalg.norm(J, axis=1)
    assert np.all(np.diff(norms[norms > 0]) >= 0)


def _imu_stream(rng, n=200, dt=0.005):
    t = np.arange(n + 1) * dt
    acc = np.stack([0.3 * np.sin(2 * t), 0.2 * np.cos(3 * t), 9.81 + 0.1 * np.sin(t)], 1) + rng.normal(0, 0.01, (n + 1, 3))
    gyr = np.stack([0.1 * np.cos(t), -0.2 * np.sin(2 * t), 0.3 + 0.05 * t], 1) + rng.normal(0, 0.001, (n + 1, 3))
    return dt, acc, gyr


NOISE = (2e-3, 1.7e-4, 3e-3, 2e-5)


def test_preintegration_matches_restatement(fv):
    """src/Preintegration.cpp:72-147: increments, Jacobian and covariance."""
    rng = np.random.default_rng(7)
    dt, acc, gyr = _imu_stream(rng)
    ba, bg = np.array([0.02, -0.01, 0.03]), np.array([1e-3, -2e-3, 5e-4])
    P = fv.Preintegration(acc[0], gyr[0], ba, bg, *NOISE)
    W = E.Preint(acc[0], gyr[0], ba, bg, *NOISE)
    for k in range(1, len(acc)):
        P.add(dt, acc[k], gyr[k])
        W.add(dt, acc[k], gyr[k])
    s = P.state()
    _close(s["delta_p"], W.dp)
    _close(s["delta_v"], W.dv)
    _close(s["delta_q"], W.dq)
    _close(s["jacobian"], W.jac)
    _close(s["covariance"], W.cov, 1e-11)
    assert abs(s["sum_dt"] - W.sum_dt) < 1e-15
    # residual and prediction (src/Preintegration.cpp:150-192)
    pose_i = np.concatenate([rng.normal(size=3), _rand_q(rng)])
    sb_i = np.concatenate([rng.normal(size=3), ba + 1e-3, bg - 1e-4])
    pose_j = np.concatenate([rng.normal(size=3), _rand_q(rng)])
    sb_j = np.concatenate([rng.normal(size=3), ba, bg])
    _close(P.evaluate(pose_i, sb_i, pose_j, sb_j), W.residual(pose_i, sb_i, pose_j, sb_j))
    pj, vj = P.predict(pose_i, sb_i[:3])
    pjw, vjw = W.predict(pose_i, sb_i[:3])
    _close(pj, pjw)
    _close(vj, vjw)
    # the predicted state at the linearisation biases has a zero residual
    # (up to the gravity-free motion model's own consistency)
    sb_i0 = np.concatenate([sb_i[:3], ba, bg])
    pj0, vj0 = P.predict(pose_i, sb_i0[:3])
    r0 = P.evaluate(pose_i, sb_i0, pj0, np.concatenate([vj0, ba, bg]))
    assert np.max(np.abs(r0)) < 1e-12


def test_preintegration_closed_forms(fv):
    """Constant specific force, no rotation: dp = a T^2 / 2, dv = a T exactly
    under the midpoint rule; constant rate about one axis: dq = the rotation
    by w T within the first-order quaternion step's error."""
    a = np.array([0.5, -0.2, 9.81])
    P = fv.Preintegration(a, np.zeros(3), np.zeros(3), np.zeros(3), *NOISE)
    for _ in range(100):
        P.add(0.01, a, np.zeros(3))
    s = P.state()
    _close(s["delta_p"], 0.5 * a * 1.0 ** 2, 1e-12)
    _close(s["delta_v"], a * 1.0, 1e-12)
    _close(s["delta_q"], [0, 0, 0, 1])
    w = np.array([0.0, 0.0, 0.4])
    P = fv.Preintegration(np.zeros(3), w, np.zeros(3), np.zeros(3), *NOISE)
    n, dt = 1000, 0.001
    for _ in range(n):
        P.add(dt, np.zeros(3), w)
    ang = 0.4 * n * dt
    assert np.max(np.abs(P.state()["delta_q"] - [0, 0, np.sin(ang / 2), np.cos(ang / 2)])) < 1e-6


def test_repropagate_about_new_biases(fv):
    rng = np.random.default_rng(9)
    dt, acc, gyr = _imu_stream(rng, n=50)
    P = fv.Preintegration(acc[0], gyr[0], np.zeros(3), np.zeros(3), *NOISE)
    for k in range(1, len(acc)):
        P.add(dt, acc[k], gyr[k])
    ba, bg = np.array([0.1, 0.0, -0.05]), np.array([0.0, 0.01, 0.0])
    P.repropagate(ba, bg)
    W = E.Preint(acc[0], gyr[0], ba, bg, *NOISE)
    for k in range(1, len(acc)):
        W.add(dt, acc[k], gyr[k])
    s = P.state()
    _close(s["delta_p"], W.dp)
    _close(s["delta_q"], W.dq)
    _close(s["covariance"], W.cov, 1e-11)


def _local_plus(block, d):
    """Perturb a pose block (p, q) by a 6-vector (dp, dtheta) on the right."""
    out = block.copy()
    out[:3] += d[:3]
    dq = np.array([d[3] / 2, d[4] / 2, d[5] / 2, 1.0])
    out[3:] = _unit(E.qmul(block[3:], dq))
    return out


def test_imu_factor_whitening_and_jacobians(fv):
    """src/ImuCostFunction.cpp:88-215.  The residual is sqrt(information)
    times the preintegration residual, and so is every Jacobian.  Unwhitened,
    the Jacobians match central differences of the preintegration residual:
    exactly in the position, velocity and bias rows, and to first order in
    the rotation rows -- at twice the differences there, because the
    reference's rotation residual is vec(dq^-1 Qi^-1 Qj) while its Jacobian
    blocks are those of 2 vec(...) (src/Preintegration.cpp:180 against
    src/ImuCostFunction.cpp:150-205)."""
    rng = np.random.default_rng(11)
    dt, acc, gyr = _imu_stream(rng, n=100)
    ba, bg = np.zeros(3), np.zeros(3)
    P = fv.Preintegration(acc[0], gyr[0], ba, bg, *NOISE)
    W = E.Preint(acc[0], gyr[0], ba, bg, *NOISE)
    for k in range(1, len(acc)):
        P.add(dt, acc[k], gyr[k])
        W.add(dt, acc[k], gyr[k])
    pose_i = np.concatenate([[0.1, 0.2, 0.3], _unit([0.1, 0.0, 0.2, 1.0])])
    sb_i = np.concatenate([[0.5, 0.0, 0.1], [0.01, 0.0, 0.0], [0.0, 0.001, 0.0]])
    pj, vj = W.predict(pose_i, sb_i[:3])
    pose_j = _local_plus(pj, np.array([0.01, -0.02, 0.005, 0.01, 0.0, -0.01]))
    sb_j = np.concatenate([vj + 0.01, [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
    r, J = P.factor(pose_i, sb_i, pose_j, sb_j)
    S = E.sqrt_information(W.cov)
    _close(r, S @ W.residual(pose_i, sb_i, pose_j, sb_j), 1e-9)
    Sinv = np.linalg.inv(S)
    raw = [Sinv @ j for j in J]
    rot = slice(3, 6)
    other = np.r_[0:3, 6:15]
    # the Jacobians take gravity as 9.8 where the residual takes 9.81
    # (include/f_vigs_slam/ImuCostFunction.hpp:19 against
    # include/f_vigs_slam/Preintegration.hpp:79): the pose_i rotation columns
    # of the position and velocity rows carry that difference
    T = W.sum_dt
    dG = E.G_FACTOR - E.G_PREINT
    Qii = E.qinv(pose_i[3:])
    grav = np.zeros((15, 3))
    grav[0:3] = E.skew(E.qrot(Qii, 0.5 * dG * T * T))
    grav[6:9] = E.skew(E.qrot(Qii, dG * T))
    h = 1e-6
    args = [pose_i, sb_i, pose_j, sb_j]
    for which in range(4):
        pose = which in (0, 2)
        Jb = raw[which]
        if pose:
            assert np.all(J[which][:, 6] == 0.0)
        for c in range(6 if pose else 9):
            ap, am = list(args), list(args)
            if pose:
                e = np.zeros(6)
                e[c] = h
                ap[which], am[which] = _local_plus(args[which], e), _local_plus(args[which], -e)
            else:
                e = np.zeros(9)
                e[c] = h
                ap[which], am[which] = args[which] + e, args[which] - e
            num = (W.residual(*ap) - W.residual(*am)) / (2 * h)
            if which == 0 and c >= 3:
                num = num + grav[:, c - 3]
            scale = max(1e-3, np.max(np.abs(num)))
            assert np.max(np.abs(Jb[other, c] - num[other])) <= 1e-6 * scale, (which, c)
            assert np.max(np.abs(Jb[rot, c] - 2.0 * num[rot])) <= 2e-2 * max(1e-3, np.max(np.abs(2.0 * num[rot]))) + 1e-9, (which, c)


def test_imu_factor_needs_samples(fv):
    P = fv.Preintegration(np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(3), *NOISE)
    pose = np.array([0, 0, 0, 0, 0, 0, 1.0])
    with pytest.raises(fv.FvgsError) as e:
        P.factor(pose, np.zeros(9), pose, np.zeros(9))
    assert e.value.status == -6


@pytest.mark.parametrize("m,n", [(6, 15), (15, 9), (3, 3)])
def test_marginalize(fv, m, n):
    """src/MarginalizationFactor.cpp:318-360: J^T J and J^T r of the prior
    reproduce the thresholded Schur complement."""
    rng = np.random.default_rng(m * 100 + n)
    N = m + n
    Jf = rng.normal(size=(2 * N, N))
    A = Jf.T @ Jf
    A[:2, :] *= 1.0  # keep symmetric
    b = rng.normal(size=N)
    J, r = fv.marginalize(A, b, m)
    As, bs = E.marginalize(A, b, m)
    Hk, Pk = E.thresholded(As, 1e-8)
    _close(J.T @ J, Hk, 1e-9)
    _close(J.T @ r, Pk @ bs, 1e-9)


def test_marginal_prior_evaluate(fv):
    """src/MarginalizationFactor.cpp:398-470: r + J dx with the pose blocks'
    local difference (sign-flipped when the relative rotation's w < 0)."""
    rng = np.random.default_rng(21)
    n = 6 + 9
    J = rng.normal(size=(n, n))
    r = rng.normal(size=n)
    x0 = [np.concatenate([rng.normal(size=3), _rand_q(rng)]), rng.normal(size=9)]
    d = np.array([0.01, -0.02, 0.03, 0.02, -0.01, 0.005])
    pose = _local_plus(x0[0], d)
    pose[3:] *= -1.0  # the same rotation with w < 0 in the relative quaternion
    sb = x0[1] + 0.01
    res, jac = fv.marginal_prior_evaluate(J, r, [(7, 0), (9, 6)], [pose, sb], x0)
    rel = E.qmul(E.qinv(x0[0][3:]), pose[3:])
    dth = 2.0 * rel[:3] * (-1.0 if rel[3] < 0 else 1.0)
    dx = np.concatenate([pose[:3] - x0[0][:3], dth, sb - x0[1]])
    _close(res, r + J @ dx)
    _close(dth, d[3:], 1e-5)
    _close(jac[0][:, :6], J[:, :6])
    assert np.all(jac[0][:, 6] == 0.0)
    _close(jac[1], J[:, 6:])


# ---------------------------------------------------------------------------
# visual-inertial normal equations (fvgs_vi_step / fvgs_vi_marginalize)
# ---------------------------------------------------------------------------
def _local_error(pose, ref):
    """(p - p_ref, 2 vec(q_ref^-1 q)): the local coordinates of the pose Plus."""
    d = E.qmul(E.qinv(ref[3:]), pose[3:])
    s = 2.0 if d[3] >= 0 else -2.0
    return np.concatenate([pose[:3] - ref[:3], s * d[:3]])


def _vi_case(fv, seed, noise=True):
    from f_vigs_slam_gb300 import synthetic as S

    tr = S.imu_trajectory(4, seed=seed, noise=noise)
    M = tr["imu_per_frame"]
    pre = fv.Preintegration(tr["acc"][0], tr["gyr"][0], np.zeros(3), np.zeros(3), tr["acc_sd"], tr["gyr_sd"], 1e-4,
                            1e-5)
    for m in range(1, M + 1):
        pre.add(tr["dt"], tr["acc"][m], tr["gyr"][m])
    rng = np.random.default_rng(seed)
    sb_i = np.concatenate([tr["imu_vel"][0], rng.normal(0, 0.01, 3), rng.normal(0, 0.001, 3)])
    pose_j, vj = pre.predict(tr["imu_pose"][0], tr["imu_vel"][0])
    pose_j[:3] += rng.normal(0, 0.01, 3)
    sb_j = np.concatenate([vj + rng.normal(0, 0.02, 3), sb_i[3:]])
    # a visual system pulling pose_j to the true pose: JtJ SPD, Jtr = JtJ e
    Q, _ = np.linalg.qr(rng.normal(size=(6, 6)))
    JtJ = Q @ np.diag(10.0 ** rng.uniform(4, 8, 6)) @ Q.T
    Jtr = JtJ @ _local_error(pose_j, tr["imu_pose"][1])
    return tr, pre, (tr["imu_pose"][0].copy(), sb_i), (pose_j, sb_j), JtJ, Jtr


def _prior(fv, seed):
    rng = np.random.default_rng(seed + 5)
    A = rng.normal(size=(30, 30))
    A = A @ A.T + 30 * np.eye(30)
    J, r = fv.marginalize(A, rng.normal(size=30), 15)
    return J, r


def _expected_step(fv, pre, JtJ, Jtr, si, sj, prior):
    """The normal equations assembled in NumPy from the library's own factor
    evaluations: H = sum J^T J, g = sum J^T r over the free local dims."""
    cols = []
    rs, Js = fv.pseudo_factor(JtJ, Jtr, 1e-4)
    Jv = np.zeros((6, 30))
    Jv[:, 15:21] = Js
    r_imu, (Jpi, Jsi, Jpj, Jsj) = pre.factor(si[0], si[1], sj[0], sj[1])
    Ji = np.zeros((15, 30))
    Ji[:, 0:6], Ji[:, 6:15], Ji[:, 15:21], Ji[:, 21:30] = Jpi[:, :6], Jsi, Jpj[:, :6], Jsj
    rows = [(rs, Jv), (r_imu, Ji)]
    if prior is not None:
        res, (Jp, Jb) = fv.marginal_prior_evaluate(prior[0], prior[1], [(7, 0), (9, 6)], [si[0], si[1]],
                                                   [prior[2][:7], prior[2][7:]])
        Jr = np.zeros((15, 30))
        Jr[:, 0:6], Jr[:, 6:15] = Jp[:, :6], Jb
        rows.append((res, Jr))
    H = sum(J.T @ J for _, J in rows)
    g = sum(J.T @ r for r, J in rows)
    cost = 0.5 * sum(float(r @ r) for r, _ in rows)
    free = np.arange(30) if prior is not None else np.arange(15, 30)
    d = np.zeros(30)
    Hf, gf = H[np.ix_(free, free)], g[free]
    d[free] = -np.linalg.solve(Hf, gf)
    return d, cost, (free, Hf, gf)


def _plus(pose, d):
    q = E.qmul(pose[3:], np.array([0.5 * d[3], 0.5 * d[4], 0.5 * d[5], 1.0]))
    return np.concatenate([pose[:3] + d[:3], q / np.linalg.norm(q)])


@pytest.mark.parametrize("with_prior", [False, True])
def test_vi_step_solves_the_normal_equations(fv, with_prior):
    """fvgs_vi_step = the Gauss-Newton step of {RGB-D pseudo factor, IMU
    factor, marginalization prior}: 15 free dims (state i fixed) or 30."""
    tr, pre, si, sj, JtJ, Jtr = _vi_case(fv, 11)
    prior = None
    if with_prior:
        J, r = _prior(fv, 11)
        x0 = np.concatenate([si[0], si[1]]).copy()
        x0[:3] += 0.003  # linearised away from the current state
        prior = (J, r, x0)
    want, want_cost, (free, Hf, gf) = _expected_step(fv, pre, JtJ, Jtr, si, sj, prior)
    (pi2, si2), (pj2, sj2), cost, d = fv.vi_step(pre, JtJ, Jtr, si, sj, prior)
    # the step solves the normal equations (relative residual at FP64 level),
    # and equals NumPy's solution to the system's conditioning
    assert np.linalg.norm(Hf @ d[free] + gf) <= 1e-9 * np.linalg.norm(gf)
    cond = np.linalg.cond(Hf)
    np.testing.assert_allclose(d, want, rtol=0, atol=max(1e-12, 1e-15 * cond) * np.abs(want).max())
    assert abs(cost - want_cost) <= 1e-10 * want_cost
    np.testing.assert_allclose(pj2, _plus(sj[0], d[15:21]), rtol=0, atol=1e-12)
    np.testing.assert_allclose(sj2, sj[1] + d[21:30], rtol=0, atol=1e-12)
    if with_prior:
        np.testing.assert_allclose(pi2, _plus(si[0], d[0:6]), rtol=0, atol=1e-12)
        np.testing.assert_allclose(si2, si[1] + d[6:15], rtol=0, atol=1e-12)
    else:
        assert np.all(d[:15] == 0) and np.array_equal(pi2, si[0]) and np.array_equal(si2, si[1])


def test_vi_marginalize_is_the_schur_complement(fv):
    tr, pre, si, sj, JtJ, Jtr = _vi_case(fv, 12)
    J0, r0 = _prior(fv, 12)
    prior = (J0, r0, np.concatenate([si[0], si[1]]))
    J, r, x0 = fv.vi_marginalize(pre, JtJ, Jtr, si, sj, prior)
    # expected: the same linearised system, state i marginalised
    rows = []
    rs, Js = fv.pseudo_factor(JtJ, Jtr, 1e-4)
    Jv = np.zeros((6, 30))
    Jv[:, 15:21] = Js
    r_imu, (Jpi, Jsi, Jpj, Jsj) = pre.factor(si[0], si[1], sj[0], sj[1])
    Ji = np.zeros((15, 30))
    Ji[:, 0:6], Ji[:, 6:15], Ji[:, 15:21], Ji[:, 21:30] = Jpi[:, :6], Jsi, Jpj[:, :6], Jsj
    res, (Jp, Jb) = fv.marginal_prior_evaluate(J0, r0, [(7, 0), (9, 6)], [si[0], si[1]], [prior[2][:7], prior[2][7:]])
    Jr = np.zeros((15, 30))
    Jr[:, 0:6], Jr[:, 6:15] = Jp[:, :6], Jb
    for rr, JJ in ((rs, Jv), (r_imu, Ji), (res, Jr)):
        rows.append((rr, JJ))
    A = sum(JJ.T @ JJ for _, JJ in rows)
    b = sum(JJ.T @ rr for rr, JJ in rows)
    As = A[15:, 15:] - A[15:, :15] @ np.linalg.solve(A[:15, :15], A[:15, 15:])
    bs = b[15:] - A[15:, :15] @ np.linalg.solve(A[:15, :15], b[:15])
    np.testing.assert_allclose(J.T @ J, As, rtol=0, atol=1e-8 * np.abs(As).max())
    np.testing.assert_allclose(J.T @ r, bs, rtol=0, atol=1e-8 * max(1.0, np.abs(bs).max()))
    np.testing.assert_array_equal(x0, np.concatenate([sj[0], sj[1]]))


def test_vi_tracker_converges_on_a_synthetic_trajectory(fv):
    """The tracking loop (preintegrate, predict, 20 Gauss-Newton steps,
    marginalise) on noisy 200 Hz IMU data with constant sensor biases and a
    visual system of the RGB-D system's magnitude pinning the camera pose: the
    IMU-frame pose follows the truth, the velocity stays on it, and the bias
    estimates (started at zero) converge towards the true biases."""
    from f_vigs_slam_gb300 import synthetic as S
    from f_vigs_slam_gb300.vi import VisualInertialTracker

    ba, bg = np.array([0.05, -0.03, 0.04]), np.array([0.002, -0.001, 0.0015])
    tr = S.imu_trajectory(16, seed=3, acc_bias=ba, gyr_bias=bg)
    truth = {}

    def visual(cam_pose):
        # camera-frame system pulling the camera to the frame's true camera pose
        t_true, q_true = truth["cam"]
        e = np.concatenate([np.asarray(cam_pose[0], np.float64) - t_true,
                            _local_error(np.concatenate([[0, 0, 0], np.asarray(cam_pose[1], np.float64)]),
                                         np.concatenate([[0, 0, 0], np.asarray(q_true, np.float64)]))[3:]])
        JtJ = np.diag([1e12, 1e12, 1e12, 1e11, 1e11, 1e11])
        return JtJ, JtJ @ e

    vt = VisualInertialTracker(visual, tr["t_imu_cam"], tr["q_imu_cam"], tr["acc_sd"], tr["gyr_sd"])
    M = tr["imu_per_frame"]
    vt.start(tr["imu_pose"][0], np.concatenate([tr["imu_vel"][0], np.zeros(6)]), tr["acc"][0], tr["gyr"][0])
    ba_err, bg_err = [], []
    for k in range(1, len(tr["frame_t"])):
        t_c, q_c = tr["cam_pose"][k]
        truth["cam"] = (np.asarray(t_c, np.float64), np.asarray(q_c, np.float64))
        sl = slice((k - 1) * M + 1, k * M + 1)
        pose, sb, costs = vt.track(tr["dt"], tr["acc"][sl], tr["gyr"][sl])
        ang, dist = S.pose_error((pose[:3], pose[3:]), (tr["imu_pose"][k][:3], tr["imu_pose"][k][3:]))
        assert ang < 1e-5 and dist < 1e-5, (k, ang, dist)
        assert np.linalg.norm(sb[:3] - tr["imu_vel"][k]) < 5e-3
        assert costs[-1] < costs[0]
        ba_err.append(float(np.linalg.norm(sb[3:6] - ba)))
        bg_err.append(float(np.linalg.norm(sb[6:9] - bg)))
    assert ba_err[-1] < 0.2 * ba_err[0] and bg_err[-1] < 0.3 * bg_err[0], (ba_err, bg_err)
