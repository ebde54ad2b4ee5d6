"""GPU parity of the fused tracking kernel against the FP64 oracle, for the
reference's approximate pose Jacobian (FVGS_Q_POSE_JAC_APPROX set) and the
analytic one (clear).

Tolerances: rendered colour and depth within
1e-5 relative; JtJ and Jtr within 1e-5 relative (Frobenius / 2-norm) of the
FP64 oracle.  The GPU blends in FP32, so a pixel whose FP32 and FP64 values
fall on opposite sides of a discrete threshold (alpha < 1/255, T < 1e-4,
T crossing 0.5) is a "flip"; flips are counted and must stay rare.
Tracking with the analytic Jacobian must reach 1e-4 rad / 1e-4 m in 20
Gauss-Newton iterations from a 1 deg / 2 cm perturbation.
"""
import numpy as np
import pytest

from conftest import make_frame, rel_err, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

IMG_RTOL = 1e-5
JAC_RTOL = 1e-5
POSE_TOL = 1e-4  # rad and m after 20 Gauss-Newton iterations

REF_JAC = 0x100 | 0x200  # FVGS_Q_POSE_JAC_APPROX | FVGS_Q_DEPTH_HUBER: the reference's Jacobian and depth weight
REF = 0x4 | 0x8 | REF_JAC  # the reference's conic layout and mapping cap, its Jacobian
INTENDED = 0x0  # every reference behaviour off: the analytic Jacobian


def _setup(oracle, fv, n, scale, seed, quirks=REF):
    W, H, K = scaled_camera(scale)
    scene = S.cam_box(n, seed=seed)
    P = oracle.default_params(quirks)
    rng = np.random.default_rng(seed + 100)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    frame = make_frame(oracle, scene, true_pose, K, W, H, P)
    s = fv.Session(n, W, H, fv.default_params(quirks))
    s.upload(scene)
    s.set_frame(0, *frame)
    return W, H, K, scene, P, frame, s


def _img_compare(g, o, rtol, floor=1e-3):
    """Per-pixel relative error |g-o| / max(|o|, floor), excluding pixels whose
    FP32/FP64 results differ by a threshold flip (abs error above 1e-3 of the
    value range).  Depth uses floor = 1 m: the median depth z + dx*phx + dy*phy
    cancels to values near zero where an FP32 result can only be accurate to
    ~1e-5 m absolute, not relative."""
    g = np.asarray(g, np.float64)
    o = np.asarray(o, np.float64)
    err = np.abs(g - o)
    scale = np.maximum(np.abs(o), floor)
    flips = err > 1e-3 * max(1.0, float(np.abs(o).max()))
    rel = (err / scale)[~flips]
    return (float(rel.max()) if rel.size else 0.0), int(flips.sum())


def test_render_parity(oracle, fvgs_lib):
    W, H, K, scene, P, frame, s = _setup(oracle, fvgs_lib, 20_000, 0.5, 7)
    pose = (np.zeros(3), S.IDENTITY_Q)
    col, dep, fT, nc = s.render(pose, K, W, H)
    b = oracle.prepare(scene, pose, K, W, H, P)
    oc, od, oT, onc = oracle.render(b, pose, K, W, H, P)
    for name, g, o, floor in (("colour", col, oc, 1e-3), ("depth", dep, od, 1.0), ("final_T", fT, oT, 1e-3)):
        rel, flips = _img_compare(g, o, IMG_RTOL, floor)
        assert rel <= IMG_RTOL, (name, rel, flips)
        assert flips <= 0.001 * W * H, (name, flips)
    assert np.mean(nc == onc) > 0.999
    s.close()


@pytest.mark.parametrize("quirks", [REF, 0x8 | REF_JAC, INTENDED, 0x4, 0x200],
                         ids=["ref", "ref_noswap", "analytic", "analytic_swap", "analytic_huber"])
def test_track_jacobian_parity(oracle, fvgs_lib, quirks):
    W, H, K, scene, P, frame, s = _setup(oracle, fvgs_lib, 20_000, 0.5, 3, quirks)
    pose = (np.zeros(3), S.IDENTITY_Q)
    JtJ, Jtr = s.track_jacobian(pose, K, 0)
    b = oracle.prepare(scene, pose, K, W, H, P)
    r = oracle.track(b, frame, pose, K, W, H, P, images=False)
    e1, e2 = rel_err(JtJ, r.JtJ), rel_err(Jtr, r.Jtr)
    print("JtJ rel", e1, "Jtr rel", e2)
    assert np.allclose(JtJ, JtJ.T)
    assert e1 <= JAC_RTOL, e1
    assert e2 <= JAC_RTOL, e2
    s.close()


@pytest.mark.parametrize("quirks", [REF, INTENDED], ids=["ref", "analytic"])
def test_track_jacobian_parity_moved_pose(oracle, fvgs_lib, quirks):
    """Away from the identity: the camera translated and rotated, so the
    per-Gaussian depths z + dx phat.x + dy phat.y of the reference's Jacobian
    cancel for other pixels, and screen offsets dx = u - x round in FP32
    where |dx| > |u|."""
    W, H, K, scene, P, frame, s = _setup(oracle, fvgs_lib, 20_000, 0.5, 31, quirks)
    for pose in ((np.array([0.003, -0.002, 0.001], np.float32), S.IDENTITY_Q),
                 S.perturb((np.zeros(3), S.IDENTITY_Q), 0.5, 1.0, np.random.default_rng(33))):
        JtJ, Jtr = s.track_jacobian(pose, K, 0)
        b = oracle.prepare(scene, pose, K, W, H, P)
        r = oracle.track(b, frame, pose, K, W, H, P, images=False)
        e1, e2 = rel_err(JtJ, r.JtJ), rel_err(Jtr, r.Jtr)
        print("JtJ rel", e1, "Jtr rel", e2)
        assert e1 <= JAC_RTOL, e1
        assert e2 <= JAC_RTOL, e2
    s.close()


@pytest.mark.parametrize("quirks", [REF, INTENDED], ids=["ref", "analytic"])
def test_track_jacobian_parity_opaque_splats(oracle, fvgs_lib, quirks):
    """Nearly opaque Gaussians (opacity in [0.9, 1]): alpha reaches the 0.99
    clamp and 1 / (1 - alpha) reaches 100, the largest factor the analytic
    Jacobian's single pass (S1 - C S2) and the reference's running remaining
    colour put on a term's rounding; pixels terminate after a few
    contributors."""
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    base = S.cam_box(20_000, seed=41)
    rng = np.random.default_rng(42)
    scene = S.Scene(base.positions, base.scales, base.orientations, base.colors,
                    rng.uniform(0.9, 1.0, base.n).astype(np.float32))
    P = oracle.default_params(quirks)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    frame = make_frame(oracle, scene, true_pose, K, W, H, P)
    pose = S.perturb(true_pose, 0.5, 1.0, rng)
    with fv.Session(scene.n, W, H, fv.default_params(quirks)) as s:
        s.upload(scene)
        s.set_frame(0, *frame)
        JtJ, Jtr = s.track_jacobian(pose, K, 0)
    b = oracle.prepare(scene, pose, K, W, H, P)
    r = oracle.track(b, frame, pose, K, W, H, P, images=False)
    e1, e2 = rel_err(JtJ, r.JtJ), rel_err(Jtr, r.Jtr)
    print("JtJ rel", e1, "Jtr rel", e2)
    assert e1 <= JAC_RTOL, e1
    assert e2 <= JAC_RTOL, e2


def test_track_deterministic(oracle, fvgs_lib):
    W, H, K, scene, P, frame, s = _setup(oracle, fvgs_lib, 10_000, 0.5, 5)
    pose = (np.array([0.01, 0, 0], np.float32), S.IDENTITY_Q)
    a = s.track_jacobian(pose, K, 0)
    b = s.track_jacobian(pose, K, 0)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    s.close()


def test_track_frame_matches_host_loop(oracle, fvgs_lib):
    """The on-device Gauss-Newton loop equals the host loop that uses the
    same Jacobians and the eigen-regularised pseudo-factor step."""
    W, H, K, scene, P, frame, s = _setup(oracle, fvgs_lib, 10_000, 0.5, 9)
    pose0 = (np.zeros(3), S.IDENTITY_Q.astype(np.float64))
    pose = pose0
    for _ in range(3):
        JtJ, Jtr = s.track_jacobian(pose, K, 0)
        pose = oracle.pose_plus(pose, oracle.gn_delta(JtJ, Jtr))
    dev_pose, _ = s.track_frame(pose0, K, iterations=3)
    ang, tr = S.pose_error(dev_pose, pose)
    assert ang < 1e-6 and tr < 1e-6, (ang, tr)
    s.close()


@pytest.mark.parametrize("quirks", [REF, INTENDED], ids=["ref", "analytic"])
def test_track_jacobian_parity_vga_50k(oracle, fvgs_lib, quirks):
    """The small plain-method workload whole: N = 50k at 640 x 480, tracked
    from the identity against a frame rendered 1 deg / 2 cm away."""
    W, H, K, scene, P, frame, s = _setup(oracle, fvgs_lib, 50_000, 1.0, 11, quirks)
    pose = (np.zeros(3), S.IDENTITY_Q)
    JtJ, Jtr = s.track_jacobian(pose, K, 0)
    b = oracle.prepare(scene, pose, K, W, H, P)
    r = oracle.track(b, frame, pose, K, W, H, P, images=False)
    e1, e2 = rel_err(JtJ, r.JtJ), rel_err(Jtr, r.Jtr)
    print("JtJ rel", e1, "Jtr rel", e2)
    assert e1 <= JAC_RTOL, e1
    assert e2 <= JAC_RTOL, e2
    s.close()


def _target_pyramid(oracle, scene, pose, K0, W, H, P, levels, seed):
    """Observed frames of every pyramid level rendered at `pose` by the oracle
    (a synthetic sensor at each resolution, intrinsics scaled by 2^-l), plus
    N(0, 0.01) colour and N(0, 0.005 m) depth noise."""
    rng = np.random.default_rng(seed)
    out = []
    for lv in range(levels):
        sc = 1.0 / (1 << lv)
        K = tuple(np.float32(k * sc) for k in K0)
        w, h = W >> lv, H >> lv
        b = oracle.prepare(scene, pose, K, w, h, P)
        col, dep, _, _ = oracle.render(b, pose, K, w, h, P)
        rgb, d = S.add_noise(col.astype(np.float32), dep.astype(np.float32), rng)
        gx, gy = S.sobel3(rgb)
        out.append((rgb, d, gx, gy))
    return out


@pytest.mark.parametrize("seed", [0, 1])
def test_intended_tracking_converges_vga_50k(oracle, fvgs_lib, seed):
    """Analytic Jacobian, coarse-to-fine over four levels (4 + 4 + 6 + 6 = 20
    Gauss-Newton iterations): from 1 deg / 2 cm the pose reaches 1e-4 rad /
    1e-4 m, and it matches the oracle's own loop over the same frames."""
    fv = fvgs_lib
    W, H, K0 = scaled_camera(1.0)
    scene = S.cam_box(50_000, seed=seed)
    P = oracle.default_params(INTENDED)
    rng = np.random.default_rng(seed + 1)
    ident = (np.zeros(3, np.float32), S.IDENTITY_Q.copy())
    true_pose = S.perturb(ident, 1.0, 2.0, rng)
    iters = (4, 4, 6, 6)
    frames = _target_pyramid(oracle, scene, true_pose, K0, W, H, P, len(iters), seed + 2)
    with fv.Session(scene.n, W, H, fv.default_params(INTENDED)) as s:
        s.upload(scene)
        for lv, fr in enumerate(frames):
            s.set_frame(lv, *fr)
        gpu_pose, _ = s.track_frame_pyramid(ident, K0, iters)
    err = S.pose_error(gpu_pose, true_pose)
    print("GPU pose error rad %.3e m %.3e" % err)
    assert err[0] <= POSE_TOL and err[1] <= POSE_TOL, err
    # the oracle's loop: same levels, same pseudo-factor step, FP64 throughout
    pose = (ident[0].astype(np.float64), ident[1].astype(np.float64))
    for lv in reversed(range(len(iters))):
        sc = 1.0 / (1 << lv)
        K = tuple(np.float32(k * sc) for k in K0)
        w, h = W >> lv, H >> lv
        for _ in range(iters[lv]):
            pf = (pose[0].astype(np.float32), pose[1].astype(np.float32))
            b = oracle.prepare(scene, pf, K, w, h, P)
            r = oracle.track(b, frames[lv], pf, K, w, h, P, images=False)
            pose = oracle.pose_plus(pose, oracle.gn_delta(r.JtJ, r.Jtr))
    d = S.pose_error(gpu_pose, pose)
    print("GPU vs oracle loop rad %.3e m %.3e" % d)
    assert d[0] <= 1e-5 and d[1] <= 1e-5, d


def test_pyramid_frame_eager_graph_and_batched_agree(oracle, fvgs_lib):
    """A coarse-to-fine frame gives the same pose eagerly
    (fvgs_track_frame_pyramid), submitted (captured as a graph, then replayed)
    and batched with another session (fvgs_frames_run_pyramid)."""
    fv = fvgs_lib
    W, H, K0 = scaled_camera(0.5)
    scene = S.cam_box(20_000, seed=21)
    P = oracle.default_params(INTENDED)
    rng = np.random.default_rng(22)
    ident = (np.zeros(3, np.float32), S.IDENTITY_Q.copy())
    true_pose = S.perturb(ident, 1.0, 2.0, rng)
    iters = (2, 3, 3)
    frames = _target_pyramid(oracle, scene, true_pose, K0, W, H, P, len(iters), 23)
    sessions = []
    for _ in range(2):
        s = fv.Session(scene.n, W, H, fv.default_params(INTENDED))
        s.upload(scene)
        for lv, fr in enumerate(frames):
            s.set_frame(lv, *fr)
        sessions.append(s)
    a, _ = sessions[0].track_frame_pyramid(ident, K0, iters)
    got = []
    for _ in range(3):
        sessions[0].frame_submit_pyramid(ident, K0, iters)
        got.append(sessions[0].frame_wait()[0])
    assert sessions[0].frame_stats()["graphed"] >= 2
    got += fv.frames_run_pyramid(sessions, [ident, ident], [K0, K0], iters)
    for p in got:
        np.testing.assert_array_equal(p[0], a[0])
        np.testing.assert_array_equal(p[1], a[1])
    for s in sessions:
        s.close()


def _tiles_to_world(tiles, q):
    """Camera-frame tile partials (translation rows without R) to the world
    frame the oracle reports: b = (R b_t, b_r), A = D A D^T, D = diag(R, I)."""
    R = S.qrot(np.asarray(q, np.float64))
    D = np.eye(6)
    D[:3, :3] = R
    iu = np.triu_indices(6)
    out = np.zeros_like(tiles, dtype=np.float64)
    for t in range(tiles.shape[0]):
        A = np.zeros((6, 6))
        A[iu] = tiles[t, 6:]
        A = A + A.T - np.diag(np.diag(A))
        Aw = D @ A @ D.T
        out[t, :6] = D @ tiles[t, :6]
        out[t, 6:] = Aw[iu]
    return out


@pytest.mark.parametrize("quirks", [REF, INTENDED], ids=["ref", "analytic"])
def test_track_tiles_room_1m_hd(oracle, fvgs_lib, quirks):
    """The large plain-method workload (N = 1 M room, 1280 x 720): per-tile
    partials of 200 tiles spread over the frame against the oracle, after a
    full binning and after an incremental one (the second evaluation, at a
    pose one Gauss-Newton-sized step away, continues the first binning)."""
    fv = fvgs_lib
    cam = S.CAM_HD
    W, H, K = cam.width, cam.height, cam.intrinsics
    scene = S.room(1_000_000, seed=0)
    traj = S.trajectory(2, seed=3)
    true_pose = traj[1]
    rng = np.random.default_rng(5)
    pose_a = S.perturb(true_pose, 0.05, 0.1, rng)
    pose_b = S.perturb(pose_a, 0.01, 0.02, rng)
    P = oracle.default_params(quirks)
    T = ((W + 15) // 16) * ((H + 15) // 16)
    sel = np.arange(0, T, T // 200)[:200]
    with fv.Session(scene.n, W, H, fv.default_params(quirks)) as s:
        s.upload(scene)
        col, dep, _, _ = s.render(true_pose, K, W, H)
        rgb, d = S.add_noise(col, dep, rng)
        gx, gy = S.sobel3(rgb)
        s.set_frame(0, rgb, d, gx, gy)
        s.upload(scene)  # no binning history: the first evaluation bins in full
        got = {}
        for name, pose in (("full", pose_a), ("incremental", pose_b)):
            s.track_jacobian(pose, K, 0)
            got[name] = (pose, s.download_tile_partials(T), s.binning_info()["incremental"])
    assert not got["full"][2] and got["incremental"][2]
    for name, (pose, tiles_gpu, _) in got.items():
        b = oracle.prepare(scene, pose, K, W, H, P)
        r = oracle.track(b, (rgb, d, gx, gy), pose, K, W, H, P, images=False, tiles=sel)
        g = _tiles_to_world(tiles_gpu[sel].astype(np.float64), pose[1])
        o = r.tiles[sel]
        e_sum_jtj = rel_err(g[:, 6:].sum(0), o[:, 6:].sum(0))
        e_sum_jtr = rel_err(g[:, :6].sum(0), o[:, :6].sum(0))
        per = np.array([rel_err(g[t], o[t]) for t in range(len(sel)) if np.linalg.norm(o[t]) > 0])
        print(name, "sum JtJ rel %.2e Jtr rel %.2e, tiles within 1e-4: %.3f (%d)" %
              (e_sum_jtj, e_sum_jtr, np.mean(per <= 1e-4), per.size))
        assert e_sum_jtj <= JAC_RTOL and e_sum_jtr <= JAC_RTOL, (name, e_sum_jtj, e_sum_jtr)
        assert per.size > 150 and np.mean(per <= 1e-4) > 0.97, (name, np.sort(per)[-5:])
