"""The allocation-free pose-Jacobian entry point (fvgs_rgbd_pose_jacobians_noalloc).

It exists for callers that cannot call cudaMalloc (a tracking thread inside
an application that owns the GPU memory budget, or a real-time loop that must
not pay cudaMalloc's synchronisation).  The test plays such a caller: it owns
every device buffer (here allocated through torch), passes them in the
reference's screen-space layout with their lengths, and checks, within the
tracking tolerance of 1e-5 relative:
  * two calls in a row against the session entry point fvgs_track_jacobian
    and against the FP64 oracle on the same binning;
  * a frame of exactly FVGS_NOALLOC_MAX_TILES tiles (4096 x 1024) against the
    session entry point, then the small frame again (the shared scratch keeps
    the large frame's contents; a smaller frame must not read them);
  * that a larger frame is rejected.
This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import make_frame, rel_err, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

RTOL = 1e-5
MAX_TILES = 16384  # FVGS_NOALLOC_MAX_TILES


def _dev(torch, a, dtype=None):
    a = np.ascontiguousarray(a if dtype is None else a.astype(dtype))
    return torch.from_numpy(a).to("cuda:0")


def _session_case(fv, scene, frame, pose, K, W, H):
    """The session entry point's result and the binned screen-space buffers it produced."""
    rgb, d, gx, gy = frame
    with fv.Session(scene.n, W, H) as s:
        s.set_debug(fv.DEBUG_PROJECTION)
        s.upload(scene)
        s.set_frame(0, rgb, d, gx, gy)
        s.project_bin(pose, K, W, H)
        proj = s.download_projection()
        _, vals, ranges = s.download_binning(W, H)
        JtJ, Jtr = s.track_jacobian(pose, K, 0)
    return proj, vals, ranges, JtJ, Jtr


def _noalloc(torch, fv, scene, frame, proj, vals, ranges, pose, K, W, H, stream=None):
    rgb, d, gx, gy = frame
    bufs = dict(
        ranges=_dev(torch, ranges.view(np.int32)), indices=_dev(torch, vals.view(np.int32)),
        uv=_dev(torch, proj["uv"]), depth=_dev(torch, proj["depth"]), inv=_dev(torch, proj["inv2d"]),
        phat=_dev(torch, proj["phat"]), col=_dev(torch, scene.colors, np.float32),
        opa=_dev(torch, scene.opacities, np.float32), gx=_dev(torch, gx), gy=_dev(torch, gy),
        rgb=_dev(torch, rgb), dep=_dev(torch, d),
    )
    torch.cuda.synchronize()
    ptr = {k: C.c_void_p(v.data_ptr()) for k, v in bufs.items()}
    JtJ = np.zeros((6, 6), np.float64)
    Jtr = np.zeros(6, np.float64)
    st = fv.load_library().fvgs_rgbd_pose_jacobians_noalloc(
        ptr["ranges"], ptr["indices"], ptr["uv"], ptr["depth"], ptr["inv"], ptr["phat"], ptr["col"], ptr["opa"],
        ptr["gx"], ptr["gy"], ptr["rgb"], ptr["dep"], C.byref(fv.make_pose(pose)), C.byref(fv.make_intr(K)),
        C.byref(fv.default_params()), C.c_int(W), C.c_int(H), C.c_uint32(scene.n), C.c_uint32(vals.shape[0]),
        C.c_void_p(JtJ.ctypes.data), C.c_void_p(Jtr.ctypes.data),
        C.c_void_p(torch.cuda.current_stream().cuda_stream if stream is None else stream),
    )
    return st, JtJ, Jtr


def test_noalloc_matches_session_entry(oracle, fvgs_lib):
    torch = pytest.importorskip("torch")
    fv = fvgs_lib
    torch.cuda.init()
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(20_000, seed=31)
    P = oracle.default_params()
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(32))
    frame = make_frame(oracle, scene, true_pose, K, W, H, P)
    pose = (np.array([0.003, -0.002, 0.001], np.float32), S.IDENTITY_Q)
    proj, vals, ranges, JtJ_ref, Jtr_ref = _session_case(fv, scene, frame, pose, K, W, H)
    b = oracle.prepare(scene, pose, K, W, H, P)
    o = oracle.track(b, frame, pose, K, W, H, P, images=False)

    results = []
    for _ in range(2):
        st, JtJ, Jtr = _noalloc(torch, fv, scene, frame, proj, vals, ranges, pose, K, W, H)
        assert st == 0, fv.STATUS_NAMES.get(st, st)
        results.append((JtJ, Jtr))
    for JtJ, Jtr in results:
        assert rel_err(JtJ, JtJ_ref) <= RTOL and rel_err(Jtr, Jtr_ref) <= RTOL
        assert rel_err(JtJ, o.JtJ) <= RTOL and rel_err(Jtr, o.Jtr) <= RTOL
    np.testing.assert_array_equal(results[0][0], results[1][0])
    np.testing.assert_array_equal(results[0][1], results[1][1])

    # a frame of exactly the static scratch's capacity: 256 x 64 tiles
    WL, HL = 4096, 1024
    assert (WL // 16) * (HL // 16) == MAX_TILES
    KL = (1400.0, 1400.0, 2047.5, 511.5)
    big = S.cam_box(60_000, seed=33)
    big.positions[:, 0] *= 3.0
    with fv.Session(big.n, WL, HL) as s:
        s.upload(big)
        col, dep, _, _ = s.render(true_pose, KL, WL, HL)
    rgbL, dL = S.add_noise(col, dep, np.random.default_rng(34))
    gxL, gyL = S.sobel3(rgbL)
    frameL = (rgbL, dL, gxL, gyL)
    projL, valsL, rangesL, JtJ_L, Jtr_L = _session_case(fv, big, frameL, pose, KL, WL, HL)
    last = rangesL[-1]
    assert last[1] > last[0] or rangesL[-64:, 1].max() > 0  # the last tile row is covered
    st, JtJ, Jtr = _noalloc(torch, fv, big, frameL, projL, valsL, rangesL, pose, KL, WL, HL)
    assert st == 0, fv.STATUS_NAMES.get(st, st)
    assert np.all(np.isfinite(JtJ)) and np.all(np.isfinite(Jtr))
    assert rel_err(JtJ, JtJ_L) <= RTOL and rel_err(Jtr, Jtr_L) <= RTOL

    # the small frame after the large one: nothing of the large call is read
    st, JtJ, Jtr = _noalloc(torch, fv, scene, frame, proj, vals, ranges, pose, K, W, H)
    assert st == 0
    np.testing.assert_array_equal(JtJ, results[0][0])
    np.testing.assert_array_equal(Jtr, results[0][1])

    # frames beyond the static scratch are rejected before any GPU work
    st, _, _ = _noalloc(torch, fv, scene, frame, proj, vals, ranges, pose, K, 4096, 1040, stream=0)
    assert st == -4  # FVGS_E_CAPACITY
