"""The allocation-free pose-Jacobian entry point (fvgs_rgbd_pose_jacobians_noalloc).

It exists for callers that cannot call cudaMalloc (a tracking thread inside
an application that owns the GPU memory budget, or a real-time loop that must
not pay cudaMalloc's synchronisation).  The test plays such a caller: it owns
every device buffer (here allocated through torch), passes them in the
reference's screen-space layout, and checks two calls in a row against the
session entry point fvgs_track_jacobian, within the tracking tolerance of
1e-5 relative.  This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import make_frame, rel_err, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _dev(torch, a, dtype=None):
    a = np.ascontiguousarray(a if dtype is None else a.astype(dtype))
    return torch.from_numpy(a).to("cuda:0")


def test_noalloc_matches_session_entry(oracle, fvgs_lib):
    torch = pytest.importorskip("torch")
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(20_000, seed=31)
    P = oracle.default_params()
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(32))
    rgb, d, gx, gy = make_frame(oracle, scene, true_pose, K, W, H, P)
    pose = (np.array([0.003, -0.002, 0.001], np.float32), S.IDENTITY_Q)

    # existing entry point, and the binned screen-space buffers it produced
    with fv.Session(scene.n, W, H) as s:
        s.set_debug(fv.DEBUG_PROJECTION)
        s.upload(scene)
        s.set_frame(0, rgb, d, gx, gy)
        s.project_bin(pose, K, W, H)
        proj = s.download_projection()
        _, vals, ranges = s.download_binning(W, H)
        JtJ_ref, Jtr_ref = s.track_jacobian(pose, K, 0)

    torch.cuda.init()
    bufs = dict(
        ranges=_dev(torch, ranges.view(np.int32)), indices=_dev(torch, vals.view(np.int32)),
        uv=_dev(torch, proj["uv"]), depth=_dev(torch, proj["depth"]), inv=_dev(torch, proj["inv2d"]),
        phat=_dev(torch, proj["phat"]), col=_dev(torch, scene.colors, np.float32),
        opa=_dev(torch, scene.opacities, np.float32), gx=_dev(torch, gx), gy=_dev(torch, gy),
        rgb=_dev(torch, rgb), dep=_dev(torch, d),
    )
    torch.cuda.synchronize()
    lib = fv.load_library()
    ptr = {k: C.c_void_p(v.data_ptr()) for k, v in bufs.items()}
    params = fv.default_params()
    results = []
    for _ in range(2):
        JtJ = np.zeros((6, 6), np.float64)
        Jtr = np.zeros(6, np.float64)
        st = lib.fvgs_rgbd_pose_jacobians_noalloc(
            ptr["ranges"], ptr["indices"], ptr["uv"], ptr["depth"], ptr["inv"], ptr["phat"], ptr["col"], ptr["opa"],
            ptr["gx"], ptr["gy"], ptr["rgb"], ptr["dep"], C.byref(fv.make_pose(pose)), C.byref(fv.make_intr(K)),
            C.byref(params), C.c_int(W), C.c_int(H), C.c_void_p(JtJ.ctypes.data), C.c_void_p(Jtr.ctypes.data),
            C.c_void_p(torch.cuda.current_stream().cuda_stream),
        )
        assert st == 0, fv.STATUS_NAMES.get(st, st)
        results.append((JtJ, Jtr))
    for JtJ, Jtr in results:
        assert rel_err(JtJ, JtJ_ref) <= RTOL
        assert rel_err(Jtr, Jtr_ref) <= RTOL
    np.testing.assert_array_equal(results[0][0], results[1][0])
    np.testing.assert_array_equal(results[0][1], results[1][1])

    # frames beyond the static scratch are rejected before any GPU work
    JtJ = np.zeros((6, 6), np.float64)
    Jtr = np.zeros(6, np.float64)
    st = lib.fvgs_rgbd_pose_jacobians_noalloc(
        ptr["ranges"], ptr["indices"], ptr["uv"], ptr["depth"], ptr["inv"], ptr["phat"], ptr["col"], ptr["opa"],
        ptr["gx"], ptr["gy"], ptr["rgb"], ptr["dep"], C.byref(fv.make_pose(pose)), C.byref(fv.make_intr(K)),
        C.byref(params), C.c_int(4096), C.c_int(1040), C.c_void_p(JtJ.ctypes.data), C.c_void_p(Jtr.ctypes.data),
        None,
    )
    assert st == -4  # FVGS_E_CAPACITY
