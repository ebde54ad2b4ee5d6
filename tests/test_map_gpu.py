"""GPU parity of the mapping step (forward with checkpoints, per-Gaussian
backward, 2D->3D chain rule, Adam) against the FP64 oracle.

Contract tolerance: Gaussian gradients within 1e-4 relative of the FP64
oracle (Frobenius norm over all Gaussians, per DeltaGaussian2D / 3D field
group).  The forward images share the tracking tolerance (1e-5).
"""
import numpy as np
import pytest

from conftest import make_frame, rel_err, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-4
ETA = 0.002

# DeltaGaussian2D field groups (columns of delta2d)
GROUPS_2D = {"meanImg": [0, 1], "invSigmaImg": [2, 3, 4], "color": [5, 6, 7], "depth": [8], "alpha": [9],
             "pHat": [10, 11]}
GROUPS_3D = {"position": [0, 1, 2], "scale": [3, 4, 5], "orientation": [6, 7, 8], "color": [9, 10, 11],
             "alpha": [12]}


def _run(oracle, fv, quirks, n=8000, scale=0.5, seed=21, bad_opacity=False):
    W, H, K = scaled_camera(scale)
    scene = S.cam_box(n, seed=seed)
    if bad_opacity:
        # every 20th Gaussian transparent, every 20th (offset) with a negative
        # opacity: neither may ever reach alpha 1/255
        scene.opacities[::20] = 0.0
        scene.opacities[7::20] = -0.3
    P = oracle.default_params(quirks)
    rng = np.random.default_rng(seed)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    rgb, d, gx, gy = make_frame(oracle, scene, true_pose, K, W, H, P)
    pose = (np.zeros(3), S.IDENTITY_Q)
    s = fv.Session(n, W, H, fv.default_params(quirks))
    s.set_debug(fv.DEBUG_MAPPING)
    s.upload(scene)
    s.set_frame(0, rgb, d, gx, gy)
    s.map_step(pose, K, ETA)
    g = s.download_map_state(W, H, deltas3d=True)
    params = s.download()
    s.close()
    b = oracle.prepare(scene, pose, K, W, H, P)
    o = oracle.map_step(scene, b, rgb, d, pose, K, W, H, P, ETA)
    return W, H, scene, g, params, o


@pytest.mark.parametrize("quirks,bad_opacity", [(0x4 | 0x8, False), (0x4, False), (0x4 | 0x8, True)])
def test_map_step_parity(oracle, fvgs_lib, quirks, bad_opacity):
    W, H, scene, g, params, o = _run(oracle, fvgs_lib, quirks, bad_opacity=bad_opacity)
    if bad_opacity:
        assert np.all(g["delta2d"][::20, 12] == 0) and np.all(g["delta2d"][7::20, 12] == 0)
    # forward images
    m = o.final_T.reshape(H, W)
    assert np.mean(g["n_contrib"] == o.n_contrib.reshape(H, W)) > 0.999
    err_c = np.abs(g["color"] - o.color.reshape(H, W, 3)) / np.maximum(np.abs(o.color.reshape(H, W, 3)), 1e-3)
    assert np.mean(err_c <= 1e-5) > 0.999
    assert np.mean(np.abs(g["final_T"] - m) <= 1e-5 * np.maximum(m, 1e-3)) > 0.999
    # gradients: Gaussians whose contribution count differs are threshold flips
    n_g = g["delta2d"][:, 12]
    n_o = o.delta2d[:, 12]
    same = n_g == n_o
    assert same.mean() > 0.99, same.mean()
    assert (n_o > 0).sum() > 100
    for name, cols in GROUPS_2D.items():
        e = rel_err(g["delta2d"][same][:, cols], o.delta2d[same][:, cols])
        print("delta2d", name, e)
        assert e <= GRAD_RTOL, (name, e)
    for name, cols in GROUPS_3D.items():
        e = rel_err(g["delta3d"][same][:, cols], o.delta3d[same][:, cols])
        print("delta3d", name, e)
        assert e <= GRAD_RTOL, (name, e)
    # Adam update: parameter changes agree to 1e-3 of the step size
    pos, scl, rot, col, opa = params
    upd = same & (n_o > 0)
    for name, gv, ov, base in (("pos", pos, o.pos, scene.positions), ("scale", scl, o.scl, scene.scales),
                               ("col", col, o.col, scene.colors)):
        dg = gv.astype(np.float64) - base
        do = ov - base
        bad = np.abs(dg - do).max(axis=1) > 1e-3 * ETA + 1e-6 * np.abs(base).max(axis=1)
        print("adam", name, bad[upd].mean())
        assert bad[upd].mean() < 0.01, name
    untouched = n_o == 0
    np.testing.assert_array_equal(pos[untouched & same], scene.positions[untouched & same])


@pytest.mark.parametrize("quirks", [0x4 | 0x8, 0x0], ids=["ref", "intended"])
def test_map_step_parity_vga_50k(oracle, fvgs_lib, quirks):
    """The small plain-method workload whole: N = 50k at 640 x 480."""
    W, H, scene, g, params, o = _run(oracle, fvgs_lib, quirks, n=50_000, scale=1.0, seed=23)
    n_g = g["delta2d"][:, 12]
    n_o = o.delta2d[:, 12]
    same = n_g == n_o
    assert same.mean() > 0.99, same.mean()
    assert (n_o > 0).sum() > 10_000
    err_c = np.abs(g["color"] - o.color.reshape(H, W, 3)) / np.maximum(np.abs(o.color.reshape(H, W, 3)), 1e-3)
    assert np.mean(err_c <= 1e-5) > 0.999
    for name, cols in GROUPS_2D.items():
        e = rel_err(g["delta2d"][same][:, cols], o.delta2d[same][:, cols])
        print("delta2d", name, e)
        assert e <= GRAD_RTOL, (name, e)
    for name, cols in GROUPS_3D.items():
        e = rel_err(g["delta3d"][same][:, cols], o.delta3d[same][:, cols])
        print("delta3d", name, e)
        assert e <= GRAD_RTOL, (name, e)
