"""The render-form image (fvgs_render_view) and GPU frame preprocessing
(fvgs_preprocess_frame) against the CPU restatement.

Render form: colour within 1e-5 relative (per image, Frobenius); depth within
1e-5 relative to max(|d|, 1 m) where both sides found the 0.5 crossing, the
1e10 "no crossing" value where the GPU found none, and the crossing decided
alike for all but 1e-4 of the pixels (FP32 and FP64 may decide it on either
side where the accumulated alpha lands within rounding of 0.5).  Preprocessing: every level's
colour, depth and gradients bit for bit (integer pyramid, explicitly rounded
FP32 everywhere else).
"""
import numpy as np
import pytest

from conftest import rel_err, scaled_camera
from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("quirks", [0x4 | 0x8, 0x8])
def test_render_view_matches_oracle(oracle, fvgs_lib, quirks):
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(20_000, seed=21)
    P = oracle.default_params(quirks)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(3))
    b = oracle.prepare(scene, pose, K, W, H, P)
    col_o, dep_o = oracle.render_view(scene, b, W, H, P)
    with fv.Session(scene.n, W, H, fv.default_params(quirks)) as s:
        s.upload(scene)
        col, dep, c8 = s.render_view(pose, K, W, H, rgb8=True)
    assert rel_err(col, col_o) <= 1e-5
    crossed_o = dep_o < 1e9
    crossed = dep < 1e9
    assert crossed_o.mean() > 0.3
    # the 0.5 crossing is decided the same way except where the accumulated
    # alpha lands within rounding of 0.5 (FP32 here, FP64 in the oracle)
    assert (crossed != crossed_o).mean() <= 1e-4
    both = crossed & crossed_o
    assert np.all(dep[~crossed] == np.float32(1e10))
    d = np.abs(dep[both] - dep_o[both]) / np.maximum(np.abs(dep_o[both]), 1.0)
    assert np.quantile(d, 0.999) <= 1e-5
    expect8 = np.clip(np.rint(np.clip(col, 0.0, 1.0) * 255.0), 0, 255).astype(np.uint8)
    assert np.abs(c8.astype(int) - expect8.astype(int)).max() <= 1


def test_render_view_signed_opacities(oracle, fvgs_lib):
    """Zero and negative opacities (outside the sigmoid's range, but valid
    input): the render form blends their weights o exp(-q/2) with the sign,
    as the reference's kernel does; same tolerances."""
    fv = fvgs_lib
    W, H, K = scaled_camera(0.5)
    scene = S.cam_box(20_000, seed=22)
    rng = np.random.default_rng(4)
    o = scene.opacities.copy()
    pick = rng.random(o.size)
    o[pick < 0.05] *= -0.2
    o[(pick >= 0.05) & (pick < 0.08)] = 0.0
    scene = S.Scene(scene.positions, scene.scales, scene.orientations, scene.colors, o.astype(np.float32))
    P = oracle.default_params(0x8)
    pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(3))
    b = oracle.prepare(scene, pose, K, W, H, P)
    col_o, dep_o = oracle.render_view(scene, b, W, H, P)
    with fv.Session(scene.n, W, H, fv.default_params(0x8)) as s:
        s.upload(scene)
        col, dep = s.render_view(pose, K, W, H)
    assert rel_err(col, col_o) <= 1e-5
    crossed_o, crossed = dep_o < 1e9, dep < 1e9
    assert (crossed != crossed_o).mean() <= 1e-4
    both = crossed & crossed_o
    d = np.abs(dep[both] - dep_o[both]) / np.maximum(np.abs(dep_o[both]), 1.0)
    assert np.quantile(d, 0.999) <= 1e-5


@pytest.mark.parametrize("depth_mm,double_scale,H,W", [(False, False, 123, 171), (True, False, 123, 171),
                                                     (False, True, 123, 171), (True, False, 9, 70),
                                                     (False, False, 3, 2)])
def test_preprocess_matches_oracle(oracle, fvgs_lib, depth_mm, double_scale, H, W):
    """Odd sizes exercise the reflect-101 borders and the (n+1)/2 levels; 9 x 70
    gives levels narrower than one 32 x 8 block row and partial blocks, 3 x 2
    levels of 2 x 1 and 1 x 1 pixels."""
    fv = fvgs_lib
    rng = np.random.default_rng(7)
    color = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    if depth_mm:
        depth = rng.integers(0, 8000, (H, W), dtype=np.uint16)
    else:
        depth = rng.uniform(0.1, 8.0, (H, W)).astype(np.float32)
    want = oracle.preprocess(color, depth, levels=3, depth_mm=depth_mm, double_scale=double_scale)
    with fv.Session(1000, W, H) as s:
        s.preprocess_frame(color, depth, levels=3, double_scale=double_scale)
        for lv in range(3):
            got = s.download_frame(lv)
            for name, g, w in zip(("rgb", "depth", "gx", "gy"), got, want[lv]):
                assert g.shape == w.shape, (lv, name)
                np.testing.assert_array_equal(g, w, err_msg="level %d %s" % (lv, name))


@pytest.mark.parametrize("where", ["host", "device"])
def test_packed_frames_equal_per_level(oracle, fvgs_lib, where):
    """fvgs_set_frames_packed (one buffer, pack_pyramid's layout; from host
    memory one copy to the device) sets every level exactly as fvgs_set_frame
    per level does."""
    import torch

    fv = fvgs_lib
    rng = np.random.default_rng(8)
    H, W = 123, 171
    color = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    depth = rng.uniform(0.1, 8.0, (H, W)).astype(np.float32)
    levels = oracle.preprocess(color, depth, levels=3, depth_mm=False, double_scale=False)
    packed = fv.pack_pyramid(levels)
    with fv.Session(1000, W, H) as s:
        if where == "host":
            s.set_frames_packed(packed, 3, W, H)
        else:
            dev = torch.from_numpy(packed).to("cuda:0")
            torch.cuda.synchronize()
            s.set_frames_packed(dev.data_ptr(), 3, W, H)
        for lv in range(3):
            got = s.download_frame(lv)
            for name, g, w in zip(("rgb", "depth", "gx", "gy"), got, levels[lv]):
                assert g.shape == w.shape, (lv, name)
                np.testing.assert_array_equal(g, w, err_msg="level %d %s" % (lv, name))


def test_session_stream_follows_set_stream(fvgs_lib):
    """fvgs_session_stream returns the stream set by fvgs_session_set_stream,
    and the session's own (non-null) stream after a reset to NULL."""
    import torch

    fv = fvgs_lib
    with fv.Session(1000, 64, 48) as s:
        own, dev = s.stream()
        assert own != 0 and dev == 0
        st = torch.cuda.Stream(device="cuda:0")
        s.set_stream(st.cuda_stream)
        assert s.stream() == (st.cuda_stream, 0)
        s.set_stream(None)
        assert s.stream() == (own, 0)
