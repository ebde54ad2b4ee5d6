"""The CUDA library's binning pinned to the reference's own GPU code: the
reference's binning kernels compiled by nvcc with the reference's flags
(oracle/ref_gpu.cu, built by oracle/ref_build.py) and launched as
GSSlam::prepareRasterization launches them, against the library and the
CPU restatement on the same inputs, at the small plain-method workload
(N = 50k, 640 x 480, culled Gaussians included) and on a 1280 x 720 room.

Bit for bit: screen means, depths, p-hat, tile counts, keys, sorted indices
and ranges.  The 2D covariance and its inverse are sums of 9 and 27 products
in the reference's source; which of them nvcc fuses into FMAs under its
default contraction is the compiler's choice, not the source's, so they are
held to 1e-5 relative (measured: a few ulps), and the tile rectangles they
feed must still give identical counts, keys and ranges.  On the CPU
(tests/test_ref_pin.py) the reference's source evaluated with one rounding
per operation equals the restatement's no-FMA build in every field."""
import numpy as np
import pytest

from f_vigs_slam_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
refbin = pytest.importorskip("refbin")

VGA = (525.0, 525.0, 319.5, 239.5)


def _cases():
    sc = S.cam_box(50_000, seed=0)
    sc.positions[:2000, 2] *= -1.0
    sc.positions[2000:4000, 0] += 40.0
    yield "vga_50k_identity", sc, (np.zeros(3, np.float32), S.IDENTITY_Q), VGA, 640, 480
    yield "vga_50k_perturbed", sc, S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, np.random.default_rng(1)), VGA, 640, 480
    room = S.room(300_000, seed=4)
    yield "room_300k_hd", room, S.trajectory(2, seed=9)[1], S.CAM_HD.intrinsics, 1280, 720


@pytest.mark.parametrize("range_mode", [0, 1], ids=["reference_range_launch", "range_per_instance"])
def test_gpu_reference_equals_library_and_restatement(oracle, fvgs_lib, range_mode):
    if not refbin.available("gpu"):
        pytest.skip("no extracted reference kernels in oracle/_ref (built where the reference's sources are)")
    fv = fvgs_lib
    q = oracle.Q_CULLED_SLOTS | (oracle.Q_RANGE_LAUNCH if range_mode == 0 else 0)
    for name, sc, pose, K, W, H in _cases():
        r = refbin.binning("gpu", sc, pose, K, W, H, range_mode=range_mode)
        b = oracle.prepare(sc, pose, K, W, H, oracle.default_params(q))
        with fv.Session(sc.n, W, H, fv.default_params(q)) as s:
            s.set_debug(fv.DEBUG_PROJECTION)
            s.upload(sc)
            n = s.project_bin(pose, K, W, H)
            proj = s.download_projection()
            keys, vals, ranges = s.download_binning(W, H)
        vis = r["counts"] > 0
        mism, rel = {}, {}
        for f, a, g, o in (("uv", r["uv"], proj["uv"], b.proj.uv), ("cov2d", r["cov2d"], proj["cov2d"], b.proj.cov2d),
                           ("inv2d", r["inv2d"], proj["inv2d"], b.proj.inv2d),
                           ("depth", r["depth"], proj["depth"], b.proj.depth),
                           ("phat", r["phat"], proj["phat"], b.proj.phat)):
            mism[f] = (int(np.sum(a.view(np.uint32) != g.view(np.uint32))),
                       int(np.sum(a.view(np.uint32) != o.view(np.uint32))))
            av, gv = a[vis].astype(np.float64), g[vis].astype(np.float64)
            scale = np.maximum(np.abs(av).max(axis=-1, keepdims=True) if av.ndim > 1 else np.abs(av), 1e-30)
            rel[f] = float(np.max(np.abs(av - gv) / scale)) if av.size else 0.0
        print(name, "projection fields differing (library, restatement):", mism, "max relative:", rel)
        for f in ("uv", "depth", "phat"):
            assert mism[f] == (0, 0), (name, f, mism)
        assert rel["cov2d"] <= 1e-5 and rel["inv2d"] <= 1e-5, (name, rel)
        # the library and the restatement agree with each other bit for bit
        np.testing.assert_array_equal(proj["cov2d"].view(np.uint32), b.proj.cov2d.view(np.uint32))
        np.testing.assert_array_equal(proj["inv2d"].view(np.uint32), b.proj.inv2d.view(np.uint32))
        np.testing.assert_array_equal(r["counts"], proj["counts"])
        assert r["n"] == n == b.keys.shape[0], name
        np.testing.assert_array_equal(r["keys"], keys)
        np.testing.assert_array_equal(r["vals"], vals)
        np.testing.assert_array_equal(r["ranges"], ranges)
        np.testing.assert_array_equal(r["keys"], b.keys)
        np.testing.assert_array_equal(r["ranges"], b.ranges)
