"""The CPU restatement pinned to the reference's own source: the reference's
binning kernels (src/GSCudaKernels.cu: projectGaussiansWorldToScreen_kernel,
countTilesPerGaussian_kernel, generateTileHashes_kernel,
computeIndicesRanges_kernel, perTileBucketCount; built by
oracle/ref_build.py into oracle/_ref/ and run thread by thread on the CPU by
oracle/ref_host.cpp) against the restatement built the same way (floating-
point contraction off): every projection output, tile count, key, value,
range and bucket count bit for bit, on the small plain-method workload
(N = 50k, 640 x 480) with culled Gaussians, and with both the reference's
range launch and one thread per instance."""
import numpy as np
import pytest

from f_vigs_slam_gb300 import synthetic as S

refbin = pytest.importorskip("refbin")

VGA = (525.0, 525.0, 319.5, 239.5)


def _scene():
    sc = S.cam_box(50_000, seed=0)
    sc.positions[:2000, 2] *= -1.0       # behind the camera
    sc.positions[2000:4000, 0] += 40.0   # outside the view
    return sc


def _compare(r, b, oracle):
    for name, a, o in (("uv", r["uv"], b.proj.uv), ("cov2d", r["cov2d"], b.proj.cov2d),
                       ("inv2d", r["inv2d"], b.proj.inv2d), ("depth", r["depth"], b.proj.depth),
                       ("phat", r["phat"], b.proj.phat)):
        np.testing.assert_array_equal(a.view(np.uint32), o.view(np.uint32), err_msg=name)
    np.testing.assert_array_equal(r["counts"], b.cnt)
    assert r["n"] == b.keys.shape[0]
    np.testing.assert_array_equal(r["keys"], b.keys)
    np.testing.assert_array_equal(r["vals"], b.vals)
    np.testing.assert_array_equal(r["ranges"], b.ranges)
    incl = np.zeros(r["ranges"].shape[0], np.uint32)
    oracle.lib().oracle_buckets(oracle._p(np.ascontiguousarray(b.ranges)), oracle.C.c_int(incl.shape[0]),
                                oracle._p(incl))
    np.testing.assert_array_equal(np.diff(np.concatenate([[0], incl.astype(np.int64)])), r["buckets"])


@pytest.mark.parametrize("range_mode", [0, 1], ids=["reference_range_launch", "range_per_instance"])
@pytest.mark.parametrize("perturbed", [False, True], ids=["identity", "perturbed"])
def test_host_reference_equals_restatement(oracle, range_mode, perturbed):
    if not refbin.available("host"):
        pytest.skip("the reference's sources are not here and oracle/_ref holds no extracted kernels")
    sc = _scene()
    pose = (np.zeros(3, np.float32), S.IDENTITY_Q)
    if perturbed:
        pose = S.perturb(pose, 1.0, 2.0, np.random.default_rng(1))
    r = refbin.binning("host", sc, pose, VGA, 640, 480, range_mode=range_mode)
    q = oracle.Q_CULLED_SLOTS | (oracle.Q_RANGE_LAUNCH if range_mode == 0 else 0)
    b = oracle.prepare(sc, pose, VGA, 640, 480, oracle.default_params(q), nofma=True)
    _compare(r, b, oracle)
    assert r["n"] > 700_000
