"""Known-answer tests pinning the CPU restatement to the reference source.

The reference ships no tests or golden data, so these values are derived by
hand from its code (file:line cited per test) and checked against the oracle.
"""
import struct

import numpy as np
import pytest

from f_vigs_slam_gb300 import synthetic as S

VGA = (525.0, 525.0, 319.5, 239.5)


def f32bits(x):
    return struct.unpack("<I", struct.pack("<f", np.float32(x)))[0]


def one(pos, scale, q=(0, 0, 0, 1), col=(0.2, 0.4, 0.6), opa=0.5):
    return S.Scene(np.array([pos], np.float32), np.array([scale], np.float32), np.array([q], np.float32),
                   np.array([col], np.float32), np.array([opa], np.float32))


IDENT = (np.zeros(3), S.IDENTITY_Q)


def test_projection_single_gaussian(oracle):
    """projectGaussiansWorldToScreen_kernel (src/GSCudaKernels.cu:345-476) at the
    identity pose: p_cam = p, u = fx x/z + cx, Sigma2D = J diag(s^2) J^T with
    J = [[fx/z, 0, -fx x/z^2], [0, fy/z, -fy y/z^2]], p_hat = (x/z^2, y/z^2)."""
    sc = one((0.5, -0.25, 2.0), (0.1, 0.05, 0.02))
    p = oracle.project(sc, IDENT, VGA, 640, 480)
    assert p.visible[0] == 1
    np.testing.assert_allclose(p.uv[0], [450.75, 173.875], rtol=1e-7)
    assert p.depth[0] == 2.0
    j00, j02, j11, j12 = 262.5, -65.625, 262.5, 32.8125
    sxx = j00 ** 2 * 0.01 + j02 ** 2 * 0.0004
    syy = j11 ** 2 * 0.0025 + j12 ** 2 * 0.0004
    sxy = j02 * j12 * 0.0004
    np.testing.assert_allclose(p.cov2d[0], [sxx, syy, sxy], rtol=1e-6)
    det = sxx * syy - sxy * sxy
    # inverse stored (xx, yy, xy) (src/GSCudaKernels.cu:469)
    np.testing.assert_allclose(p.inv2d[0], [syy / det, sxx / det, -sxy / det], rtol=1e-5)
    np.testing.assert_allclose(p.phat[0], [0.125, -0.0625], rtol=1e-7)


def test_culling(oracle):
    """Culled when z <= 0 (:381) or u/v outside [0,W)x[0,H) (:391)."""
    sc = S.Scene(np.array([[0, 0, -1], [10, 0, 1], [0, 0, 1]], np.float32), np.full((3, 3), 0.1, np.float32),
                 np.tile(S.IDENTITY_Q, (3, 1)), np.zeros((3, 3), np.float32), np.full(3, 0.5, np.float32))
    p = oracle.project(sc, IDENT, VGA, 640, 480)
    assert list(p.visible) == [0, 0, 1]


def test_tile_count_and_keys(oracle):
    """countTilesPerGaussian_kernel (:549-593) and generateTileHashes_kernel
    (:596-667): 3-sigma box from sqrt of the diagonal, tiles of 16, key =
    tile << 32 | bits(z + phx*dx + phy*dy) at the tile centre (t+0.5)*16."""
    sc = one((0.5, -0.25, 2.0), (0.1, 0.05, 0.02))
    P = oracle.default_params()
    b = oracle.prepare(sc, IDENT, VGA, 640, 480, P)
    # sigma_x = 26.28 px -> [371.9, 529.6] -> tiles 23..33; sigma_y = 13.14 -> [134.4, 213.3] -> 8..13
    assert list(b.rect[0]) == [23, 8, 33, 13]
    assert b.cnt[0] == 11 * 6
    # first key (row-major loop): tile (23, 8); dx = 376 - 450.75, dy = 136 - 173.875
    d = 2.0 + 0.125 * (376 - 450.75) + (-0.0625) * (136 - 173.875)
    assert d == -4.9765625  # exact in binary
    assert int(b.keys_gen[0]) == (8 * 40 + 23) << 32 | f32bits(d)
    # negative depths have the sign bit set and sort after every positive one
    assert np.all(np.diff(b.keys.astype(np.uint64)) >= 0)


def test_stable_sort_ties_keep_generation_order(oracle):
    """thrust::sort_by_key is a stable radix sort (src/GSSlam.cu:624-628):
    identical keys keep Gaussian-index order."""
    sc = S.Scene(np.array([[0.0, 0.0, 2.0]] * 3, np.float32), np.full((3, 3), 0.01, np.float32),
                 np.tile(S.IDENTITY_Q, (3, 1)), np.zeros((3, 3), np.float32), np.full(3, 0.5, np.float32))
    b = oracle.prepare(sc, IDENT, VGA, 640, 480, oracle.default_params())
    for t in range(b.ranges.shape[0]):
        s, e = b.ranges[t]
        if e > s:
            assert list(b.vals[s:e]) == sorted(b.vals[s:e])


def test_straddling_four_tiles(oracle):
    """A small Gaussian centred on a tile corner covers 4 tiles whose keys use
    the four tile centres (+-8 px from the centre)."""
    # u = v = 16 exactly: fx=fy=16, cx=cy=0, x/z = y/z = 1
    K = (16.0, 16.0, 0.0, 0.0)
    sc = one((2.0, 2.0, 2.0), (0.05, 0.05, 0.05))
    b = oracle.prepare(sc, IDENT, K, 64, 64, oracle.default_params())
    assert b.cnt[0] == 4
    tiles = sorted(int(k >> 32) for k in b.keys_gen)
    assert tiles == [0, 1, 4, 5]
    ph = b.proj.phat[0]
    for k in b.keys_gen:
        t = int(k >> 32)
        tx, ty = t % 4, t // 4
        d = np.float32(np.float32(2.0) + np.float32(ph[0]) * np.float32((tx + 0.5) * 16 - 16)
                       + np.float32(ph[1]) * np.float32((ty + 0.5) * 16 - 16))
        assert abs(float(np.frombuffer(np.uint32(int(k) & 0xffffffff).tobytes(), np.float32)[0]) - float(d)) < 1e-6


def test_range_launch_quirk(oracle):
    """computeIndicesRanges_kernel launched with ceil(T/256)*256 threads over
    instances (src/GSSlam.cu:633-640): only the first 256*ceil(T/256)
    instances set boundaries; instance 0 returns without closing its tile."""
    keys = np.array([(t << 32) for t in [0, 0, 1, 1, 1, 3]], np.uint64)
    vals = np.arange(6, dtype=np.uint32)
    P = oracle.default_params(oracle.Q_RANGE_LAUNCH)
    _, _, r = oracle.sort_ranges(keys, vals, 64, 16, P)  # 4 tiles -> 256 threads cover all 6
    assert r.tolist() == [[0, 2], [2, 5], [0, 0], [5, 6]]
    # a single instance: the thread 0 early return leaves the end at 0
    _, _, r1 = oracle.sort_ranges(keys[:1], vals[:1], 64, 16, P)
    assert r1.tolist()[0] == [0, 0]
    P0 = oracle.default_params(0)
    _, _, r2 = oracle.sort_ranges(keys[:1], vals[:1], 64, 16, P0)
    assert r2.tolist()[0] == [0, 1]


def test_culled_slot_quirk(oracle):
    """With the reference's culled slots a Gaussian behind the camera keeps a
    zero record: one instance in tile 0 with key 0 (sorts first there)."""
    sc = S.Scene(np.array([[0, 0, -1], [0.1, 0.1, 2]], np.float32), np.full((2, 3), 0.01, np.float32),
                 np.tile(S.IDENTITY_Q, (2, 1)), np.zeros((2, 3), np.float32), np.full(2, 0.5, np.float32))
    b = oracle.prepare(sc, IDENT, VGA, 640, 480, oracle.default_params(oracle.Q_CULLED_SLOTS | oracle.Q_INVSIGMA_SWAP))
    assert b.cnt[0] == 1 and int(b.keys_gen[0]) == 0
    b2 = oracle.prepare(sc, IDENT, VGA, 640, 480, oracle.default_params())
    assert b2.cnt[0] == 0


def test_center_pixel_skip_and_neighbour(oracle):
    """Forward blend (src/GSCudaKernels.cu:979-1041): v <= 0 is skipped, so a
    Gaussian centred exactly on a pixel leaves that pixel at the background;
    the neighbour gets alpha = min(0.99, o exp(-v/2)) with v from the
    consumed inverse covariance, colour = rgb alpha (background black)."""
    K = (100.0, 100.0, 0.0, 0.0)
    sc = one((2.0, 1.0, 2.0), (0.05, 0.05, 0.05), col=(0.3, 0.6, 0.9), opa=0.8)  # u = 100, v = 50
    P = oracle.default_params()
    b = oracle.prepare(sc, IDENT, K, 160, 96, P)
    assert tuple(b.proj.uv[0]) == (100.0, 50.0)
    col, dep, T, nc = oracle.render(b, IDENT, K, 160, 96, P)
    assert np.all(col[50, 100] == 0.0) and T[50, 100] == 1.0
    r = b.rec[0]
    dx = 100.0 - 101.0
    v = np.float64(r[4]) * dx * dx
    a = min(np.float64(np.float32(0.99)), np.float64(np.float32(0.8)) * np.exp(-0.5 * v))
    np.testing.assert_allclose(col[50, 101], np.array([0.3, 0.6, 0.9], np.float32).astype(np.float64) * a,
                               rtol=1e-12)
    np.testing.assert_allclose(T[50, 101], 1 - a, rtol=1e-12)


def test_empty_tile(oracle):
    """An empty tile has range (0,0) and renders the background, T = 1."""
    sc = one((0.5, 0.5, 2.0), (0.01, 0.01, 0.01))
    P = oracle.default_params()
    b = oracle.prepare(sc, IDENT, VGA, 640, 480, P)
    assert b.ranges[0].tolist() == [0, 0]
    col, dep, T, nc = oracle.render(b, IDENT, VGA, 640, 480, P)
    assert np.all(col[:16, :16] == 0) and np.all(T[:16, :16] == 1.0) and np.all(nc[:16, :16] == 0)


def test_self_rendered_target_has_zero_jtr(oracle):
    """Observed frame = exact render at the same pose: colour and depth
    residuals vanish, so Jtr = 0 exactly while JtJ is positive semi-definite."""
    W, H, K = 160, 120, (131.25, 131.25, 79.875, 59.875)
    sc = S.cam_box(2000, seed=5)
    P = oracle.default_params()
    b = oracle.prepare(sc, IDENT, K, W, H, P)
    col, dep, _, _ = oracle.render(b, IDENT, K, W, H, P)
    rgb, d = col.astype(np.float32), dep.astype(np.float32)
    # exact float copies of the render: residuals are the float rounding only
    gx, gy = S.sobel3(rgb)
    r = oracle.track(b, (rgb, d, gx, gy), IDENT, K, W, H, P, images=False)
    assert np.linalg.norm(r.Jtr) <= 1e-5 * np.sqrt(np.abs(np.diag(r.JtJ)).max())
    assert np.linalg.eigvalsh(r.JtJ).min() >= -1e-9 * np.abs(r.JtJ).max()


def test_pseudo_factor(oracle):
    """RgbdPoseCostFunction (src/RgbdPoseCost.cu:57-78): J*^T J* = JtJ with
    eigenvalues <= eps dropped, and J*^T r* = the projection of Jtr."""
    rng = np.random.default_rng(0)
    A = rng.normal(size=(6, 6))
    H = A @ A.T
    w, U = np.linalg.eigh(H)
    w[0] = 1e-6  # below eps
    H = (U * w) @ U.T
    g = rng.normal(size=6)
    r, J = oracle.pseudo_factor(H, g, 1e-4)
    keep = w > 1e-4
    Hk = (U[:, keep] * w[keep]) @ U[:, keep].T
    np.testing.assert_allclose(J.T @ J, Hk, atol=1e-9)
    np.testing.assert_allclose(J.T @ r, U[:, keep] @ (U[:, keep].T @ g), atol=1e-9)
    d = oracle.gn_delta(H, g, 1e-4)
    np.testing.assert_allclose(d, -(U[:, keep] / w[keep]) @ (U[:, keep].T @ g), atol=1e-9)


def test_pose_plus():
    """PoseLocalParameterization::Plus (src/PoseLocalParameterization.cpp:22-44):
    p += dp; q = normalise(q (x) [dtheta/2, 1])."""
    import oracle as O

    t, q = O.pose_plus((np.zeros(3), np.array([0, 0, 0, 1.0])), np.array([1, 2, 3, 0.2, 0, 0]))
    assert list(t) == [1, 2, 3]
    np.testing.assert_allclose(q, np.array([0.1, 0, 0, 1]) / np.sqrt(1.01))


def test_adam_first_step(oracle):
    """updateGaussiansParametersAdam_kernel (src/GSCudaKernels.cu:2779-2882):
    the first step moves a parameter by eta * g / sqrt(g^2 + eps) (bias-corrected
    moments equal g and g^2); n == 0 leaves it untouched."""
    import ctypes as C

    L = oracle.lib()
    n = 2
    pos = np.zeros((n, 3))
    scl = np.full((n, 3), 0.1)
    rot = np.tile([0, 0, 0, 1.0], (n, 1))
    col = np.full((n, 3), 0.5)
    opa = np.full(n, 0.5)
    adam = np.zeros((n, 27))
    d3 = np.zeros((n, 14))
    d3[0, 0:3] = [0.3, -0.2, 1e-3]
    d3[0, 13] = 5
    P = oracle.default_params()
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    L.oracle_adam(p(pos), p(scl), p(rot), p(col), p(opa), p(adam), p(d3), C.c_int(n), C.c_float(0.002), C.byref(P))
    g = d3[0, 0:3]
    np.testing.assert_allclose(pos[0], 0.002 * g / np.sqrt(g * g + np.float64(np.float32(1e-8))), rtol=1e-6)
    assert np.all(pos[1] == 0) and adam[1, 26] == 0 and adam[0, 26] == 1


def test_kat_pyrdown_impulse(oracle):
    """cv::pyrDown of a 5x5 impulse at (2, 2): weights [1 4 6 4 1]/16 per
    axis with reflect-101 borders give the centre 6/16 and each border
    output 1/16 + 1/16 (the impulse is reached from both sides), so the 3x3
    result is 255 * (2, 6, 2)^T (2, 6, 2) / 256, rounded: (4, 12, 4),
    (12, 36, 12), (4, 12, 4)."""
    import numpy as np

    img = np.zeros((5, 5), np.uint8)
    img[2, 2] = 255
    out = oracle.pyrdown(img)
    np.testing.assert_array_equal(out, np.array([[4, 12, 4], [12, 36, 12], [4, 12, 4]], np.uint8))
    outf = oracle.pyrdown(img.astype(np.float32))
    np.testing.assert_allclose(outf, np.outer([2, 6, 2], [2, 6, 2]) * 255.0 / 256.0, rtol=1e-6)


def test_kat_render_view_single_gaussian(oracle):
    """forwardPassTileKernel with one Gaussian of opacity 0.5 centred on pixel
    (3, 2), inverse covariance diag(1, 1), colour (1, 0, 0), depth 2, zero
    phat: that pixel gets colour 0.5 and, as 1 - A falls from 1 to 0.5
    (crossing 0.5), depth 2; its neighbour (4, 2) gets 0.5 exp(-1/2) and no
    crossing (depth 1e10)."""
    import ctypes as C

    import numpy as np

    W, H = 8, 4
    uv = np.array([[3.0, 2.0]], np.float32)
    inv2d = np.array([[1.0, 1.0, 0.0]], np.float32)  # (xx, yy, xy)
    depth = np.array([2.0], np.float32)
    phat = np.zeros((1, 2), np.float32)
    col = np.array([[1.0, 0.0, 0.0]], np.float32)
    opa = np.array([0.5], np.float32)
    ranges = np.array([0, 1], np.uint32)  # one 16x16 tile
    vals = np.array([0], np.uint32)
    out_c = np.zeros((H, W, 3), np.float64)
    out_d = np.zeros((H, W), np.float64)
    p = lambda a: C.c_void_p(a.ctypes.data)
    oracle.lib().oracle_render_view(p(uv), p(inv2d), p(depth), p(phat), p(col), p(opa), p(ranges), p(vals),
                                    C.c_int(W), C.c_int(H), C.c_int(16), C.c_int(16), p(out_c), p(out_d))
    assert abs(out_c[2, 3, 0] - 0.5) < 1e-15 and out_d[2, 3] == 2.0
    assert abs(out_c[2, 4, 0] - 0.5 * np.exp(-0.5)) < 1e-15 and out_d[2, 4] == 1e10


class _Bin:
    """A hand-made binned view: records rec[12N], one tile list."""

    def __init__(self, rec, order):
        self.rec = np.ascontiguousarray(rec, np.float32)
        self.vals = np.asarray(order, np.uint32)
        self.ranges = np.array([[0, len(order)]], np.uint32)


def _rec(u, v, z, opa, c=(1.0, 0.0, 1.0), phat=(0.0, 0.0)):
    return [u, v, z, opa, c[0], c[1], c[2], phat[0], phat[1], 0.5, 0.5, 0.5]


def test_kat_visibility(oracle):
    """computeGaussiansVisibility_kernel (src/GSCudaKernels.cu:1455-1537), one
    tile of 8x4 pixels: g0 (opacity 0.6 on pixel (1,1)) is seen and stops that
    pixel (T = 0.4 < 0.5); g1 (0.9, same place, behind g0) is seen from pixel
    (2,1), where g0 leaves T = 1 - 0.6 e^-1/2; g2 is far outside the image;
    g3 (opacity 0.003) never reaches alpha 1/255.  With a cap of one Gaussian
    per tile only g0 is considered."""
    b = _Bin([_rec(1, 1, 1, 0.6), _rec(1, 1, 2, 0.9), _rec(100, 100, 1, 0.9), _rec(5, 2, 1, 0.003)],
             [0, 1, 2, 3])
    P = oracle.default_params()
    np.testing.assert_array_equal(oracle.visibility(b, 8, 4, P, cap=0), [1, 1, 0, 0])
    np.testing.assert_array_equal(oracle.visibility(b, 8, 4, P, cap=1), [1, 0, 0, 0])
    # seen only through pixel (1,1): g1 first in the list hides g0 there, but
    # g0 still reaches alpha >= 1/255 on other pixels
    np.testing.assert_array_equal(oracle.visibility(_Bin(b.rec, [1, 0]), 8, 4, P, cap=0), [1, 1, 0, 0])


def test_kat_outlier_scores_and_states(oracle):
    """computeOutliers_kernel / removeOutliers_kernel (src/GSCudaKernels.cu:
    1620-1739): one Gaussian of opacity 0.5 at pixel (3,2), unit inverse
    covariance, depth 2, zero phat, over an 8x4 image whose observed depth is
    3 for x < 4 (rendered 2 < 0.8 * 3: outlier evidence) and 2 elsewhere;
    a second Gaussian at depth -1 never counts (rendered depth <= 0)."""
    W, H = 8, 4
    b = _Bin([_rec(3, 2, 2, 0.5), _rec(3, 2, -1, 0.5)], [0, 1])
    obs = np.full((H, W), 2.0, np.float32)
    obs[:, :4] = 3.0
    ta, op = oracle.outlier_scores(b, obs, W, H, oracle.default_params())
    want_t = want_o = 0.0
    for y in range(H):
        for x in range(W):
            a = float(np.float32(0.5 * np.exp(-0.5 * ((x - 3) ** 2 + (y - 2) ** 2))))
            if a < 1 / 255:
                continue
            want_t += a
            want_o += a if x < 4 else 0.0
    assert ta[0] == want_t and op[0] == want_o and ta[1] == 0.0 and op[1] == 0.0
    share = want_o / want_t
    assert want_t > 1.0 and 0.65 < share < 0.75
    np.testing.assert_array_equal(oracle.outlier_states(ta, op, 0.6), [0xff, 0])
    np.testing.assert_array_equal(oracle.outlier_states(ta, op, 0.75), [0, 0])
    # FP32 edges: a share of exactly 0.6f is not above 0.6f; an infinite
    # total gives a share of 0 (or NaN): kept; a total of at most 1: kept
    ta2 = np.array([0.5, 2.0, 2.0, 2.0, np.inf, np.inf])
    op2 = np.array([0.5, 1.3, 1.1, 1.2, 1.0, np.inf])
    np.testing.assert_array_equal(oracle.outlier_states(ta2, op2, 0.6), [0, 0xff, 0, 0, 0, 0])


def test_kat_prune_states(oracle):
    """pruneGaussians_kernel (src/GSCudaKernels.cu:1566-1618) with the
    reference's thresholds 0.05 / 0.05 / 0.005."""
    scales = np.array([[0.1, 0.1, 0.1], [0.1, 0.1, 0.1], [0.1, 0.1, 0.1], [0.1, 0.004, 0.1],
                       [0.1, 0.004, 0.0001], [0.004, 0.004, 0.004], [0.0049, 0.0049, 0.006]], np.float32)
    opac = np.array([0.5, 0.04, 0.05, 0.5, 0.5, 0.5, 0.5], np.float32)
    sc = S.Scene(np.zeros((7, 3), np.float32), scales, np.tile(S.IDENTITY_Q, (7, 1)),
                 np.zeros((7, 3), np.float32), opac)
    #        keep, transparent, at threshold, flat but wide, needle, tiny, max >= 0.005
    want = [0, 0xff, 0, 0, 0xff, 0xff, 0]
    np.testing.assert_array_equal(oracle.prune_states(sc), want)


def test_kat_compaction_order_and_covisibility(oracle):
    """thrust::sort_by_key on 0 / 0xff states (src/GSSlam.cu:1536-1548) keeps
    the survivors in order, then the removed ones; computeCovisibilityRatio
    (src/GSSlam.cu:1713-1904) divides |a and b| by |a or b|."""
    np.testing.assert_array_equal(oracle.compact_order([0, 0xff, 0, 0xff, 0]), [0, 2, 4, 1, 3])
    assert oracle.covisibility([1, 1, 0, 1, 0], [0, 1, 1, 1, 0]) == (2, 4, np.float32(0.5))
    assert oracle.covisibility([0, 0], [0, 0]) == (0, 0, np.float32(0.0))


def test_backward_colour_terms_are_loss_gradients(oracle):
    """optimizeGaussiansPerGaussianPass (src/GSCudaKernels.cu:2265-2502), colour
    part (depth and distortion weights 0), in the intended semantics (quirks
    off: consumed conic = true inverse covariance, no 256 cap): with
    L = 0.5 sum_p |C_p - obs_p|^2 and C the forward blend, the per-Gaussian 2D
    accumulations are
      dmx, dmy = -dL/du, -dL/dv;  dix, diz = -dL/da, -dL/dc and
      diy = -dL/db / 2 for the consumed conic (a, b, c);
      dcr, dcg, dcb = -dL/d colour;  dal = +o dL/do (the opposite sign)
    checked against central differences of the oracle's FP64 forward blend on
    the same tile lists (records perturbed in place).  With the reference's
    conic-layout quirk the quadratic form can be indefinite and alpha clamped
    at 0.99, where the backward (which ignores the clamp) is no longer the
    loss gradient."""
    rng = np.random.default_rng(5)
    n, W, H = 6, 32, 32
    K = (40.0, 40.0, 15.5, 15.5)
    pos = np.column_stack([rng.uniform(-0.5, 0.5, n), rng.uniform(-0.5, 0.5, n), rng.uniform(1.5, 2.5, n)])
    scene = S.Scene(pos.astype(np.float32), np.full((n, 3), 0.12, np.float32),
                    np.tile(np.array([0, 0, 0, 1], np.float32), (n, 1)), rng.uniform(0.2, 0.8, (n, 3)).astype(np.float32),
                    np.full(n, 0.45, np.float32))
    P = oracle.default_params(0)
    P.w_depth = 0.0
    P.w_dist = 0.0
    b = oracle.prepare(scene, IDENT, K, W, H, P)
    obs = rng.uniform(0, 1, (H, W, 3)).astype(np.float32)
    depth = np.ones((H, W), np.float32)
    m = oracle.map_step(scene, b, obs, depth, IDENT, K, W, H, P, 0.0)
    rec0 = b.rec.copy()

    def loss(g, col, h):
        b.rec = rec0.copy()
        b.rec[g, col] = np.float32(rec0[g, col] + h)
        c, _, _, _ = oracle.render(b, IDENT, K, W, H, P)
        return 0.5 * float(np.sum((np.asarray(c).reshape(H, W, 3) - obs) ** 2))

    def fd(g, col, h):
        """Central, forward and backward differences: a pixel whose alpha
        crosses the 1/255 cut inside the step makes one side jump; the
        gradient must match the central difference or a one-sided one."""
        hp = float(np.float32(rec0[g, col] + h) - rec0[g, col])
        hm = float(rec0[g, col] - np.float32(rec0[g, col] - h))
        l0, lp, lm = loss(g, col, 0.0), loss(g, col, hp), loss(g, col, -hm)
        return np.array([(lp - lm) / (hp + hm), (lp - l0) / hp, (l0 - lm) / hm])

    def check(got, cands, name):
        scale = np.abs(cands[:, 0]).max()
        for i, (gv, c) in enumerate(zip(got, cands)):
            err = np.abs(c - gv)
            # central differences agree to 1e-3; one-sided ones to first order in h
            ok = err[0] <= 1e-3 * max(abs(c[0]), scale) or min(err[1:]) <= 2e-2 * max(abs(gv), scale)
            assert ok, (name, i, gv, c)

    # record columns: u v z o | c.x c.y c.z | phat | r g b
    # delta2d: dmx dmy dix diy diz dcr dcg dcb dz dal dpx dpy n
    checks = [(0, 0, -1.0, 1e-3), (1, 1, -1.0, 1e-3), (4, 2, -1.0, 1e-4), (5, 3, -0.5, 1e-4), (6, 4, -1.0, 1e-4),
              (9, 5, -1.0, 1e-3), (10, 6, -1.0, 1e-3), (11, 7, -1.0, 1e-3)]
    active = [g for g in range(n) if m.delta2d[g, 12] > 0]
    assert len(active) >= 4
    for col, k, sgn, h in checks:
        check(m.delta2d[active, k], np.array([sgn * fd(g, col, h) for g in active]), "record column %d" % col)
    o = rec0[active, 3].astype(np.float64)
    check(m.delta2d[active, 9], o[:, None] * np.array([fd(g, 3, 1e-4) for g in active]), "opacity")
    b.rec = rec0
