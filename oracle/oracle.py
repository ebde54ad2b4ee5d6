"""ctypes wrapper of the CPU restatement (oracle/fvgs_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the library.  Builds
oracle/_build/liboracle.so on first use if it is missing.

Parity unpinned by reference outputs (the reference has no tests or fixtures
and cannot be built here); pinned by hand-derived known-answer tests.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "fvgs_oracle.cpp")


LIB_NOFMA = os.path.join(BUILD, "liboracle_nofma.so")


def build(force: bool = False, nofma: bool = False) -> str:
    """Compile the oracle with -ffp-contract=off (bit-exact FP32 keys) and OpenMP.
    nofma: the variant without the reference's FMA contractions (every product
    and sum rounded on its own), compared with the reference's source compiled
    the same way."""
    lib = LIB_NOFMA if nofma else LIB
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= os.path.getmtime(SRC):
        return lib
    os.makedirs(BUILD, exist_ok=True)
    tmp = lib + ".tmp%d" % os.getpid()
    cmd = [
        "g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
        "-fPIC", "-shared", "-o", tmp, SRC,
    ] + (["-DFVGS_ORACLE_NO_FMA"] if nofma else [])
    subprocess.check_call(cmd)
    os.replace(tmp, lib)
    return lib


class Pose(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("orientation", C.c_float * 4)]


class Intr(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float)]


class Params(C.Structure):
    _fields_ = [
        ("tile_w", C.c_int32), ("tile_h", C.c_int32), ("radius_sigma", C.c_float),
        ("bg", C.c_float * 3), ("alpha_thresh", C.c_float), ("color_thresh", C.c_float),
        ("depth_thresh", C.c_float), ("w_depth", C.c_float), ("w_dist", C.c_float),
        ("lambda_iso", C.c_float), ("adam_beta1", C.c_float), ("adam_beta2", C.c_float),
        ("adam_eps", C.c_float), ("quirks", C.c_uint32), ("eig_eps", C.c_double),
    ]


Q_CULLED_SLOTS = 0x1
Q_RANGE_LAUNCH = 0x2
Q_INVSIGMA_SWAP = 0x4
Q_MAP_CAP256 = 0x8
Q_VIS_CAP256 = 0x10
Q_ADAM_STAY = 0x20
Q_POSE_WXYZ = 0x40
Q_COLOR_RESCALE = 0x80
Q_POSE_JAC_APPROX = 0x100
Q_DEPTH_HUBER = 0x200
QUIRKS_DEFAULT = (Q_INVSIGMA_SWAP | Q_MAP_CAP256 | Q_VIS_CAP256 | Q_ADAM_STAY | Q_POSE_WXYZ
                  | Q_COLOR_RESCALE | Q_POSE_JAC_APPROX | Q_DEPTH_HUBER)
QUIRKS_INTENDED = 0


def default_params(quirks: int = QUIRKS_DEFAULT, tile=(16, 16)) -> Params:
    p = Params()
    p.tile_w, p.tile_h = tile
    p.radius_sigma = 3.0
    p.bg[:] = [0.0, 0.0, 0.0]
    p.alpha_thresh, p.color_thresh, p.depth_thresh = 0.2, 0.1, 0.2
    p.w_depth, p.w_dist, p.lambda_iso = 1.0, 0.1, 0.01
    p.adam_beta1, p.adam_beta2, p.adam_eps = 0.9, 0.999, 1e-8
    p.quirks = quirks
    p.eig_eps = 1e-4
    return p


def make_pose(pose) -> Pose:
    t, q = pose
    p = Pose()
    p.position[:] = [float(v) for v in np.asarray(t, np.float32)]
    p.orientation[:] = [float(v) for v in np.asarray(q, np.float32)]
    return p


def make_intr(K) -> Intr:
    i = Intr()
    i.fx, i.fy, i.cx, i.cy = [float(np.float32(v)) for v in K]
    return i


_libs = {}


def lib(nofma: bool = False):
    if nofma not in _libs:
        L = C.CDLL(build(nofma=nofma))
        L.oracle_emit_keys.restype = C.c_int64
        L.oracle_buckets.restype = C.c_int64
        _libs[nofma] = L
    return _libs[nofma]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Projection:
    def __init__(self, uv, cov2d, inv2d, depth, phat, visible):
        self.uv, self.cov2d, self.inv2d = uv, cov2d, inv2d
        self.depth, self.phat, self.visible = depth, phat, visible


def project(scene, pose, K, W, H, nofma: bool = False) -> Projection:
    n = scene.n
    uv = np.zeros((n, 2), np.float32)
    cov = np.zeros((n, 3), np.float32)
    inv = np.zeros((n, 3), np.float32)
    dep = np.zeros(n, np.float32)
    ph = np.zeros((n, 2), np.float32)
    vis = np.zeros(n, np.uint8)
    pos, scl, rot = _f32(scene.positions), _f32(scene.scales), _f32(scene.orientations)
    lib(nofma).oracle_project(
        _p(pos), _p(scl), _p(rot), C.c_int(n), C.byref(make_pose(pose)), C.byref(make_intr(K)),
        C.c_int(W), C.c_int(H), _p(uv), _p(cov), _p(inv), _p(dep), _p(ph), _p(vis),
    )
    return Projection(uv, cov, inv, dep, ph, vis)


def count(proj: Projection, W, H, params: Params, nofma: bool = False):
    n = proj.uv.shape[0]
    cnt = np.zeros(n, np.uint32)
    rect = np.zeros((n, 4), np.int32)
    lib(nofma).oracle_count(
        _p(proj.uv), _p(proj.cov2d), _p(proj.visible), C.c_int(n), C.c_int(W), C.c_int(H),
        C.c_int(params.tile_w), C.c_int(params.tile_h), C.c_float(params.radius_sigma),
        C.c_uint32(params.quirks), _p(cnt), _p(rect),
    )
    return cnt, rect


def emit_keys(proj: Projection, cnt, rect, W, params: Params, nofma: bool = False):
    n = proj.uv.shape[0]
    total = int(cnt.astype(np.int64).sum())
    keys = np.zeros(max(total, 1), np.uint64)
    vals = np.zeros(max(total, 1), np.uint32)
    got = lib(nofma).oracle_emit_keys(
        _p(proj.uv), _p(proj.depth), _p(proj.phat), _p(cnt), _p(rect), C.c_int(n), C.c_int(W),
        C.c_int(params.tile_w), C.c_int(params.tile_h), C.c_int64(total), _p(keys), _p(vals),
    )
    assert got == total
    return keys[:total].copy(), vals[:total].copy()


def num_tiles(W, H, params: Params):
    return ((W + params.tile_w - 1) // params.tile_w) * ((H + params.tile_h - 1) // params.tile_h)


def sort_ranges(keys, vals, W, H, params: Params):
    keys = keys.copy()
    vals = vals.copy()
    T = num_tiles(W, H, params)
    ranges = np.zeros((T, 2), np.uint32)
    lib().oracle_sort_ranges(
        _p(keys), _p(vals), C.c_int64(keys.shape[0]), C.c_int(T), C.c_uint32(params.quirks), _p(ranges)
    )
    return keys, vals, ranges


def make_records(proj: Projection, scene, params: Params):
    n = proj.uv.shape[0]
    rec = np.zeros((n, 12), np.float32)
    lib().oracle_make_records(
        _p(proj.uv), _p(proj.inv2d), _p(proj.depth), _p(proj.phat), _p(_f32(scene.colors)),
        _p(_f32(scene.opacities)), C.c_int(n), C.c_uint32(params.quirks), _p(rec),
    )
    return rec


def cam3d(scene, pose):
    """FP64 camera-frame mean and 3D covariance of every Gaussian, (N, 9) =
    (x, y, z, Sxx, Sxy, Sxz, Syy, Syz, Szz): the geometry the analytic pose
    Jacobian differentiates."""
    n = scene.n
    out = np.zeros((max(n, 1), 9), np.float64)
    pos, scl, rot = _f32(scene.positions), _f32(scene.scales), _f32(scene.orientations)
    lib().oracle_cam3d(_p(pos), _p(scl), _p(rot), C.c_int(n), C.byref(make_pose(pose)), _p(out))
    return out[:n]


class Binning:
    """Everything prepareRasterization produces (src/GSSlam.cu:408-646), plus
    the FP64 camera-frame geometry the analytic pose Jacobian needs."""

    def __init__(self, proj, cnt, rect, keys_gen, vals_gen, keys, vals, ranges, rec, geo=None):
        self.proj, self.cnt, self.rect = proj, cnt, rect
        self.keys_gen, self.vals_gen = keys_gen, vals_gen
        self.keys, self.vals, self.ranges, self.rec = keys, vals, ranges, rec
        self.geo = geo


def prepare(scene, pose, K, W, H, params: Params, nofma: bool = False) -> Binning:
    """nofma: the binning without the reference's FMA contractions (see build)."""
    proj = project(scene, pose, K, W, H, nofma)
    cnt, rect = count(proj, W, H, params, nofma)
    kg, vg = emit_keys(proj, cnt, rect, W, params, nofma)
    ks, vs, ranges = sort_ranges(kg, vg, W, H, params)
    rec = make_records(proj, scene, params)
    geo = None if (params.quirks & Q_POSE_JAC_APPROX) else cam3d(scene, pose)
    return Binning(proj, cnt, rect, kg, vg, ks, vs, ranges, rec, geo)


class TrackResult:
    def __init__(self, JtJ, Jtr, tiles, color, depth, final_T, n_contrib):
        self.JtJ, self.Jtr, self.tiles = JtJ, Jtr, tiles
        self.color, self.depth, self.final_T, self.n_contrib = color, depth, final_T, n_contrib


def track(b: Binning, frame, pose, K, W, H, params: Params, images: bool = True,
          pixel_jacobians: bool = False, tiles=None) -> TrackResult:
    """frame = (rgb (H,W,3), depth (H,W), gx (H,W,3), gy (H,W,3)) float32.

    With Q_POSE_JAC_APPROX set in params.quirks this is the reference's
    getRgbdPoseJacobians; clear, the analytic pose Jacobian
    (oracle_track_intended; the gradient images are not read).  With
    pixel_jacobians (analytic mode only) the result also carries the
    per-pixel colour Jacobian jc (H, W, 3, 6) and depth Jacobian jd (H, W, 6).
    tiles: optional tile ids to evaluate (the others get zero partials; JtJ
    and Jtr then sum the evaluated tiles only)."""
    mask = None
    if tiles is not None:
        mask = np.zeros(num_tiles(W, H, params), np.uint8)
        mask[np.asarray(tiles, np.int64)] = 1
    if not (params.quirks & Q_POSE_JAC_APPROX):
        return _track_intended(b, frame, pose, K, W, H, params, images, pixel_jacobians, mask)
    rgb, depth, gx, gy = [_f32(a) for a in frame]
    T = num_tiles(W, H, params)
    tiles = np.zeros((T, 27), np.float64)
    JtJ = np.zeros((6, 6), np.float64)
    Jtr = np.zeros(6, np.float64)
    if images:
        col = np.zeros((H, W, 3), np.float64)
        dep = np.zeros((H, W), np.float64)
        fT = np.zeros((H, W), np.float64)
        nc = np.zeros((H, W), np.uint32)
        ptrs = (_p(col), _p(dep), _p(fT), _p(nc))
    else:
        col = dep = fT = nc = None
        ptrs = (None, None, None, None)
    lib().oracle_track(
        _p(b.rec), _p(b.ranges), _p(b.vals), _p(rgb), _p(depth), _p(gx), _p(gy),
        C.byref(make_pose(pose)), C.byref(make_intr(K)), C.byref(params), C.c_int(W), C.c_int(H),
        _p(tiles), _p(JtJ), _p(Jtr), *ptrs, _p(mask) if mask is not None else None,
    )
    return TrackResult(JtJ, Jtr, tiles, col, dep, fT, nc)


def _track_intended(b: Binning, frame, pose, K, W, H, params: Params, images: bool, pixel_jacobians: bool,
                    mask=None):
    rgb, depth = _f32(frame[0]), _f32(frame[1])
    if b.geo is None:
        raise ValueError("binning was prepared without the geometry of the analytic Jacobian")
    geo = np.ascontiguousarray(b.geo, np.float64)
    T = num_tiles(W, H, params)
    tiles = np.zeros((T, 27), np.float64)
    JtJ = np.zeros((6, 6), np.float64)
    Jtr = np.zeros(6, np.float64)
    if images or pixel_jacobians:
        col = np.zeros((H, W, 3), np.float64)
        dep = np.zeros((H, W), np.float64)
        fT = np.zeros((H, W), np.float64)
        nc = np.zeros((H, W), np.uint32)
        ptrs = (_p(col), _p(dep), _p(fT), _p(nc))
    else:
        col = dep = fT = nc = None
        ptrs = (None, None, None, None)
    jc = np.zeros((H, W, 3, 6), np.float64) if pixel_jacobians else None
    jd = np.zeros((H, W, 6), np.float64) if pixel_jacobians else None
    lib().oracle_track_intended(
        _p(b.rec), _p(geo), _p(b.ranges), _p(b.vals), _p(rgb), _p(depth), C.byref(make_pose(pose)),
        C.byref(make_intr(K)), C.byref(params), C.c_int(W), C.c_int(H), _p(tiles), _p(JtJ), _p(Jtr), *ptrs,
        _p(jc) if jc is not None else None, _p(jd) if jd is not None else None,
        _p(mask) if mask is not None else None,
    )
    r = TrackResult(JtJ, Jtr, tiles, col, dep, fT, nc)
    r.jc, r.jd = jc, jd
    return r


def forward64(scene, b: Binning, pose64, K, W, H, params: Params):
    """The tracking forward blend in FP64 at the FP64 pose (t, q (x,y,z,w))
    over b's tile lists: colour (H,W,3), median depth (H,W) and the per-pixel
    branch signature (H,W,3) (blended count, median position, n_contrib)."""
    t, q = pose64
    t = np.ascontiguousarray(t, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    col = np.zeros((H, W, 3), np.float64)
    dep = np.zeros((H, W), np.float64)
    sig = np.zeros((H, W, 3), np.uint32)
    lib().oracle_forward64(
        _p(_f32(scene.positions)), _p(_f32(scene.scales)), _p(_f32(scene.orientations)), _p(_f32(scene.colors)),
        _p(_f32(scene.opacities)), C.c_int(scene.n), _p(t), _p(q), C.byref(make_intr(K)), C.byref(params),
        C.c_int(W), C.c_int(H), _p(b.ranges), _p(b.vals), _p(col), _p(dep), _p(sig))
    return col, dep, sig


def render(b: Binning, pose, K, W, H, params: Params):
    """Forward blend of the tracking kernel for every pixel (observed depth
    treated as valid everywhere): colour (H,W,3), depth, final T, n_contrib."""
    ones = np.ones((H, W), np.float32)
    z3 = np.zeros((H, W, 3), np.float32)
    r = track(b, (z3, ones, z3, z3), pose, K, W, H, params, images=True)
    return r.color, r.depth, r.final_T, r.n_contrib


def render_view(scene, b: Binning, W, H, params: Params):
    """Render-form forward pass (forwardPassTileKernel, src/GSCudaKernels.cu:710-859)
    in FP64: colour (H,W,3) without background, median depth (H,W), 1e10 where
    the accumulated alpha never crosses 0.5."""
    col = np.zeros((H, W, 3), np.float64)
    dep = np.zeros((H, W), np.float64)
    p = b.proj
    lib().oracle_render_view(
        _p(_f32(p.uv)), _p(_f32(p.inv2d)), _p(_f32(p.depth)), _p(_f32(p.phat)), _p(_f32(scene.colors)),
        _p(_f32(scene.opacities)), _p(b.ranges), _p(b.vals), C.c_int(W), C.c_int(H), C.c_int(params.tile_w),
        C.c_int(params.tile_h), _p(col), _p(dep))
    return col, dep


def pyrdown(img):
    """One cv::pyrDown step (5-tap binomial, reflect-101 borders) of an (H, W)
    or (H, W, C) uint8 or float32 image (src/GSSlam.cu:1942-1944)."""
    a = np.ascontiguousarray(img)
    H, W = a.shape[:2]
    c = 1 if a.ndim == 2 else a.shape[2]
    shape = ((H + 1) // 2, (W + 1) // 2) + (() if a.ndim == 2 else (c,))
    if a.dtype == np.uint8:
        out = np.zeros(shape, np.uint8)
        lib().oracle_pyrdown_u8(_p(a), C.c_int(W), C.c_int(H), C.c_int(c), _p(out))
    else:
        a = a.astype(np.float32)
        out = np.zeros(shape, np.float32)
        lib().oracle_pyrdown_f32(_p(a), C.c_int(W), C.c_int(H), C.c_int(c), _p(out))
    return out


def preprocess(color_u8, depth, levels=3, depth_mm=False, double_scale=False):
    """GSSlam::initAndCopyImgs (src/GSSlam.cu:1913-1969) for one frame: per
    pyramid level the colour as float [0,1] (x 1/255 once more with
    double_scale, the scaling computeRgbdPoseJacobians adds, 2158), the depth
    in metres (uint16 millimetres x 0.001), and the 3x3 Sobel gradients of the
    float colour.  Returns a list of (rgb, depth, gx, gy)."""
    from f_vigs_slam_gb300 import synthetic as S

    col = np.ascontiguousarray(color_u8, np.uint8)
    dep = (depth.astype(np.float32) * np.float32(0.001)) if depth_mm else np.ascontiguousarray(depth, np.float32)
    out = []
    for lv in range(levels):
        if lv > 0:
            col = pyrdown(col)
            dep = pyrdown(dep)
        f = col.astype(np.float32) * np.float32(1.0 / 255.0)
        gx, gy = S.sobel3(f)
        rgb = f * np.float32(1.0 / 255.0) if double_scale else f
        out.append((rgb, dep.copy(), gx, gy))
    return out


class MapResult:
    pass


def map_step(scene, b: Binning, frame_rgb, frame_depth, pose, K, W, H, params: Params, eta: float,
             adam_state=None):
    """One optimizeGaussiansKeyframe step (src/GSSlam.cu:1083-1320) in FP64.
    Returns a MapResult with forward images, delta2d (N,13), delta3d (N,14)
    and the updated parameters / Adam state (float64)."""
    L = lib()
    n = scene.n
    T = num_tiles(W, H, params)
    BS = params.tile_w * params.tile_h
    bucket_incl = np.zeros(T, np.uint32)
    nb = int(L.oracle_buckets(_p(b.ranges), C.c_int(T), _p(bucket_incl)))
    P = W * H
    r = MapResult()
    r.final_T = np.zeros(P, np.float64)
    r.n_contrib = np.zeros(P, np.uint32)
    r.max_contrib = np.zeros(T, np.uint32)
    r.color = np.zeros((P, 3), np.float64)
    r.depth = np.zeros(P, np.float64)
    r.color_err = np.zeros((P, 3), np.float64)
    r.depth_obs = np.zeros(P, np.float64)
    r.sampled_T = np.zeros(max(nb, 1) * BS, np.float64)
    r.sampled_ar = np.zeros((max(nb, 1) * BS, 3), np.float64)
    rgb, dep = _f32(frame_rgb), _f32(frame_depth)
    L.oracle_map_forward(
        _p(b.rec), _p(b.ranges), _p(b.vals), _p(bucket_incl), _p(rgb), _p(dep), C.byref(params),
        C.c_int(W), C.c_int(H), _p(r.final_T), _p(r.n_contrib), _p(r.max_contrib), _p(r.color),
        _p(r.depth), _p(r.color_err), _p(r.depth_obs), _p(r.sampled_T), _p(r.sampled_ar),
    )
    r.delta2d = np.zeros((n, 13), np.float64)
    L.oracle_map_backward(
        _p(b.rec), _p(b.ranges), _p(b.vals), _p(bucket_incl), _p(r.sampled_T), _p(r.sampled_ar),
        _p(r.n_contrib), _p(r.max_contrib), _p(r.color), _p(r.depth), _p(r.color_err),
        _p(r.depth_obs), C.byref(params), C.c_int(W), C.c_int(H), _p(r.delta2d),
    )
    r.delta3d = np.zeros((n, 14), np.float64)
    pos, scl, rot = _f32(scene.positions), _f32(scene.scales), _f32(scene.orientations)
    L.oracle_delta3d(
        _p(pos), _p(scl), _p(rot), _p(r.delta2d), C.c_int(n), C.byref(make_pose(pose)),
        C.byref(make_intr(K)), C.c_float(params.lambda_iso), _p(r.delta3d),
    )
    r.pos = scene.positions.astype(np.float64).copy()
    r.scl = scene.scales.astype(np.float64).copy()
    r.rot = scene.orientations.astype(np.float64).copy()
    r.col = scene.colors.astype(np.float64).copy()
    r.opa = scene.opacities.astype(np.float64).copy()
    r.adam = np.zeros((n, 27), np.float64) if adam_state is None else adam_state.astype(np.float64).copy()
    L.oracle_adam(
        _p(r.pos), _p(r.scl), _p(r.rot), _p(r.col), _p(r.opa), _p(r.adam), _p(r.delta3d), C.c_int(n),
        C.c_float(eta), C.byref(params),
    )
    r.bucket_incl = bucket_incl
    r.num_buckets = nb
    return r


# ----------------------------------------------------------------------------
# Host FP64 post-processing (src/GSSlam.cu:2233-2243, src/RgbdPoseCost.cu:57-106,
# src/PoseLocalParameterization.cpp:22-44)
# ----------------------------------------------------------------------------
def pseudo_factor(JtJ, Jtr, eps=1e-4):
    """Eigen-regularised pseudo residual r* = S^-1/2 U^T Jtr and Jacobian
    J* = S^1/2 U^T (eigenvalues <= eps dropped)."""
    w, U = np.linalg.eigh(JtJ)
    keep = w > eps
    S = np.where(keep, w, 0.0)
    Sinv = np.where(keep, 1.0 / np.where(keep, w, 1.0), 0.0)
    Jstar = np.sqrt(S)[:, None] * U.T
    rstar = np.sqrt(Sinv) * (U.T @ Jtr)
    return rstar, Jstar


def gn_delta(JtJ, Jtr, eps=1e-4):
    """Gauss-Newton step of the pseudo factor: solve J*^T J* d = -J*^T r*."""
    rstar, Jstar = pseudo_factor(JtJ, Jtr, eps)
    return -np.linalg.lstsq(Jstar, rstar, rcond=None)[0]


def pose_plus(pose, delta):
    """PoseLocalParameterization::Plus: p += dp, q = normalise(q (x) [1, dth/2])."""
    t, q = pose
    t2 = np.asarray(t, np.float64) + delta[:3]
    dq = np.array([0.5 * delta[3], 0.5 * delta[4], 0.5 * delta[5], 1.0])
    x = np.asarray(q, np.float64)
    ax, ay, az, aw = x
    bx, by, bz, bw = dq
    q2 = np.array(
        [
            aw * bx + bw * ax + ay * bz - az * by,
            aw * by + bw * ay + az * bx - ax * bz,
            aw * bz + bw * az + ax * by - ay * bx,
            aw * bw - ax * bx - ay * by - az * bz,
        ]
    )
    q2 /= np.linalg.norm(q2)
    return t2, q2


# ----------------------------------------------------------------------------
# map maintenance (src/GSCudaKernels.cu:1455-1739, src/GSSlam.cu:1467-1904)
# ----------------------------------------------------------------------------
def visibility(b: Binning, W, H, params: Params, cap: int | None = None):
    """computeGaussiansVisibility_kernel over the binned view: uint8 mask per
    Gaussian (1 = some pixel blends it before its T falls below 0.5).  cap
    defaults to 256 with Q_VIS_CAP256 set in params.quirks, else all."""
    n = b.rec.shape[0]
    if cap is None:
        cap = 256 if (params.quirks & Q_VIS_CAP256) else 0
    vis = np.zeros(max(n, 1), np.uint8)
    lib().oracle_visibility(_p(b.rec), _p(b.ranges), _p(b.vals), C.c_int(n), C.c_int(W), C.c_int(H),
                            C.c_int(params.tile_w), C.c_int(params.tile_h), C.c_int(cap), _p(vis))
    return vis[:n]


def outlier_scores(b: Binning, obs_depth, W, H, params: Params):
    """computeOutliers_kernel sums in FP64: (total_alpha, outlier_prob) per Gaussian."""
    n = b.rec.shape[0]
    ta = np.zeros(max(n, 1), np.float64)
    op = np.zeros(max(n, 1), np.float64)
    lib().oracle_outlier_scores(_p(b.rec), _p(b.ranges), _p(b.vals), C.c_int(n), _p(_f32(obs_depth)), C.c_int(W),
                                C.c_int(H), C.c_int(params.tile_w), C.c_int(params.tile_h), _p(ta), _p(op))
    return ta[:n], op[:n]


def outlier_states(total_alpha, outlier_prob, threshold: float = 0.6):
    """removeOutliers_kernel: 0xff where total_alpha > 1 and the outlier share > threshold."""
    ta = np.ascontiguousarray(total_alpha, np.float64)
    op = np.ascontiguousarray(outlier_prob, np.float64)
    st = np.zeros(max(ta.shape[0], 1), np.uint8)
    lib().oracle_outlier_states(_p(ta), _p(op), C.c_int(ta.shape[0]), C.c_float(threshold), _p(st))
    return st[:ta.shape[0]]


def prune_states(scene, alpha_threshold=0.05, scale_ratio_threshold=0.05, min_scale=0.005):
    """pruneGaussians_kernel in FP32: 0xff for Gaussians to prune."""
    sc, op = _f32(scene.scales), _f32(scene.opacities)
    st = np.zeros(max(scene.n, 1), np.uint8)
    lib().oracle_prune_states(_p(sc), _p(op), C.c_int(scene.n), C.c_float(alpha_threshold),
                              C.c_float(scale_ratio_threshold), C.c_float(min_scale), _p(st))
    return st[:scene.n]


def compact_order(states):
    """Order of thrust::sort_by_key on the 0 / 0xff states (radix sort of
    unsigned char keys, stable): survivors in order, then the removed ones."""
    return np.argsort(np.asarray(states, np.uint8), kind="stable")


def covisibility(vis_a, vis_b):
    """computeGaussiansCovisibility_kernel + the driver's ratio: (inter, union,
    inter / union as float32, 0 for an empty union)."""
    a = np.asarray(vis_a) != 0
    b = np.asarray(vis_b) != 0
    inter, uni = int(np.sum(a & b)), int(np.sum(a | b))
    return inter, uni, (np.float32(inter) / np.float32(uni)) if uni else np.float32(0.0)


def seed(mode: str, bgr, depth, K, pose_t, pose_q_raw, sample: int, init_scale=2.0, init_opacity=0.8, mask=None,
         max_out: int | None = None):
    """initGaussiansFromRgbd_kernel (mode 'init') or densifyGaussians_kernel
    (mode 'densify', with a W x H float mask) in FP32, seeds in row-major order
    of their sample cell: (positions, scales, orientations raw (w,x,y,z),
    colors, opacities)."""
    bgr = np.ascontiguousarray(bgr, np.uint8)
    H, W = bgr.shape[:2]
    dep = _f32(depth)
    msk = _f32(mask) if mask is not None else np.zeros((H, W), np.float32)
    cap = W * H if max_out is None else max_out
    pos = np.zeros((max(cap, 1), 3), np.float32)
    scl = np.zeros((max(cap, 1), 3), np.float32)
    rot = np.zeros((max(cap, 1), 4), np.float32)
    col = np.zeros((max(cap, 1), 3), np.float32)
    opa = np.zeros(max(cap, 1), np.float32)
    t = _f32(pose_t)
    q = _f32(pose_q_raw)
    n = lib().oracle_seed(C.c_int(0 if mode == "init" else 1), _p(bgr), _p(dep), _p(msk), C.c_int(W), C.c_int(H),
                          C.c_int(sample), C.byref(make_intr(K)), _p(t), _p(q), C.c_float(init_scale),
                          C.c_float(init_opacity), C.c_int(cap), _p(pos), _p(scl), _p(rot), _p(col), _p(opa))
    return pos[:n], scl[:n], rot[:n], col[:n], opa[:n]


def density_mask(b: Binning, obs_depth, W, H, params: Params):
    """computeDensityMask_kernel in FP64: (H, W) mask."""
    n = b.rec.shape[0]
    m = np.zeros((H, W), np.float64)
    lib().oracle_density_mask(_p(b.rec), _p(b.ranges), _p(b.vals), C.c_int(n), _p(_f32(obs_depth)), C.c_int(W),
                              C.c_int(H), C.c_int(params.tile_w), C.c_int(params.tile_h), _p(m))
    return m
