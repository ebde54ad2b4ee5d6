"""Python binding of the fvgs C-ABI (include/fvgs.h) via ctypes.

This is the host-side mirror of the reference's GSSlam device calls used by
tests and the benchmark.  There is no CPU fallback: if libfvgs.so is missing
or has no GPU to run on, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfvgs.so")

FVGS_OK = 0
STATUS_NAMES = {
    0: "FVGS_OK", -1: "FVGS_E_INVALID", -2: "FVGS_E_NOMEM", -3: "FVGS_E_CUDA", -4: "FVGS_E_CAPACITY",
    -5: "FVGS_E_TIMEOUT", -6: "FVGS_E_STATE", -7: "FVGS_E_ADMISSION",
}

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
# every reference behaviour off: the analytic pose Jacobian, Tukey depth weight
QUIRKS_INTENDED = 0
MAX_LEVELS = 4  # FVGS_MAX_LEVELS

PRECISION_FP32 = 0
PRECISION_REDUCED = 1

DEBUG_PROJECTION = 0x1
DEBUG_IMAGES = 0x2
DEBUG_MAPPING = 0x4
DEBUG_RADIX_SORT = 0x8
DEBUG_NO_CANDIDATES = 0x10

TRACK_VARIANTS = 8  # FVGS_TRACK_VARIANTS
KERNEL_CLASSES = ["project", "scan", "emit", "sort", "ranges", "track", "reduce", "gn", "map_fwd", "map_bwd",
                  "map_update", "render", "maint"]
K = {name: i for i, name in enumerate(KERNEL_CLASSES)}


class FvgsError(RuntimeError):
    def __init__(self, status: int, what: str, msg: str = ""):
        self.status = status
        super().__init__("%s failed: %s (%s) %s" % (what, STATUS_NAMES.get(status, status), status, msg))


class Pose(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("orientation", C.c_float * 4)]


class Intrinsics(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float)]


class Params(C.Structure):
    _fields_ = [
        ("tile_w", C.c_int32), ("tile_h", C.c_int32), ("radius_sigma", C.c_float),
        ("bg", C.c_float * 3), ("alpha_thresh", C.c_float), ("color_thresh", C.c_float),
        ("depth_thresh", C.c_float), ("w_depth", C.c_float), ("w_dist", C.c_float),
        ("lambda_iso", C.c_float), ("adam_beta1", C.c_float), ("adam_beta2", C.c_float),
        ("adam_eps", C.c_float), ("quirks", C.c_uint32), ("eig_eps", C.c_double),
    ]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libfvgs.so (build it with f_vigs_slam_gb300.build first)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(
                "libfvgs.so not found at %s: build the CUDA library (python -m f_vigs_slam_gb300.build)" % path
            )
        lib = C.CDLL(path)
        lib.fvgs_status_string.restype = C.c_char_p
        lib.fvgs_status_string.argtypes = [C.c_int]
        _lib = lib
    return _lib


def _check(status: int, what: str):
    if status != FVGS_OK:
        msg = load_library().fvgs_status_string(status).decode()
        raise FvgsError(status, what, msg)


def default_params(quirks: int = QUIRKS_DEFAULT) -> Params:
    p = Params()
    _check(load_library().fvgs_params_default(C.byref(p)), "fvgs_params_default")
    p.quirks = quirks
    return p


def make_pose(pose) -> Pose:
    t, q = pose
    p = Pose()
    p.position[:] = [float(v) for v in np.asarray(t, np.float32)]
    p.orientation[:] = [float(v) for v in np.asarray(q, np.float32)]
    return p


def make_intr(K) -> Intrinsics:
    i = Intrinsics()
    i.fx, i.fy, i.cx, i.cy = [float(np.float32(v)) for v in K]
    return i


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Session:
    """One SLAM map resident on one GPU (fvgs_session)."""

    def __init__(self, capacity: int, max_width: int, max_height: int, params: Params | None = None,
                 device: int = 0):
        self.lib = load_library()
        self.params = params if params is not None else default_params()
        h = C.c_void_p()
        _check(
            self.lib.fvgs_session_create(C.byref(self.params), C.c_int(device), C.c_uint32(capacity),
                                         C.c_int(max_width), C.c_int(max_height), C.byref(h)),
            "fvgs_session_create",
        )
        self.h = h
        self.n = 0
        self.tile = (self.params.tile_w, self.params.tile_h)

    def close(self):
        if self.h:
            self.lib.fvgs_session_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- state
    def set_debug(self, flags: int):
        _check(self.lib.fvgs_session_set_debug(self.h, C.c_uint32(flags)), "fvgs_session_set_debug")

    def set_stream(self, stream_handle: int | None):
        _check(self.lib.fvgs_session_set_stream(self.h, C.c_void_p(stream_handle or 0)), "fvgs_session_set_stream")

    def stream(self):
        """(cudaStream_t as an int, CUDA device) the session's work runs on (fvgs_session_stream)."""
        st, dev = C.c_void_p(), C.c_int()
        _check(self.lib.fvgs_session_stream(self.h, C.byref(st), C.byref(dev)), "fvgs_session_stream")
        return int(st.value or 0), int(dev.value)

    def sync(self):
        _check(self.lib.fvgs_session_sync(self.h), "fvgs_session_sync")

    def set_timing(self, classes=()):
        mask = 0
        for c in classes:
            mask |= 1 << K[c]
        _check(self.lib.fvgs_session_set_timing(self.h, C.c_uint32(mask)), "fvgs_session_set_timing")

    def get_timing(self, reset: bool = False):
        n = len(KERNEL_CLASSES)
        ms = np.zeros(n, np.float64)
        launches = np.zeros(n, np.uint64)
        timed = np.zeros(n, np.uint64)
        _check(self.lib.fvgs_session_get_timing(self.h, _ptr(ms), _ptr(launches), _ptr(timed), C.c_int(int(reset))),
               "fvgs_session_get_timing")
        return {c: dict(ms=float(ms[i]), launches=int(launches[i]), timed=int(timed[i]))
                for i, c in enumerate(KERNEL_CLASSES)}

    def set_precision(self, precision: int):
        """Precision form (fvgs_session_set_precision): PRECISION_FP32 or PRECISION_REDUCED."""
        _check(self.lib.fvgs_session_set_precision(self.h, C.c_int(precision)), "fvgs_session_set_precision")

    def autotune(self, pose, K, level: int = 0, reps: int = 5):
        """fvgs_session_autotune: (chosen variant, median ms per variant)."""
        v = C.c_int()
        ms = np.zeros(TRACK_VARIANTS, np.float32)
        _check(self.lib.fvgs_session_autotune(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)), C.c_int(level),
                                              C.c_int(reps), C.byref(v), _ptr(ms)), "fvgs_session_autotune")
        return int(v.value), ms

    def set_autotune(self, enabled: bool):
        _check(self.lib.fvgs_session_set_autotune(self.h, C.c_int(int(enabled))), "fvgs_session_set_autotune")

    def set_track_variant(self, level: int, variant: int):
        _check(self.lib.fvgs_session_set_track_variant(self.h, C.c_int(level), C.c_int(variant)),
               "fvgs_session_set_track_variant")

    def footprint(self) -> int:
        b = C.c_uint64()
        _check(self.lib.fvgs_session_footprint(self.h, C.byref(b)), "fvgs_session_footprint")
        return int(b.value)

    def binning_info(self) -> dict:
        """How the last binning read back by the host was formed (see fvgs_session_binning_info)."""
        n, inc, ne, nc = C.c_uint32(), C.c_int(), C.c_uint32(), C.c_uint32()
        _check(self.lib.fvgs_session_binning_info(self.h, C.byref(n), C.byref(inc), C.byref(ne), C.byref(nc)),
               "fvgs_session_binning_info")
        return dict(n_instances=int(n.value), incremental=bool(inc.value), n_entering=int(ne.value),
                    n_changed=int(nc.value))

    def upload(self, scene):
        pos, scl, rot = _f32(scene.positions), _f32(scene.scales), _f32(scene.orientations)
        col, opa = _f32(scene.colors), _f32(scene.opacities)
        _check(
            self.lib.fvgs_upload_gaussians(self.h, _ptr(pos), _ptr(scl), _ptr(rot), _ptr(col), _ptr(opa),
                                           C.c_uint32(scene.n)),
            "fvgs_upload_gaussians",
        )
        self.n = scene.n

    def download(self):
        n = self.n
        pos = np.zeros((n, 3), np.float32)
        scl = np.zeros((n, 3), np.float32)
        rot = np.zeros((n, 4), np.float32)
        col = np.zeros((n, 3), np.float32)
        opa = np.zeros(n, np.float32)
        _check(
            self.lib.fvgs_download_gaussians(self.h, _ptr(pos), _ptr(scl), _ptr(rot), _ptr(col), _ptr(opa),
                                             C.c_uint32(n)),
            "fvgs_download_gaussians",
        )
        return pos, scl, rot, col, opa

    def set_frame(self, level: int, rgb, depth, gx, gy):
        rgb, depth, gx, gy = _f32(rgb), _f32(depth), _f32(gx), _f32(gy)
        H, W = depth.shape
        _check(
            self.lib.fvgs_set_frame(self.h, C.c_int(level), _ptr(rgb), _ptr(depth), _ptr(gx), _ptr(gy),
                                    C.c_int(W), C.c_int(H)),
            "fvgs_set_frame",
        )

    def set_frames_packed(self, packed, levels: int, W: int, H: int):
        """Frames of levels 0..levels-1 from one packed buffer (pack_pyramid's
        layout): a numpy array (host memory: one copy to the device) or a
        device pointer (int)."""
        ptr = C.c_void_p(packed) if isinstance(packed, int) else _ptr(_f32(packed))
        _check(self.lib.fvgs_set_frames_packed(self.h, ptr, C.c_int(levels), C.c_int(W), C.c_int(H)),
               "fvgs_set_frames_packed")

    # -------------------------------------------------------------- binning
    def project_bin(self, pose, K, W, H) -> int:
        n = C.c_uint32()
        _check(
            self.lib.fvgs_project_bin(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)), C.c_int(W),
                                      C.c_int(H), C.byref(n)),
            "fvgs_project_bin",
        )
        return int(n.value)

    def download_projection(self, debug: bool = True):
        n = self.n
        uv = np.zeros((n, 2), np.float32)
        dep = np.zeros(n, np.float32)
        ph = np.zeros((n, 2), np.float32)
        cnt = np.zeros(n, np.uint32)
        cov = np.zeros((n, 3), np.float32) if debug else None
        inv = np.zeros((n, 3), np.float32) if debug else None
        vis = np.zeros(n, np.uint8) if debug else None
        _check(
            self.lib.fvgs_download_projection(self.h, _ptr(uv), _ptr(cov), _ptr(inv), _ptr(dep), _ptr(ph),
                                              _ptr(vis), _ptr(cnt)),
            "fvgs_download_projection",
        )
        return dict(uv=uv, cov2d=cov, inv2d=inv, depth=dep, phat=ph, visible=vis, counts=cnt)

    def num_tiles(self, W, H):
        tw, th = self.tile
        return ((W + tw - 1) // tw) * ((H + th - 1) // th)

    def binning_grid(self):
        """(tile_w, tile_h, number of tiles) of the last binning."""
        tw, th, T = C.c_int(), C.c_int(), C.c_int()
        _check(self.lib.fvgs_session_binning_grid(self.h, C.byref(tw), C.byref(th), C.byref(T)),
               "fvgs_session_binning_grid")
        return int(tw.value), int(th.value), int(T.value)

    def candidates(self):
        """The projection's candidate list after the work enqueued so far:
        (held, length, position[3], orientation[4], view-cone half-angle)."""
        valid, n, p, cone = C.c_int(), C.c_uint32(), Pose(), C.c_float()
        _check(self.lib.fvgs_session_candidates(self.h, C.byref(valid), C.byref(n), C.byref(p), C.byref(cone)),
               "fvgs_session_candidates")
        return bool(valid.value), int(n.value), list(p.position), list(p.orientation), float(cone.value)

    def download_binning(self, W, H, max_instances: int | None = None):
        n = C.c_uint32()
        _check(self.lib.fvgs_download_binning(self.h, None, None, None, C.c_uint64(0), C.byref(n)),
               "fvgs_download_binning")
        cnt = int(n.value)
        keys = np.zeros(max(cnt, 1), np.uint64)
        vals = np.zeros(max(cnt, 1), np.uint32)
        T = self.binning_grid()[2]
        ranges = np.zeros((max(T, 1), 2), np.uint32)
        _check(
            self.lib.fvgs_download_binning(self.h, _ptr(keys), _ptr(vals), _ptr(ranges), C.c_uint64(cnt),
                                           C.byref(n)),
            "fvgs_download_binning",
        )
        return keys[:cnt], vals[:cnt], ranges[:T]

    # ------------------------------------------------------------- tracking
    def track_jacobian(self, pose, K, level: int = 0):
        JtJ = np.zeros((6, 6), np.float64)
        Jtr = np.zeros(6, np.float64)
        _check(
            self.lib.fvgs_track_jacobian(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)), C.c_int(level),
                                         _ptr(JtJ), _ptr(Jtr)),
            "fvgs_track_jacobian",
        )
        return JtJ, Jtr

    def download_tile_partials(self, T: int):
        out = np.zeros((T, 27), np.float32)
        _check(self.lib.fvgs_download_tile_partials(self.h, _ptr(out), C.c_int(T)), "fvgs_download_tile_partials")
        return out

    def download_track_images(self, W, H):
        col = np.zeros((H, W, 3), np.float32)
        dep = np.zeros((H, W), np.float32)
        fT = np.zeros((H, W), np.float32)
        nc = np.zeros((H, W), np.uint32)
        _check(self.lib.fvgs_download_track_images(self.h, _ptr(col), _ptr(dep), _ptr(fT), _ptr(nc)),
               "fvgs_download_track_images")
        return col, dep, fT, nc

    def track_frame(self, pose, K, iterations: int = 20, level: int = 0):
        p = make_pose(pose)
        step = np.zeros(6, np.float64)
        _check(
            self.lib.fvgs_track_frame(self.h, C.byref(p), C.byref(make_intr(K)), C.c_int(level),
                                      C.c_int(iterations), _ptr(step)),
            "fvgs_track_frame",
        )
        return (np.array(p.position[:], np.float32), np.array(p.orientation[:], np.float32)), step

    def track_frame_pyramid(self, pose, K0, iterations=(4, 4, 6, 6)):
        """Coarse-to-fine frame (fvgs_track_frame_pyramid): iterations[l] Gauss-Newton steps at level l,
        from the coarsest level down; K0 are the level-0 intrinsics."""
        p = make_pose(pose)
        step = np.zeros(6, np.float64)
        it = (C.c_int * len(iterations))(*iterations)
        _check(self.lib.fvgs_track_frame_pyramid(self.h, C.byref(p), C.byref(make_intr(K0)), it,
                                                 C.c_int(len(iterations)), _ptr(step)),
               "fvgs_track_frame_pyramid")
        return (np.array(p.position[:], np.float32), np.array(p.orientation[:], np.float32)), step

    def render_view(self, pose, K, W, H, rgb8: bool = False):
        """Render-form image (fvgs_render_view): float rgb (H,W,3), depth (H,W), optional 8-bit rgb."""
        col = np.zeros((H, W, 3), np.float32)
        dep = np.zeros((H, W), np.float32)
        c8 = np.zeros((H, W, 3), np.uint8) if rgb8 else None
        _check(self.lib.fvgs_render_view(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)), C.c_int(W),
                                         C.c_int(H), _ptr(col), _ptr(dep), _ptr(c8)), "fvgs_render_view")
        return (col, dep, c8) if rgb8 else (col, dep)

    def preprocess_frame(self, color_u8, depth, levels: int = 3, double_scale: bool = False):
        """Camera frame -> pyramid levels on the device (fvgs_preprocess_frame); depth float32 metres or
        uint16 millimetres."""
        col = np.ascontiguousarray(color_u8, np.uint8)
        H, W = col.shape[:2]
        if depth.dtype == np.uint16:
            dep, mm = np.ascontiguousarray(depth), 1
        else:
            dep, mm = np.ascontiguousarray(depth, np.float32), 0
        _check(self.lib.fvgs_preprocess_frame(self.h, _ptr(col), _ptr(dep), C.c_int(mm), C.c_int(W), C.c_int(H),
                                              C.c_int(levels), C.c_int(int(double_scale))), "fvgs_preprocess_frame")

    def download_frame(self, level: int = 0):
        w, h = C.c_int(), C.c_int()
        _check(self.lib.fvgs_download_frame(self.h, C.c_int(level), None, None, None, None, C.byref(w), C.byref(h)),
               "fvgs_download_frame")
        W, H = w.value, h.value
        rgb = np.zeros((H, W, 3), np.float32)
        dep = np.zeros((H, W), np.float32)
        gx = np.zeros((H, W, 3), np.float32)
        gy = np.zeros((H, W, 3), np.float32)
        _check(self.lib.fvgs_download_frame(self.h, C.c_int(level), _ptr(rgb), _ptr(dep), _ptr(gx), _ptr(gy),
                                            None, None), "fvgs_download_frame")
        return rgb, dep, gx, gy

    def render(self, pose, K, W, H):
        col = np.zeros((H, W, 3), np.float32)
        dep = np.zeros((H, W), np.float32)
        fT = np.zeros((H, W), np.float32)
        nc = np.zeros((H, W), np.uint32)
        _check(
            self.lib.fvgs_render(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)), C.c_int(W), C.c_int(H),
                                 _ptr(col), _ptr(dep), _ptr(fT), _ptr(nc)),
            "fvgs_render",
        )
        return col, dep, fT, nc

    # -------------------------------------------------------------- mapping
    def map_step(self, pose, K, eta: float = 0.002, level: int = 0):
        _check(
            self.lib.fvgs_map_step(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)), C.c_int(level),
                                   C.c_float(eta)),
            "fvgs_map_step",
        )

    def download_map_state(self, W, H, deltas3d: bool = False):
        n = self.n
        fT = np.zeros((H, W), np.float32)
        nc = np.zeros((H, W), np.uint32)
        col = np.zeros((H, W, 3), np.float32)
        dep = np.zeros((H, W), np.float32)
        d2 = np.zeros((n, 16), np.float32)
        d3 = np.zeros((n, 16), np.float32) if deltas3d else None
        _check(
            self.lib.fvgs_download_map_state(self.h, _ptr(fT), _ptr(nc), _ptr(col), _ptr(dep), _ptr(d2), _ptr(d3)),
            "fvgs_download_map_state",
        )
        n2 = d2[:, 12].copy().view(np.uint32).astype(np.float64)
        d2f = d2[:, :13].astype(np.float64)
        d2f[:, 12] = n2
        return dict(final_T=fT, n_contrib=nc, color=col, depth=dep, delta2d=d2f,
                    delta3d=None if d3 is None else d3[:, :14].astype(np.float64))

    def download_adam_state(self):
        """Optimiser state (fvgs_download_adam_state): (9, n, 4) float32 planes."""
        n = self.n
        st = np.zeros((9, n, 4), np.float32)
        _check(self.lib.fvgs_download_adam_state(self.h, _ptr(st), C.c_uint32(n)), "fvgs_download_adam_state")
        return st

    # ---- map maintenance
    def remove_outliers(self, pose, K, level: int = 0, threshold: float = 0.6, remove: bool = True) -> int:
        """GSSlam::removeOutliers (fvgs_remove_outliers): number of Gaussians marked (removed when remove)."""
        m = C.c_uint32()
        _check(self.lib.fvgs_remove_outliers(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)), C.c_int(level),
                                             C.c_float(threshold), C.c_int(int(remove)), C.byref(m)),
               "fvgs_remove_outliers")
        if remove:
            self.n -= int(m.value)
        return int(m.value)

    def prune(self, alpha_threshold: float = 0.05, scale_ratio_threshold: float = 0.05, min_scale: float = 0.005,
              remove: bool = True) -> int:
        """GSSlam::prune (fvgs_prune): number of Gaussians marked (removed when remove)."""
        m = C.c_uint32()
        _check(self.lib.fvgs_prune(self.h, C.c_float(alpha_threshold), C.c_float(scale_ratio_threshold),
                                   C.c_float(min_scale), C.c_int(int(remove)), C.byref(m)), "fvgs_prune")
        if remove:
            self.n -= int(m.value)
        return int(m.value)

    def download_marks(self, n: int, scores: bool = False):
        """States of the last marking (and outlier scores): states or (states, total_alpha, outlier_prob)."""
        st = np.zeros(n, np.uint8)
        ta = np.zeros(n, np.float32) if scores else None
        op = np.zeros(n, np.float32) if scores else None
        _check(self.lib.fvgs_download_marks(self.h, _ptr(st), _ptr(ta), _ptr(op), C.c_uint32(n)),
               "fvgs_download_marks")
        return (st, ta, op) if scores else st

    def visibility(self, pose, K, W, H):
        """computeGaussiansVisibility_kernel (fvgs_visibility): (uint8 mask per Gaussian, count)."""
        vis = np.zeros(self.n, np.uint8)
        c = C.c_uint32()
        _check(self.lib.fvgs_visibility(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)), C.c_int(W),
                                        C.c_int(H), _ptr(vis), C.byref(c)), "fvgs_visibility")
        return vis, int(c.value)

    def covisibility(self, pose_a, K_a, W_a, H_a, pose_b, K_b, W_b, H_b):
        """GSSlam::computeCovisibilityRatio (fvgs_covisibility): (inter, union, ratio)."""
        i, u, r = C.c_uint32(), C.c_uint32(), C.c_float()
        _check(self.lib.fvgs_covisibility(self.h, C.byref(make_pose(pose_a)), C.byref(make_intr(K_a)), C.c_int(W_a),
                                          C.c_int(H_a), C.byref(make_pose(pose_b)), C.byref(make_intr(K_b)),
                                          C.c_int(W_b), C.c_int(H_b), C.byref(i), C.byref(u), C.byref(r)),
               "fvgs_covisibility")
        return int(i.value), int(u.value), float(r.value)

    def init_gaussians(self, pose, K, sample_px: int = 10, init_scale: float = 2.0, init_opacity: float = 0.8) -> int:
        """GSSlam::initializeGaussiansFromRgbd (fvgs_init_gaussians) from the last preprocessed camera frame:
        the new Gaussian count."""
        n = C.c_uint32()
        _check(self.lib.fvgs_init_gaussians(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)),
                                            C.c_int(sample_px), C.c_float(init_scale), C.c_float(init_opacity),
                                            C.byref(n)), "fvgs_init_gaussians")
        self.n = int(n.value)
        return self.n

    def densify(self, pose, K, sample_px: int = 10, W: int | None = None, H: int | None = None):
        """GSSlam::densify (fvgs_densify) against the last preprocessed camera frame: Gaussians added, and the
        density mask (H, W) when W and H are given."""
        m = np.zeros((H, W), np.float32) if W is not None else None
        a = C.c_uint32()
        _check(self.lib.fvgs_densify(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)), C.c_int(sample_px),
                                     _ptr(m), C.byref(a)), "fvgs_densify")
        self.n += int(a.value)
        return (int(a.value), m) if m is not None else int(a.value)

    # ---- asynchronous frames (CUDA-graph replay once the binning history is valid)
    def frame_submit(self, pose, K, iterations: int = 20, level: int = 0, map_eta: float | None = None):
        _check(self.lib.fvgs_frame_submit(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K)), C.c_int(level),
                                          C.c_int(iterations), C.c_float(-1.0 if map_eta is None else map_eta)),
               "fvgs_frame_submit")

    def frame_submit_pyramid(self, pose, K0, iterations=(4, 4, 6, 6), map_eta: float | None = None):
        it = (C.c_int * len(iterations))(*iterations)
        _check(self.lib.fvgs_frame_submit_pyramid(self.h, C.byref(make_pose(pose)), C.byref(make_intr(K0)), it,
                                                  C.c_int(len(iterations)),
                                                  C.c_float(-1.0 if map_eta is None else map_eta)),
               "fvgs_frame_submit_pyramid")

    def frame_poll(self) -> bool:
        d = C.c_int()
        _check(self.lib.fvgs_frame_poll(self.h, C.byref(d)), "fvgs_frame_poll")
        return bool(d.value)

    def frame_wait(self):
        p = Pose()
        step = np.zeros(6, np.float64)
        _check(self.lib.fvgs_frame_wait(self.h, C.byref(p), _ptr(step)), "fvgs_frame_wait")
        return (np.array(p.position[:], np.float32), np.array(p.orientation[:], np.float32)), step

    def set_track_tiles(self, level: int, tile_w: int, tile_h: int):
        """Tile shape of a pyramid level's tracking (fvgs_session_set_track_tiles): 16x16, 8x8 or 32x8."""
        _check(self.lib.fvgs_session_set_track_tiles(self.h, C.c_int(level), C.c_int(tile_w), C.c_int(tile_h)),
               "fvgs_session_set_track_tiles")

    def frame_stats(self) -> dict:
        g, e = C.c_uint64(), C.c_uint64()
        _check(self.lib.fvgs_session_frame_stats(self.h, C.byref(g), C.byref(e)), "fvgs_session_frame_stats")
        return dict(graphed=int(g.value), eager=int(e.value))


def frames_run(sessions, poses, Ks, iterations: int = 20, levels=None, map_etas=None):
    """One frame on each session, overlapped on the device (fvgs_frames_run)."""
    lib = load_library()
    n = len(sessions)
    hs = (C.c_void_p * n)(*[s.h for s in sessions])
    ps = (Pose * n)(*[make_pose(p) for p in poses])
    ks = (Intrinsics * n)(*[make_intr(k) for k in Ks])
    lv = None if levels is None else (C.c_int * n)(*levels)
    et = None if map_etas is None else (C.c_float * n)(*[(-1.0 if e is None else e) for e in map_etas])
    _check(lib.fvgs_frames_run(hs, ps, ks, lv, C.c_int(iterations), et, C.c_int(n)), "fvgs_frames_run")
    return [(np.array(p.position[:], np.float32), np.array(p.orientation[:], np.float32)) for p in ps]


def frames_run_pyramid(sessions, poses, K0s, iterations=(4, 4, 6, 6), map_etas=None):
    """One coarse-to-fine frame on each session, overlapped on the device (fvgs_frames_run_pyramid)."""
    lib = load_library()
    n = len(sessions)
    hs = (C.c_void_p * n)(*[s.h for s in sessions])
    ps = (Pose * n)(*[make_pose(p) for p in poses])
    ks = (Intrinsics * n)(*[make_intr(k) for k in K0s])
    it = (C.c_int * len(iterations))(*iterations)
    et = None if map_etas is None else (C.c_float * n)(*[(-1.0 if e is None else e) for e in map_etas])
    _check(lib.fvgs_frames_run_pyramid(hs, ps, ks, it, C.c_int(len(iterations)), et, C.c_int(n)),
           "fvgs_frames_run_pyramid")
    return [(np.array(p.position[:], np.float32), np.array(p.orientation[:], np.float32)) for p in ps]


TILE_SHAPES = ((16, 16), (8, 8), (32, 8))
STAGE_BATCHES = (128, 256, 512)


class Batch:
    """Keyframe batching in one persistent launch per Gauss-Newton iteration (fvgs_batch_*)."""

    def __init__(self, sessions):
        self.lib = load_library()
        self.sessions = list(sessions)
        n = len(self.sessions)
        hs = (C.c_void_p * n)(*[s.h for s in self.sessions])
        self.h = C.c_void_p()
        _check(self.lib.fvgs_batch_create(hs, C.c_int(n), C.byref(self.h)), "fvgs_batch_create")

    def close(self):
        if self.h:
            _check(self.lib.fvgs_batch_destroy(self.h), "fvgs_batch_destroy")
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_level(self, level: int, tile_w: int, tile_h: int, batch: int = 256):
        _check(self.lib.fvgs_batch_set_level(self.h, C.c_int(level), C.c_int(tile_w), C.c_int(tile_h),
                                             C.c_int(batch)), "fvgs_batch_set_level")

    def autotune(self, poses, K0s, iterations=(4, 4, 6, 6), reps: int = 5):
        """Per level: the fastest (tile_w, tile_h, batch) and the 9 medians (ms, shape-major)."""
        n = len(self.sessions)
        ps = (Pose * n)(*[make_pose(p) for p in poses])
        ks = (Intrinsics * n)(*[make_intr(k) for k in K0s])
        it = (C.c_int * len(iterations))(*iterations)
        cfg = np.zeros(3 * MAX_LEVELS, np.int32)
        ms = np.full(9 * MAX_LEVELS, np.nan, np.float32)
        _check(self.lib.fvgs_batch_autotune(self.h, ps, ks, it, C.c_int(len(iterations)), C.c_int(reps),
                                            _ptr(cfg), _ptr(ms)), "fvgs_batch_autotune")
        return ({l: tuple(int(v) for v in cfg[3 * l:3 * l + 3]) for l in range(len(iterations)) if iterations[l] > 0},
                {l: ms[9 * l:9 * l + 9].reshape(3, 3) for l in range(len(iterations)) if iterations[l] > 0})

    def run_pyramid(self, poses, K0s, iterations=(4, 4, 6, 6)):
        n = len(self.sessions)
        ps = (Pose * n)(*[make_pose(p) for p in poses])
        ks = (Intrinsics * n)(*[make_intr(k) for k in K0s])
        it = (C.c_int * len(iterations))(*iterations)
        _check(self.lib.fvgs_batch_run_pyramid(self.h, ps, ks, it, C.c_int(len(iterations))),
               "fvgs_batch_run_pyramid")
        return [(np.array(p.position[:], np.float32), np.array(p.orientation[:], np.float32)) for p in ps]

    def stats(self) -> dict:
        g, e, bl = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(self.lib.fvgs_batch_stats(self.h, C.byref(g), C.byref(e), C.byref(bl)), "fvgs_batch_stats")
        return dict(graphed=int(g.value), eager=int(e.value), batch_launches=int(bl.value))


def pack_pyramid(levels):
    """Pack per-level frames [(rgb, depth, gx, gy), ...] (level 0 first) into one float32 array in the
    layout of fvgs_server_request.pyr_frames: per level rgb[3P], depth[P], grad_x[3P], grad_y[3P]."""
    parts = []
    for rgb, d, gx, gy in levels:
        parts += [np.ravel(_f32(rgb)), np.ravel(_f32(d)), np.ravel(_f32(gx)), np.ravel(_f32(gy))]
    return np.concatenate(parts)


# ---- serving (include/fvgs_server.h) ----
class ServerRequest(C.Structure):
    _fields_ = [("pose", Pose), ("K", Intrinsics), ("level", C.c_int), ("iterations", C.c_int),
                ("map_eta", C.c_float), ("tag", C.c_uint64), ("t_arrival", C.c_double),
                ("rgb", C.c_void_p), ("depth", C.c_void_p), ("grad_x", C.c_void_p), ("grad_y", C.c_void_p),
                ("width", C.c_int), ("height", C.c_int), ("raw_color", C.c_void_p), ("raw_depth", C.c_void_p),
                ("raw_depth_u16_mm", C.c_int), ("raw_levels", C.c_int), ("raw_double_scale", C.c_int),
                ("pyr_levels", C.c_int), ("pyr_iterations", C.c_int * MAX_LEVELS), ("pyr_frames", C.c_void_p)]


class ServerResult(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("slot", C.c_int), ("status", C.c_int), ("pose", Pose),
                ("last_step", C.c_double * 6), ("t_arrival", C.c_double), ("t_launch", C.c_double),
                ("t_done", C.c_double)]


class Server:
    """Continuous-batching server over many sessions (fvgs_server_*)."""

    def __init__(self, memory_budget_bytes: int, max_inflight: int = 16):
        self.lib = load_library()
        self.h = C.c_void_p()
        _check(self.lib.fvgs_server_create(C.c_uint64(memory_budget_bytes), C.c_int(max_inflight),
                                           C.byref(self.h)), "fvgs_server_create")

    def close(self):
        if self.h:
            _check(self.lib.fvgs_server_destroy(self.h), "fvgs_server_destroy")
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def admit(self, session) -> int:
        slot = C.c_int()
        _check(self.lib.fvgs_server_admit(self.h, session.h, C.byref(slot)), "fvgs_server_admit")
        return int(slot.value)

    def release(self, slot: int):
        _check(self.lib.fvgs_server_release(self.h, C.c_int(slot)), "fvgs_server_release")

    @staticmethod
    def now() -> float:
        t = C.c_double()
        _check(load_library().fvgs_server_now(C.byref(t)), "fvgs_server_now")
        return float(t.value)

    def submit(self, slot: int, pose, K, iterations: int = 20, level: int = 0, map_eta: float | None = None,
               tag: int = 0, t_arrival: float = 0.0, frame=None, raw=None, pyramid=None, pyramid_frames=None):
        """frame: optional (rgb_ptr, depth_ptr, gx_ptr, gy_ptr, W, H) of memory that stays valid (pinned
        host or device) until the result is back, for `level`; raw: optional (color_u8_ptr, depth_ptr, W,
        H[, depth_u16]) camera frame, preprocessed on the device (level 0); pyramid: optional per-level
        iteration counts of a coarse-to-fine frame (K is then the level-0 intrinsics); pyramid_frames:
        optional (ptr, W, H) of every level's frame packed in one buffer (pack_pyramid's layout)."""
        r = ServerRequest()
        r.pose = make_pose(pose)
        r.K = make_intr(K)
        r.level, r.iterations = level, iterations
        if pyramid is not None:
            r.pyr_levels = len(pyramid)
            for i, v in enumerate(pyramid):
                r.pyr_iterations[i] = int(v)
            if pyramid_frames is not None:
                r.pyr_frames, r.width, r.height = pyramid_frames
        r.map_eta = -1.0 if map_eta is None else map_eta
        r.tag, r.t_arrival = tag, t_arrival
        if frame is not None:
            r.rgb, r.depth, r.grad_x, r.grad_y, r.width, r.height = frame
        if raw is not None:
            r.raw_color, r.raw_depth, r.width, r.height = raw[:4]
            r.raw_depth_u16_mm = int(raw[4]) if len(raw) > 4 else 0
            r.raw_levels = 1
        _check(self.lib.fvgs_server_submit(self.h, C.c_int(slot), C.byref(r)), "fvgs_server_submit")

    def results(self, wait_for: int = 0, max_results: int = 4096):
        buf = (ServerResult * max_results)()
        n = C.c_int()
        _check(self.lib.fvgs_server_results(self.h, buf, C.c_int(max_results), C.c_int(wait_for), C.byref(n)),
               "fvgs_server_results")
        out = []
        for r in buf[:n.value]:
            out.append(dict(tag=int(r.tag), slot=int(r.slot), status=int(r.status),
                            pose=(np.array(r.pose.position[:], np.float32), np.array(r.pose.orientation[:], np.float32)),
                            t_arrival=r.t_arrival, t_launch=r.t_launch, t_done=r.t_done))
        return out

    def stats(self) -> dict:
        ab, inf, la, co = C.c_uint64(), C.c_int(), C.c_uint64(), C.c_uint64()
        _check(self.lib.fvgs_server_stats(self.h, C.byref(ab), C.byref(inf), C.byref(la), C.byref(co)),
               "fvgs_server_stats")
        return dict(admitted_bytes=int(ab.value), inflight=int(inf.value), launched=int(la.value),
                    completed=int(co.value))


# ----------------------------------------------------------------------------
# host FP64 estimator glue (include/fvgs_estimator.h)
# ----------------------------------------------------------------------------
def _d(a, n=None):
    a = np.ascontiguousarray(a, np.float64)
    if n is not None and a.size != n:
        raise ValueError("expected %d values, got %d" % (n, a.size))
    return a


def jacobian_cam_to_imu(JtJ, Jtr, q_imu_cam, t_imu_cam, q_imu):
    """fvgs_jacobian_cam_to_imu: the IMU-frame 6x6 system (quaternions x, y, z, w)."""
    H = np.zeros((6, 6))
    g = np.zeros(6)
    _check(load_library().fvgs_jacobian_cam_to_imu(_ptr(_d(JtJ, 36)), _ptr(_d(Jtr, 6)), _ptr(_d(q_imu_cam, 4)),
                                                   _ptr(_d(t_imu_cam, 3)), _ptr(_d(q_imu, 4)), _ptr(H), _ptr(g)),
           "fvgs_jacobian_cam_to_imu")
    return H, g


def pseudo_factor(JtJ, Jtr, eps=1e-4):
    """fvgs_pseudo_factor: (r* [6], J* [6x6])."""
    r = np.zeros(6)
    J = np.zeros((6, 6))
    _check(load_library().fvgs_pseudo_factor(_ptr(_d(JtJ, 36)), _ptr(_d(Jtr, 6)), C.c_double(eps), _ptr(r), _ptr(J)),
           "fvgs_pseudo_factor")
    return r, J


class Preintegration:
    """fvgs_preint_*: IMU preintegration between two keyframes."""

    def __init__(self, acc0, gyr0, ba, bg, acc_n, gyr_n, acc_w, gyr_w):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib.fvgs_preint_create(_ptr(_d(acc0, 3)), _ptr(_d(gyr0, 3)), _ptr(_d(ba, 3)), _ptr(_d(bg, 3)),
                                           C.c_double(acc_n), C.c_double(gyr_n), C.c_double(acc_w),
                                           C.c_double(gyr_w), C.byref(h)), "fvgs_preint_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.fvgs_preint_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, dt, acc, gyr):
        _check(self.lib.fvgs_preint_add(self.h, C.c_double(dt), _ptr(_d(acc, 3)), _ptr(_d(gyr, 3))), "fvgs_preint_add")

    def repropagate(self, ba, bg):
        _check(self.lib.fvgs_preint_repropagate(self.h, _ptr(_d(ba, 3)), _ptr(_d(bg, 3))), "fvgs_preint_repropagate")

    def state(self):
        dp, dq, dv = np.zeros(3), np.zeros(4), np.zeros(3)
        T = C.c_double()
        jac, cov = np.zeros((15, 15)), np.zeros((15, 15))
        _check(self.lib.fvgs_preint_state(self.h, _ptr(dp), _ptr(dq), _ptr(dv), C.byref(T), _ptr(jac), _ptr(cov)),
               "fvgs_preint_state")
        return dict(delta_p=dp, delta_q=dq, delta_v=dv, sum_dt=T.value, jacobian=jac, covariance=cov)

    def evaluate(self, pose_i, sb_i, pose_j, sb_j):
        r = np.zeros(15)
        _check(self.lib.fvgs_preint_evaluate(self.h, _ptr(_d(pose_i, 7)), _ptr(_d(sb_i, 9)), _ptr(_d(pose_j, 7)),
                                             _ptr(_d(sb_j, 9)), _ptr(r)), "fvgs_preint_evaluate")
        return r

    def predict(self, pose_i, v_i):
        pj, vj = np.zeros(7), np.zeros(3)
        _check(self.lib.fvgs_preint_predict(self.h, _ptr(_d(pose_i, 7)), _ptr(_d(v_i, 3)), _ptr(pj), _ptr(vj)),
               "fvgs_preint_predict")
        return pj, vj

    def factor(self, pose_i, sb_i, pose_j, sb_j, jacobians=True):
        """fvgs_imu_factor: whitened residual [15] and Jacobians (15x7, 15x9, 15x7, 15x9)."""
        r = np.zeros(15)
        J = [np.zeros((15, 7)), np.zeros((15, 9)), np.zeros((15, 7)), np.zeros((15, 9))] if jacobians else [None] * 4
        _check(self.lib.fvgs_imu_factor(self.h, _ptr(_d(pose_i, 7)), _ptr(_d(sb_i, 9)), _ptr(_d(pose_j, 7)),
                                        _ptr(_d(sb_j, 9)), _ptr(r), *(_ptr(j) for j in J)), "fvgs_imu_factor")
        return (r, J) if jacobians else r


def marginalize(A, b, m, eps=1e-8):
    """fvgs_marginalize: prior (J [n x n], r [n]) of the kept n = dim - m dimensions."""
    A = _d(A)
    N = A.shape[0]
    n = N - m
    J, r = np.zeros((n, n)), np.zeros(n)
    _check(load_library().fvgs_marginalize(_ptr(A), _ptr(_d(b, N)), C.c_int(m), C.c_int(n), C.c_double(eps),
                                           _ptr(J), _ptr(r)), "fvgs_marginalize")
    return J, r


def marginal_prior_evaluate(J, r, blocks, x, x0, jacobians=True):
    """fvgs_marginal_prior_evaluate: blocks = [(global size, local offset)]."""
    J, r = _d(J), _d(r)
    n = r.size
    k = len(blocks)
    sizes = (C.c_int * k)(*[b[0] for b in blocks])
    idx = (C.c_int * k)(*[b[1] for b in blocks])
    xs = [_d(v) for v in x]
    x0s = [_d(v) for v in x0]
    xp = (C.c_void_p * k)(*[v.ctypes.data for v in xs])
    x0p = (C.c_void_p * k)(*[v.ctypes.data for v in x0s])
    res = np.zeros(n)
    jac = [np.zeros((n, b[0])) for b in blocks] if jacobians else []
    jp = (C.c_void_p * k)(*[j.ctypes.data for j in jac]) if jacobians else None
    _check(load_library().fvgs_marginal_prior_evaluate(_ptr(J), _ptr(r), C.c_int(n), C.c_int(k), sizes, idx, xp, x0p,
                                                       _ptr(res), jp), "fvgs_marginal_prior_evaluate")
    return (res, jac) if jacobians else res


def _prior_args(prior):
    if prior is None:
        return None, None, None, ()
    J, r, x0 = _d(prior[0], 225), _d(prior[1], 15), _d(prior[2], 16)
    return _ptr(J), _ptr(r), _ptr(x0), (J, r, x0)


def vi_step(preint, JtJ_imu, Jtr_imu, state_i, state_j, prior=None, eps=1e-4):
    """fvgs_vi_step: one Gauss-Newton step of the visual-inertial problem.

    state_* = (pose [7: p, q x y z w], speedbias [9]); prior = (J 15x15, r 15,
    x0 16) on state i or None (state i fixed).  Returns the updated
    (state_i, state_j), the cost before the step and the 30 local increments."""
    pi, si = _d(state_i[0], 7).copy(), _d(state_i[1], 9).copy()
    pj, sj = _d(state_j[0], 7).copy(), _d(state_j[1], 9).copy()
    Jp, rp, xp, keep = _prior_args(prior)
    cost = C.c_double()
    delta = np.zeros(30)
    _check(load_library().fvgs_vi_step(preint.h, _ptr(_d(JtJ_imu, 36)), _ptr(_d(Jtr_imu, 6)), C.c_double(eps), Jp,
                                       rp, xp, _ptr(pi), _ptr(si), _ptr(pj), _ptr(sj), C.byref(cost), _ptr(delta)),
           "fvgs_vi_step")
    del keep
    return (pi, si), (pj, sj), cost.value, delta


def vi_marginalize(preint, JtJ_imu, Jtr_imu, state_i, state_j, prior=None, eps=1e-4):
    """fvgs_vi_marginalize: the prior (J 15x15, r 15, x0 16) on state j for the next frame."""
    Jp, rp, xp, keep = _prior_args(prior)
    J, r, x0 = np.zeros((15, 15)), np.zeros(15), np.zeros(16)
    _check(load_library().fvgs_vi_marginalize(preint.h, _ptr(_d(JtJ_imu, 36)), _ptr(_d(Jtr_imu, 6)),
                                              C.c_double(eps), Jp, rp, xp, _ptr(_d(state_i[0], 7)),
                                              _ptr(_d(state_i[1], 9)), _ptr(_d(state_j[0], 7)),
                                              _ptr(_d(state_j[1], 9)), _ptr(J), _ptr(r), _ptr(x0)),
           "fvgs_vi_marginalize")
    del keep
    return J, r, x0
