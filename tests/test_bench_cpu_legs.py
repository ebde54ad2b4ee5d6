"""The CPU legs of bench.py's render / preprocessing measurement, on CPU:
the comparison of a session's render and preprocessed levels with the
oracle's (here a stand-in session that returns the oracle's own outputs, so
the render matches to FP32 rounding and the levels exactly), and the
algorithmic byte count of the preprocessing."""
import numpy as np

from f_vigs_slam_gb300 import synthetic as S


class _Session:
    """download() / download_frame() of a session holding `scene` and `levels`."""

    def __init__(self, scene, levels):
        self.scene, self.levels = scene, levels

    def download(self):
        sc = self.scene
        return sc.positions, sc.scales, sc.orientations, sc.colors, sc.opacities

    def download_frame(self, lv):
        return self.levels[lv]


def test_render_preprocess_cpu_leg(oracle):
    import bench

    W, H = 160, 120
    K = (131.25, 131.25, 79.5, 59.5)
    scene = S.cam_box(5000, seed=4)
    pose = (np.zeros(3, np.float32), np.array(S.IDENTITY_Q, np.float32))
    P = oracle.default_params(bench.QUIRKS)
    b = oracle.prepare(scene, pose, K, W, H, P)
    col, dep = oracle.render_view(scene, b, W, H, P)
    rng = np.random.default_rng(1)
    c8 = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    mm = rng.integers(0, 8000, (H, W), dtype=np.uint16)
    levels = oracle.preprocess(c8, mm, levels=bench.ROOM_LEVELS, depth_mm=True)
    r = bench.cpu_render_preprocess_sample(None, _Session(scene, levels), pose, K, W, H, c8, mm,
                                           col.astype(np.float32), dep.astype(np.float32))
    assert r["preprocess_levels_bit_exact"]
    assert r["render_parity"]["colour_rel_err"] < 1e-6
    assert r["render_parity"]["crossing_differs_share"] == 0.0
    # a level off by one value is caught
    bad = [tuple(a.copy() for a in lv) for lv in levels]
    bad[1][0][0, 0, 0] += np.float32(1e-3)
    r = bench.cpu_render_preprocess_sample(None, _Session(scene, bad), pose, K, W, H, c8, mm,
                                           col.astype(np.float32), dep.astype(np.float32))
    assert not r["preprocess_levels_bit_exact"]


def test_preprocess_bytes():
    import bench

    # 1280x720, three levels: 5 B per camera pixel in, 40 B per pixel of 1280x720, 640x360, 320x180 out
    assert bench.preprocess_bytes(1280, 720) == 5 * 921600 + 40 * (921600 + 230400 + 57600)
    # odd sizes use the (n + 1) / 2 levels
    assert bench.preprocess_bytes(5, 3) == 5 * 15 + 40 * (15 + 3 * 2 + 2 * 1)
