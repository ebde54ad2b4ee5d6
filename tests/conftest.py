import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libfvgs.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O  # noqa: E402  (oracle/oracle.py)

    O.build()
    return O


@pytest.fixture(scope="session")
def fvgs_lib():
    """The built CUDA library (built in-tree on first use)."""
    from f_vigs_slam_gb300 import build

    build.build()
    from f_vigs_slam_gb300 import fvgs

    return fvgs


def scaled_camera(scale: float):
    from f_vigs_slam_gb300 import synthetic as S

    c = S.CAM_VGA
    # intrinsics scaled as GSSlam::computeRgbdPoseJacobians does per pyramid level
    return int(c.width * scale), int(c.height * scale), (c.fx * scale, c.fy * scale, c.cx * scale, c.cy * scale)


def make_frame(oracle_mod, scene, pose, K, W, H, params, seed=3):
    """Observed RGB-D frame: oracle render at `pose` + noise, Sobel gradients."""
    from f_vigs_slam_gb300 import synthetic as S

    b = oracle_mod.prepare(scene, pose, K, W, H, params)
    col, dep, _, _ = oracle_mod.render(b, pose, K, W, H, params)
    rng = np.random.default_rng(seed)
    rgb, d = S.add_noise(col.astype(np.float32), dep.astype(np.float32), rng)
    gx, gy = S.sobel3(rgb)
    return rgb, d, gx, gy


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))
