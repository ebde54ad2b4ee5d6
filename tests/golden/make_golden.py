"""Generate the golden fixtures of the CPU restatement (tests/golden/*.npz).

The reference publishes no golden data, so these fixtures freeze the oracle's
outputs on small seeded inputs (regression guard for the oracle; the GPU
tests also compare the CUDA path against them).  The oracle itself is pinned
to the reference source by tests/test_oracle_kat.py.

Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from f_vigs_slam_gb300 import synthetic as S  # noqa: E402

REF_JAC = O.Q_POSE_JAC_APPROX | O.Q_DEPTH_HUBER  # the reference's pose Jacobian and depth weight

CASES = {
    # name: (n, W, H, K, scene seed, pose seed, quirks)
    "small_default": (300, 64, 48, (52.5, 52.5, 31.95, 23.95), 101, 7, O.QUIRKS_DEFAULT),
    # every other reference behaviour off, the reference's Jacobian
    "small_quirks_off_refjac": (300, 64, 48, (52.5, 52.5, 31.95, 23.95), 102, 8, REF_JAC),
    # everything intended: the analytic pose Jacobian
    "small_intended": (300, 64, 48, (52.5, 52.5, 31.95, 23.95), 104, 10, O.QUIRKS_INTENDED),
    "small_culled_slots": (300, 64, 48, (52.5, 52.5, 31.95, 23.95), 103, 9,
                           O.Q_CULLED_SLOTS | O.Q_INVSIGMA_SWAP | REF_JAC),
}


def scene_for(n, seed):
    sc = S.cam_box(n, seed=seed)
    # a few Gaussians behind the camera and outside the view
    sc.positions[: n // 20, 2] *= -1.0
    sc.positions[n // 20: n // 10, 0] += 40.0
    return sc


def make(name):
    n, W, H, K, s_seed, p_seed, quirks = CASES[name]
    P = O.default_params(quirks)
    sc = scene_for(n, s_seed)
    rng = np.random.default_rng(p_seed)
    true_pose = S.perturb((np.zeros(3), S.IDENTITY_Q), 1.0, 2.0, rng)
    b_true = O.prepare(sc, true_pose, K, W, H, P)
    col, dep, _, _ = O.render(b_true, true_pose, K, W, H, P)
    rgb, d = S.add_noise(col.astype(np.float32), dep.astype(np.float32), rng)
    gx, gy = S.sobel3(rgb)
    pose = (np.zeros(3, np.float32), S.IDENTITY_Q)
    b = O.prepare(sc, pose, K, W, H, P)
    tr = O.track(b, (rgb, d, gx, gy), pose, K, W, H, P, images=True)
    out = dict(
        W=W, H=H, K=np.array(K, np.float32), quirks=quirks,
        positions=sc.positions, scales=sc.scales, orientations=sc.orientations, colors=sc.colors,
        opacities=sc.opacities, rgb=rgb, depth=d, gx=gx, gy=gy,
        uv=b.proj.uv, cov2d=b.proj.cov2d, inv2d=b.proj.inv2d, zdepth=b.proj.depth, phat=b.proj.phat,
        visible=b.proj.visible, counts=b.cnt, keys=b.keys, vals=b.vals, ranges=b.ranges,
        JtJ=tr.JtJ, Jtr=tr.Jtr, tiles=tr.tiles, img_color=tr.color, img_depth=tr.depth, img_T=tr.final_T,
        img_nc=tr.n_contrib,
    )
    if quirks & O.Q_CULLED_SLOTS == 0:
        m = O.map_step(sc, b, rgb, d, pose, K, W, H, P, 0.002)
        out.update(delta2d=m.delta2d, delta3d=m.delta3d, new_pos=m.pos, new_scl=m.scl, new_rot=m.rot,
                   new_col=m.col, new_opa=m.opa)
    return out


def main():
    for name in CASES:
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **make(name))
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
