"""ctypes wrapper of the reference's own binning kernels (oracle/ref_host.cpp,
oracle/ref_gpu.cu, built into oracle/_ref/ by oracle/ref_build.py).

TEST INFRASTRUCTURE ONLY: the ground truth the CPU restatement and the CUDA
library are compared with.  `available(kind)` says whether a harness could be
built here ("host": needs the reference's sources or the files oracle/_ref/
already holds; "gpu": also nvcc and, to run, a GPU).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_libs = {}


def _load(kind: str):
    if kind not in _libs:
        import ref_build

        paths = ref_build.build(gpu=(kind == "gpu"), host=(kind == "host"))
        path = paths.get(kind)
        _libs[kind] = C.CDLL(path) if path else None
    return _libs[kind]


def available(kind: str) -> bool:
    try:
        return _load(kind) is not None
    except Exception:
        return False


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def binning(kind: str, scene, pose, K, W, H, range_mode: int = 1):
    """The reference's prepareRasterization on `scene` at `pose` (t, q raw
    float4), K = (fx, fy, cx, cy): projection outputs, tile counts, the sorted
    keys and values, ranges and bucket counts.  range_mode 0 = the
    reference's range launch (ceil(T / 256) blocks), 1 = one thread per
    instance."""
    L = _load(kind)
    if L is None:
        raise RuntimeError("reference harness %r unavailable" % kind)
    fn = L.ref_binning_host if kind == "host" else L.ref_binning_gpu
    n = scene.n
    f32 = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
    pos, scl, rot = f32(scene.positions), f32(scene.scales), f32(scene.orientations)
    t = f32(pose[0])
    q = f32(pose[1])
    K4 = f32(K)
    T = ((W + 15) // 16) * ((H + 15) // 16)
    out = {"uv": np.zeros((n, 2), np.float32), "cov2d": np.zeros((n, 3), np.float32),
           "inv2d": np.zeros((n, 3), np.float32), "depth": np.zeros(n, np.float32),
           "phat": np.zeros((n, 2), np.float32), "counts": np.zeros(n, np.uint32),
           "ranges": np.zeros((T, 2), np.uint32), "buckets": np.zeros(T, np.uint32)}
    cap = max(1, 64 * n)
    for _ in range(2):
        keys = np.zeros(cap, np.uint64)
        vals = np.zeros(cap, np.uint32)
        ninst = C.c_uint64()
        rc = fn(_p(pos), _p(scl), _p(rot), C.c_int(n), _p(t), _p(q), _p(K4), C.c_int(W), C.c_int(H),
                C.c_int(range_mode), _p(out["uv"]), _p(out["cov2d"]), _p(out["inv2d"]), _p(out["depth"]),
                _p(out["phat"]), _p(out["counts"]), _p(keys), _p(vals), C.c_uint64(cap), _p(out["ranges"]),
                _p(out["buckets"]), C.byref(ninst))
        if rc == 1:
            cap = int(ninst.value)
            continue
        if rc != 0:
            raise RuntimeError("reference binning failed (%d)" % rc)
        m = int(ninst.value)
        out["keys"], out["vals"], out["n"] = keys[:m].copy(), vals[:m].copy(), m
        return out
    raise RuntimeError("reference binning: instance buffer")
