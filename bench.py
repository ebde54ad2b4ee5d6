#!/usr/bin/env python
"""Tracking benchmark of the GB300 Gaussian-splatting hot path.

Workload (the large plain-method configuration): N = 1,000,000 Gaussians
uniform in a 10 x 10 x 4 m room, a camera trajectory random-walking 1 cm /
0.5 deg per frame, 1280x720 RGB-D frames (fx = fy = 1050, 16x16 tiles).  One
step = one frame = 20 Gauss-Newton tracking iterations (binning + fused
Jacobian kernel + on-device 6x6 pseudo-factor step) + 1 mapping step
(forward, backward, 2D->3D, Adam) on that frame.  Observed frames are rendered
at the true pose with N(0,0.01) colour / N(0,0.005 m) depth noise and Sobel
gradients (synthetic data; the reference names no dataset).

Metric: tracking frames/s (whole job, all ranks).  `value` runs with the
frames already resident in HBM; `e2e` runs the same steps through the C-ABI
with the frames in pinned host memory (host->device copy of rgb, depth and
both gradient images plus the pose read-back inside the timed region).

Multi-GPU: replicas only (every GPU tracks its own trajectory segment; no
collective on the data path); the elapsed time is the max over ranks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tracking frames/s & p99 latency, served+batched vs plain, 1 GB300, same pose err"
N_GAUSS = 1_000_000
ITERS = 20
ETA = 0.002


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_GAUSS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


# ----------------------------------------------------------------------------
# workload
# ----------------------------------------------------------------------------
def make_workload(sess, n_frames, seed):
    from f_vigs_slam_gb300 import synthetic as S

    cam = S.CAM_HD
    W, H, K = cam.width, cam.height, cam.intrinsics
    traj = S.trajectory(200, seed=seed)
    rng = np.random.default_rng(seed + 1)
    frames = []
    for k in range(n_frames):
        pose = traj[(k + 1) % len(traj)]
        col, dep, _, _ = sess.render(pose, K, W, H)
        rgb, d = S.add_noise(col, dep, rng)
        gx, gy = S.sobel3(rgb)
        frames.append(dict(rgb=rgb, depth=d, gx=gx, gy=gy, pose=pose, prev=traj[k % len(traj)]))
    return W, H, K, frames


class ClockSampler:
    """nvidia-smi clocks / throttle reasons every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_track_bytes(n_inst, W, H):
    """Algorithmic HBM bytes of one fused tracking launch: every instance's
    48-byte blending record read once, 40 B/pixel of observed rgb, depth and
    the two gradient images, 108 B per tile written."""
    T = ((W + 15) // 16) * ((H + 15) // 16)
    return 48 * n_inst + 40 * W * H + 108 * T


def algorithmic_bytes(cls, n_g, n_inst, W, H):
    """Per-launch algorithmic bytes of each kernel class."""
    P = W * H
    T = ((W + 15) // 16) * ((H + 15) // 16)
    return {
        "project": 64 * n_g + 84 * n_g,
        "scan": 8 * n_g,
        "emit": 36 * n_g + 12 * n_inst,
        "sort": 24 * n_inst,
        "ranges": 8 * n_inst + 8 * T,
        "track": algorithmic_track_bytes(n_inst, W, H),
        "map_fwd": 48 * n_inst + 16 * P + 40 * P,
        "map_bwd": 48 * n_inst + 52 * P + 52 * n_g,
        "map_update": (64 + 64 + 144) * n_g + (64 + 144) * n_g,
    }.get(cls)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def max_over_ranks(values, device, world):
    """Elapsed times are the max over ranks (the slowest replica bounds the job)."""
    if world <= 1:
        return list(values)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def replica_throughput(steps, world, max_ms):
    """Whole-job frames/s: every rank tracks `steps` frames of its own trajectory."""
    return steps * world / (max_ms / 1000.0)


# ----------------------------------------------------------------------------
# CPU baseline (the CPU restatement of the reference, FP64, all host threads)
# ----------------------------------------------------------------------------
def cpu_sample(n, band_rows=720, seed=0):
    """Time the oracle on a bounded sample of one frame: projection + tile
    counts of all N Gaussians, then keys / sort / tracking Jacobian / mapping
    step on a horizontal band of `band_rows` pixel rows through the image
    centre (intrinsics shifted so the band is the same pixels of the full
    frame).  Extrapolates one frame = 21 binnings + 20 Jacobians + 1 mapping
    step, with band costs scaled by H / band_rows."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from f_vigs_slam_gb300 import synthetic as S

    O.build()
    cam = S.CAM_HD
    W, H = cam.width, cam.height
    scene = S.room(n, seed=seed)
    traj = S.trajectory(3, seed=seed)
    pose, prev = traj[1], traj[0]
    P = O.default_params()
    band_rows = max(16, min(H, (band_rows // 16) * 16))
    y0 = ((H - band_rows) // 2 // 16) * 16
    K_band = (cam.fx, cam.fy, cam.cx, cam.cy - y0)
    # observed band: oracle render at the true pose over the band only
    b_true = O.prepare(scene, pose, K_band, W, band_rows, P)
    col, dep, _, _ = O.render(b_true, pose, K_band, W, band_rows, P)
    rng = np.random.default_rng(seed + 1)
    rgb, d = S.add_noise(col.astype(np.float32), dep.astype(np.float32), rng)
    gx, gy = S.sobel3(rgb)
    t0 = time.perf_counter()
    proj = O.project(scene, prev, cam.intrinsics, W, H)
    O.count(proj, W, H, P)
    t_proj = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = O.prepare(scene, prev, K_band, W, band_rows, P)
    t_bin_band_all = time.perf_counter() - t0
    t_bin_band = max(t_bin_band_all - t_proj, 0.0)
    t0 = time.perf_counter()
    O.track(b, (rgb, d, gx, gy), prev, K_band, W, band_rows, P, images=False)
    t_track = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.map_step(scene, b, rgb, d, prev, K_band, W, band_rows, P, ETA)
    t_map_all = time.perf_counter() - t0
    t_map = max(t_map_all - 0.0, 0.0)
    scale = H / band_rows
    frame_s = 21 * t_proj + scale * (21 * t_bin_band + ITERS * t_track + t_map)
    wall = t_proj + t_bin_band_all + t_track + t_map_all
    return dict(frame_s=frame_s, wall_s=wall, t_proj=t_proj, t_bin_band=t_bin_band, t_track=t_track, t_map=t_map,
                band_rows=band_rows, threads=os.cpu_count() or 1)


def run_reference(args):
    """CPU arm: the CPU restatement of the reference's path (FP64, all host
    threads), one bounded sample per step, extrapolated to frames/s."""
    rank, _, world = dist_info()
    if rank != 0:
        return 0
    budget_s = 180.0
    total = args.warmup + args.steps
    first = cpu_sample(args.n, band_rows=720, seed=0)
    rows = 720
    if first["wall_s"] * total > budget_s:
        rows = max(16, int(720 * budget_s / (first["wall_s"] * total)) // 16 * 16)
    samples = []
    for i in range(total):
        r = first if (i == 0 and rows == 720) else cpu_sample(args.n, band_rows=rows, seed=i % 3)
        if i >= args.warmup:
            samples.append(r)
    fs = [1.0 / r["frame_s"] for r in samples]
    v = float(np.median(fs))
    sample = ("per step: one binning (projection, counts, keys, stable sort, ranges) + one tracking Jacobian + one "
              "mapping step of %d Gaussians on %d of the 720 rows of a 1280x720 frame, extrapolated to 21 binnings "
              "+ 20 Jacobians + 1 mapping step per frame" % (args.n, samples[0]["band_rows"]))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "frames/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.median([r["wall_s"] for r in samples])),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "room N=%d, 1280x720, 20 GN iterations + 1 mapping step per frame" % args.n,
                   "path": "CPU restatement of the reference (FP64, OpenMP); the reference itself cannot be built "
                           "here (needs Eigen in device code, OpenCV-CUDA, Ceres, ROS 2)"},
        "cpu_baseline": {"value": v, "unit": "frames/s", "cores": samples[0]["threads"], "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
def run_ours(args):
    import torch

    from f_vigs_slam_gb300 import build as B

    B.build()
    from f_vigs_slam_gb300 import fvgs
    from f_vigs_slam_gb300 import synthetic as S

    rank, local_rank, world = dist_info()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)

    n_frames = args.warmup + args.steps
    scene = S.room(args.n, seed=0)
    sess = fvgs.Session(args.n, 1280, 720, device=local_rank)
    sess.set_stream(stream.cuda_stream)
    sess.upload(scene)
    W, H, K, frames = make_workload(sess, n_frames, seed=17 * rank)
    # device-resident frames for the `value` leg, pinned host frames for e2e
    dframes, hframes = [], []
    for f in frames:
        dframes.append({k: torch.from_numpy(np.ascontiguousarray(f[k])).to(dev) for k in ("rgb", "depth", "gx", "gy")})
        hframes.append({k: torch.from_numpy(np.ascontiguousarray(f[k])).pin_memory() for k in ("rgb", "depth", "gx", "gy")})
    torch.cuda.synchronize()

    def set_frame_ptr(fr):
        st = sess.lib.fvgs_set_frame(sess.h, 0, *(fvgs.C.c_void_p(fr[k].data_ptr()) for k in ("rgb", "depth", "gx", "gy")),
                                     W, H)
        if st != 0:
            raise fvgs.FvgsError(st, "fvgs_set_frame")

    def step(k, src):
        fr = src[k % len(src)]
        set_frame_ptr(fr)
        pose, _ = sess.track_frame(frames[k % len(frames)]["prev"], K, iterations=ITERS)
        sess.map_step(pose, K, ETA)
        return pose

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up (also grows the instance buffers to the workload's size)
    for k in range(args.warmup):
        step(k, dframes)
    torch.cuda.synchronize()
    # per-kernel-class CUDA-event times for the roofline and the shares, from
    # separate untimed frames (the events would otherwise sit in the timed region)
    sess.set_timing(fvgs.KERNEL_CLASSES)
    sess.get_timing(reset=True)
    for k in range(min(2, args.steps)):
        step(args.warmup + k, dframes)
    torch.cuda.synchronize()
    timing = sess.get_timing(reset=True)
    sess.set_timing(())

    clocks = ClockSampler(local_rank)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    step_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    errs = []
    ev0.record(stream)
    for i in range(args.steps):
        k = args.warmup + i
        step_ev[i][0].record(stream)
        pose = step(k, dframes)
        step_ev[i][1].record(stream)
        errs.append(S.pose_error(pose, frames[k % len(frames)]["pose"]))
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    lat = sorted(a.elapsed_time(b) for a, b in step_ev)
    # kernel launch counts are kept without events: these are the timed steps'
    timed_launches = sess.get_timing(reset=True)
    n_inst = int(sess.project_bin(frames[-1]["pose"], K, W, H))

    # e2e leg: pinned host frames through the C-ABI
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(args.steps):
        step(args.warmup + i, hframes)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    e2e_wall = (time.perf_counter() - t0) * 1000.0

    ms, e2e_ms = max_over_ranks([ms, e2e_ms], dev, world)
    value = replica_throughput(args.steps, world, ms)
    e2e_value = replica_throughput(args.steps, world, e2e_ms)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r = cpu_sample(args.n, band_rows=720, seed=0)
        cpu = {"value": 1.0 / r["frame_s"], "unit": "frames/s", "cores": r["threads"], "kind": "port",
               "sample": ("one binning + one tracking Jacobian + one mapping step of %d Gaussians on %d rows of "
                          "a 1280x720 frame (%.1f s of CPU work), extrapolated to one frame = 21 binnings + 20 "
                          "Jacobians + 1 mapping step" % (args.n, r["band_rows"], r["wall_s"]))}

    if rank == 0:
        dominant = max((c for c in timing if timing[c]["timed"]), key=lambda c: timing[c]["ms"])
        peak, peak_kind = load_peaks()
        per_launch_ms = timing[dominant]["ms"] / max(1, timing[dominant]["timed"])
        algo = algorithmic_bytes(dominant, args.n, n_inst, W, H)
        achieved = algo / (per_launch_ms / 1000.0) / 1e9
        traffic = load_traffic().get(dominant)
        gpu_launches = int(sum(v["launches"] for v in timed_launches.values()))
        shares = {c: round(v["ms"] / max(1e-9, sum(x["ms"] for x in timing.values())), 4)
                  for c, v in timing.items() if v["ms"] > 0}
        line = {
            "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "room N=%d, 1280x720, 16x16 tiles, 20 GN iterations + 1 mapping step per frame"
                                   % args.n,
                       "form": "plain per-frame GPU path", "parallelism": "replicas" if world > 1 else "single",
                       "l2": "not flushed: per-frame working set (instances %.0f MB + Gaussians %.0f MB) exceeds "
                             "the 129 MB L2" % (n_inst * 24 / 1e6, args.n * 64 / 1e6),
                       "instances_per_binning": n_inst},
            "p50_ms": lat[len(lat) // 2], "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
            "pose_error_median": {"rad": float(np.median([e[0] for e in errs])),
                                  "m": float(np.median([e[1] for e in errs]))},
            "e2e": {"value": e2e_value, "unit": "frames/s", "h2d_bytes_per_step": 40 * W * H,
                    "d2h_bytes_per_step": 160, "wall_ms": e2e_wall},
            "gpu_launches": gpu_launches,
            "kernel_share": shares,
            "roofline": {"kernel": dominant, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": algo, "ms_per_launch": per_launch_ms},
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    sess.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
