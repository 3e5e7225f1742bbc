#!/usr/bin/env python3
"""Benchmark: batched serving vs the plain one-session-per-launch path.

Workload ("serving mix"): 64 scanning sessions, each with its own seeded
synthetic scene (spheres/boxes on a ground plane, camera orbit of radius
0.9 m, Kinect-style axial noise, 1.5 % dropout in 8x8 blobs, depth cut at
2.5 m) and its own length drawn from U{50..500} frames.  Frame sizes cycle
through 320x240 (fx = fy = 285), 512x424 (fx = fy = 365) and 640x480
(fx = fy = 525); volumes are 128^3 to 512^3 int16 TSDF + uint16 weight over a
1.5 m cube (at most 512 MiB each), truncation max(2 cm, 5 voxels), ICP
10/5/4 iterations with 10 cm / 20 degree rejection, compensated (two-sum)
reduction.

A step is one batched pass of the whole pipeline (ingest, bilateral filter,
pyramid, input normal maps, ICP, integration, ray-cast of three levels) over
the frame of every session that is still running: step r carries frame r of
each session longer than r frames.  Every session is first advanced through
steps 0 .. D-1 untimed (the warm depth, --warm-depth, default 100 frames), so
the timed steps D .. D+K-1 (--steps K) run on volumes at mid-session fill.

  value      frames/s of the batched form over the K timed steps: frames
             resident in HBM, steps enqueued back to back, CUDA events on the
             launching stream.  A step's working set (up to 64 frames, the
             active sub-cubes of 64 volumes, 13 GB of volumes in all) is far
             larger than L2, so L2 is not flushed.
  e2e        the same steps through the C ABI with host frames
             (vs_batch_step_host: pinned uint16 frames in, poses out, every
             step); e2e_pageable the same from pageable host memory.
  plain      the same frames through the plain path, one session per launch
             (vs_scan_frame per frame, one graph per frame), from the same
             warm state.
  serving    open-loop Poisson arrivals through the serving loop (vs_server_*)
             at 2000 frames/s aggregate, host frames in, results polled out;
             latency = result on the host - scheduled arrival.  The plain path
             serves the same schedule first-come first-served, one frame per
             launch.
  serving_sustained
             the offered rate raised until p99 latency reaches 10 ms or the
             frames fall behind the arrivals, for the serving loop and for the
             plain path: the highest rate each sustains, and their ratio.
  ate        every session's camera trajectory against the FP64 oracle run of
             the same frames (all sessions, every frame of the timed steps),
             and the frames each side lost.

`--impl reference` times the CPU restatement of the reference's path (the
reference itself does not build on Linux) on the CPU sample that
`cpu_baseline` times, with all host threads; that process maps the oracle's
library only.  Under torchrun every rank runs its own copy of the workload
(sessions are independent: replicas, weak scaling); rank 0 prints the line.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "vcl-volume-scanner_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

MIX = dict(name="serving_mix_64", sessions=64, seed=5, length=(50, 500),
           sizes=[(320, 240, 285.0, 160.0, 120.0), (512, 424, 365.0, 255.5, 211.5), (640, 480, 525.0, 319.5, 239.5)],
           volumes=(128, 256, 384, 512), size_m=1.5, mu=0.02, mu_voxels=5.0, icp_iters=(10, 5, 4),
           th_icp=0.1 ** 2, normal_deg=20.0, dropout_blob=0.015, max_depth=2.5, arrival_fps=2000.0,
           hbm_budget_gb=150, p99_bound_ms=10.0,
           serving_rates=(2000, 4000, 6000, 7000, 8000, 8500, 9000, 9250, 9500, 10000, 11000, 12000, 14000, 16000),
           server_shapes=((3, 1), (1, 2)),
           plain_rates=(250, 500, 750, 1000, 1250, 1500, 1750, 2000, 2500))
CPU_SESSIONS = 3  # the CPU sample: sessions 0..2, one of each frame size


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="serving mix: timed batched steps after the warm depth (default 60); plain_vga: timed "
                         "frames (default 295); precision: frames (default 30)")
    ap.add_argument("--workload", default="serving_mix", choices=["serving_mix", "plain_vga"])
    ap.add_argument("--study", default=None, choices=["precision"])
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--warm-depth", type=int, default=100,
                    help="frames every session runs untimed before the timed steps")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sessions", type=int, default=MIX["sessions"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU baseline sample")
    ap.add_argument("--ref-seconds", type=float, default=240.0, help="budget of the reference arm")
    ap.add_argument("--serving-seconds", type=float, default=2.5, help="arrival span of one serving run")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ate", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    a = ap.parse_args()
    if a.steps is None:
        a.steps = 30 if a.study == "precision" else (295 if a.workload == "plain_vga" else 60)
    a.warmup = max(0, a.warmup)
    return a


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def session_specs(n, seed):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        w, h, f, cx, cy = MIX["sizes"][i % 3]
        dim = int(MIX["volumes"][int(rng.integers(0, len(MIX["volumes"])))])
        length = int(rng.integers(MIX["length"][0], MIX["length"][1] + 1))
        specs.append(dict(w=w, h=h, f=f, cx=cx, cy=cy, dim=dim, length=length, seed=1000 + seed * 100 + i))
    return specs


def session_mu(vox):
    """truncation of a session: 2 cm, or 5 voxels where that is more (the
    reference's own rule is 5 voxels, VCL_Volume_Scanner_View.cpp:423; at
    1.7 voxels, 2 cm in a 128^3 volume over 1.5 m, the ray-cast misses most of
    the thin first-frame band and tracking fails, in the oracle as here)"""
    return max(MIX["mu"], MIX["mu_voxels"] * float(vox))


def generate(spec, n_frames, oracle=False):
    """depth frames 0..n_frames-1, ground-truth poses and scene centre of a
    session; oracle=True uses the oracle library's copy of the generator (the
    same source, bit-identical frames), so a CPU-only run maps no library of
    the package"""
    if oracle:
        import oracle_py as M
    else:
        import vs_scanner as M
    sc = M.synth_config(spec["w"], spec["h"], fx=spec["f"], fy=spec["f"], cx=spec["cx"], cy=spec["cy"],
                        n_frames=max(1, int(n_frames)), seed=spec["seed"], dropout_blob=MIX["dropout_blob"],
                        max_depth=MIX["max_depth"])
    return M.synth_generate(sc)


def session_params(spec, centre):
    """every configuration value of a session (plain numbers)"""
    vox = float(np.float32(MIX["size_m"]) / np.float32(spec["dim"]))
    origin = [float(c) - MIX["size_m"] / 2.0 for c in np.asarray(centre, np.float64)]
    return dict(width=spec["w"], height=spec["h"], fx=spec["f"], fy=spec["f"], cx=spec["cx"], cy=spec["cy"],
                dim=(spec["dim"],) * 3, origin=origin, voxel_size=vox, mu=session_mu(vox), th_icp=MIX["th_icp"],
                cos_normal=float(np.cos(np.radians(MIX["normal_deg"]))), icp_iters=MIX["icp_iters"])


def make_config(spec, centre):
    import vs_scanner as V

    p = session_params(spec, centre)
    return V.default_config(p["width"], p["height"], fx=p["fx"], fy=p["fy"], cx=p["cx"], cy=p["cy"], dim=p["dim"],
                            origin=p["origin"], voxel_size=p["voxel_size"], mu=p["mu"], th_icp=p["th_icp"],
                            cos_normal=p["cos_normal"], icp_iters=p["icp_iters"], tsdf_type=V.VS_TSDF_INT16,
                            reduce_mode=V.VS_REDUCE_KAHAN)


def oracle_config(spec, centre, reduce_mode, tsdf_store):
    """the same session for the oracle: reduce_mode 0 / tsdf_store 0 is the
    reference's own arithmetic (its reduction tree, float TSDF), 3 / 0 the
    FP64 pipeline"""
    import oracle_py as O

    p = session_params(spec, centre)
    return O.make_config(p["width"], p["height"], p["fx"], p["fy"], p["cx"], p["cy"], p["dim"], p["origin"],
                         p["voxel_size"], p["mu"], th_icp=p["th_icp"], cos_normal=p["cos_normal"],
                         icp_iters=p["icp_iters"], tsdf_store=tsdf_store, reduce_mode=reduce_mode)


def frames_needed(spec, warm_depth, steps):
    return min(spec["length"], warm_depth + steps)


def build_workload(specs, warm_depth, steps):
    seqs = []
    for sp in specs:
        depth, gt, centre = generate(sp, frames_needed(sp, warm_depth, steps))
        seqs.append(dict(spec=sp, depth=depth, gt=gt, centre=centre, cfg=make_config(sp, centre)))
    return seqs


def config_json(args, specs, world):
    sizes, vols = {}, {}
    for sp in specs:
        k = "%dx%d" % (sp["w"], sp["h"])
        sizes[k] = sizes.get(k, 0) + 1
        k = "%d^3" % sp["dim"]
        vols[k] = vols.get(k, 0) + 1
    D, K = args.warm_depth, args.steps
    timed = sum(max(0, min(sp["length"], D + K) - D) for sp in specs)
    return {"workload": "%s: %d sessions, lengths U{%d..%d}, frame sizes %s, volumes %s int16+uint16 over %.1f m, "
                        "mu max(%.0f cm, %.0f voxels), ICP %d/%d/%d, 10 cm / 20 deg rejection, Poisson %.0f "
                        "frames/s aggregate, HBM budget %d GB; every session warmed untimed through frames 0..%d, "
                        "then %d timed steps (frames %d..%d)" % (
                            MIX["name"], len(specs), MIX["length"][0], MIX["length"][1], sizes, vols, MIX["size_m"],
                            MIX["mu"] * 100, MIX["mu_voxels"], *MIX["icp_iters"], MIX["arrival_fps"],
                            MIX["hbm_budget_gb"], D - 1, K, D, D + K - 1),
            "warm_depth_frames": D, "timed_frames": int(timed),
            "sessions_in_timed_steps": int(sum(1 for sp in specs if sp["length"] > D)),
            "sessions_per_gpu": len(specs), "parallelism": "replicas x%d" % world,
            "l2": "not flushed: a step's working set (up to 64 frames, active sub-cubes of 64 volumes) is far "
                  "above L2",
            "scene": "seeded synthetic spheres/boxes on a ground plane, orbit 0.9 m, session seeds 1000+%d*100+i"
                     % MIX["seed"]}


# ---------------------------------------------------------------------------
# measurement helpers
# ---------------------------------------------------------------------------
def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            v = float(json.load(f)["hbm_gbs"])
        return v, "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_unit(kernel_key, unit_key):
    """DRAM bytes (or warp instructions) per unit of work of a kernel, from
    the committed ncu summary (profiles/ncu_traffic.txt: `kernel key value ...`)"""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for line in open(p):
            parts = line.split()
            if len(parts) >= 3 and parts[0] == kernel_key and parts[1] == unit_key:
                return float(parts[2])
    except (OSError, ValueError):
        pass
    return None


def raycast_per_unit(key):
    """(per ray, per sub-cube) figure of the ray-cast stage's kernels from the
    committed ncu summary: the march-and-shade kernel per ray, the two passes
    of the band distance field per sub-cube; key "dram_bytes" or "warp_inst" """
    r = traffic_per_unit("k_ray_fused", key + "_per_ray")
    bx = traffic_per_unit("k_band_xy", key + "_per_brick")
    bz = traffic_per_unit("k_band_z", key + "_per_brick")
    if r is None or bx is None or bz is None:
        return None
    return r, bx + bz


def level_bricks(cfg):
    return (cfg.dim[0] // 8) * (cfg.dim[1] // 8) * (cfg.dim[2] // 8)


def level_pixels(cfg):
    return [(cfg.width >> l) * (cfg.height >> l) for l in range(cfg.levels)]


class ClockSampler:
    """nvidia-smi samples during the timed region"""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        # raw samples; the summary goes into the JSON line
        self.path = os.path.join(os.environ.get("VS_BENCH_CLOCKS_DIR", os.path.join(ROOT, "_bench")),
                                 "clocks_bench_%d.csv" % gpu_index)

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(value, world):
    """the largest value over the ranks of the job (gloo on CPU tensors, NCCL
    on the current CUDA device)"""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier_all(world):
    import torch

    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def pct(a, q):
    return float(np.percentile(np.asarray(a, np.float64), q)) if len(a) else None


def centres(poses):
    return np.array([-np.asarray(T, np.float64)[:3, :3].T @ np.asarray(T, np.float64)[:3, 3] for T in poses])


def set_omp_threads(n):
    try:
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(int(n))
    except OSError:
        pass


def arrival_schedule(counts, fps_total, seed):
    """(t, session index, frame) sorted by t: session i a Poisson stream of
    fps_total / len(counts) frames/s from t = 0, counts[i] frames"""
    rng = np.random.default_rng(seed)
    rate = fps_total / len(counts)
    ev = []
    for i, c in enumerate(counts):
        t = np.cumsum(rng.exponential(1.0 / rate, size=int(c)))
        ev += [(float(t[k]), i, k) for k in range(len(t))]
    ev.sort()
    return ev


# ---------------------------------------------------------------------------
# the CPU sample (cpu_baseline and the reference arm time the same frames)
# ---------------------------------------------------------------------------
def cpu_sample(args, threads, budget_s):
    """The oracle in the reference's own arithmetic (reduction tree, float
    TSDF) on sessions 0..2 of the mix (one of each frame size), round robin:
    frames 0..W-1 untimed (W = --warmup), then up to K rounds (--steps) of
    one frame per session, timed, within budget_s.  Maps the oracle's library
    only (frames from its copy of the generator)."""
    import oracle_py as O

    O.load()
    set_omp_threads(threads)
    specs = session_specs(max(args.sessions, CPU_SESSIONS), MIX["seed"])[:CPU_SESSIONS]
    W, K = args.warmup, args.steps
    sess = []
    for sp in specs:
        depth, _, centre = generate(sp, min(sp["length"], W + K), oracle=True)
        sess.append((O.Session(oracle_config(sp, centre, reduce_mode=0, tsdf_store=0)), depth))
    for k in range(W):
        for s, d in sess:
            if k < d.shape[0]:
                s.frame(d[k])
    rounds, frames, total = 0, 0, 0.0
    for k in range(W, W + K):
        t0 = time.perf_counter()
        n = 0
        for s, d in sess:
            if k < d.shape[0]:
                s.frame(d[k])
                n += 1
        if n == 0:
            break
        total += time.perf_counter() - t0
        rounds += 1
        frames += n
        if total > budget_s:
            break
    sample = ("sessions 0..%d of the serving mix (320x240 %d^3, 512x424 %d^3, 640x480 %d^3): frames 0..%d untimed, "
              "then %d rounds of one frame per session (frames %d..%d, %d frames, %.1f s); the oracle in the "
              "reference's arithmetic (its reduction tree, float TSDF), %d thread%s" % (
                  CPU_SESSIONS - 1, specs[0]["dim"], specs[1]["dim"], specs[2]["dim"], W - 1, rounds, W,
                  W + rounds - 1, frames, total, threads, "" if threads == 1 else "s"))
    return {"value": frames / total if total > 0 else 0.0, "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": sample, "rounds": rounds, "frames": frames, "seconds": total}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    cb = cpu_sample(args, threads, args.ref_seconds)
    specs = session_specs(args.sessions, MIX["seed"])
    line = {"impl": "reference", "metric": "frames/s", "value": cb["value"], "unit": "frames/s",
            "n_gpus": args.gpus, "steps": cb["rounds"], "warmup": args.warmup,
            "ms_per_step": 1000.0 * cb["seconds"] / max(1, cb["rounds"]), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_json(args, specs, world),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "a step is one frame of each of the %d sampled sessions" % CPU_SESSIONS}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# ATE against the FP64 oracle (spawned worker processes, one session each)
# ---------------------------------------------------------------------------
def _ate_worker_init():
    os.environ["OMP_NUM_THREADS"] = "1"


def _ate_worker(job):
    """oracle poses and tracked flags of one session over frames 0..n-1: the
    FP64 pipeline, or (job[2] = (reduction mode, TSDF storage)) the float
    pipeline with those arithmetic choices; (2, 1), compensated sums and int16
    TSDF, are the benchmark's own"""
    spec, n = job[0], job[1]
    variant = job[2] if len(job) > 2 else None
    fp32 = variant is not None
    import oracle_py as O

    O.load()
    set_omp_threads(1)
    depth, gt, centre = generate(spec, n, oracle=True)
    if fp32:
        s = O.Session(oracle_config(spec, centre, reduce_mode=variant[0], tsdf_store=variant[1]), f64=False)
    else:
        s = O.Session(oracle_config(spec, centre, reduce_mode=3, tsdf_store=0), f64=True)
    poses, tracked = [], []
    for k in range(n):
        tracked.append(bool(s.frame(depth[k])))
        poses.append(s.pose().astype(np.float64) if fp32 else s.pose_f64())
    return np.array(poses), np.array(tracked), np.asarray(gt[:n])


def ate_all_sessions(specs, ours, ours_tracked, warm_depth, steps):
    """camera-centre error of every session's GPU trajectory (all frames
    0..D+K-1) against the FP64 oracle's, over the timed frames D..D+K-1
    (RMS per session, worst session, worst frame) and over all frames"""
    import multiprocessing as mp

    jobs = [(sp, len(ours[i])) for i, sp in enumerate(specs)]
    t0 = time.perf_counter()
    ctx = mp.get_context("spawn")
    pool = ctx.Pool(max(1, os.cpu_count() or 1), initializer=_ate_worker_init)
    ref = pool.map(_ate_worker, jobs, chunksize=1)
    dt = time.perf_counter() - t0
    per, worst, worst_i, worst_frame, all_rms = {}, 0.0, None, 0.0, 0.0
    lost_gpu, lost_oracle, sq, n_timed = {}, {}, 0.0, 0
    sq_each, n_each = {}, {}
    for i, sp in enumerate(specs):
        rp, rt, _ = ref[i]
        d = np.linalg.norm(centres(ours[i]) - centres(rp), axis=1) * 1e3
        win = d[warm_depth:]
        if win.size:
            n_timed += win.size
            sq += float(np.sum(win ** 2))
            sq_each[i], n_each[i] = float(np.sum(win ** 2)), win.size
            rms = float(np.sqrt(np.mean(win ** 2)))
            per["%d" % i] = round(rms, 5)
            if rms > worst:
                worst, worst_i = rms, i
            worst_frame = max(worst_frame, float(win.max()))
        all_rms = max(all_rms, float(np.sqrt(np.mean(d ** 2))))
        g_lost = [k for k, t in enumerate(ours_tracked[i]) if not t and k > 0]
        o_lost = [k for k, t in enumerate(rt) if not t and k > 0]
        if g_lost:
            lost_gpu["%d" % i] = g_lost[:20]
        if o_lost:
            lost_oracle["%d" % i] = o_lost[:20]
    rest = [i for i in sq_each if i != worst_i]
    out = {"vs_fp64_oracle_mm": worst, "pooled_rms_mm": float(np.sqrt(sq / max(1, n_timed))),
           "pooled_rms_mm_without_worst_session": float(np.sqrt(sum(sq_each[i] for i in rest) /
                                                                max(1, sum(n_each[i] for i in rest)))),
           "sessions_within_1mm": int(sum(1 for v in per.values() if v < 1.0)), "worst_frame_mm": worst_frame,
           "all_frames_worst_session_mm": all_rms, "sessions": len(per), "timed_frames_compared": int(n_timed),
           "per_session_rms_mm": per, "sessions_with_lost_frames": {"gpu": lost_gpu, "fp64_oracle": lost_oracle},
           "oracle_seconds": dt, "oracle_workers": os.cpu_count() or 1,
           "note": "RMS of camera-centre differences over frames %d..%d of every session running then (both "
                   "trajectories start at the identity); the FP64 oracle runs every frame from frame 0" %
                   (warm_depth, warm_depth + steps - 1)}
    if worst_i is not None:
        # how sensitive that session is: the float oracle, run step by step in
        # every combination of the reference's arithmetic choices (reduction:
        # the reference's tree, plain, compensated, FP64 sums; TSDF: float,
        # int16), against the FP64 one, and the FP64 pipeline against the
        # generator's ground truth.  A session whose float variants spread
        # over more than the 1 mm bound bifurcates: the rounding of any float
        # implementation decides which way its trajectory goes.
        n_w = len(ours[worst_i])
        variants = [(rm, ts) for rm in (0, 1, 2, 3) for ts in (0, 1)]
        fl = pool.map(_ate_worker, [(specs[worst_i], n_w, v) for v in variants], chunksize=1)
        rp = ref[worst_i][0]
        gt = fl[0][2]
        spread = {}
        for v, (fp, _, _) in zip(variants, fl):
            dfl = np.linalg.norm(centres(fp) - centres(rp), axis=1)[warm_depth:] * 1e3
            spread["%s_%s" % (("reference_tree", "plain", "compensated", "fp64_sums")[v[0]],
                              ("float", "int16")[v[1]])] = round(float(np.sqrt(np.mean(dfl ** 2))), 4)
        dgt = np.linalg.norm(centres(rp) - centres(gt), axis=1) * 1e3
        out["worst_session"] = {"session": worst_i, "size": "%dx%d" % (specs[worst_i]["w"], specs[worst_i]["h"]),
                                "volume": specs[worst_i]["dim"], "gpu_rms_mm": worst,
                                "fp32_oracle_vs_fp64_rms_mm": spread["compensated_int16"],
                                "float_oracle_variants_vs_fp64_rms_mm": spread,
                                "float_variants_beyond_1mm": int(sum(1 for x in spread.values() if x >= 1.0)),
                                "fp64_vs_ground_truth_rms_mm": float(np.sqrt(np.mean(dgt ** 2)))}
    pool.close()
    pool.join()
    return out


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def stage_bytes(cfg, st):
    """algorithmic bytes per frame and stage (st: active sub-cubes, voxels updated)"""
    W, H = cfg.width, cfg.height
    lv = [(W >> l) * (H >> l) for l in range(3)]
    it = MIX["icp_iters"]
    return {"filter": 6.0 * W * H + sum(lv[l] * (4 + 4 + 32) for l in range(3)),
            "track": sum(28.0 * lv[l] * it[l] for l in range(3)),
            "integrate": 4.0 * 512 * st[0] + 4.0 * st[1] + 2.0 * W * H + 8.0 * st[0],
            "raycast": 28.0 * sum(lv)}


def run_ours(args):
    import torch

    import vs_scanner as V

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        barrier_all(world)

    D, K = args.warm_depth, args.steps
    specs = session_specs(args.sessions, MIX["seed"])
    t_gen = time.perf_counter()
    seqs = build_workload(specs, D, K)
    t_gen = time.perf_counter() - t_gen
    n_s = len(seqs)
    avail = [s["depth"].shape[0] for s in seqs]
    frames_dev = [torch.from_numpy(s["depth"].view(np.int16)).cuda() for s in seqs]
    pinned = [torch.from_numpy(s["depth"].view(np.int16)).pin_memory() for s in seqs]
    host = [p.numpy().view(np.uint16) for p in pinned]
    pageable = [s["depth"] for s in seqs]
    st = torch.cuda.Stream()

    sessions = [V.Session(s["cfg"]) for s in seqs]
    batch = V.Batch()
    members = [[i for i in range(n_s) if avail[i] > r] for r in range(D + K)]
    handles = [[sessions[i] for i in m] for m in members]
    ptrs = [[frames_dev[i][r].data_ptr() for i in m] for r, m in enumerate(members)]
    window = [r for r in range(D, D + K) if members[r]]
    n_frames = int(sum(len(members[r]) for r in window))
    if not window:
        raise SystemExit("no session runs past the warm depth %d" % D)

    # ---- warm-up: graph capture and first launches on throwaway sessions ----
    n_warm = min(16, n_s)
    warm = [V.Session(seqs[i]["cfg"]) for i in range(n_warm)]
    for k in range(args.warmup):
        batch.step(warm, [frames_dev[i][min(k, avail[i] - 1)].data_ptr() for i in range(n_warm)], st.cuda_stream)
    batch.sync()
    # autotuner: launch shapes, timed on the warm-up sessions
    tuned = None
    if not args.no_autotune:
        shape, ms = batch.autotune(warm, reps=3)
        tuned = {"ray_tile": "%dx%d" % (1 << shape[0], 32 >> shape[0]), "march_blocks_per_sm": shape[1],
                 "shade_blocks_per_sm": shape[2], "bilateral_tile": "32x%d" % shape[3],
                 "integrate_blocks_per_sm": shape[4] or "all resident", "raycast_ms_warm_sessions": ms}
    for w in warm:
        w.close()

    def warm_state():
        """every session reset and advanced through steps 0..D-1 (untimed)"""
        for s in sessions:
            s.reset()
        for r in range(D):
            if members[r]:
                batch.step(handles[r], ptrs[r], st.cuda_stream)
        batch.sync()

    # ---- batched form, device-resident frames: the timed region ----
    warm_state()
    clk = ClockSampler(local)
    barrier()
    clk.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(window) + 1)]
    # VS_BENCH_NVTX=1 marks the timed steps as an NVTX range (for profilers
    # that filter on it, e.g. ncu --nvtx --nvtx-include "timed_steps/")
    nvtx = os.environ.get("VS_BENCH_NVTX") == "1"
    if nvtx:
        torch.cuda.nvtx.range_push("timed_steps")
    t_wall = time.perf_counter()
    ev[0].record(st)
    for j, r in enumerate(window):
        batch.step(handles[r], ptrs[r], st.cuda_stream)
        ev[j + 1].record(st)
    st.synchronize()
    if nvtx:
        torch.cuda.nvtx.range_pop()
    t_wall = time.perf_counter() - t_wall
    barrier()
    clocks = clk.stop()
    step_ms = np.array([ev[j].elapsed_time(ev[j + 1]) for j in range(len(window))])
    total_ms = max_over_ranks(float(ev[0].elapsed_time(ev[-1])), world)
    fps_batched = world * n_frames / (total_ms / 1000.0)
    kps = batch.kernels_per_step()
    final_batched = [s.pose()[1] for s in sessions]

    # ---- stage breakdown of the same steps (separate, synchronous pass) ----
    warm_state()
    batch.set_stage_timing(True)
    stage_steps = window[:20]
    stage = np.zeros((len(stage_steps), 4))
    alg = {k: 0.0 for k in ("filter", "track", "integrate", "raycast")}
    for j, r in enumerate(stage_steps):
        batch.step(handles[r], ptrs[r], st.cuda_stream)
        batch.sync()
        stage[j] = batch.stage_times()
        for i in members[r]:
            fs = sessions[i].frame_stats()
            for k, v in stage_bytes(seqs[i]["cfg"], fs).items():
                alg[k] += v
    batch.set_stage_timing(False)
    names = ["filter", "track", "integrate", "raycast"]
    stage_sum = stage.sum(axis=0)
    stage_mean = stage.mean(axis=0)

    # ---- e2e: the same steps with host frames through the C ABI ----
    def e2e_pass(frames_host, record):
        for s in sessions:
            s.reset()
        batch.sync()
        for r in range(D):
            if members[r]:
                T, tr = batch.step_host(handles[r], [frames_host[i][r] for i in members[r]])
                if record is not None:
                    for j, i in enumerate(members[r]):
                        record[0][i].append(T[j].astype(np.float64))
                        record[1][i].append(bool(tr[j]))
        barrier()
        t0 = time.perf_counter()
        for r in window:
            T, tr = batch.step_host(handles[r], [frames_host[i][r] for i in members[r]])
            if record is not None:
                for j, i in enumerate(members[r]):
                    record[0][i].append(T[j].astype(np.float64))
                    record[1][i].append(bool(tr[j]))
        return max_over_ranks(time.perf_counter() - t0, world)

    traj = ([[] for _ in range(n_s)], [[] for _ in range(n_s)])
    e2e_s = e2e_pass(host, traj)
    fps_e2e = world * n_frames / e2e_s
    e2e_pageable_s = e2e_pass(pageable, None)
    h2d = int(round(sum(host[i][0].nbytes for r in window for i in members[r]) / len(window)))
    d2h = 64 * 80  # pose heads of every slot, one copy per step

    # ---- plain path: one session per launch, same frames, same warm state ----
    warm_state()
    torch.cuda.synchronize()
    pev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    barrier()
    pev[0].record(st)
    with torch.cuda.stream(st):
        for r in window:
            for i in members[r]:
                sessions[i].scan_frame(frames_dev[i][r].data_ptr(), st.cuda_stream)
    pev[1].record(st)
    st.synchronize()
    plain_ms = max_over_ranks(float(pev[0].elapsed_time(pev[1])), world)
    fps_plain = world * n_frames / (plain_ms / 1000.0)
    # the batched and plain runs of every session end on the same FP64 pose
    plain_equal = all(np.array_equal(sessions[i].pose()[1], final_batched[i]) for i in range(n_s))

    # ---- serving: open-loop Poisson arrivals ----
    serving = plain_serving = sustained = None
    if not args.no_serving:
        for s in sessions:
            s.reset()
        torch.cuda.synchronize()
        # a failure here is reported in the line, not allowed to lose the
        # timed results above
        try:
            sustained = serving_sweeps(V, seqs, host, sessions, args.serving_seconds)
            serving = sustained.pop("at_2000", None)
            plain_serving = sustained.pop("plain_at_2000", None)
        except Exception as e:  # noqa: BLE001
            sustained = {"error": "%s: %s" % (type(e).__name__, e)}
    batch.close()
    for s in sessions:
        s.close()
    del frames_dev
    torch.cuda.empty_cache()

    if rank != 0:
        return
    peak, peak_kind = measured_peak_hbm()
    dom_i = int(np.argmax(stage_sum))
    dom = names[dom_i]
    achieved = {k: alg[k] / (stage_sum[names.index(k)] * 1e-3) / 1e9 for k in names}
    kernel_key = {"integrate": "k_integrate", "raycast": "k_band_xy+k_band_z+k_ray_fused", "track": "k_icp_iter",
                  "filter": "k_bilateral_batch"}[dom]
    # measured DRAM bytes of one step of the stage: per-unit figures of the
    # committed ncu captures times this workload's units per step
    rays = np.mean([sum(sum(level_pixels(seqs[i]["cfg"])) for i in members[r]) for r in stage_steps])
    bricks = np.mean([sum(level_bricks(seqs[i]["cfg"]) for i in members[r]) for r in stage_steps])
    traffic = None
    if dom == "raycast":
        pu = raycast_per_unit("dram_bytes")
        if pu is not None:
            traffic = pu[0] * rays + pu[1] * bricks
    elif dom == "track":
        px = traffic_per_unit("k_icp_iter", "dram_bytes_per_pixel")
        if px is not None:
            traffic = px * np.mean([sum(sum(p * it for p, it in zip(level_pixels(seqs[i]["cfg"]), MIX["icp_iters"]))
                                        for i in members[r]) for r in stage_steps])
    roofline = {"bound": "hbm", "kernel": kernel_key, "stage": dom,
                "achieved": achieved[dom], "peak": peak, "unit": "GB/s", "frac": achieved[dom] / peak,
                "traffic": traffic,
                "traffic_note": "DRAM bytes per step: bytes per unit from profiles/ncu_traffic.txt x units per step "
                                "(%.0f rays, %.0f sub-cubes)" % (rays, bricks),
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
                "fallback 6800 GB/s",
                "note": "algorithmic bytes of the stage per step (the first %d timed steps) / its event-timed "
                        "duration; the ray-cast is issue-bound, not HBM-bound (see profiles/)" % len(stage_steps),
                "algorithmic_bytes_per_step": alg[dom] / len(stage_steps),
                "stages_gbs": achieved, "stages_frac": {k: v / peak for k, v in achieved.items()}}
    if dom == "raycast":
        # the ray-cast's own bound is instruction issue: warp instructions per
        # ray from the committed ncu captures times this workload's rays, over
        # the event-timed stage, against one warp instruction per scheduler per
        # cycle (4 per SM) at the SM clock sampled during the timed region
        pu = raycast_per_unit("warp_inst")
        mhz = (clocks or {}).get("sm_mhz")
        if pu is not None and mhz:
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            got = (pu[0] * rays + pu[1] * bricks) / (stage_sum[dom_i] / len(stage_steps) * 1e-3)
            top = 4.0 * sms * mhz * 1e6
            roofline["issue"] = {"achieved": got, "peak": top, "unit": "warp instructions/s", "frac": got / top,
                                 "warp_inst_per_ray": pu[0], "warp_inst_per_subcube": pu[1],
                                 "note": "warp instructions per ray and per sub-cube from profiles/ncu_traffic.txt x "
                                         "%.0f rays and %.0f sub-cubes per step / the stage's event time; peak = 4 x "
                                         "%d SMs x %.0f MHz" % (rays, bricks, sms, mhz)}

    cpu = ate = None
    if not args.no_cpu:
        try:
            cb = cpu_sample(args, 1, args.cpu_seconds)
            cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        except Exception as e:  # noqa: BLE001
            cpu = {"error": "%s: %s" % (type(e).__name__, e)}
    if not args.no_ate:
        try:
            ate = ate_all_sessions(specs, traj[0], traj[1], D, K)
        except Exception as e:  # noqa: BLE001
            ate = {"error": "%s: %s" % (type(e).__name__, e)}

    line = {"metric": "frames/s", "value": fps_batched, "unit": "frames/s", "n_gpus": world, "steps": len(window),
            "warmup": args.warmup, "ms_per_step": float(step_ms.mean()), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_json(args, specs, world),
            "frames_per_step": n_frames / len(window),
            "step_ms": {"p50": pct(step_ms, 50), "p99": pct(step_ms, 99), "max": float(step_ms.max())},
            "plain": {"value": fps_plain, "unit": "frames/s", "ms": plain_ms,
                      "note": "one session per launch (vs_scan_frame), same frames and warm state, device-resident",
                      "final_poses_equal_batched": bool(plain_equal)},
            "batched_over_plain": fps_batched / fps_plain,
            "serving": serving, "plain_serving": plain_serving, "serving_sustained": sustained,
            "stages_ms_per_step": {n_: float(v) for n_, v in zip(names, stage_mean)},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": fps_e2e, "unit": "frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "note": "vs_batch_step_host per step: pinned host frames in (read over the host link by the step's "
                             "first kernel), pose heads out"},
            "e2e_pageable": {"value": world * n_frames / e2e_pageable_s, "unit": "frames/s",
                             "note": "the same from pageable host frames"},
            "gpu_launches": int(kps * len(window)),
            "autotune": tuned,
            "clocks": clocks,
            "ate": ate,
            "tracked_last_frame": int(sum(1 for i in range(n_s) if traj[1][i] and traj[1][i][-1])),
            "generation_s": t_gen, "wall_s_timed_region": t_wall}
    print(json.dumps(line), flush=True)


def run_serving(V, seqs, host, rate, span_s, seed, **server_kw):
    """open-loop arrivals through vs_server at `rate` frames/s aggregate for
    about span_s seconds (every session a Poisson stream of rate / n frames/s
    from its frame 0); latency from the scheduled arrival"""
    n = len(seqs)
    counts = [min(h.shape[0] - 1, max(4, int(math.ceil(rate * span_s / n)))) for h in host]
    sched = [(t, i, k + 1) for t, i, k in arrival_schedule(counts, rate, seed)]
    srv = V.Server(hbm_budget=MIX["hbm_budget_gb"] << 30, **server_kw)
    ids = [srv.open(s["cfg"]) for s in seqs]
    # frame 0 of every session first, untimed: the runners capture their
    # graphs on their first steps
    for i, sid in enumerate(ids):
        while not srv.submit(sid, host[i][0]):
            time.sleep(0.0002)
    srv.drain()
    while srv.poll(timeout_ms=0):
        pass
    results = []
    done = threading.Event()

    def poller():
        while not done.is_set():
            results.extend(srv.poll(timeout_ms=50))
        while True:
            got = srv.poll(timeout_ms=0)
            if not got:
                break
            results.extend(got)

    th = threading.Thread(target=poller)
    th.start()
    t0 = srv.clock() + 0.05
    busy = 0
    try:
        for t, i, k in sched:
            while True:
                now = srv.clock()
                if now >= t0 + t:
                    break
                time.sleep(min(0.0005, t0 + t - now))
            while not srv.submit(ids[i], host[i][k]):
                busy += 1
                time.sleep(0.0002)
        srv.drain()
    finally:
        done.set()
        th.join()
    stats = srv.stats()
    srv.close()
    index = {sid: i for i, sid in enumerate(ids)}
    arr = {(i, k): t0 + t for t, i, k in sched}
    lat = [1000.0 * (r["t_done"] - arr[(index[r["session"]], r["frame"])]) for r in results]
    t_first = t0 + sched[0][0]
    t_last = max(r["t_done"] for r in results)
    span_arr = sched[-1][0] - sched[0][0]
    return {"offered_fps": rate, "offered_fps_mean": len(sched) / span_arr, "frames": len(results),
            "achieved_fps": len(results) / (t_last - t_first), "span_s": t_last - t_first,
            "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "max_ms": float(max(lat)),
            "mean_batch": stats["mean_batch"], "max_batch": stats["max_batch_seen"], "steps": stats["steps"],
            "submit_retries": busy, "sessions_admitted": len(ids),
            "hbm_resident_gb": stats["bytes_resident"] / 2 ** 30 if stats["bytes_resident"] else None}


def run_plain_serving(sessions, host, rate, span_s, seed):
    """the same kind of arrivals served first-come first-served, one frame per
    launch (vs_scan_frame_host), after the same untimed frame 0 of every
    session"""
    n = len(sessions)
    counts = [min(h.shape[0] - 1, max(4, int(math.ceil(rate * span_s / n)))) for h in host]
    sched = [(t, i, k + 1) for t, i, k in arrival_schedule(counts, rate, seed)]
    for i, s in enumerate(sessions):
        s.reset()
        s.scan_frame_host(host[i][0])
    lat = []
    t0 = time.perf_counter() + 0.05
    for t, i, k in sched:
        now = time.perf_counter()
        if now < t0 + t:
            time.sleep(t0 + t - now)
        sessions[i].scan_frame_host(host[i][k])
        lat.append(1000.0 * (time.perf_counter() - (t0 + t)))
    span = time.perf_counter() - (t0 + sched[0][0])
    span_arr = sched[-1][0] - sched[0][0]
    return {"offered_fps": rate, "offered_fps_mean": len(sched) / span_arr, "frames": len(lat),
            "achieved_fps": len(lat) / span, "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "max_ms": float(max(lat))}


def sustains(r):
    return r["p99_ms"] < MIX["p99_bound_ms"] and r["achieved_fps"] >= 0.95 * r["offered_fps_mean"]


def serving_sweeps(V, seqs, host, sessions, span_s):
    """offered rate raised until p99 reaches 10 ms or the results fall behind
    the arrivals, for the serving loop and for the plain path"""
    out = {"p99_bound_ms": MIX["p99_bound_ms"], "criterion": "p99 < %.0f ms and achieved >= 0.95 x offered" %
           MIX["p99_bound_ms"], "span_s": span_s,
           "note": "each run opens the 64 sessions, runs frame 0 of each untimed, then Poisson arrivals of frames 1.."}
    best, out["batched"] = None, {}
    for lanes, pipeline in MIX["server_shapes"]:
        runs, top = [], None
        for k, rate in enumerate(MIX["serving_rates"]):
            r = run_serving(V, seqs, host, float(rate), span_s, MIX["seed"] + 17 + k, lanes=lanes, pipeline=pipeline)
            r["lanes"], r["pipeline"] = lanes, pipeline
            runs.append(r)
            if rate == MIX["arrival_fps"] and (lanes, pipeline) == tuple(MIX["server_shapes"][0]):
                out["at_2000"] = r
            if not sustains(r):
                break
            top = r
        out["batched"]["lanes%d_pipeline%d" % (lanes, pipeline)] = runs
        if top and (best is None or top["achieved_fps"] > best["achieved_fps"]):
            best = top
    prun, pbest = [], None
    for k, rate in enumerate(MIX["plain_rates"]):
        r = run_plain_serving(sessions, host, float(rate), span_s, MIX["seed"] + 117 + k)
        prun.append(r)
        if rate == MIX["arrival_fps"]:
            out["plain_at_2000"] = r
        if not sustains(r):
            break
        pbest = r
    if "plain_at_2000" not in out:
        out["plain_at_2000"] = run_plain_serving(sessions, host, MIX["arrival_fps"], span_s, MIX["seed"] + 17)
    out["plain"] = prun
    out["sustained_fps"] = best["achieved_fps"] if best else None
    out["sustained_offered_fps"] = best["offered_fps"] if best else None
    out["sustained_server"] = {"lanes": best["lanes"], "pipeline": best["pipeline"]} if best else None
    out["plain_sustained_fps"] = pbest["achieved_fps"] if pbest else None
    out["plain_sustained_offered_fps"] = pbest["offered_fps"] if pbest else None
    out["ratio_over_plain"] = (best["achieved_fps"] / pbest["achieved_fps"]) if best and pbest else None
    return out


# ---------------------------------------------------------------------------
# --workload plain_vga: one session, 640x480, 512^3
# ---------------------------------------------------------------------------
VGA = dict(name="plain_vga_512", width=640, height=480, fx=525.0, fy=525.0, cx=319.5, cy=239.5, volume=512,
           size_m=1.5, mu=0.02, icp_iters=(10, 5, 4), th_icp=0.1 ** 2, normal_deg=20.0, dropout_blob=0.015,
           max_depth=2.5, seed=2)
L2_FLUSH_BYTES = 256 << 20


def vga_frames(n):
    import vs_scanner as V

    w = VGA
    sc = V.synth_config(w["width"], w["height"], fx=w["fx"], fy=w["fy"], cx=w["cx"], cy=w["cy"], n_frames=n,
                        seed=w["seed"], dropout_blob=w["dropout_blob"], max_depth=w["max_depth"])
    return V.synth_generate(sc)


def vga_config(centre):
    import vs_scanner as V

    w = VGA
    origin, vox = V.cube_around(centre, w["size_m"], w["volume"])
    return V.default_config(w["width"], w["height"], fx=w["fx"], fy=w["fy"], cx=w["cx"], cy=w["cy"],
                            dim=(w["volume"],) * 3, origin=origin, voxel_size=vox, mu=w["mu"], th_icp=w["th_icp"],
                            cos_normal=float(np.cos(np.radians(w["normal_deg"]))), icp_iters=w["icp_iters"],
                            tsdf_type=V.VS_TSDF_INT16, reduce_mode=V.VS_REDUCE_KAHAN)


def vga_config_json(args, world):
    w = VGA
    return {"workload": "%s: 1 session, %dx%d uint16 depth, %d^3 int16+uint16 TSDF over %.1f m, mu %.0f cm, "
                        "ICP %d/%d/%d, 10 cm / 20 deg rejection" % (
                            w["name"], w["width"], w["height"], w["volume"], w["size_m"], w["mu"] * 100,
                            *w["icp_iters"]),
            "frames": args.steps, "sessions_per_gpu": 1, "parallelism": "replicas x%d" % world,
            "l2": "flushed between frames (256 MB write outside the timed events)",
            "scene": "seeded synthetic spheres/boxes on a ground plane, orbit 0.9 m, seed %d" % w["seed"]}


def run_plain_vga_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle_py as O

    n_threads = os.cpu_count() or 1
    O.load()
    set_omp_threads(n_threads)
    warm = min(args.warmup, 3)
    depth, gt, centre = vga_frames(warm + args.steps)
    s = O.Session(O.config_from_vs(vga_config(centre), reduce_mode=0))
    for k in range(warm):
        s.frame(depth[k])
    times = []
    t_start = time.perf_counter()
    for k in range(warm, warm + args.steps):
        t0 = time.perf_counter()
        s.frame(depth[k])
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > args.ref_seconds:
            break
    total = sum(times)
    fps = len(times) / total
    sample = "%d frames of the VGA sequence after %d warm-up frames, oracle port (reference FP32 semantics), " \
             "%d threads" % (len(times), warm, n_threads)
    print(json.dumps({"impl": "reference", "metric": "frames/s", "value": fps, "unit": "frames/s",
                      "n_gpus": args.gpus, "steps": len(times), "warmup": warm, "ms_per_step": 1000.0 * total / len(times),
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                      "data": "synthetic", "config": vga_config_json(args, 1),
                      "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": n_threads, "kind": "port",
                                       "sample": sample},
                      "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


def run_plain_vga(args):
    import torch

    import vs_scanner as V

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    depth, gt, centre = vga_frames(args.warmup + args.steps)
    cfg = vga_config(centre)
    frames_dev = torch.from_numpy(depth.view(np.int16)).cuda()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()
    sess = V.Session(cfg)
    sess.set_stage_timing(True)
    with torch.cuda.stream(st):
        for k in range(args.warmup):
            flush.zero_()
            sess.scan_frame(frames_dev[k].data_ptr(), st.cuda_stream)
    st.synchronize()
    clk = ClockSampler(local)
    barrier_all(world)
    clk.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stage = np.zeros((args.steps, 4))
    stats = np.zeros((args.steps, 4))
    with torch.cuda.stream(st):
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(st)
            sess.scan_frame(frames_dev[args.warmup + i].data_ptr(), st.cuda_stream)
            ev[i][1].record(st)
            stage[i] = sess.stage_times()
            stats[i] = sess.frame_stats()
    st.synchronize()
    barrier_all(world)
    clocks = clk.stop()
    frame_ms = np.array([a.elapsed_time(b) for a, b in ev])
    total_ms = max_over_ranks(float(frame_ms.sum()), world)
    fps = world * args.steps / (total_ms / 1000.0)
    kpf = sess.kernels_per_frame()
    # end to end: host frames through vs_scan_frame_host
    sess.set_stage_timing(False)
    sess.reset()
    host = torch.from_numpy(depth.view(np.int16)).pin_memory().numpy().view(np.uint16)
    for k in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        sess.scan_frame_host(host[k])
    e2e_t, poses = [], []
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        T, _ = sess.scan_frame_host(host[args.warmup + i])
        e2e_t.append(time.perf_counter() - t0)
    e2e_fps = world * args.steps / max_over_ranks(sum(e2e_t), world)
    sess.close()
    if rank != 0:
        return
    names = ["filter", "track", "integrate", "raycast"]
    stage_mean = stage.mean(axis=0)
    peak, peak_kind = measured_peak_hbm()
    st_ = (stats[:, 0].mean(), stats[:, 1].mean())
    alg = stage_bytes(cfg, st_)
    dom = names[int(np.argmax(stage_mean))]
    achieved = {k: alg[k] / (stage_mean[names.index(k)] * 1e-3) / 1e9 for k in names}
    rays = sum(level_pixels(cfg))
    traffic = None
    if dom == "raycast":
        pu = raycast_per_unit("dram_bytes")
        if pu is not None:
            traffic = pu[0] * rays + pu[1] * level_bricks(cfg)
    elif dom == "track":
        px = traffic_per_unit("k_icp_iter", "dram_bytes_per_pixel")
        if px is not None:
            traffic = px * sum(p * it for p, it in zip(level_pixels(cfg), VGA["icp_iters"]))
    cpu = ate = None
    if not args.no_cpu:
        import oracle_py as O

        O.load()
        set_omp_threads(1)
        s = O.Session(O.config_from_vs(cfg, reduce_mode=0))
        n, t0 = 0, time.perf_counter()
        while n < depth.shape[0] and (time.perf_counter() - t0 < args.cpu_seconds or n < 2):
            s.frame(depth[n])
            n += 1
        dt = time.perf_counter() - t0
        cpu = {"value": n / dt, "unit": "frames/s", "cores": 1, "kind": "port",
               "sample": "first %d frames of the sequence (%.1f s), oracle port, reference FP32 semantics, 1 thread"
                         % (n, dt)}
        nf = min(n, args.ate_frames)
        set_omp_threads(os.cpu_count() or 1)
        s64 = O.Session(O.config_from_vs(cfg, reduce_mode=3, tsdf_store=0), f64=True)
        s2 = V.Session(cfg)
        ours, ref = [], []
        for k in range(nf):
            T, _ = s2.scan_frame_host(host[k])
            ours.append(T.astype(np.float64))
            s64.frame(depth[k])
            ref.append(s64.pose_f64())
        s2.close()
        d = np.linalg.norm(centres(ours) - centres(ref), axis=1)
        ate = {"vs_fp64_oracle_mm": float(np.sqrt(np.mean(d ** 2)) * 1e3), "frames": nf,
               "max_mm": float(d.max() * 1e3)}
    line = {"metric": "frames/s", "value": fps, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(frame_ms.mean()), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": vga_config_json(args, world),
            "latency_ms": {"p50": pct(frame_ms, 50), "p99": pct(frame_ms, 99), "max": float(frame_ms.max())},
            "stages_ms": {n_: float(v) for n_, v in zip(names, stage_mean)},
            "roofline": {"bound": "hbm", "kernel": {"raycast": "k_band_xy+k_band_z+k_ray_fused", "track": "k_icp_iter",
                                                    "integrate": "k_integrate", "filter": "k_bilateral_batch"}[dom],
                         "stage": dom, "achieved": achieved[dom], "peak": peak, "unit": "GB/s",
                         "frac": achieved[dom] / peak, "traffic": traffic,
                         "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
                         "fallback 6800 GB/s", "stages_gbs": achieved},
            "integrate": {"active_subcubes": st_[0], "voxels_updated": st_[1],
                          "achieved_gbs": achieved["integrate"], "frac": achieved["integrate"] / peak},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": cfg.width * cfg.height * 2,
                    "d2h_bytes_per_step": 80},
            "gpu_launches": int(kpf * args.steps), "clocks": clocks, "ate": ate}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# --study precision: reductions x TSDF storage against the FP64 oracle
# ---------------------------------------------------------------------------
def _solve_ldl_f64(A, b):
    """FP64 L D L^T solve of a 6x6 system (the device's solve, restated)"""
    n = 6
    L = np.eye(n)
    D = np.zeros(n)
    for j in range(n):
        D[j] = A[j, j] - np.sum(L[j, :j] ** 2 * D[:j])
        for i in range(j + 1, n):
            L[i, j] = (A[i, j] - np.sum(L[i, :j] * L[j, :j] * D[:j])) / D[j]
    y = np.zeros(n)
    for i in range(n):
        y[i] = b[i] - np.dot(L[i, :i], y[:i])
    z = y / D
    x = np.zeros(n)
    for i in reversed(range(n)):
        x[i] = z[i] - np.dot(L[i + 1:, i], x[i + 1:])
    return x


def _solve_f32_refined(A, b, steps=2):
    """float L D L^T factors with `steps` FP64 refinement steps (the device's
    previous solve, restated)"""
    A32 = A.astype(np.float32)
    n = 6
    L = np.eye(n, dtype=np.float32)
    D = np.zeros(n, np.float32)
    for j in range(n):
        D[j] = A32[j, j] - np.float32(np.sum((L[j, :j] ** 2 * D[:j]).astype(np.float32), dtype=np.float32))
        for i in range(j + 1, n):
            L[i, j] = (A32[i, j] - np.float32(np.sum(L[i, :j] * L[j, :j] * D[:j], dtype=np.float32))) / D[j]

    def fsolve(r):
        r = r.astype(np.float32)
        y = np.zeros(n, np.float32)
        for i in range(n):
            y[i] = r[i] - np.float32(np.dot(L[i, :i], y[:i]))
        z = y / D
        x = np.zeros(n, np.float32)
        for i in reversed(range(n)):
            x[i] = z[i] - np.float32(np.dot(L[i + 1:, i], x[i + 1:]))
        return x

    x = fsolve(b).astype(np.float64)
    for _ in range(steps):
        x = x + fsolve(b - A @ x).astype(np.float64)
    return x


def _device_inverse(T64):
    """the float camera-to-global pose a session integrates with: the rigid
    inverse of its FP64 pose in FP64, in the device's operation order,
    rounded to float (a float inversion of the float pose differs in the last
    bits, enough to move a sub-cube across the activation boundary)"""
    T = np.asarray(T64, np.float64)
    out = np.zeros((4, 4), np.float64)
    for r in range(3):
        for c in range(3):
            out[r, c] = T[c, r]
        out[r, 3] = -(float(T[0, r]) * float(T[0, 3]) + float(T[1, r]) * float(T[1, 3]) + float(T[2, r]) * float(T[2, 3]))
    out[3, 3] = 1.0
    return out.astype(np.float32)


def _rot_err(A, B):
    R = np.asarray(A, np.float64)[:3, :3].T @ np.asarray(B, np.float64)[:3, :3]
    w = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2.0
    return float(np.arctan2(np.linalg.norm(w), (np.trace(R) - 1.0) / 2.0))


def _trans_err(A, B):
    return float(np.linalg.norm(np.asarray(A, np.float64)[:3, 3] - np.asarray(B, np.float64)[:3, 3]))


def _system(sums):
    A = np.zeros((6, 6))
    k = 0
    for i in range(6):
        for j in range(i, 6):
            A[i, j] = A[j, i] = sums[k]
            k += 1
    return A, np.asarray(sums[21:27], np.float64)


def run_precision(args):
    """Configuration-1 workload (one 320x240 session, fx = fy = 285, cx = 160,
    cy = 120, 1 % dropout, ICP 10/5/4, mu 3 cm) with the TSDF in a 512^3 volume
    over 1 m.  Every reduction mode x every TSDF storage runs on the GPU,
    stage by stage.  Two kinds of error are reported for each variant:

    * per frame, on identical inputs (the tolerance): at every frame the FP64
      oracle's tracker takes the GPU session's own inputs (model maps,
      filtered pyramid, previous FP64 pose) and the GPU's pose is compared
      with its result.  The float oracle (the reference's own arithmetic)
      takes the same inputs too: where its pose and the FP64 one differ by
      more than 1e-5 rad / 0.01 mm the frame's solution is set by rounding
      (ICP stopped at its iteration cap with correspondences still flipping),
      and the tolerance is stated over the other, well-posed frames as well as
      over all of them; at sample frames the FP32 oracle integrates the frame
      into the GPU's own volume at the GPU's pose (TSDF error in int16 steps
      over the updated voxels) and ray-casts the GPU's volume (share of
      vertices within 1 mm of the GPU's);
    * end to end (drift): the GPU trajectory against the FP64 oracle pipeline
      run on the same frames from frame 0, and both against the generator's
      ground truth.

    The solve of every frame's last ICP system is checked against numpy's
    FP64 solve of the same sums (relative error, condition number), and on
    systems made ill-conditioned on purpose the device's FP64 L D L^T
    (restated) is compared with the float-factor-plus-two-refinements solve."""
    import oracle_py as O
    import torch
    import vs_scanner as V

    rank, world, _ = dist_env()
    if rank != 0:
        return
    nf = args.steps
    sc = V.synth_config(320, 240, fx=285.0, fy=285.0, cx=160.0, cy=120.0, n_frames=nf, seed=1, dropout_iid=0.01)
    depth, gt, centre = V.synth_generate(sc)
    origin, vox = V.cube_around(centre, 1.0, 512)
    sample = sorted(set([min(10, nf - 1), nf - 1]))

    def cfg_of(reduce_mode, tsdf_type):
        return V.default_config(320, 240, fx=285.0, fy=285.0, cx=160.0, cy=120.0, dim=(512,) * 3, origin=origin,
                                voxel_size=vox, mu=0.03, th_icp=0.1 ** 2, icp_iters=(10, 5, 4),
                                tsdf_type=tsdf_type, reduce_mode=reduce_mode)

    O.load()
    set_omp_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    ref = O.Session(O.config_from_vs(cfg_of(V.VS_REDUCE_FP64, V.VS_TSDF_FP32), reduce_mode=3, tsdf_store=0), f64=True)
    ref_poses = []
    for k in range(nf):
        ref.frame(depth[k])
        ref_poses.append(ref.pose_f64())
    t_oracle = time.perf_counter() - t0
    gt_c = centres([np.asarray(g) for g in gt])
    light = np.array([0, 0, -1], np.float32)

    def ate(a, b):
        d = np.linalg.norm(centres(a) - centres(b), axis=1)
        return float(np.sqrt(np.mean(d ** 2)) * 1e3)

    rows = []
    solve_err, solve_cond = [], []
    for rm, rname in ((V.VS_REDUCE_FP32, "fp32"), (V.VS_REDUCE_KAHAN, "two-sum fp32"), (V.VS_REDUCE_FP64, "fp64")):
        for tt, tname in ((V.VS_TSDF_INT16, "int16"), (V.VS_TSDF_FP16, "fp16"), (V.VS_TSDF_FP32, "fp32")):
            cfg = cfg_of(rm, tt)
            ocfg64 = O.config_from_vs(cfg, reduce_mode=3)
            ocfg32 = O.config_from_vs(cfg, reduce_mode=0, tsdf_store=0)
            s = V.Session(cfg)
            poses, rot, trans, tsdf_steps, ray_within, ray_agree = [], [], [], [], [], []
            floor_rot, floor_trans, wp_rot, wp_trans = [], [], [], []
            for k in range(nf):
                Tp, Tp64, _ = s.pose()
                mv = [s.maps(l)["model_vertex"] for l in range(3)]
                mn = [s.maps(l)["model_normal"] for l in range(3)]
                d = torch.from_numpy(np.ascontiguousarray(depth[k]).view(np.int16)).cuda()
                s.stage_filter(d.data_ptr())
                s.stage_track()
                T, T64, info = s.pose()
                if k > 0 and info[0]:
                    ind = [s.maps(l)["input_depth"] for l in range(3)]
                    ok, dT, _ = O.track(ocfg64, ind, mv, mn, Tp64, f64=True)
                    # the same inputs through the float oracle (the reference's
                    # own arithmetic): how far FP32 rounding alone moves this
                    # frame's solution
                    ok32, fT, _ = O.track(ocfg32, ind, mv, mn, Tp, f64=False)
                    if ok and ok32:
                        r_, t_ = _rot_err(T64, dT), _trans_err(T64, dT) * 1e3
                        rot.append(r_)
                        trans.append(t_)
                        rf, tf = _rot_err(fT, dT), _trans_err(fT, dT) * 1e3
                        floor_rot.append(rf)
                        floor_trans.append(tf)
                        if rf < 1e-5 and tf < 1e-2:
                            wp_rot.append(r_)
                            wp_trans.append(t_)
                    sums, x = s.icp_system()
                    A, b = _system(sums)
                    if sums[27] > 0:
                        xr = np.linalg.solve(A, b)
                        solve_err.append(float(np.linalg.norm(x.astype(np.float64) - xr) /
                                               max(np.linalg.norm(xr), 1e-30)))
                        solve_cond.append(float(np.linalg.cond(A)))
                before = s.volume() if k in sample else None
                s.stage_integrate()
                s.stage_raycast()
                s.sync()
                poses.append(s.pose()[1])
                if before is not None:
                    Tg = np.ascontiguousarray(s.pose()[0], np.float32)
                    Tc = _device_inverse(s.pose()[1])
                    vol = O.Volume(ocfg32)
                    vol.set(*before)
                    vol.integrate(O.depth_to_m(depth[k]), Tg, Tc)
                    ot, ow = vol.get()
                    t_, w_ = s.volume()
                    upd = ow > before[1]
                    if upd.any():
                        tsdf_steps.append(float(np.max(np.abs(t_[upd].astype(np.float64) - ot[upd])) * 32767.0))
                    vol.set(t_, w_)
                    od, ov, _, _ = vol.raycast(0, Tg, Tc, np.ascontiguousarray(Tc[:3, 3]), light)
                    m0 = s.maps(0)
                    gv, gd = m0["model_vertex"].reshape(-1, 3), m0["model_depth"].reshape(-1)
                    both = (od.reshape(-1) > 0) & (gd > 0)
                    ray_agree.append(float(((od.reshape(-1) > 0) == (gd > 0)).mean()))
                    if both.any():
                        e = np.linalg.norm(gv[both] - ov.reshape(-1, 3)[both], axis=1)
                        ray_within.append(float(np.mean(e <= 1e-3)))
            s.close()
            rows.append({"reduction": rname, "tsdf": tname,
                         "per_frame_rot_max_rad": max(rot) if rot else None,
                         "per_frame_trans_max_mm": max(trans) if trans else None,
                         "per_frame_frames": len(rot),
                         "fp32_oracle_per_frame_rot_max_rad": max(floor_rot) if floor_rot else None,
                         "fp32_oracle_per_frame_trans_max_mm": max(floor_trans) if floor_trans else None,
                         "well_posed_frames": len(wp_rot),
                         "well_posed_rot_max_rad": max(wp_rot) if wp_rot else None,
                         "well_posed_trans_max_mm": max(wp_trans) if wp_trans else None,
                         "per_frame_tsdf_max_int16_steps": max(tsdf_steps) if tsdf_steps else None,
                         "per_frame_raycast_within_1mm_min": min(ray_within) if ray_within else None,
                         "per_frame_raycast_hit_agree_min": min(ray_agree) if ray_agree else None,
                         "drift_ate_vs_fp64_mm": ate(poses, ref_poses),
                         "drift_max_vs_fp64_mm": float(np.max(np.linalg.norm(centres(poses) - centres(ref_poses),
                                                                             axis=1)) * 1e3),
                         "ate_vs_ground_truth_mm": float(np.sqrt(np.mean(np.linalg.norm(
                             centres(poses) - gt_c, axis=1) ** 2)) * 1e3)})
    # the two solves on systems of growing condition number: a real frame's
    # system with its smallest eigenvalues scaled down
    rng = np.random.default_rng(7)
    base = None
    with V.Session(cfg_of(V.VS_REDUCE_KAHAN, V.VS_TSDF_INT16)) as s:
        for k in range(3):
            s.scan_frame_host(depth[k])
        base = _system(s.icp_system()[0])
    ill = []
    if base is not None and np.isfinite(base[0]).all() and base[0][0, 0] > 0:
        A0, b0 = base
        ev, U = np.linalg.eigh(A0)
        for target in (1e2, 1e4, 1e6, 1e8):
            e2 = ev.copy()
            e2[:3] = ev[-1] / target * np.array([1.0, 3.0, 10.0])
            A = (U * e2) @ U.T
            A = 0.5 * (A + A.T)
            b = A @ rng.standard_normal(6)
            xr = np.linalg.solve(A, b)
            n = max(np.linalg.norm(xr), 1e-30)
            ill.append({"cond": float(np.linalg.cond(A)),
                        "fp64_ldlt_rel_err": float(np.linalg.norm(_solve_ldl_f64(A, b) - xr) / n),
                        "f32_factor_2_refinements_rel_err": float(np.linalg.norm(_solve_f32_refined(A, b) - xr) / n)})
    out = {"study": "precision", "workload": "config 1: 320x240, %d frames, fx=fy=285, 512^3 over 1 m, mu 3 cm, "
                                             "ICP 10/5/4" % nf,
           "reference": "FP64 oracle (double arithmetic, FP64 sums, double TSDF) on the host, %.1f s" % t_oracle,
           "fp64_oracle_ate_vs_ground_truth_mm": float(np.sqrt(np.mean(np.linalg.norm(
               centres(ref_poses) - gt_c, axis=1) ** 2)) * 1e3),
           "tolerances": {"per_frame_pose": "1e-4 rad, 0.1 mm", "tsdf": "1 int16 step (int16 storage)",
                          "raycast": "99.9 % of vertices within 1 mm"},
           "sample_frames": sample,
           "variants": rows,
           "device_solve_vs_numpy_fp64": {"max_rel_err": max(solve_err) if solve_err else None,
                                          "max_cond": max(solve_cond) if solve_cond else None,
                                          "systems": len(solve_err)},
           "ill_conditioned_solves": ill}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.study == "precision":
        run_precision(args)
    elif args.workload == "plain_vga":
        (run_plain_vga_reference if args.impl == "reference" else run_plain_vga)(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
