#!/usr/bin/env python3
"""Benchmark: batched serving vs the plain one-session-per-launch path.

Workload ("serving mix"): 64 scanning sessions, each with its own seeded
synthetic scene (spheres/boxes on a ground plane, camera orbit of radius
0.9 m, Kinect-style axial noise, 1.5 % dropout in 8x8 blobs, depth cut at
2.5 m) and its own length drawn from U{50..500} frames.  Frame sizes cycle
through 320x240 (fx = fy = 285), 512x424 (fx = fy = 365) and 640x480
(fx = fy = 525); volumes are 128^3 to 512^3 int16 TSDF + uint16 weight over a
1.5 m cube (at most 512 MiB each), truncation 2 cm, ICP 10/5/4 iterations with
10 cm / 20 degree rejection, compensated (two-sum) reduction.

A step is one batched pass of the whole pipeline (ingest, bilateral filter,
pyramid, input normal maps, ICP, integration, ray-cast of three levels) over
the frame of every session that is still running: step r carries frame r of
each session longer than r frames.

  value      frames/s of the batched form: all frames resident in HBM, steps
             enqueued back to back, CUDA events on the launching stream around
             the timed steps.  The working set of a step (64 frames, the
             active sub-cubes of 64 volumes, 13 GB of volumes in all) is far
             larger than L2, so L2 is not flushed.
  e2e        the same steps through the C ABI with host frames
             (vs_batch_step_host: pinned uint16 frames in, poses out, every
             step).
  plain      the same frames through the plain path, one session per launch
             (vs_scan_frame per frame, one graph per frame).
  serving    open-loop arrivals through the serving loop (vs_server_*): every
             session sends frames as a Poisson stream of 31.25 frames/s
             (2000 frames/s aggregate while all 64 run), host frames in,
             results polled out; latency = result on the host - scheduled
             arrival.  The plain path serves the same arrival schedule
             first-come first-served, one frame per launch.

`--impl reference` times the CPU restatement of the reference's path (the
reference itself does not build on Linux) on the same session mix with all
host threads.  Under torchrun every rank runs its own copy of the workload
(sessions are independent: replicas, weak scaling); rank 0 prints the line.
"""
import argparse
import ctypes
import json
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
           volumes=(128, 256, 384, 512), size_m=1.5, mu=0.02, icp_iters=(10, 5, 4), th_icp=0.1 ** 2,
           normal_deg=20.0, dropout_blob=0.015, max_depth=2.5, arrival_fps=2000.0, hbm_budget_gb=150)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="serving mix: batched steps (session lengths are capped at it, default 500); "
                         "plain_vga: timed frames (default 295); precision: frames (default 30)")
    ap.add_argument("--workload", default="serving_mix", choices=["serving_mix", "plain_vga"])
    ap.add_argument("--study", default=None, choices=["precision"])
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sessions", type=int, default=MIX["sessions"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU baseline sample")
    ap.add_argument("--ref-seconds", type=float, default=90.0, help="budget of the reference arm")
    ap.add_argument("--ate-frames", type=int, default=12)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    a = ap.parse_args()
    if a.steps is None:
        a.steps = 30 if a.study == "precision" else (295 if a.workload == "plain_vga" else 500)
    return a


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def session_specs(n, max_len, seed):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        w, h, f, cx, cy = MIX["sizes"][i % 3]
        dim = int(MIX["volumes"][int(rng.integers(0, len(MIX["volumes"])))])
        length = int(min(max_len, rng.integers(MIX["length"][0], MIX["length"][1] + 1)))
        specs.append(dict(w=w, h=h, f=f, cx=cx, cy=cy, dim=dim, length=max(1, length), seed=1000 + seed * 100 + i))
    return specs


def generate(spec):
    import vs_scanner as V

    sc = V.synth_config(spec["w"], spec["h"], fx=spec["f"], fy=spec["f"], cx=spec["cx"], cy=spec["cy"],
                        n_frames=spec["length"], seed=spec["seed"], dropout_blob=MIX["dropout_blob"],
                        max_depth=MIX["max_depth"])
    depth, gt, centre = V.synth_generate(sc)
    return depth, gt, centre


def session_mu(vox):
    """truncation of a session: 2 cm, or 5 voxels where that is more (the
    reference's own rule is 5 voxels, VCL_Volume_Scanner_View.cpp:423; at
    1.7 voxels, 2 cm in a 128^3 volume over 1.5 m, the ray-cast misses most of
    the thin first-frame band and tracking fails, in the oracle as here)"""
    return max(MIX["mu"], 5.0 * float(vox))


def make_config(spec, centre):
    import vs_scanner as V

    origin, vox = V.cube_around(centre, MIX["size_m"], spec["dim"])
    return V.default_config(spec["w"], spec["h"], fx=spec["f"], fy=spec["f"], cx=spec["cx"], cy=spec["cy"],
                            dim=(spec["dim"],) * 3, origin=origin, voxel_size=vox, mu=session_mu(vox),
                            th_icp=MIX["th_icp"], cos_normal=float(np.cos(np.radians(MIX["normal_deg"]))),
                            icp_iters=MIX["icp_iters"], tsdf_type=V.VS_TSDF_INT16, reduce_mode=V.VS_REDUCE_KAHAN)


def build_workload(n, max_len, seed):
    specs = session_specs(n, max_len, seed)
    seqs = []
    for sp in specs:
        depth, gt, centre = generate(sp)
        seqs.append(dict(spec=sp, depth=depth, gt=gt, centre=centre, cfg=make_config(sp, centre)))
    return seqs


def config_json(args, seqs, world):
    lens = [s["spec"]["length"] for s in seqs]
    sizes = {}
    for s in seqs:
        k = "%dx%d" % (s["spec"]["w"], s["spec"]["h"])
        sizes[k] = sizes.get(k, 0) + 1
    vols = {}
    for s in seqs:
        k = "%d^3" % s["spec"]["dim"]
        vols[k] = vols.get(k, 0) + 1
    return {"workload": "%s: %d sessions, lengths U{%d..%d} (capped at %d), frame sizes %s, volumes %s int16+uint16 "
                        "over %.1f m, mu %.0f cm, ICP %d/%d/%d, 10 cm / 20 deg rejection, Poisson %.0f frames/s "
                        "aggregate, HBM budget %d GB" % (
                            MIX["name"], len(seqs), MIX["length"][0], MIX["length"][1], args.steps, sizes, vols,
                            MIX["size_m"], MIX["mu"] * 100, *MIX["icp_iters"], MIX["arrival_fps"],
                            MIX["hbm_budget_gb"]),
            "frames": int(sum(lens)), "sessions_per_gpu": len(seqs), "parallelism": "replicas x%d" % world,
            "l2": "not flushed: a step's working set (64 frames, active sub-cubes of 64 volumes) is far above L2",
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
    """DRAM bytes per unit of work of a kernel, from the committed ncu summary
    (profiles/ncu_traffic.txt: `kernel key value ...`)"""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for line in open(p):
            parts = line.split()
            if len(parts) >= 3 and parts[0] == kernel_key and parts[1] == unit_key:
                return float(parts[2])
    except (OSError, ValueError):
        pass
    return None


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


def arrival_schedule(seqs, fps_total, seed):
    """(t, session index, frame) sorted by t: each session a Poisson stream of
    fps_total / n_sessions frames/s from t = 0"""
    rng = np.random.default_rng(seed)
    rate = fps_total / len(seqs)
    ev = []
    for i, s in enumerate(seqs):
        gaps = rng.exponential(1.0 / rate, size=s["spec"]["length"])
        t = np.cumsum(gaps)
        ev += [(float(t[k]), i, k) for k in range(len(t))]
    ev.sort()
    return ev


# ---------------------------------------------------------------------------
# reference arm: the CPU restatement on the same mix
# ---------------------------------------------------------------------------
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle_py as O

    n_threads = os.cpu_count() or 1
    O.load()
    set_omp_threads(n_threads)
    specs = session_specs(args.sessions, args.steps, MIX["seed"])
    # a bounded sample: the first frames of the first sessions (one of each
    # size in turn), round robin, until the time budget or K frames
    sample_sessions = min(6, len(specs))
    seqs = []
    for sp in specs[:sample_sessions]:
        sp = dict(sp, length=min(sp["length"], 40))
        depth, gt, centre = generate(sp)
        seqs.append((O.Session(O.config_from_vs(make_config(sp, centre), reduce_mode=0)), depth))
    for k in range(min(args.warmup, 2)):
        for s, d in seqs:
            s.frame(d[k])
    times, n, k = [], 0, min(args.warmup, 2)
    t_start = time.perf_counter()
    while n < args.steps and time.perf_counter() - t_start < args.ref_seconds:
        for s, d in seqs:
            if k >= d.shape[0]:
                continue
            t0 = time.perf_counter()
            s.frame(d[k])
            times.append(time.perf_counter() - t0)
            n += 1
        k += 1
        if all(k >= d.shape[0] for _, d in seqs):
            break
    total = sum(times)
    fps = len(times) / total
    sample = ("%d frames: sessions 0..%d of the serving mix round robin (sizes 320x240/512x424/640x480), frames "
              "%d.. of each, oracle port (reference FP32 semantics), %d threads" % (
                  len(times), sample_sessions - 1, min(args.warmup, 2), n_threads))
    line = {"impl": "reference", "metric": "frames/s", "value": fps, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": len(times), "warmup": min(args.warmup, 2), "ms_per_step": 1000.0 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": "%s (bounded CPU sample, see cpu_baseline.sample)" %
                                                        MIX["name"]},
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": n_threads, "kind": "port", "sample": sample},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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

    t_gen = time.perf_counter()
    seqs = build_workload(args.sessions, args.steps, MIX["seed"])
    t_gen = time.perf_counter() - t_gen
    n_s = len(seqs)
    lens = [s["spec"]["length"] for s in seqs]
    rounds = max(lens)
    n_frames = int(sum(lens))
    frames_dev = [torch.from_numpy(s["depth"].view(np.int16)).cuda() for s in seqs]
    pinned = [torch.from_numpy(s["depth"].view(np.int16)).pin_memory() for s in seqs]
    host = [p.numpy().view(np.uint16) for p in pinned]
    st = torch.cuda.Stream()

    sessions = [V.Session(s["cfg"]) for s in seqs]
    batch = V.Batch()

    # ---- warm-up: graph capture and first launches on throwaway sessions ----
    n_warm = min(16, n_s)
    warm = [V.Session(seqs[i]["cfg"]) for i in range(n_warm)]
    for k in range(args.warmup):
        batch.step(warm, [frames_dev[i][min(k, lens[i] - 1)].data_ptr() for i in range(n_warm)], st.cuda_stream)
    batch.sync()
    # autotuner: the ray-cast launch shape, timed on the warm-up sessions
    tuned = None
    if not args.no_autotune:
        shape, ms = batch.autotune(warm, reps=3)
        tuned = {"ray_tile": "%dx%d" % (1 << shape[0], 32 >> shape[0]), "march_blocks_per_sm": shape[1],
                 "shade_blocks_per_sm": shape[2], "raycast_ms_warm_sessions": ms}
    for w in warm:
        w.close()

    # ---- batched form, device-resident frames: the timed region ----
    members = [[i for i in range(n_s) if lens[i] > r] for r in range(rounds)]
    handles = [[sessions[i] for i in m] for m in members]
    ptrs = [[frames_dev[i][r].data_ptr() for i in m] for r, m in enumerate(members)]
    clk = ClockSampler(local)
    barrier()
    clk.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(rounds + 1)]
    t_wall = time.perf_counter()
    ev[0].record(st)
    for r in range(rounds):
        batch.step(handles[r], ptrs[r], st.cuda_stream)
        ev[r + 1].record(st)
    st.synchronize()
    t_wall = time.perf_counter() - t_wall
    barrier()
    clocks = clk.stop()
    step_ms = np.array([ev[r].elapsed_time(ev[r + 1]) for r in range(rounds)])
    total_ms = max_over_ranks(float(ev[0].elapsed_time(ev[rounds])), world)
    fps_batched = world * n_frames / (total_ms / 1000.0)
    kps = batch.kernels_per_step()
    tracked_batched = [int(s.pose()[2][0]) for s in sessions]
    final_batched = [s.pose()[1] for s in sessions]

    # ---- stage breakdown of full steps (separate, synchronous pass) ----
    for s in sessions:
        s.reset()
    batch.set_stage_timing(True)
    n_stage = min(20, rounds)
    stage = np.zeros((n_stage, 4))
    alg = {k: 0.0 for k in ("filter", "track", "integrate", "raycast")}
    for r in range(n_stage):
        batch.step(handles[r], ptrs[r], st.cuda_stream)
        batch.sync()
        stage[r] = batch.stage_times()
        for i in members[r]:
            fs = sessions[i].frame_stats()
            for k, v in stage_bytes(seqs[i]["cfg"], fs).items():
                alg[k] += v
    batch.set_stage_timing(False)
    names = ["filter", "track", "integrate", "raycast"]
    stage_sum = stage.sum(axis=0)
    stage_mean = stage.mean(axis=0)

    # ---- e2e: the same steps with host frames through the C ABI ----
    for s in sessions:
        s.reset()
    batch.sync()
    e2e_poses = {i: [] for i in range(min(3, n_s))}
    barrier()
    t0 = time.perf_counter()
    for r in range(rounds):
        T, _ = batch.step_host(handles[r], [host[i][r] for i in members[r]])
        for j, i in enumerate(members[r]):
            if i in e2e_poses and len(e2e_poses[i]) < args.ate_frames:
                e2e_poses[i].append(T[j].astype(np.float64))
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    fps_e2e = world * n_frames / e2e_s
    h2d = int(round(sum(h.nbytes for h in host) / rounds))  # mean host frame bytes per step
    d2h = 64 * 80  # pose heads of every slot, one copy per step

    # ---- plain path: one session per launch, same frames ----
    for s in sessions:
        s.reset()
    torch.cuda.synchronize()
    pev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    barrier()
    pev[0].record(st)
    with torch.cuda.stream(st):
        for r in range(rounds):
            for i in members[r]:
                sessions[i].scan_frame(frames_dev[i][r].data_ptr(), st.cuda_stream)
    pev[1].record(st)
    st.synchronize()
    plain_ms = max_over_ranks(float(pev[0].elapsed_time(pev[1])), world)
    fps_plain = world * n_frames / (plain_ms / 1000.0)
    # the batched and plain runs of every session end on the same FP64 pose
    plain_equal = all(np.array_equal(sessions[i].pose()[1], final_batched[i]) for i in range(n_s))

    # ---- serving: open-loop Poisson arrivals ----
    serving = None
    plain_serving = None
    if not args.no_serving:
        sched = arrival_schedule(seqs, MIX["arrival_fps"], MIX["seed"] + 17)
        serving = run_serving(V, seqs, host, sched)
        for s in sessions:
            s.reset()
        plain_serving = run_plain_serving(sessions, host, sched)
    batch.close()
    for s in sessions:
        s.close()

    if rank != 0:
        return
    peak, peak_kind = measured_peak_hbm()
    dom_i = int(np.argmax(stage_sum))
    dom = names[dom_i]
    achieved = {k: alg[k] / (stage_sum[names.index(k)] * 1e-3) / 1e9 for k in names}
    kernel_key = {"integrate": "k_integrate", "raycast": "k_ray_march+k_ray_shade", "track": "k_icp_iter",
                  "filter": "k_bilateral_batch"}[dom]
    # measured DRAM bytes of one step of the stage: per-unit figures of the
    # committed ncu captures times this workload's units per step
    rays = np.mean([sum(sum(level_pixels(seqs[i]["cfg"])) for i in members[r]) for r in range(n_stage)])
    traffic = None
    if dom == "raycast":
        a_, b_ = traffic_per_unit("k_ray_march", "dram_bytes_per_ray"), traffic_per_unit("k_ray_shade",
                                                                                          "dram_bytes_per_ray")
        if a_ is not None and b_ is not None:
            traffic = (a_ + b_) * rays
    elif dom == "track":
        px = traffic_per_unit("k_icp_iter", "dram_bytes_per_pixel")
        if px is not None:
            traffic = px * np.mean([sum(sum(p * it for p, it in zip(level_pixels(seqs[i]["cfg"]), MIX["icp_iters"]))
                                        for i in members[r]) for r in range(n_stage)])
    roofline = {"bound": "hbm", "kernel": kernel_key, "stage": dom,
                "achieved": achieved[dom], "peak": peak, "unit": "GB/s", "frac": achieved[dom] / peak,
                "traffic": traffic,
                "traffic_note": "DRAM bytes per step: bytes per unit from profiles/ncu_traffic.txt x units per step "
                                "(%.0f rays)" % rays,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
                "fallback 6800 GB/s",
                "note": "algorithmic bytes of the stage per full step (the sessions of the first %d steps) / its "
                        "event-timed duration; the ray-cast is issue-bound, not HBM-bound (see profiles/)" % n_stage,
                "algorithmic_bytes_per_step": alg[dom] / n_stage,
                "stages_gbs": achieved, "stages_frac": {k: v / peak for k, v in achieved.items()}}
    if dom == "raycast":
        # the ray-cast's own bound is instruction issue: warp instructions per
        # ray from the committed ncu captures times this workload's rays, over
        # the event-timed stage, against one warp instruction per scheduler per
        # cycle (4 per SM) at the SM clock sampled during the timed region
        ia = traffic_per_unit("k_ray_march", "warp_inst_per_ray")
        ib = traffic_per_unit("k_ray_shade", "warp_inst_per_ray")
        mhz = (clocks or {}).get("sm_mhz")
        if ia is not None and ib is not None and mhz:
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            got = (ia + ib) * rays / (stage_sum[dom_i] / n_stage * 1e-3)
            top = 4.0 * sms * mhz * 1e6
            roofline["issue"] = {"achieved": got, "peak": top, "unit": "warp instructions/s", "frac": got / top,
                                 "warp_inst_per_ray": ia + ib,
                                 "note": "warp instructions per ray from profiles/ncu_traffic.txt x %.0f rays per "
                                         "step / the stage's event time; peak = 4 x %d SMs x %.0f MHz" %
                                         (rays, sms, mhz)}

    cpu = None
    ate = None
    if not args.no_cpu:
        cpu = cpu_baseline(seqs, args.cpu_seconds)
        ate = ate_vs_fp64(seqs, e2e_poses, args.ate_frames)

    line = {"metric": "frames/s", "value": fps_batched, "unit": "frames/s", "n_gpus": world, "steps": rounds,
            "warmup": args.warmup, "ms_per_step": float(step_ms.mean()), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_json(args, seqs, world),
            "frames_per_step": n_frames / rounds,
            "step_ms": {"p50": pct(step_ms, 50), "p99": pct(step_ms, 99), "max": float(step_ms.max())},
            "plain": {"value": fps_plain, "unit": "frames/s", "ms": plain_ms,
                      "note": "one session per launch (vs_scan_frame), same frames, device-resident",
                      "final_poses_equal_batched": bool(plain_equal)},
            "batched_over_plain": fps_batched / fps_plain,
            "serving": serving, "plain_serving": plain_serving,
            "stages_ms_per_step": {n_: float(v) for n_, v in zip(names, stage_mean)},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": fps_e2e, "unit": "frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "note": "vs_batch_step_host per step: pinned host frames in, pose heads out"},
            "gpu_launches": int(kps * rounds),
            "autotune": tuned,
            "clocks": clocks,
            "ate": ate,
            "tracked_last_frame": int(sum(tracked_batched)),
            "generation_s": t_gen, "wall_s_timed_region": t_wall}
    print(json.dumps(line), flush=True)


def run_serving(V, seqs, host, sched):
    """open-loop arrivals through vs_server; latency from the scheduled arrival"""
    srv = V.Server(hbm_budget=MIX["hbm_budget_gb"] << 30)
    ids = [srv.open(s["cfg"]) for s in seqs]
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
    arr = {(i, k): t0 + t for t, i, k in sched}
    lat = [1000.0 * (r["t_done"] - arr[(ids.index(r["session"]), r["frame"])]) for r in results]
    t_first = t0 + sched[0][0]
    t_last = max(r["t_done"] for r in results)
    span_arr = sched[-1][0] - sched[0][0]
    return {"offered_fps_peak": MIX["arrival_fps"], "offered_fps_mean": len(sched) / span_arr,
            "frames": len(results), "achieved_fps": len(results) / (t_last - t_first),
            "span_s": t_last - t_first, "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "max_ms": float(max(lat)),
            "mean_batch": stats["mean_batch"], "max_batch": stats["max_batch_seen"], "steps": stats["steps"],
            "submit_retries": busy, "sessions_admitted": len(ids),
            "hbm_resident_gb": stats["bytes_resident"] / 2 ** 30 if stats["bytes_resident"] else None}


def run_plain_serving(sessions, host, sched):
    """the same arrivals served first-come first-served, one frame per launch"""
    lat = []
    t0 = time.perf_counter() + 0.05
    for t, i, k in sched:
        now = time.perf_counter()
        if now < t0 + t:
            time.sleep(t0 + t - now)
        sessions[i].scan_frame_host(host[i][k])
        lat.append(1000.0 * (time.perf_counter() - (t0 + t)))
    span = time.perf_counter() - (t0 + sched[0][0])
    return {"offered_fps_peak": MIX["arrival_fps"], "frames": len(lat), "achieved_fps": len(lat) / span,
            "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "max_ms": float(max(lat))}


def cpu_baseline(seqs, seconds):
    """The oracle (reference semantics, FP32, reference reduction tree), one
    thread, on a bounded sample: the first frames of sessions 0..2 (one of
    each frame size), round robin."""
    import oracle_py as O

    O.load()
    set_omp_threads(1)
    ss = [(O.Session(O.config_from_vs(seqs[i]["cfg"], reduce_mode=0)), seqs[i]["depth"]) for i in range(min(3, len(seqs)))]
    n, k = 0, 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds or n < 3:
        progressed = False
        for s, d in ss:
            if k < d.shape[0]:
                s.frame(d[k])
                n += 1
                progressed = True
        k += 1
        if not progressed:
            break
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "frames/s", "cores": 1, "kind": "port",
            "sample": "%d frames (first %d of sessions 0..2: 320x240, 512x424, 640x480), %.1f s, oracle port, "
                      "reference FP32 semantics, 1 thread" % (n, k, dt)}


def ate_vs_fp64(seqs, poses, nf):
    """RMS camera-centre error of the batched poses against the FP64 oracle
    run of the same frames (both trajectories start at the identity)"""
    import oracle_py as O

    set_omp_threads(os.cpu_count() or 1)
    out = {}
    worst = 0.0
    for i, ours in poses.items():
        s = O.Session(O.config_from_vs(seqs[i]["cfg"], reduce_mode=3, tsdf_store=0), f64=True)
        ref = []
        for k in range(len(ours)):
            s.frame(seqs[i]["depth"][k])
            ref.append(s.pose_f64())
        d = np.linalg.norm(centres(ours) - centres(ref), axis=1)
        rms = float(np.sqrt(np.mean(d ** 2)) * 1e3)
        out["session_%d_%dx%d" % (i, seqs[i]["spec"]["w"], seqs[i]["spec"]["h"])] = {"rms_mm": rms, "frames": len(ours),
                                                                                       "max_mm": float(d.max() * 1e3)}
        worst = max(worst, rms)
    return {"vs_fp64_oracle_mm": worst, "sessions": out}


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
        a_, b_ = traffic_per_unit("k_ray_march", "dram_bytes_per_ray"), traffic_per_unit("k_ray_shade",
                                                                                          "dram_bytes_per_ray")
        if a_ is not None and b_ is not None:
            traffic = (a_ + b_) * rays
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
            "roofline": {"bound": "hbm", "kernel": {"raycast": "k_ray_march+k_ray_shade", "track": "k_icp_iter",
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
def run_precision(args):
    """Configuration-1 workload (one 320x240 session, fx = fy = 285, cx = 160,
    cy = 120, 1 % dropout, ICP 10/5/4, mu 3 cm) with the TSDF in a 512^3 volume
    over 1 m.  Every reduction mode x every TSDF storage runs on the GPU; the
    FP64 oracle (double arithmetic, FP64 sums, double TSDF) runs the same
    frames on the CPU.  Errors: per-frame pose against the FP64 oracle's pose
    of the same frame, ATE against the FP64 trajectory and the generator's
    ground truth, final TSDF and level-0 model maps against the oracle's."""
    import oracle_py as O
    import vs_scanner as V

    rank, world, _ = dist_env()
    if rank != 0:
        return
    nf = args.steps
    sc = V.synth_config(320, 240, fx=285.0, fy=285.0, cx=160.0, cy=120.0, n_frames=nf, seed=1, dropout_iid=0.01)
    depth, gt, centre = V.synth_generate(sc)
    origin, vox = V.cube_around(centre, 1.0, 512)

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
    ref_t, ref_w = ref.volume().get()
    ref_maps = ref.maps(0)
    t_oracle = time.perf_counter() - t0
    gt_c = centres([np.asarray(g) for g in gt])

    def ate(a, b):
        d = np.linalg.norm(centres(a) - centres(b), axis=1)
        return float(np.sqrt(np.mean(d ** 2)) * 1e3)

    rows = []
    for rm, rname in ((V.VS_REDUCE_FP32, "fp32"), (V.VS_REDUCE_KAHAN, "two-sum fp32"), (V.VS_REDUCE_FP64, "fp64")):
        for tt, tname in ((V.VS_TSDF_INT16, "int16"), (V.VS_TSDF_FP16, "fp16"), (V.VS_TSDF_FP32, "fp32")):
            s = V.Session(cfg_of(rm, tt))
            poses = []
            for k in range(nf):
                s.scan_frame_host(depth[k])
                poses.append(s.pose()[1])
            t, w = s.volume()
            m = s.maps(0)
            s.close()
            rot = [float(np.arctan2(np.linalg.norm([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2,
                                    (np.trace(R) - 1) / 2))
                   for R in (np.asarray(a)[:3, :3].T @ np.asarray(b)[:3, :3] for a, b in zip(poses, ref_poses))]
            trans = [float(np.linalg.norm(np.asarray(a)[:3, 3] - np.asarray(b)[:3, 3]) * 1e3)
                     for a, b in zip(poses, ref_poses)]
            both = (w > 0) & (ref_w > 0)
            dt_ = np.abs(t[both].astype(np.float64) - ref_t[both].astype(np.float64))
            va = m["model_vertex"].reshape(-1, 3)
            vb = ref_maps["model_vertex"].reshape(-1, 3)
            valid = (va[:, 0] != -100.0) & (vb[:, 0] != -100.0)
            dv = np.linalg.norm(va[valid] - vb[valid], axis=1) * 1e3
            rows.append({"reduction": rname, "tsdf": tname,
                         "pose_rot_max_rad": max(rot), "pose_trans_max_mm": max(trans),
                         "ate_vs_fp64_mm": ate(poses, ref_poses),
                         "ate_vs_ground_truth_mm": float(np.sqrt(np.mean(np.linalg.norm(
                             centres(poses) - gt_c, axis=1) ** 2)) * 1e3),
                         "tsdf_abs_err_mean": float(dt_.mean()) if dt_.size else None,
                         "tsdf_abs_err_max": float(dt_.max()) if dt_.size else None,
                         "weight_mismatch_voxels": int(np.count_nonzero(w != ref_w)),
                         "raycast_vertex_err_mean_mm": float(dv.mean()) if dv.size else None,
                         "raycast_within_1mm": float(np.mean(dv < 1.0)) if dv.size else None,
                         "raycast_valid_agree": float(np.mean((va[:, 0] != -100.0) == (vb[:, 0] != -100.0)))})
    out = {"study": "precision", "workload": "config 1: 320x240, %d frames, fx=fy=285, 512^3 over 1 m, mu 3 cm, "
                                             "ICP 10/5/4" % nf,
           "reference": "FP64 oracle (double arithmetic, FP64 sums, double TSDF) on the host, %.1f s" % t_oracle,
           "fp64_oracle_ate_vs_ground_truth_mm": float(np.sqrt(np.mean(np.linalg.norm(
               centres(ref_poses) - gt_c, axis=1) ** 2)) * 1e3),
           "variants": rows}
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
