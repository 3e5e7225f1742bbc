#!/usr/bin/env python3
"""Benchmark of the per-frame reconstruction path on GB300.

Workload ("plain method at VGA"): one scanning session, 640x480 uint16 depth
frames (fx = fy = 525, cx = 319.5, cy = 239.5) from the seeded synthetic scene
generator with Kinect-style axial noise, 1.5 % dropout in 8x8 blobs and a
2.5 m cut-off; a 512^3 int16 TSDF + uint16 weight volume over 1.5 m,
truncation 2 cm; ICP 10/5/4 iterations with a 10 cm distance and 20 degree
normal rejection.  A step is one frame through vs_scan_frame: ingest, bilateral
filter, pyramid, input vertex/normal maps, ICP, TSDF integration, ray-cast of
three levels.

  value   frames/s on the device: inputs resident in HBM, each frame timed
          with CUDA events on its stream, L2 flushed (256 MB write) between
          frames outside the timed events.
  e2e     frames/s through the C ABI with host buffers: vs_scan_frame_host
          copies the uint16 frame in and the pose out every frame.

`--impl reference` times the CPU restatement of the reference's path (the
reference itself does not build on Linux) on the host cores with all threads.
Under torchrun every rank runs its own session (sessions are independent:
replicas, weak scaling); rank 0 prints the JSON line.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "vcl-volume-scanner_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

WORKLOAD = dict(name="plain_vga_512", width=640, height=480, fx=525.0, fy=525.0, cx=319.5, cy=239.5,
                volume=512, size_m=1.5, mu=0.02, icp_iters=(10, 5, 4), th_icp=0.1 ** 2, normal_deg=20.0,
                dropout_blob=0.015, max_depth=2.5, seed=2, sequence_frames=300)
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=295)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def make_frames(n, seed_offset=0):
    import vs_scanner as V

    w = WORKLOAD
    sc = V.synth_config(w["width"], w["height"], fx=w["fx"], fy=w["fy"], cx=w["cx"], cy=w["cy"], n_frames=n,
                        seed=w["seed"] + seed_offset, dropout_blob=w["dropout_blob"], max_depth=w["max_depth"])
    depth, gt, centre = V.synth_generate(sc)
    return depth, gt, centre


def make_config(centre):
    import vs_scanner as V

    w = WORKLOAD
    origin, vox = V.cube_around(centre, w["size_m"], w["volume"])
    return V.default_config(w["width"], w["height"], fx=w["fx"], fy=w["fy"], cx=w["cx"], cy=w["cy"],
                            dim=(w["volume"],) * 3, origin=origin, voxel_size=vox, mu=w["mu"],
                            th_icp=w["th_icp"], cos_normal=float(np.cos(np.radians(w["normal_deg"]))),
                            icp_iters=w["icp_iters"], tsdf_type=V.VS_TSDF_INT16, reduce_mode=V.VS_REDUCE_KAHAN)


def config_json(args, world):
    w = WORKLOAD
    return {"workload": "%s: 1 session, %dx%d uint16 depth, %d^3 int16+uint16 TSDF over %.1f m, mu %.0f cm, "
                        "ICP %d/%d/%d, 10 cm / 20 deg rejection" % (
                            w["name"], w["width"], w["height"], w["volume"], w["size_m"], w["mu"] * 100,
                            *w["icp_iters"]),
            "frames": args.steps, "sessions_per_gpu": 1, "parallelism": "replicas x%d" % world,
            "l2": "flushed between steps (256 MB write outside the timed events)",
            "scene": "seeded synthetic spheres/boxes on a ground plane, orbit 0.9 m, seed %d" % w["seed"]}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            v = float(json.load(f)["hbm_gbs"])
        return v, "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profiles(kernel_key):
    """DRAM bytes per launch of a kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for line in open(p):
            parts = line.split()
            if len(parts) >= 3 and parts[0] == kernel_key and parts[1] == "dram_bytes_per_launch":
                return float(parts[2])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi samples during the timed region"""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", "clocks_bench_%d.csv" % gpu_index)

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


def cpu_baseline(depth, centre, seconds, threads):
    """The oracle (reference semantics, FP32, reference reduction tree) on a
    bounded prefix of the same sequence."""
    import oracle_py as O

    lib = O.load()
    del lib
    try:
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(int(threads))
    except OSError:
        pass
    cfg = make_config(centre)
    ocfg = O.config_from_vs(cfg, reduce_mode=0)
    s = O.Session(ocfg)
    n = 0
    t0 = time.perf_counter()
    poses = []
    while n < depth.shape[0]:
        s.frame(depth[n])
        poses.append(s.pose().astype(np.float64))
        n += 1
        if time.perf_counter() - t0 > seconds and n >= 2:
            break
    dt = time.perf_counter() - t0
    return n / dt, n, dt, poses


def fp64_trajectory(depth, centre, n, threads):
    import oracle_py as O

    try:
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(int(threads))
    except OSError:
        pass
    cfg = make_config(centre)
    s = O.Session(O.config_from_vs(cfg, reduce_mode=3, tsdf_store=0), f64=True)
    out = []
    for k in range(n):
        s.frame(depth[k])
        out.append(s.pose_f64())
    return out


def centres(poses):
    return np.array([-np.asarray(T)[:3, :3].T @ np.asarray(T)[:3, 3] for T in poses])


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    n_threads = os.cpu_count() or 1
    depth, gt, centre = make_frames(args.warmup + args.steps)
    import oracle_py as O

    O.load()
    try:
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(n_threads)
    except OSError:
        pass
    cfg = make_config(centre)
    s = O.Session(O.config_from_vs(cfg, reduce_mode=0))
    for k in range(args.warmup):
        s.frame(depth[k])
    times = []
    for k in range(args.warmup, args.warmup + args.steps):
        t0 = time.perf_counter()
        s.frame(depth[k])
        times.append(time.perf_counter() - t0)
    total = sum(times)
    fps = args.steps / total
    sample = "%d frames of the workload after %d warm-up frames, oracle port (reference FP32 semantics), %d threads" % (
        args.steps, args.warmup, n_threads)
    line = {"impl": "reference", "metric": "frames/s", "value": fps, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_json(args, 1),
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": n_threads, "kind": "port", "sample": sample},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    import vs_scanner as V

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    n = args.warmup + args.steps
    depth, gt, centre = make_frames(n, seed_offset=0)
    cfg = make_config(centre)
    frames_dev = torch.from_numpy(depth.view(np.int16)).cuda()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    sess = V.Session(cfg)
    sess.set_stage_timing(True)
    kpf = sess.kernels_per_frame()
    frame_bytes = cfg.width * cfg.height * 2

    # ---- warm-up (untimed) ----
    with torch.cuda.stream(st):
        for k in range(args.warmup):
            flush.zero_()
            sess.scan_frame(frames_dev[k].data_ptr(), st.cuda_stream)
    st.synchronize()

    # ---- timed region: K frames, device events per frame ----
    clk = ClockSampler(local)
    barrier()
    clk.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stage = np.zeros((args.steps, 4))
    stats = np.zeros((args.steps, 4))
    poses = []
    t_wall = time.perf_counter()
    with torch.cuda.stream(st):
        for i in range(args.steps):
            k = args.warmup + i
            flush.zero_()
            ev[i][0].record(st)
            sess.scan_frame(frames_dev[k].data_ptr(), st.cuda_stream)
            ev[i][1].record(st)
            stage[i] = sess.stage_times()
            stats[i] = sess.frame_stats()
    st.synchronize()
    t_wall = time.perf_counter() - t_wall
    barrier()
    clocks = clk.stop()
    frame_ms = np.array([a.elapsed_time(b) for a, b in ev])
    _, T64, info = sess.pose()
    total_ms = float(frame_ms.sum())
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    fps = world * args.steps / (total_ms / 1000.0)

    # ---- end to end through the C ABI with host buffers ----
    sess.set_stage_timing(False)
    sess.reset()
    pinned = torch.from_numpy(depth.view(np.int16)).pin_memory()
    host = pinned.numpy().view(np.uint16)
    e2e_poses = []
    for k in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        sess.scan_frame_host(host[k])
    barrier()
    e2e_t = []
    for i in range(args.steps):
        k = args.warmup + i
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        T, tracked = sess.scan_frame_host(host[k])
        e2e_t.append(time.perf_counter() - t0)
        e2e_poses.append(T.astype(np.float64))
    barrier()
    e2e_total = sum(e2e_t)
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([e2e_total], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_fps = world * args.steps / e2e_total

    if rank != 0:
        return
    # ---- roofline of the dominant stage ----
    stage_mean = stage.mean(axis=0)
    names = ["filter", "track", "integrate", "raycast"]
    peak, peak_kind = measured_peak_hbm()
    W, H = cfg.width, cfg.height
    active, nupd = stats[:, 0].mean(), stats[:, 1].mean()
    # algorithmic bytes per launch (one frame):
    #   integrate: 4 B per swept voxel pair (512 per active sub-cube) read,
    #              4 B per updated voxel written, 2 B per depth pixel, 8 B of
    #              flag + list per active sub-cube
    b_int = 4.0 * 512 * active + 4.0 * nupd + 2.0 * W * H + 8.0 * active
    lv = [(W >> l) * (H >> l) for l in range(3)]
    iters = WORKLOAD["icp_iters"]
    b_icp = sum(28.0 * lv[l] * iters[l] for l in range(3))
    b_filter = 6.0 * W * H + sum(lv[l] * (4 + 4 + 32) for l in range(3))
    b_ray = 28.0 * sum(lv)
    alg = {"filter": b_filter, "track": b_icp, "integrate": b_int, "raycast": b_ray}
    dom = names[int(np.argmax(stage_mean))]
    achieved = alg[dom] / (stage_mean[names.index(dom)] * 1e-3) / 1e9
    kernel_key = {"integrate": "k_integrate", "raycast": "k_raycast", "track": "k_icp_iter",
                  "filter": "k_bilateral"}[dom]
    traffic = traffic_from_profiles(kernel_key)
    roofline = {"bound": "hbm", "kernel": kernel_key, "stage": dom, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind if peak_kind == "measured" else
                "fallback 6800 GB/s",
                "note": "algorithmic bytes of the stage per frame / its event-timed duration"}
    integ = {"achieved_gbs": b_int / (stage_mean[2] * 1e-3) / 1e9, "frac": b_int / (stage_mean[2] * 1e-3) / 1e9 / peak,
             "active_subcubes": active, "voxels_updated": nupd, "algorithmic_bytes": b_int}

    # ---- CPU baseline and FP64 trajectory check on a bounded prefix ----
    cpu = None
    ate = None
    if not args.no_cpu:
        fps_cpu, ncpu, tcpu, cpu_poses = cpu_baseline(depth, centre, args.cpu_seconds, 1)
        cpu = {"value": fps_cpu, "unit": "frames/s", "cores": 1, "kind": "port",
               "sample": "first %d frames of the same sequence (%.1f s), oracle port, reference FP32 semantics, "
                         "1 thread" % (ncpu, tcpu)}
        nf = min(ncpu, len(e2e_poses) + args.warmup)
        ref64 = fp64_trajectory(depth, centre, nf, os.cpu_count() or 1)
        # the e2e run restarted from frame 0 after reset: frames 0..warmup-1 untimed
        ours = []
        sess2 = V.Session(cfg)
        for k in range(nf):
            T, _ = sess2.scan_frame_host(host[k])
            ours.append(T.astype(np.float64))
        sess2.close()
        d = np.linalg.norm(centres(ours) - centres(ref64), axis=1)
        ate = {"vs_fp64_oracle_mm": float(np.sqrt(np.mean(d ** 2)) * 1e3), "frames": nf,
               "max_mm": float(d.max() * 1e3)}
    gt_err = np.linalg.norm(centres([gt[args.warmup + args.steps - 1]]) - centres([T64]), axis=1)[0]

    line = {"metric": "frames/s", "value": fps, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(frame_ms.mean()), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_json(args, world),
            "latency_ms": {"p50": float(np.percentile(frame_ms, 50)), "p99": float(np.percentile(frame_ms, 99)),
                           "max": float(frame_ms.max())},
            "stages_ms": {n_: float(v) for n_, v in zip(names, stage_mean)},
            "roofline": roofline, "integrate": integ,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": frame_bytes,
                    "d2h_bytes_per_step": 80},
            "gpu_launches": int(kpf * args.steps),
            "clocks": clocks,
            "ate": ate,
            "tracking": {"last_frame_tracked": int(info[0]), "camera_err_vs_generator_mm": float(gt_err * 1e3)},
            "wall_s_timed_region": t_wall}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
