#!/usr/bin/env python
"""Odometry-step benchmark of the GB300 hot path (one JSON line on stdout).

A step is LIOBuilder::process on one LiDAR package in the LIO_MAPPING state:
time sort, IMU predict chain, undistortion, downsample, iterated EKF update
(ieskf_max_iter residual launches) and the voxel-map update.

Workload (default, `--workload urban`): the seeded synthetic 100 x 100 x 20 m
urban block -- ground, random facades, 5 % clutter points -- seen by a
spinning 128-beam LiDAR, 200 000 rays per scan at 10 Hz (about 173 000 returns),
float32 points, 3 cm range noise, 200 Hz IMU, 0.1 m scan downsample, 0.5 m
voxels, LRU capacity 4 M voxels, 4 IEKF iterations per scan.

Arms:
  value  scans/s with every package already in HBM (vmp_process_device),
         per-step CUDA events on the library's stream, L2 flushed (256 MB
         write) before each step outside the timed events;
  e2e    scans/s through vmp_process from pinned host buffers: each step's
         host->device copy of the scan + IMU samples and the device->host
         result copy are inside the (wall-clock) timing;
  cpu_baseline  the CPU oracle (restated reference, one thread as the
         reference's MP_PROC_NUM=1) on a bounded sample of the same scans.
`--impl reference` times that CPU restatement with all host threads instead.

Multi-GPU: streams shard by GPU (one independent sensor stream per rank,
seed 0x5EED0000 + rank), no collective on the data path; "scaling": "weak".
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "scans/s & p99 scan latency: 64-stream served vs plain 1-stream GPU vs CPU ref"

# SURVEY 8(d)-style algorithmic bytes per unit for each profiled phase:
# (bytes per unit, unit name).  Units are the points the phase processes.
ALGO_BYTES = {
    "residual": (64.0, "downsampled point x IEKF iteration"),   # 16 B point + 16 B slot + 32 B plane record
    "map_state": (220.0, "inserted point"),                       # K-INS
    "undistort": (32.0, "raw point"),                             # K-UND
    "downsample": (32.0, "raw point"),                            # K-DS (+16 B per output point, not counted)
}
PROF_NAMES = ["upload", "time_sort", "predict", "undistort", "downsample", "body_cov", "residual", "residual_idle",
              "update_other", "map_batch", "map_group", "map_state", "map_finish", "result"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="urban", choices=["urban", "room"])
    ap.add_argument("--points", type=int, default=None, help="rays per scan (default: workload's)")
    ap.add_argument("--cpu-sample", type=int, default=None, help="CPU-baseline scans (default: bounded)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--flush-mb", type=int, default=256)
    return ap.parse_args()


def workload(args, rank):
    from voxelmapplus_fastlio2_gb300 import abi, synth
    if args.workload == "urban":
        kind, pts, leaf, cap, iters = synth.KIND_URBAN, 200000, 0.1, 4000000, 4
        name = "urban block 100x100x20 m, spinning 128-beam, 200k rays/scan"
    else:
        kind, pts, leaf, cap, iters = synth.KIND_ROOM, 20000, 0.2, 100000, 5
        name = "room 20x20x5 m, rosette, 20k rays/scan"
    if args.points:
        pts = args.points
    cfg = abi.default_config(scan_resolution=leaf, map_capacity=cap, ieskf_max_iter=iters,
                             max_scan_points=max(1024, pts + 64))
    seed = 0x5EED0000 + rank
    return kind, pts, cfg, seed, name


def make_packages(kind, pts, seed, count):
    from voxelmapplus_fastlio2_gb300 import synth
    seq = synth.Sequence(kind, seed=seed, points_per_scan=pts)
    return [seq.next() for _ in range(count)]


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(phase):
    """DRAM bytes per launch of the phase's main kernel from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(phase)
    except Exception:
        return None


def pkg_arrays(p):
    pts = np.ctypeslib.as_array(C.cast(p.points, C.POINTER(C.c_float)), shape=(p.n, 4)).copy()
    imu = np.ctypeslib.as_array(C.cast(p.imus, C.POINTER(C.c_double)), shape=(p.n_imu, 7)).copy()
    return pts, imu


def run_value(args, pkgs, cfg, n_init, barrier):
    """Inputs resident in HBM; per-step CUDA events on the library's stream."""
    import torch
    from voxelmapplus_fastlio2_gb300 import lio
    g = lio.LIOBuilder(cfg)
    for p in pkgs[:n_init]:
        g.process(p)
    dev = []
    for p in pkgs[n_init:]:
        pts, imu = pkg_arrays(p)
        dev.append((torch.from_numpy(pts).cuda(), torch.from_numpy(imu).cuda(), p))
    stream = torch.cuda.ExternalStream(g.lib.vmp_cuda_stream(g.h))
    flush = torch.empty(args.flush_mb << 20, dtype=torch.uint8, device="cuda")
    W, K = args.warmup, args.steps
    for i in range(W):
        d_pts, d_imu, p = dev[i]
        g.process_device(d_pts.data_ptr(), p.n, p.t_start, p.t_end, d_imu.data_ptr(), p.n_imu)
    torch.cuda.synchronize()
    barrier()
    g.lib.vmp_profile_enable(g.h, 1)
    launches0 = g.lib.vmp_launch_count()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    evs = []
    n_raw, n_down, res = [], [], None
    t_wall = time.perf_counter()
    for i in range(W, W + K):
        d_pts, d_imu, p = dev[i]
        with torch.cuda.stream(stream):
            flush.fill_(i & 255)  # > L2 (129 MB): evicts the previous step's lines
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
        res = g.process_device(d_pts.data_ptr(), p.n, p.t_start, p.t_end, d_imu.data_ptr(), p.n_imu)
        with torch.cuda.stream(stream):
            b.record(stream)
        evs.append((a, b))
        n_raw.append(res.n_raw)
        n_down.append(res.n_down)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    barrier()
    clk = clocks.stop()
    launches = g.lib.vmp_launch_count() - launches0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms = (C.c_double * 16)()
    nl = (C.c_longlong * 16)()
    it = (C.c_longlong * 16)()
    g.lib.vmp_profile_read(g.h, ms, nl, it)
    prof = {PROF_NAMES[k]: {"ms": ms[k], "launches": nl[k], "items": it[k]} for k in range(len(PROF_NAMES))}
    g.lib.vmp_profile_enable(g.h, 0)
    out = {"step_ms": step_ms, "wall_s": t_wall, "launches": launches, "clocks": clk, "prof": prof,
           "n_raw": float(np.mean(n_raw)), "n_down": float(np.mean(n_down)), "map_size": int(res.map_size),
           "iters_last": int(res.iters)}
    g.close()
    return out


def run_e2e(args, pkgs, cfg, n_init, barrier):
    """Through vmp_process from pinned host buffers (copies inside the timing)."""
    import torch
    from voxelmapplus_fastlio2_gb300 import abi, lio
    g = lio.LIOBuilder(cfg)
    for p in pkgs[:n_init]:
        g.process(p)
    host = []
    for p in pkgs[n_init:]:
        pts, imu = pkg_arrays(p)
        hp = torch.from_numpy(pts).pin_memory()
        hi = torch.from_numpy(imu).pin_memory()
        scan = abi.vmp_scan(C.cast(C.c_void_p(hp.data_ptr()), C.POINTER(abi.vmp_point)), p.n, p.t_start, p.t_end)
        host.append((hp, hi, scan, p))
    W, K = args.warmup, args.steps
    res = abi.vmp_result()

    def step(i):
        hp, hi, scan, p = host[i]
        code = g.lib.vmp_process(g.h, C.byref(scan), C.cast(C.c_void_p(hi.data_ptr()), C.POINTER(abi.vmp_imu)),
                                 p.n_imu, C.byref(res))
        if code != 0:
            raise RuntimeError(g.lib.vmp_last_error(g.h))

    for i in range(W):
        step(i)
    torch.cuda.synchronize()
    barrier()
    h0, d0 = C.c_longlong(), C.c_longlong()
    g.lib.vmp_io_bytes(g.h, C.byref(h0), C.byref(d0))
    walls = []
    for i in range(W, W + K):
        t0 = time.perf_counter()
        step(i)
        walls.append(time.perf_counter() - t0)
    torch.cuda.synchronize()
    barrier()
    h1, d1 = C.c_longlong(), C.c_longlong()
    g.lib.vmp_io_bytes(g.h, C.byref(h1), C.byref(d1))
    g.close()
    return {"walls": walls, "h2d": (h1.value - h0.value) / K, "d2h": (d1.value - d0.value) / K}


def run_cpu(pkgs, cfg, n_init, warmup, sample, threads):
    """The CPU oracle over init + warm-up scans, timing `sample` scans."""
    import oracle
    o = oracle.Oracle(cfg, threads=threads)
    for p in pkgs[:n_init + warmup]:
        o.process(p)
    t = []
    for p in pkgs[n_init + warmup:n_init + warmup + sample]:
        t0 = time.perf_counter()
        o.process(p)
        t.append(time.perf_counter() - t0)
    return t


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws <= 1:
        return rank, ws, (lambda: None), (lambda x: x), None
    import torch
    import torch.distributed as dist
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        dist.barrier()

    def allmax(x):
        t = torch.tensor([float(x)], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return rank, ws, barrier, allmax, dist


def main():
    args = parse()
    from voxelmapplus_fastlio2_gb300 import build as vbuild
    rank, ws, barrier, allmax, dist = dist_setup(args)
    kind, pts, cfg, seed, wname = workload(args, rank)
    n_init = 2  # IMU_INIT + MAP_INIT packages
    if args.impl == "reference":
        if rank != 0:
            return
        import oracle
        oracle.build() if not os.path.exists(oracle.ORACLE_SO) else None
        vbuild.build_synth()
        threads = os.cpu_count() or 1
        pkgs = make_packages(kind, pts, seed, n_init + args.warmup + args.steps)
        t = run_cpu(pkgs, cfg, n_init, args.warmup, args.steps, threads)
        v = len(t) / sum(t)
        line = {"metric": METRIC, "value": v, "unit": "scans/s", "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(t) / len(t),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generator)",
                "config": {"workload": wname, "rays_per_scan": pts, "ieskf_max_iter": cfg.ieskf_max_iter},
                "latency_ms": {"p50": 1e3 * float(np.percentile(t, 50)), "p99": 1e3 * float(np.percentile(t, 99))},
                "cpu_baseline": {"value": v, "unit": "scans/s", "cores": threads, "kind": "port",
                                 "sample": f"{len(t)} mapping scans after {args.warmup} warm-up scans; CPU "
                                           f"restatement of the reference, residual loop on {threads} OpenMP threads"},
                "e2e": {"value": v, "unit": "scans/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    vbuild.build_all()
    import torch
    pkgs = make_packages(kind, pts, seed, n_init + args.warmup + args.steps)
    val = run_value(args, pkgs, cfg, n_init, barrier)
    e2e = None if args.no_e2e else run_e2e(args, pkgs, cfg, n_init, barrier)
    step_s = sum(val["step_ms"]) / 1e3
    step_s_max = allmax(step_s)
    value = ws * args.steps / step_s_max
    line = {"metric": METRIC, "value": value, "unit": "scans/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * step_s_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": wname, "rays_per_scan": pts, "returns_per_scan": val["n_raw"],
                       "points_after_downsample": val["n_down"], "ieskf_max_iter": cfg.ieskf_max_iter,
                       "voxel_size": cfg.voxel_size, "scan_resolution": cfg.scan_resolution,
                       "map_capacity": cfg.map_capacity, "map_voxels_at_end": val["map_size"],
                       "streams_per_gpu": 1, "parallelism": f"stream-sharded x{ws}",
                       "l2": f"flushed before every timed step ({args.flush_mb} MB write, outside the step events)"},
            "latency_ms": {"p50": float(np.percentile(val["step_ms"], 50)),
                           "p99": float(np.percentile(val["step_ms"], 99))}}
    if e2e is not None:
        ev = ws * args.steps / allmax(sum(e2e["walls"]))
        line["e2e"] = {"value": ev, "unit": "scans/s", "h2d_bytes_per_step": int(e2e["h2d"]),
                       "d2h_bytes_per_step": int(e2e["d2h"]),
                       "latency_ms": {"p50": 1e3 * float(np.percentile(e2e["walls"], 50)),
                                      "p99": 1e3 * float(np.percentile(e2e["walls"], 99))}}
    # roofline of the dominant profiled phase with an algorithmic byte count
    prof = val["prof"]
    dom = max(ALGO_BYTES, key=lambda k: prof[k]["ms"])
    per_unit, unit_name = ALGO_BYTES[dom]
    launches = max(1, prof[dom]["launches"])
    avg_ms = prof[dom]["ms"] / launches
    bytes_per_launch = per_unit * prof[dom]["items"] / launches
    peak, peak_src = load_peaks()
    achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9 if avg_ms > 0 else 0.0
    line["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": load_traffic(dom),
                        "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_ms,
                        "bytes_per_unit": per_unit, "unit_of_work": unit_name, "peak_source": peak_src}
    line["profile_ms_per_step"] = {k: v["ms"] / args.steps for k, v in prof.items()}
    line["clocks"] = val["clocks"]
    line["gpu_launches"] = val["launches"]
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        sample = args.cpu_sample
        if sample is None:
            t_probe = run_cpu(pkgs, cfg, n_init, 0, 1, 1)[0]
            sample = int(max(3, min(args.steps, 15.0 / max(t_probe, 1e-3))))
        t = run_cpu(pkgs, cfg, n_init, args.warmup, sample, 1)
        line["cpu_baseline"] = {"value": len(t) / sum(t), "unit": "scans/s", "cores": 1, "kind": "port",
                                "sample": f"{len(t)} mapping scans (after {args.warmup} warm-up scans) of the same "
                                          f"sequence, CPU restatement of the reference on 1 thread",
                                "host_cores": os.cpu_count()}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
