#!/usr/bin/env python
"""Benchmark of the GB300 odometry hot path (one JSON line on stdout).

Metric: scans/s and p99 per-scan latency of the 64-stream served form, next
to the plain one-stream GPU path and the CPU reference restatement.  A step
(scan) is LIOBuilder::process on one LiDAR package in the LIO_MAPPING state:
time sort, IMU predict chain, undistortion, downsample, iterated EKF update
and the voxel-map update.

Default workload (`--workload serve`): 64 independent sensor streams on one
GPU, each with its own seeded scene and trajectory -- even streams the
20 x 20 x 5 m room seen by a rosette LiDAR, odd ones the 100 x 100 x 20 m
urban block seen by a spinning 128-beam LiDAR -- with rays per scan drawn
uniformly from [2k, 200k], 200 Hz IMU, 0.5 m voxels, admitted under a 150 GB
HBM budget, served by libvmp's server (vmp_submit / vmp_poll).
  value     scans/s of all streams: `--steps` mapping scans per stream, the
            packages already in HBM (vmp_submit_device), all submitted at
            once, wall time until the last result is on the host;
  e2e       the same scans from the same map states on a second server,
            packages from host memory (vmp_submit copies each package; the
            host->device copies and the result reads are inside the timing);
  latency   open loop: each stream a Poisson process at 10 Hz, p50 / p99 of
            (result on host - submission);
  plain_1stream  the same streams and packages with one package on the GPU
            at a time (one worker), and the one-stream urban block (200k
            rays, 4 M voxel capacity) with its per-phase CUDA-event profile,
            which gives the kernel roofline: HBM bytes of the dominant phase
            against the measured copy bandwidth, and (roofline.fp64) the
            FP64-bound phases against the FP64 pipe's issue rate;
  cpu_baseline  the CPU oracle (restated reference, one thread as the
            reference's MP_PROC_NUM=1) on a bounded sample of the streams.
The line ends with latency_ms and served_over_plain_same_mix (the metric's
two halves); per-phase detail goes to stderr ("bench detail: {...}").
`--impl reference` runs the CPU restatement on all streams of the served
workload, one single-threaded oracle per stream, all host cores.

`--workload urban|room` runs the plain one-stream path alone (value: HBM
resident with per-step CUDA events and an L2 flush between steps; e2e: from
pinned host buffers).  `--workload planefit` is the batched plane fit and its
precision study (1 M voxels), `--workload corridor` the long-horizon stress
(16 corridor streams under the LRU cap, drift against the oracle and the
ground truth), `--workload io` the steps either side of the path (Livox
decode, output clouds, plane-marker export, STD plane voxels).

Multi-GPU: streams shard by GPU (each rank serves its own streams), no
collective on the data path; "scaling": "weak".
"""
import argparse
import ctypes as C
import json
import os
import resource
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

# Algorithmic (minimum unique) bytes per unit of work for each profiled phase:
# (bytes per unit, unit name).  Units are the points the phase processes.
ALGO_BYTES = {
    "residual": (64.0, "downsampled point x IEKF iteration"),   # 16 B point + 16 B slot + 32 B plane record
    "map_state": (220.0, "inserted point"),                       # K-INS
    "undistort": (32.0, "raw point"),                             # K-UND
    "downsample": (32.0, "raw point"),                            # K-DS (+16 B per output point, not counted)
}
PROF_NAMES = ["upload", "time_sort", "predict", "undistort", "downsample", "body_cov", "residual", "residual_idle",
              "update_other", "map_batch", "map_group", "map_state", "map_finish", "result", "residual_step"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed scans (per stream for the served workload; default 16 there, 60 otherwise)")
    ap.add_argument("--warmup", type=int, default=None, help="warm-up scans (default 10 served, 3 corridor, 5 otherwise)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="serve", choices=["serve", "urban", "room", "planefit", "corridor", "io"])
    ap.add_argument("--voxels", type=int, default=1_000_000, help="planefit workload: voxels per batch")
    ap.add_argument("--fit-mode", default="fp32c", choices=["fp64", "fp32", "fp32c"],
                    help="planefit workload: arithmetic mode of the headline value")
    ap.add_argument("--streams", type=int, default=64, help="served workload: concurrent sensor streams")
    ap.add_argument("--workers", type=int, default=0, help="served workload: server worker threads (0: streams, <= 32)")
    ap.add_argument("--open-loop-scans", type=int, default=15, help="served workload: 10 Hz scans per stream")
    ap.add_argument("--hbm-budget-gb", type=float, default=150.0)
    ap.add_argument("--plain-steps", type=int, default=30, help="served workload: steps of the plain urban run")
    ap.add_argument("--points", type=int, default=None, help="rays per scan (default: workload's)")
    ap.add_argument("--map-capacity", type=int, default=None, help="plain workloads: LRU voxel capacity")
    ap.add_argument("--cpu-sample", type=int, default=None, help="CPU-baseline scans (default: bounded)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--flush-mb", type=int, default=256)
    a = ap.parse_args()
    if a.steps is None:
        a.steps = {"serve": 16, "planefit": 200, "corridor": 400}.get(a.workload, 60)
    if a.warmup is None:
        # served streams: past the first scans of map growth, whose extra map
        # work would make whichever phase runs first look ~12 % slower
        a.warmup = {"serve": 10, "corridor": 3}.get(a.workload, 5)
    if a.workload == "corridor" and "--streams" not in sys.argv:
        a.streams = 16
    return a


def workload(args, rank, name=None):
    from voxelmapplus_fastlio2_gb300 import abi, synth
    if (name or args.workload) == "urban":
        kind, pts, leaf, cap, iters = synth.KIND_URBAN, 200000, 0.1, 4000000, 4
        name = "urban block 100x100x20 m, spinning 128-beam, {}k rays/scan"
    else:
        kind, pts, leaf, cap, iters = synth.KIND_ROOM, 20000, 0.2, 100000, 5
        name = "room 20x20x5 m, rosette, {}k rays/scan"
    if args.points:
        pts = args.points
    name = name.format(f"{pts / 1000:g}")
    if getattr(args, "map_capacity", None):
        cap = args.map_capacity
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


# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) per unit of
# work of each profiled phase, from ncu captures on GB300: one steady scan of
# the urban block at 50k rays for the scan phases, k_fit<FP32C> on 200 000
# voxels / 13.16 M points for the fit.  The traffic grows in proportion to
# the units, so a launch's traffic is this times its units.
TRAFFIC_PER_UNIT = {
    "residual": 138.0,   # per downsampled point x IEKF iteration (k_residual<6, 4>)
    "map_state": 534.0,  # per inserted point: k_seg_chain + k_refit_eig + k_cov_terms + k_seg_cov
    "undistort": 17.3,   # per raw point
    "fit_fp32c": 51.5,   # per point
}


# FP64 warp instructions (ncu sm__inst_executed_pipe_fp64.sum) per unit of
# work of the FP64-bound phases: means over six steady scans of the 200k-ray
# urban block (a one-pass capture of this bench's own urban workload).
# These phases are bound by the FP64 pipe, not by
# HBM: an FP64 warp instruction holds an SM sub-partition's FP64 pipe for 64
# cycles whatever its active lanes (a dependent-DFMA micro-probe on this
# GB300), so the pipe's peak is 4 x SMs x clock / 64 warp instructions/s.
# The map-state kernels (k_seg_chain + k_refit_eig + k_cov_terms +
# k_seg_cov) are left out: their count per inserted point follows the scan's
# plane refits (19.0-25.6 over the six scans, and falling as voxels freeze),
# so no constant gives an honest rate for them.
FP64_PER_UNIT = {
    "residual": 5.81,   # per downsampled point x IEKF iteration
    "undistort": 7.11,  # per raw point
    "body_cov": 6.21,   # per downsampled point
    "map_batch": 5.59,  # per batch point
}
FP64_CYCLES_PER_WARP_INSTR = 64


def fp64_peak():
    """FP64 warp instructions/s of the whole GPU at its maximum SM clock."""
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            mhz = float(json.load(f)["sm_max_mhz"])
    except Exception:
        mhz = 2070.0
    return 4 * sms * mhz * 1e6 / FP64_CYCLES_PER_WARP_INSTR


def load_traffic(phase, units_per_launch):
    """DRAM bytes per launch of the phase (TRAFFIC_PER_UNIT x units), or None
    where no capture covers it."""
    t = TRAFFIC_PER_UNIT.get(phase)
    return None if t is None else t * units_per_launch


def pkg_arrays(p):
    pts = np.ctypeslib.as_array(C.cast(p.points, C.POINTER(C.c_float)), shape=(p.n, 4)).copy()
    imu = np.ctypeslib.as_array(C.cast(p.imus, C.POINTER(C.c_double)), shape=(p.n_imu, 7)).copy()
    return pts, imu


PROFILE_STEPS = 10


def run_value(args, pkgs, cfg, n_init, barrier):
    """Inputs resident in HBM; per-step CUDA events on the library's stream.
    The timed steps run as in production (captured scan graphs); the
    per-phase profile comes from PROFILE_STEPS further scans with the
    library's CUDA-event profiler on (direct launches, same kernels)."""
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
    P = min(PROFILE_STEPS, len(dev) - W - K)
    for i in range(W):
        d_pts, d_imu, p = dev[i]
        g.process_device(d_pts.data_ptr(), p.n, p.t_start, p.t_end, d_imu.data_ptr(), p.n_imu)
    torch.cuda.synchronize()
    barrier()
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
    g.lib.vmp_profile_enable(g.h, 1)
    m_calls, m_rounds, m_phase = [], [], []
    for i in range(W + K, W + K + P):
        d_pts, d_imu, p = dev[i]
        with torch.cuda.stream(stream):
            flush.fill_(i & 255)
        g.process_device(d_pts.data_ptr(), p.n, p.t_start, p.t_end, d_imu.data_ptr(), p.n_imu)
        # merge statistics of the scan (these reads wait for the stream; the
        # profiled scans are not timed)
        m_calls.append(g.lib.vmp_last_merge_calls(g.h))
        m_rounds.append(g.lib.vmp_last_merge_rounds(g.h))
        mp = (C.c_double * 64)()
        nmp = g.lib.vmp_last_merge_profile(g.h, mp, 64)
        if nmp > 2:
            m_phase.append([float(mp[k]) for k in range(nmp)])
    torch.cuda.synchronize()
    ms = (C.c_double * 16)()
    nl = (C.c_longlong * 16)()
    it = (C.c_longlong * 16)()
    g.lib.vmp_profile_read(g.h, ms, nl, it)
    prof = {PROF_NAMES[k]: {"ms": ms[k], "launches": nl[k], "items": it[k]} for k in range(len(PROF_NAMES))}
    g.lib.vmp_profile_enable(g.h, 0)
    out = {"step_ms": step_ms, "wall_s": t_wall, "launches": launches, "clocks": clk, "prof": prof,
           "prof_steps": max(P, 1), "n_raw": float(np.mean(n_raw)), "n_down": float(np.mean(n_down)),
           "map_size": int(res.map_size), "iters_last": int(res.iters),
           "merge": {"calls_per_scan": float(np.mean(m_calls)) if m_calls else 0.0,
                     "rounds_per_scan": float(np.mean(m_rounds)) if m_rounds else 0.0,
                     "rounds_max": int(max(m_rounds)) if m_rounds else 0,
                     "fixpoint_us": _merge_phases(m_phase)}}
    g.close()
    return out


def _merge_phases(runs):
    """Mean phase times (us) of the merge fixed point over the profiled
    scans: setup, the call tests and the merging calls of each round (over
    the scans that ran that round), and CTA 0's write-back."""
    if not runs:
        return None
    rounds = []
    for k in range(max((len(r) - 2) // 2 for r in runs)):
        rs = [r for r in runs if len(r) - 2 >= 2 * (k + 1)]
        rounds.append({"tests": round(float(np.mean([r[1 + 2 * k] for r in rs])), 2),
                       "merges": round(float(np.mean([r[2 + 2 * k] for r in rs])), 2), "scans": len(rs)})
    return {"setup": float(np.mean([r[0] for r in runs])), "rounds": rounds,
            "write_back": float(np.mean([r[-1] for r in runs])), "total": float(np.mean([sum(r) for r in runs]))}


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


# ------------------------------------------------------------------ served
def serve_streams(args, rank):
    """The served workload: per stream (kind, rays per scan, config, seed).
    Even streams are rooms, odd ones urban blocks, each with its own seeded
    scene and trajectory; rays per scan uniform in [2k, 200k]."""
    from voxelmapplus_fastlio2_gb300 import abi, synth
    rng = np.random.default_rng(0x5EED + rank)
    out = []
    for s in range(args.streams):
        kind = synth.KIND_ROOM if s % 2 == 0 else synth.KIND_URBAN
        rays = int(rng.integers(2000, 200001))
        if kind == synth.KIND_URBAN:
            cfg = abi.default_config(scan_resolution=0.1, map_capacity=400000, ieskf_max_iter=4,
                                     max_scan_points=rays + 64)
        else:
            cfg = abi.default_config(scan_resolution=0.2, map_capacity=100000, max_scan_points=rays + 64)
        out.append((kind, rays, cfg, 0x5EED0000 + 1000 * rank + 16 + s))
    return out


def make_serve_packages(streams, count):
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=4) as ex:
        return list(ex.map(lambda st: make_packages(st[0], st[1], st[3], count), streams))


def _drain(srv, total, timeout_s=600.0):
    res, t_end = [], time.perf_counter() + timeout_s
    while len(res) < total:
        if time.perf_counter() > t_end:
            raise RuntimeError(f"served run timed out with {len(res)} of {total} results")
        for r in srv.poll(max_results=1024, timeout_ms=200):
            if r.status != 0:
                raise RuntimeError(f"stream {r.stream_id} package {r.cookie}: status {r.status}")
            res.append(r)
    return res


def _stage_device(pk):
    import torch
    pts, imu = pkg_arrays(pk)
    return torch.from_numpy(pts).cuda(), torch.from_numpy(imu).cuda()


def run_served(args, streams, pkgs, workers, phases, barrier, keep_results=False):
    """One server, all streams.  Per stream the packages run in order:
    IMU_INIT + MAP_INIT + warm-up, then the phases:
      "device": K packages per stream, already in HBM, all submitted at once;
      "host":   K packages per stream from host memory (vmp_submit copies);
      "open":   open loop, each stream a Poisson process at 10 Hz for L
                packages, host memory.
    Returns per phase: scans/s, latencies, launches, clocks."""
    import torch
    from voxelmapplus_fastlio2_gb300 import lio as vlio
    from voxelmapplus_fastlio2_gb300.serve import Server
    W, K, L = args.warmup, args.steps, args.open_loop_scans
    srv = Server(hbm_budget_bytes=args.hbm_budget_gb * 1e9, max_streams=len(streams), workers=workers,
                 queue_depth=max(64, K + L + 8))
    out = {}
    try:
        sids = [srv.open_stream(cfg) for (_, _, cfg, _) in streams]
        out["budget_used_gb"] = srv.info()["budget_used"] / 1e9
        n0 = 2 + W
        for k in range(n0):
            for sid, pk in zip(sids, pkgs):
                srv.submit(sid, pk[k], cookie=k)
        _drain(srv, n0 * len(sids))
        nxt = n0
        lib = vlio.load()
        for ph in phases:
            if ph == "device":
                dev = [[_stage_device(pk[nxt + k]) for k in range(K)] for pk in pkgs]
                torch.cuda.synchronize()
            barrier()
            clocks = ClockSampler(torch.cuda.current_device())
            clocks.start()
            time.sleep(0.3)
            l0 = lib.vmp_launch_count()
            ru0 = resource.getrusage(resource.RUSAGE_SELF)
            t0 = time.perf_counter()
            if ph in ("device", "host"):
                for k in range(K):
                    for i, (sid, pk) in enumerate(zip(sids, pkgs)):
                        p = pk[nxt + k]
                        if ph == "device":
                            d_pts, d_imu = dev[i][k]
                            srv.submit_device(sid, d_pts.data_ptr(), p.n, p.t_start, p.t_end, d_imu.data_ptr(),
                                              p.n_imu, cookie=nxt + k)
                        else:
                            srv.submit(sid, p, cookie=nxt + k)
                res = _drain(srv, K * len(sids))
                nxt += K
            else:
                rng = np.random.default_rng(7)
                events = []
                for i in range(len(sids)):
                    t = float(rng.uniform(0.0, 0.1))
                    for k in range(L):
                        events.append((t, i, nxt + k))
                        t += float(rng.exponential(0.1))
                events.sort()
                got = []
                th = threading.Thread(target=lambda: got.extend(_drain(srv, len(events))))
                th.start()
                for t, i, k in events:
                    dt = t0 + t - time.perf_counter()
                    if dt > 0:
                        time.sleep(dt)
                    srv.submit(sids[i], pkgs[i][k], cookie=k)
                th.join()
                res = got
                nxt += L
            wall = time.perf_counter() - t0
            ru1 = resource.getrusage(resource.RUSAGE_SELF)
            cpu_s = (ru1.ru_utime - ru0.ru_utime) + (ru1.ru_stime - ru0.ru_stime)
            launches = lib.vmp_launch_count() - l0
            clk = clocks.stop()
            barrier()
            lat = [r.end_ms - r.submit_ms for r in res]
            svc = [r.end_ms - r.start_ms for r in res]
            out[ph] = {"scans": len(res), "wall_s": wall, "scans_per_s": len(res) / wall,
                       "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
                       "service_ms": {"p50": float(np.percentile(svc, 50)), "p99": float(np.percentile(svc, 99))},
                       "launches": launches, "clocks": clk, "host_cpu_cores_busy": cpu_s / wall,
                       "n_down_mean": float(np.mean([r.result.n_down for r in res]))}
            if keep_results:
                out[ph]["results"] = [(sids.index(r.stream_id), r.cookie, np.array(r.result.x.pos[:]),
                                       np.array(r.result.x.rot[:]).reshape(3, 3), r.result.evicted,
                                       r.result.map_size, np.array(r.result.P[:])) for r in res]
            if ph == "device":
                del dev
        out["tuning"] = srv.tuning()
    finally:
        srv.close()
    return out


def run_cpu_served(streams, pkgs, warmup, steps, threads, stream_ids, collect=None):
    """The CPU oracle on the served workload: the listed streams' packages,
    streams in parallel on `threads` host threads (one oracle per stream, as
    the reference runs one single-threaded node per sensor).  With a dict
    `collect`, the timed scans' results are stored in it by (stream, package
    index)."""
    from concurrent.futures import ThreadPoolExecutor
    import oracle

    def one(i):
        o = oracle.Oracle(streams[i][2], threads=1)
        for p in pkgs[i][:2 + warmup]:
            o.process(p)
        return o

    with ThreadPoolExecutor(max_workers=threads) as ex:
        ors = list(ex.map(one, stream_ids))

    def timed(j):
        i = stream_ids[j]
        for k, p in enumerate(pkgs[i][2 + warmup:2 + warmup + steps]):
            r = ors[j].process(p)
            if collect is not None:
                collect[(i, 2 + warmup + k)] = r

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(timed, range(len(stream_ids))))
    wall = time.perf_counter() - t0
    return len(stream_ids) * steps / wall, wall


def pose_errors(gpu, cpu):
    """Per-scan errors of served results against the oracle's: position (m),
    rotation angle (rad, by atan2) and the covariance P (max abs difference
    over max abs entry).  gpu: {(stream, package): (pos, rot, P)}."""
    dp, da, dP = [], [], []
    for key, ro in cpu.items():
        if key not in gpu:
            continue
        pos, rot, P = gpu[key]
        dp.append(float(np.linalg.norm(pos - np.array(ro.x.pos[:]))))
        Rd = rot.T @ np.array(ro.x.rot[:]).reshape(3, 3)
        sk = 0.5 * np.linalg.norm([Rd[2, 1] - Rd[1, 2], Rd[0, 2] - Rd[2, 0], Rd[1, 0] - Rd[0, 1]])
        da.append(float(np.arctan2(sk, (np.trace(Rd) - 1.0) / 2.0)))
        Po = np.array(ro.P[:])
        dP.append(float(np.max(np.abs(P - Po)) / max(float(np.max(np.abs(Po))), 1e-300)))
    if not dp:
        return None
    return {"scans": len(dp), "pos_m_max": max(dp), "rot_rad_max": max(da), "P_rel_max": max(dP)}


def dist_setup(args, backend=None):
    """One process per GPU (torchrun): rank, world size, a barrier and a max
    over ranks.  NCCL where GPUs are visible; gloo (CPU tensors) where none
    is, which is how the multi-rank path is tested on CPU."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws <= 1:
        return rank, ws, (lambda: None), (lambda x: x), None
    import torch
    import torch.distributed as dist
    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        dev = "cuda"
    else:
        dist.init_process_group("gloo")
        dev = "cpu"

    def barrier():
        dist.barrier()

    def allmax(x):
        t = torch.tensor([float(x)], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return rank, ws, barrier, allmax, dist


def aggregate_value(ws, scans_per_rank, wall_s, allmax):
    """Whole-job scans/s: every rank's scans over the slowest rank's time
    (weak scaling: each rank serves its own streams)."""
    return ws * scans_per_rank / allmax(wall_s)


def roofline_of(prof):
    """Roofline of the dominant profiled phase with an algorithmic byte count."""
    dom = max(ALGO_BYTES, key=lambda k: prof[k]["ms"])
    per_unit, unit_name = ALGO_BYTES[dom]
    launches = max(1, prof[dom]["launches"])
    avg_ms = prof[dom]["ms"] / launches
    bytes_per_launch = per_unit * prof[dom]["items"] / launches
    peak, peak_src = load_peaks()
    achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9 if avg_ms > 0 else 0.0
    phases = {}
    for k, (pu, _) in ALGO_BYTES.items():  # every phase with a byte count, the dominant one included
        nl = max(1, prof[k]["launches"])
        ms = prof[k]["ms"] / nl
        if ms > 0:
            a = pu * prof[k]["items"] / nl / (ms * 1e-3) / 1e9
            phases[k] = {"achieved": a, "frac": a / peak, "avg_launch_ms": ms}
    # the same phases against the FP64 pipe, which is what bounds them
    p64 = fp64_peak()
    f64 = {}
    for k, per in FP64_PER_UNIT.items():
        nl = max(1, prof[k]["launches"])
        ms = prof[k]["ms"] / nl
        if ms > 0 and prof[k]["items"] > 0:
            a = per * prof[k]["items"] / nl / (ms * 1e-3)
            f64[k] = {"achieved": a, "frac": a / p64, "avg_launch_ms": ms, "instr_per_unit": per}
    fp64 = {"bound": "fp64", "unit": "FP64 warp instructions/s", "peak": p64,
            "peak_source": "4 x SMs x max SM clock / 64 cycles per FP64 warp instruction (micro-probe)",
            "phases": f64}
    if f64:  # the FP64 phase with the most device time
        d64 = max(f64, key=lambda k: prof[k]["ms"])
        fp64.update({"kernel": d64, "achieved": f64[d64]["achieved"], "frac": f64[d64]["frac"]})
    return {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": load_traffic(dom, prof[dom]["items"] / launches),
            "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_ms,
            "bytes_per_unit": per_unit, "unit_of_work": unit_name, "peak_source": peak_src,
            "phases": phases, "fp64": fp64}


SERVE_NAME = ("64 independent streams, each its own seeded scene and trajectory (even: 20x20x5 m room, "
              "rosette; odd: 100x100x20 m urban block, 128-beam), rays/scan uniform 2k-200k, 10 Hz, "
              "HBM admission budget 150 GB")


def main_serve(args, rank, ws, barrier, allmax, dist):
    from voxelmapplus_fastlio2_gb300 import abi
    from voxelmapplus_fastlio2_gb300 import build as vbuild
    streams = serve_streams(args, rank)
    W, K, L = args.warmup, args.steps, args.open_loop_scans
    if args.workload == "serve" and args.streams != 64:
        name = SERVE_NAME.replace("64 independent", f"{args.streams} independent")
    else:
        name = SERVE_NAME
    rays = [s[1] for s in streams]
    cfg_line = {"workload": name, "streams_per_gpu": args.streams,
                "rays_per_scan": {"min": min(rays), "max": max(rays), "mean": round(float(np.mean(rays)))},
                "ieskf_max_iter": {"room": 5, "urban": 4}, "scan_resolution": {"room": 0.2, "urban": 0.1},
                "voxel_size": 0.5, "map_capacity": {"room": 100000, "urban": 400000},
                "parallelism": f"stream-sharded x{ws}, {args.streams} streams per GPU"}
    if args.impl == "reference":
        if rank != 0:
            return
        import oracle
        oracle.build() if not os.path.exists(oracle.ORACLE_SO) else None
        vbuild.build_synth()
        threads = os.cpu_count() or 1
        pkgs = make_serve_packages(streams, 2 + W + K)
        v, wall = run_cpu_served(streams, pkgs, W, K, threads, list(range(len(streams))))
        line = {"metric": METRIC, "value": v, "unit": "scans/s", "impl": "reference", "n_gpus": args.gpus,
                "steps": K, "warmup": W, "ms_per_step": 1e3 / v, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)", "config": cfg_line,
                "cpu_baseline": {"value": v, "unit": "scans/s", "cores": threads, "kind": "port",
                                 "sample": f"{K} mapping scans per stream of all {len(streams)} streams after "
                                           f"{W} warm-up scans; CPU restatement of the reference, one "
                                           f"single-threaded oracle per stream, {threads} streams at a time"},
                "e2e": {"value": v, "unit": "scans/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    vbuild.build_all()
    pkgs = make_serve_packages(streams, 2 + W + K + L)
    workers = args.workers or min(32, len(streams))
    # value (packages in HBM) and e2e (host buffers) on two servers fed the
    # same packages: the same scans from the same map states
    served = run_served(args, streams, pkgs, workers, ["device", "open"], barrier, keep_results=True)
    gpu_res = {(r[0], r[1]): (r[2], r[3], r[6]) for r in served["device"].pop("results")}
    served["open"].pop("results", None)
    served_host = run_served(args, streams, pkgs, workers, ["host"], barrier)
    plain_mix = run_served(args, streams, pkgs, 1, ["device"], barrier)
    # plain one-stream urban block (per-phase profile: the kernel roofline)
    kind, pts, ucfg, seed, uname = workload(args, rank, "urban")
    upk = make_packages(kind, pts, seed, 2 + W + args.plain_steps + PROFILE_STEPS)
    uargs = argparse.Namespace(**vars(args))
    uargs.steps = args.plain_steps
    uval = run_value(uargs, upk, ucfg, 2, barrier)
    uval_s = sum(uval["step_ms"]) / 1e3
    dv = served["device"]
    value = aggregate_value(ws, dv["scans"], dv["wall_s"], allmax)
    hv = served_host["host"]
    h2d = float(np.mean([p.n * C.sizeof(abi.vmp_point) + p.n_imu * C.sizeof(abi.vmp_imu)
                         for pk in pkgs for p in pk[2 + W:2 + W + K]]))
    roof = roofline_of(uval["prof"])
    detail = {"served": {"streams": args.streams, "workers": workers, "hbm_budget_gb": args.hbm_budget_gb,
                         "budget_used_gb": served["budget_used_gb"], "autotuner": served["tuning"],
                         "device_resident": dv, "host_buffers": hv, "open_loop_10hz": served["open"]},
              "rays_per_scan": rays, "roofline_phases": roof.pop("phases"),
              "fp64_phases": roof["fp64"].pop("phases"),
              "profile_ms_per_step_urban200k": {k: v["ms"] / uval["prof_steps"] for k, v in uval["prof"].items()}}
    roof["measured_on"] = "plain one-stream urban block run"
    line = {"metric": METRIC, "value": value, "unit": "scans/s", "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": 1e3 * allmax(dv["wall_s"]) / dv["scans"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": cfg_line,
            "steps_meaning": f"{K} mapping scans per stream, all submitted at once; value = scans of all streams "
                             "/ wall time; e2e = the same scans from the same map states on a second server, "
                             "packages from host memory",
            "e2e": {"value": ws * hv["scans"] / allmax(hv["wall_s"]), "unit": "scans/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(C.sizeof(abi.vmp_result)),
                    "latency_ms": hv["latency_ms"]},
            "plain_1stream": {
                "same_mix_scans_per_s": plain_mix["device"]["scans_per_s"],
                "urban200k": {"scans_per_s": len(uval["step_ms"]) / uval_s,
                              "latency_ms": {"p50": float(np.percentile(uval["step_ms"], 50)),
                                             "p99": float(np.percentile(uval["step_ms"], 99))}}},
            "roofline": roof, "clocks": dv["clocks"], "gpu_launches": dv["launches"]}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        ids = list(range(min(4, len(streams))))
        cpk = [pkgs[i][:2 + W + K] if i in ids else [] for i in range(len(streams))]
        cres = {}
        v1, wall = run_cpu_served(streams, cpk, W, K, 1, ids, collect=cres)
        line["pose_vs_oracle"] = pose_errors(gpu_res, cres)
        line["cpu_baseline"] = {"value": v1, "unit": "scans/s", "cores": 1, "kind": "port",
                                "sample": f"{K} mapping scans of each of streams {ids} (rays/scan "
                                          f"{[streams[i][1] for i in ids]}) after {W} warm-up scans; CPU "
                                          "restatement of the reference on 1 thread",
                                "host_cores": os.cpu_count()}
    # the metric's two halves last, so that a record keeping only the end of
    # the line still holds them
    line["latency_ms"] = dict(served["open"]["latency_ms"], arrivals="Poisson 10 Hz per stream",
                              streams=args.streams)
    line["served_over_plain_same_mix"] = dv["scans_per_s"] / plain_mix["device"]["scans_per_s"]
    if rank == 0:
        print("bench detail: " + json.dumps(detail), file=sys.stderr)
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


CORRIDOR_NAME = ("long-horizon stress: {s} independent streams, each a 1 km corridor (walls, floor, ceiling, "
                 "pillars; its own seed and trajectory) seen by a spinning 32-beam LiDAR, 100k rays/scan, 10 Hz, "
                 "{k} mapping scans per stream, LRU capacity {cap} voxels per stream")


def main_corridor(args, rank, ws, barrier, allmax, dist):
    """Long-horizon stress (1 km corridors): many corridor streams served
    with the LRU cap in force; throughput, latency, eviction counts, and the
    drift of stream 0 against the oracle and against the ground truth."""
    from voxelmapplus_fastlio2_gb300 import abi, synth
    from voxelmapplus_fastlio2_gb300 import build as vbuild
    cap = args.map_capacity or 8000
    W, K = args.warmup, args.steps
    cfg = abi.default_config(scan_resolution=0.2, map_capacity=cap, max_scan_points=100000 + 64)
    streams = [(synth.KIND_CORRIDOR, 100000, cfg, 0x5EED0000 + 1000 * rank + 64 + s) for s in range(args.streams)]
    name = CORRIDOR_NAME.format(s=args.streams, k=K, cap=cap)
    from concurrent.futures import ThreadPoolExecutor
    L = args.open_loop_scans
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        pkgs = list(ex.map(lambda st: make_packages(st[0], st[1], st[3], 2 + W + K + L), streams))
    if args.impl == "reference":
        if rank != 0:
            return
        threads = os.cpu_count() or 1
        v, wall = run_cpu_served(streams, pkgs, W, K, threads, list(range(len(streams))))
        print(json.dumps({"metric": METRIC, "value": v, "unit": "scans/s", "impl": "reference", "n_gpus": args.gpus,
                          "steps": K, "warmup": W, "ms_per_step": 1e3 / v, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
                          "config": {"workload": name},
                          "cpu_baseline": {"value": v, "unit": "scans/s", "cores": threads, "kind": "port",
                                           "sample": f"{K} mapping scans of each of {len(streams)} streams, one "
                                                     "single-threaded oracle per stream"},
                          "e2e": {"value": v, "unit": "scans/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    vbuild.build_all()
    workers = args.workers or min(32, len(streams))
    served = run_served(args, streams, pkgs, workers, ["device", "open"], barrier, keep_results=True)
    dv = served["device"]
    value = aggregate_value(ws, dv["scans"], dv["wall_s"], allmax)
    # stream 0 against the oracle (same packages) and the ground truth
    import oracle
    res0 = sorted([r for r in dv["results"] if r[0] == 0], key=lambda r: r[1])
    o = oracle.Oracle(cfg)
    seq = synth.Sequence(synth.KIND_CORRIDOR, seed=streams[0][3], points_per_scan=100000)
    d_oracle, d_truth_g, d_truth_o, p_first = [], [], [], None
    ro = None
    for k, pk in enumerate(pkgs[0][:2 + W + K]):
        ro = o.process(pk)
        if k < 2 + W:
            continue
        r = res0[k - 2 - W]
        _, pg = seq.pose(pk.t_end)
        if p_first is None:
            p_first = pg - np.array(ro.x.pos[:])
        Rd = r[3].T @ np.array(ro.x.rot[:]).reshape(3, 3)  # angle by atan2: accurate near 0
        sk = 0.5 * np.linalg.norm([Rd[2, 1] - Rd[1, 2], Rd[0, 2] - Rd[2, 0], Rd[1, 0] - Rd[0, 1]])
        d_oracle.append((float(np.linalg.norm(r[2] - np.array(ro.x.pos[:]))),
                         float(np.arctan2(sk, (np.trace(Rd) - 1.0) / 2.0))))
        d_truth_g.append(float(np.linalg.norm(r[2] - (pg - p_first))))
        d_truth_o.append(float(np.linalg.norm(np.array(ro.x.pos[:]) - (pg - p_first))))
    evicted = int(sum(r[4] for r in dv["results"]))
    line = {"metric": METRIC, "value": value, "unit": "scans/s", "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": 1e3 * allmax(dv["wall_s"]) / dv["scans"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": name, "streams_per_gpu": args.streams, "map_capacity": cap,
                       "scan_resolution": 0.2, "voxel_size": 0.5,
                       "capacity_note": "a 1 km corridor holds ~1e5 surface voxels at 0.5 m, so a 20 M cap never "
                                        "evicts; the cap is set below the visible voxel set to keep the LRU "
                                        "eviction path busy"},
            "latency_ms": served["open"]["latency_ms"], "latency_note": f"open loop: each stream a Poisson "
                                                                          f"process at 10 Hz for {L} scans",
            "service_ms": dv["service_ms"],
            "evicted_voxels_total": evicted, "evicted_per_scan": evicted / max(1, dv["scans"]),
            "map_size_end_stream0": int(res0[-1][5]) if res0 else None,
            "stream0_vs_oracle": {"pos_m_max": max(d[0] for d in d_oracle), "rot_rad_max": max(d[1] for d in d_oracle),
                                  "scans": len(d_oracle)},
            "stream0_drift_vs_truth_m": {"gpu_end": d_truth_g[-1], "gpu_max": max(d_truth_g),
                                         "oracle_end": d_truth_o[-1], "oracle_max": max(d_truth_o)},
            "clocks": dv["clocks"], "gpu_launches": dv["launches"]}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


IO_METRIC = "points/s: Livox decode, output clouds, plane-marker export, STD plane voxels (device vs CPU restatement)"


def _wall(fn, reps):
    t = time.perf_counter()
    out = None
    for _ in range(reps):
        out = fn()
    return (time.perf_counter() - t) / reps, out


def main_io(args, rank, ws, barrier, allmax, dist):
    """The steps either side of the path, through their public entry points
    with host buffers (copies inside the timing), next to the CPU
    restatement: livox2pcl on the urban sequence's messages, lidarToBody +
    lidarToWorld of the undistorted cloud, the plane-marker walk of the map,
    and STD plane voxels of a 10-scan key cloud."""
    import oracle
    from voxelmapplus_fastlio2_gb300 import abi, fit, lio
    from voxelmapplus_fastlio2_gb300 import build as vbuild
    if rank != 0:
        return
    kind, pts, cfg, seed, uname = workload(args, rank, "urban")
    K = max(3, min(args.steps, 20))
    pkgs = make_packages(kind, pts, seed, 2 + K)
    rng = np.random.default_rng(3)
    msgs = []
    for p in pkgs:
        a = pkg_arrays(p)[0]
        m = np.zeros(p.n, dtype=abi.livox_dtype())
        m["x"], m["y"], m["z"] = a[:, 0], a[:, 1], a[:, 2]
        m["offset_time"] = np.rint(a[:, 3].astype(np.float64) * 1e6).astype(np.uint32)
        m["reflectivity"] = rng.integers(0, 256, p.n)
        m["tag"] = rng.choice(np.array([0x00, 0x10, 0x20], dtype=np.uint8), p.n, p=[0.6, 0.35, 0.05])
        m["line"] = rng.choice(np.array([0, 1, 2, 3, 4], dtype=np.uint8), p.n, p=[0.24] * 4 + [0.04])
        msgs.append(m)
    ours = args.impl != "reference"
    if ours:
        vbuild.build_all()
        g = lio.LIOBuilder(cfg)
        l0 = g.lib.vmp_launch_count()
    o = oracle.Oracle(cfg)
    world, comp = [], {}
    t_dec_g = t_dec_c = t_out_g = t_out_c = 0.0
    n_dec = 0
    for k, (p, m) in enumerate(zip(pkgs, msgs)):
        t0 = time.perf_counter()
        op, oi = oracle.livox_decode(m, 1, 0.1, 200.0)
        t_dec_c += time.perf_counter() - t0
        o.process_points(op, p.t_start, p.t_end, p.imus, p.n_imu, oi)
        if ours:
            t0 = time.perf_counter()
            g.livox_decode(m, 1, 0.1, 200.0, copy_out=False)  # count and last time only, as the node needs
            t_dec_g += time.perf_counter() - t0
            g.process_decoded(p.t_start, p.t_end, p.imus, p.n_imu)
        n_dec += len(op)
        if k >= 2:
            t0 = time.perf_counter()
            cw, _ = o.output_cloud(1)
            o.output_cloud(0)
            t_out_c += time.perf_counter() - t0
            world.append(cw)
            if ours:
                t0 = time.perf_counter()
                g.output_cloud(1)
                g.output_cloud(0)
                t_out_g += time.perf_counter() - t0
    n_in = sum(len(m) for m in msgs)
    n_out = 2 * sum(len(w) for w in world)
    key = np.ascontiguousarray(np.concatenate(world[-10:]))
    # back to back (the timings inside the sequence above interleave the
    # CPU restatement's scans, during which the GPU idles and clocks down):
    # both output clouds of the last scan, then every message decoded again
    R = len(world)
    n_out_b = 2 * R * len(world[-1])
    tc_out, _ = _wall(lambda: (o.output_cloud(1), o.output_cloud(0)), R)
    tc_dec, _ = _wall(lambda: [oracle.livox_decode(m, 1, 0.1, 200.0) for m in msgs], 1)
    comp["livox_decode"] = {"messages": len(msgs), "points_in": n_in, "points_kept": n_dec,
                            "cpu_points_per_s": n_in / tc_dec, "cpu_points_per_s_in_sequence": n_in / t_dec_c}
    comp["output_clouds"] = {"points": n_out_b, "cpu_points_per_s": n_out_b / (R * tc_out),
                             "cpu_points_per_s_in_sequence": n_out / t_out_c}
    if ours:
        g.output_cloud(1)
        tg_out, _ = _wall(lambda: (g.output_cloud(1), g.output_cloud(0)), R)
        g.livox_decode(msgs[0], 1, 0.1, 200.0, copy_out=False)
        tg_dec, _ = _wall(lambda: [g.livox_decode(m, 1, 0.1, 200.0, copy_out=False) for m in msgs], 1)
    mk = np.zeros(100000, dtype=abi.plane_marker_dtype())
    tc, nm = _wall(lambda: o.lib.orc_map_planes(o.h, mk.ctypes.data_as(C.POINTER(abi.vmp_plane_marker)), 100000), 3)
    info = abi.vmp_map_info()
    o.lib.orc_map_info(o.h, C.byref(info))
    comp["map_planes"] = {"map_voxels": int(info.size), "markers": int(nm), "cpu_ms": 1e3 * tc}
    so = np.zeros(len(key), dtype=abi.std_voxel_dtype())
    tc, ns = _wall(lambda: o.lib.orc_std_plane_voxels(key.ctypes.data_as(C.POINTER(C.c_float)), 4, len(key), 1.0, 10,
                                                        0.01, so.ctypes.data_as(C.POINTER(abi.vmp_std_voxel)),
                                                        len(key)), 2)
    comp["std_plane_voxels"] = {"points": int(len(key)), "voxels": int(ns), "cpu_ms": 1e3 * tc}
    base = {"metric": IO_METRIC, "unit": "points/s", "n_gpus": 1, "steps": K, "warmup": 2, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)"}
    cfg_line = {"workload": uname + "; Livox messages made from its scans (20 B per point), key cloud = the last "
                                    "10 world clouds", "components": comp}
    cpu = {"value": n_in / tc_dec, "unit": "points/s", "cores": 1, "kind": "port",
           "sample": f"{len(msgs)} Livox messages back to back, CPU restatement of livox2pcl on 1 thread"}
    if not ours:
        print(json.dumps(dict(base, value=cpu["value"], impl="reference", ms_per_step=1e3 * tc_dec / len(msgs),
                              config=cfg_line, cpu_baseline=cpu,
                              e2e={"value": cpu["value"], "unit": "points/s", "h2d_bytes_per_step": 0,
                                   "d2h_bytes_per_step": 0})))
        return
    tg, ng = _wall(lambda: g.map.planes(100000), 5)
    comp["map_planes"].update({"gpu_ms": 1e3 * tg, "gpu_markers": int(len(ng))})
    tg, gs = _wall(lambda: fit.std_plane_voxels(key, 1.0, 10, 0.01), 3)
    comp["std_plane_voxels"].update({"gpu_ms": 1e3 * tg, "gpu_voxels": int(len(gs))})
    comp["livox_decode"].update({"gpu_points_per_s": n_in / tg_dec, "gpu_points_per_s_in_sequence": n_in / t_dec_g})
    comp["output_clouds"].update({"gpu_points_per_s": n_out_b / (R * tg_out),
                                  "gpu_points_per_s_in_sequence": n_out / t_out_g})
    # the served form: the raw messages through vmp_submit_livox (decoded by
    # the workers), 8 streams each with its own map and filter fed the same
    # message sequence, all submitted at once; the whole sequence (IMU and
    # map initialisation included) until the last result is polled
    from voxelmapplus_fastlio2_gb300.serve import Server
    S = 8
    scfg = abi.default_config(scan_resolution=cfg.scan_resolution, map_capacity=400000,
                              ieskf_max_iter=cfg.ieskf_max_iter, max_scan_points=cfg.max_scan_points)
    srv = Server(hbm_budget_bytes=150e9, max_streams=S, workers=S)
    try:
        sids = [srv.open_stream(scfg) for _ in range(S)]
        t0 = time.perf_counter()
        for k, (p, m) in enumerate(zip(pkgs, msgs)):
            for sid in sids:
                srv.submit_livox(sid, m, p.t_start, p.imus, p.n_imu, filter_num=1, range_min=0.1, range_max=200.0,
                                 cookie=k)
        got, bad = 0, 0
        while got < S * len(msgs):
            rs = srv.poll(max_results=256, timeout_ms=1000)
            got += len(rs)
            bad += sum(1 for r in rs if r.status != abi.VMP_OK)
        t_srv = time.perf_counter() - t0
    finally:
        srv.close()
    comp["served_livox"] = {"streams": S, "messages": S * len(msgs), "failed": bad,
                            "messages_per_s": S * len(msgs) / t_srv, "points_per_s": S * n_in / t_srv,
                            "note": "vmp_submit_livox: decode + the whole scan step per message, from host buffers"}
    v = n_in / tg_dec
    print(json.dumps(dict(base, value=v, ms_per_step=1e3 * tg_dec / len(msgs), config=cfg_line,
                          e2e={"value": v, "unit": "points/s", "h2d_bytes_per_step": int(20 * n_in / len(msgs)),
                               "d2h_bytes_per_step": 8},
                          gpu_launches=int(g.lib.vmp_launch_count() - l0), cpu_baseline=cpu)))
    g.close()


PLANEFIT_METRIC = "voxels/s: batched plane fit (updatePlane over every voxel), FP32 compensated vs FP32 vs FP64"
PLANEFIT_NAME = ("batched plane fit + precision study: {v} voxels of a 0.5 m grid over +-100 x +-100 x +-10 m, "
                 "points/voxel lognormal (median 40, sigma 1) clipped to [5, 4000], 1 cm normal noise, "
                 "10% isotropic voxels")


def planefit_bytes(off, rec):
    """Algorithmic (unique) bytes of one fit call: every point's xyz (12 B),
    the covariance of the points of plane voxels (24 B; a non-plane voxel's
    plane covariance is not formed), the offsets (8 B per voxel) and the 296 B
    record written per voxel."""
    counts = np.diff(off)
    plane = (rec["flags"] & 2) != 0
    V, N = len(counts), int(off[-1])
    Np = int(counts[plane].sum())
    return {"fit": 12.0 * N + 24.0 * Np + (8 + 296) * V, "points": N, "plane_points": Np}


def main_planefit(args, rank, ws, barrier, allmax, dist):
    """Batched plane fitting (1 M voxels): value = voxels/s of the chosen
    mode with the batch resident in HBM; e2e = the host-buffer call
    (vmp_fit_planes) with the copies inside; precision of all three modes
    against the oracle (FP64, the reference's sequential arithmetic)."""
    from voxelmapplus_fastlio2_gb300 import abi, fit
    import oracle
    modes = {"fp64": fit.FP64, "fp32": fit.FP32, "fp32c": fit.FP32C}
    xyz, cov, off = fit.synth_voxels(args.voxels, seed=0x5EED0000 + rank)
    V, N = len(off) - 1, xyz.shape[1]
    name = PLANEFIT_NAME.format(v=V)
    olib = oracle.load()
    threads = os.cpu_count() or 1

    def oracle_fit(lo, hi, nthreads):
        o = off[lo:hi + 1] - off[lo]
        px = np.ascontiguousarray(xyz[:, off[lo]:off[hi]])
        pc = np.ascontiguousarray(cov[:, off[lo]:off[hi]])
        out = np.zeros(hi - lo, dtype=abi.fit_rec_dtype())
        olib.orc_fit_planes(px.ctypes.data_as(C.POINTER(C.c_float)), pc.ctypes.data_as(C.POINTER(C.c_float)),
                            o.ctypes.data_as(C.POINTER(C.c_longlong)), hi - lo, px.shape[1], 10, 0.01,
                            out.ctypes.data_as(C.POINTER(abi.vmp_fit_rec)), nthreads)
        return out

    if args.impl == "reference":
        if rank != 0:
            return
        sample = min(V, 50_000)
        ts = []
        for i in range(args.warmup + args.steps):
            lo = (i * sample) % max(1, V - sample + 1)
            t0 = time.perf_counter()
            oracle_fit(lo, lo + sample, threads)
            if i >= args.warmup:
                ts.append(time.perf_counter() - t0)
        v = sample * len(ts) / sum(ts)
        print(json.dumps({"metric": PLANEFIT_METRIC, "value": v, "unit": "voxels/s", "impl": "reference",
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1e3 * sum(ts) / len(ts), "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
                          "config": {"workload": name, "voxels": V, "points": N},
                          "cpu_baseline": {"value": v, "unit": "voxels/s", "cores": threads, "kind": "port",
                                           "sample": f"{sample} consecutive voxels per step, CPU restatement "
                                                     f"of addPoint + updatePlane on {threads} OpenMP threads"},
                          "e2e": {"value": v, "unit": "voxels/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return
    from voxelmapplus_fastlio2_gb300 import build as vbuild
    from voxelmapplus_fastlio2_gb300._lib import load
    vbuild.build_all()
    import torch
    lib = load()
    stream = torch.cuda.Stream()
    d_xyz = torch.from_numpy(xyz).cuda()
    d_cov = torch.from_numpy(cov).cuda()
    d_off = torch.from_numpy(off).cuda()
    rs = abi.fit_rec_dtype().itemsize
    d_out = torch.zeros(V * rs, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()

    def run(mode):
        fit.fit_planes_device(d_xyz.data_ptr(), d_cov.data_ptr(), d_off.data_ptr(), V, N, d_out.data_ptr(),
                              mode=mode, cuda_stream=stream.cuda_stream)

    # precision of every mode against the oracle on the whole batch
    t0 = time.perf_counter()
    ref = oracle_fit(0, V, threads)
    t_oracle = time.perf_counter() - t0
    precision, per_mode = {}, {}
    for mname, mode in modes.items():
        run(mode)
        stream.synchronize()
        rec = d_out.cpu().numpy().view(abi.fit_rec_dtype()).reshape(-1)
        precision[mname] = fit.compare(rec, ref)
    bytes_ = planefit_bytes(off, ref)
    mode = modes[args.fit_mode]
    for mname, m in modes.items():  # short timing of every mode
        for _ in range(2):
            run(m)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 10 if mname == "fp64" else 30
        a.record(stream)
        for _ in range(reps):
            run(m)
        b.record(stream)
        b.synchronize()
        per_mode[mname] = {"voxels_per_s": V * reps / (a.elapsed_time(b) * 1e-3),
                           "ms_per_call": a.elapsed_time(b) / reps}
    for _ in range(args.warmup):
        run(mode)
    stream.synchronize()
    barrier()
    l0 = lib.vmp_launch_count()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    evs = []
    for _ in range(args.steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        run(mode)
        b.record(stream)
        evs.append((a, b))
    stream.synchronize()
    barrier()
    clk = clocks.stop()
    launches = lib.vmp_launch_count() - l0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    t_step = allmax(sum(step_ms) / 1e3)
    value = ws * V * args.steps / t_step
    # the kernel's own device time (profiled calls: events around the launch)
    lib.vmp_fit_profile(1)
    P = 10
    for _ in range(P):
        run(mode)
    ms = C.c_double()
    calls = C.c_longlong()
    lib.vmp_fit_profile_read(C.byref(ms), C.byref(calls))
    lib.vmp_fit_profile(0)
    kms = ms.value / max(1, calls.value)
    peak, peak_src = load_peaks()
    achieved = bytes_["fit"] / (kms * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": "k_fit<" + args.fit_mode + ">", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak,
            "traffic": load_traffic("fit_" + args.fit_mode, bytes_["points"]),
            "algorithmic_bytes_per_launch": bytes_["fit"], "avg_launch_ms": kms, "peak_source": peak_src,
            "bytes_per_unit": "12 B per point + 24 B per plane-voxel point + 304 B per voxel"}
    # e2e: the host-buffer entry point from pinned memory, copies inside
    h_xyz = torch.from_numpy(xyz).pin_memory()
    h_cov = torch.from_numpy(cov).pin_memory()
    h_off = torch.from_numpy(off).pin_memory()
    h_out = torch.zeros(V * rs, dtype=torch.uint8).pin_memory()
    p = fit.params(mode)
    walls = []
    E = max(3, min(20, args.steps // 10))
    for i in range(1 + E):
        t0 = time.perf_counter()
        rc = lib.vmp_fit_planes(C.c_void_p(h_xyz.data_ptr()), C.c_void_p(h_cov.data_ptr()),
                                C.c_void_p(h_off.data_ptr()), V, N, C.byref(p), C.c_void_p(h_out.data_ptr()))
        if rc != 0:
            raise RuntimeError(f"vmp_fit_planes: status {rc}")
        if i > 0:
            walls.append(time.perf_counter() - t0)
    e2e_v = ws * V * len(walls) / allmax(sum(walls))
    # CPU baseline: the oracle on the whole batch, all host threads (it is
    # also the precision reference above), and one thread on a slice
    t1 = time.perf_counter()
    n1 = min(V, 20_000)
    oracle_fit(0, n1, 1)
    t1 = time.perf_counter() - t1
    line = {"metric": PLANEFIT_METRIC, "value": value, "unit": "voxels/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_step / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": {"fp64": "f64", "fp32": "f32", "fp32c": "f32"}[args.fit_mode],
            "data": "synthetic (seeded generator)",
            "config": {"workload": name, "voxels": V, "points": N, "mode": args.fit_mode,
                       "update_point_thresh": 10, "plane_thresh": 0.01,
                       "l2": f"inputs {(36 * N) / 1e9:.2f} GB > L2 (129 MB): no flush"},
            "e2e": {"value": e2e_v, "unit": "voxels/s", "h2d_bytes_per_step": int(36 * N + 8 * (V + 1)),
                    "d2h_bytes_per_step": int(rs * V)},
            "roofline": roof, "clocks": clk, "gpu_launches": int(launches), "modes": per_mode,
            "precision_vs_oracle": precision,
            "cpu_baseline": {"value": V / t_oracle, "unit": "voxels/s", "cores": threads, "kind": "port",
                             "sample": f"all {V} voxels, CPU restatement of addPoint + updatePlane on {threads} "
                                       f"OpenMP threads; one thread: {n1 / t1:.0f} voxels/s on {n1} voxels"}}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    from voxelmapplus_fastlio2_gb300 import build as vbuild
    if args.workload == "serve":
        # 64 streams need more than the default 8 hardware work queues (set
        # before the process creates its CUDA context)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    rank, ws, barrier, allmax, dist = dist_setup(args)
    if args.workload == "serve":
        return main_serve(args, rank, ws, barrier, allmax, dist)
    if args.workload == "planefit":
        return main_planefit(args, rank, ws, barrier, allmax, dist)
    if args.workload == "corridor":
        return main_corridor(args, rank, ws, barrier, allmax, dist)
    if args.workload == "io":
        return main_io(args, rank, ws, barrier, allmax, dist)
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
    pkgs = make_packages(kind, pts, seed, n_init + args.warmup + args.steps + PROFILE_STEPS)
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
    prof = val["prof"]
    line["roofline"] = roofline_of(prof)
    line["profile_ms_per_step"] = {k: v["ms"] / val["prof_steps"] for k, v in prof.items()}
    line["merge"] = dict(val["merge"], map_finish_ms_per_scan=prof["map_finish"]["ms"] / val["prof_steps"],
                         note="map_finish = the merge fixed point (one cooperative launch) + LRU queue + finalize")
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
