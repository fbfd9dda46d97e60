#!/usr/bin/env python
"""Scan->map throughput of the GB300 G-VOM path (one JSON line on rank 0).

Workload (default): OS1-64-shaped scans (64 x 1024 = 65,536 float32 points)
plus world-fixed vegetation at 20 points/m^2 inside the map footprint, along a
seeded 100-scan trajectory (0.4 m and up to 3 deg yaw per scan, float32 4x4
transforms); grid 256 x 256 x 64 at 0.15 m, buffer 4.  Synthetic, seeded
(gvom_gb300.synthetic): the reference publishes no dataset.

One step = one scan through Process_pointcloud followed by combine_maps (the
plain per-scan form of the path).  Metric: points/sec = points ingested per
step / step time.

  value    device-resident inputs (points already in HBM, maps written to
           device buffers), per-step CUDA events on the launching stream,
           L2 flushed (256 MB write) before every step outside the timed span
  e2e      the public API with host buffers: numpy points in, numpy maps out
           (host<->device copies inside the timed span), wall clock
  roofline per-kernel CUDA-event durations inside the timed region; the
           dominant kernel's algorithmic bytes / its mean launch time against
           the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (restatement of the reference path) on all
           host threads, a time-bounded sample of the same workload

--impl reference: the reference's own path cannot run on this machine (no numba,
no compiled parts), so the reference arm times the CPU restatement of it with
all host threads, on the same workload / metric.

Multi-GPU (torchrun): independent replicas, one map instance per GPU, no
collective on the data path; value = all ranks' points / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "scan->map points/sec (process_pointcloud + combine_maps per scan)"
UNIT = "points/s"
L2_FLUSH_BYTES = 256 << 20

# per-stage algorithmic bytes; see DESIGN.md "Roofline accounting"
def stage_bytes(name, n, V, Vext, X2, C_slot, C_sum, Cc, Cc_last, nsrc):
    if name == "k_voxelize_trace":
        return 12 * n + 64
    if name == "k_assign":
        return 8 * Vext + 4 * V + 12 * C_slot
    if name == "k_scatter":
        return 20 * n + 16 * n
    if name == "k_cell_moments":
        return 20 * n + 16 * n + 48 * C_slot
    if name == "k_voxel_stats":
        return 52 * C_slot + 27 * 56 * C_slot
    if name == "k_cleanup":
        return 20 * n
    if name == "k_merge":
        return 4 * V * nsrc + 4 * V + 4 * Cc + 8 * X2 * ((V // X2 + 7) // 8)
    if name == "k_merge_stats":
        return 4 * Cc + 4 * nsrc * Cc + 64 * (C_sum + Cc_last) + 64 * Cc
    if name == "k_columns":
        return 8 * X2 * ((V // X2 + 7) // 8) + 28 * X2
    if name == "k_maps2d":
        return 20 * X2 + 20 * X2 + 24 * X2
    return 0


def env_rank():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", str(r)))
    return r, w, lr


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.p = None
        self.gpu = gpu_index
        self.path = os.path.join(HERE, "gpurun_out", f"clocks_gpu{gpu_index}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-i", str(self.gpu), "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(5)
        except Exception:
            self.p.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(dict(sm=float(parts[1]), smax=float(parts[2]), active=parts[4],
                                 hw=parts[5], hwt=parts[6], swt=parts[7], swp=parts[8]))
            except ValueError:
                continue
        if not rows:
            return None
        reasons = set()
        for r in rows:
            for k, nm in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                          ("swp", "sw_power_cap")):
                if r[k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(r["sm"] for r in rows), "sm_max_mhz": max(r["smax"] for r in rows),
                "samples": len(rows), "reasons": sorted(reasons)}


def measured_peak_hbm():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(kernel, workload):
    """Per-launch DRAM bytes of `kernel` from a committed ncu summary, or None."""
    try:
        with open(os.path.join(HERE, "profiles", "dram_traffic.json")) as f:
            d = json.load(f)
        return d.get(workload, {}).get(kernel)
    except Exception:
        return None


def make_scans(w, n, device):
    from gvom_gb300.synthetic import make_workload_scans
    return make_workload_scans(w, n, device=device)


def cpu_baseline(w, scans, budget_s=12.0, threads=None):
    """Time the CPU oracle (all host threads) on a bounded sample of the workload."""
    from oracle.oracle import OracleGvom
    threads = threads or os.cpu_count() or 1
    o = OracleGvom(*w.gvom_args(), threads=threads)
    pts = 0
    steps = 0
    t0 = time.perf_counter()
    while True:
        s = scans[steps % len(scans)]
        o.Process_pointcloud(s.points, s.ego, s.transform)
        o.combine_maps()
        pts += s.points.shape[0]
        steps += 1
        if time.perf_counter() - t0 >= budget_s and steps >= 3:
            break
    dt = time.perf_counter() - t0
    return {"value": pts / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} steps (process+combine) of {w.name}, {pts} points, {dt:.1f} s"}


def run_reference(args, w):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    scans = make_scans(w, min(100, max(8, args.steps + args.warmup)), device="cpu" if not _has_cuda() else "cuda")
    from oracle.oracle import OracleGvom
    threads = os.cpu_count() or 1
    o = OracleGvom(*w.gvom_args(), threads=threads)
    tw = time.perf_counter()
    for i in range(max(1, args.warmup)):
        s = scans[i % len(scans)]
        o.Process_pointcloud(s.points, s.ego, s.transform)
        o.combine_maps()
    est = (time.perf_counter() - tw) / max(1, args.warmup)
    # bounded sample: at most ~60 s of CPU work whatever --steps asks for
    n_run = int(min(args.steps, max(3, 60.0 / max(est, 1e-3))))
    times = []
    pts = 0
    t_start = time.perf_counter()
    for k in range(n_run):
        s = scans[(args.warmup + k) % len(scans)]
        t0 = time.perf_counter()
        o.Process_pointcloud(s.points, s.ego, s.transform)
        o.combine_maps()
        times.append(time.perf_counter() - t0)
        pts += s.points.shape[0]
    total = time.perf_counter() - t_start
    v = pts / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": n_run,
        "steps_requested": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (reference typing)", "data": "synthetic",
        "config": {"workload": w.name, "grid": [w.xy_size, w.xy_size, w.z_size], "voxel_m": w.res,
                   "buffer_size": w.buffer_size, "points_per_scan": int(pts / n_run)},
        "latency_ms": {"p50": 1e3 * float(np.percentile(times, 50)), "p99": 1e3 * float(np.percentile(times, 99))},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n_run} steps of {w.name} on the CPU restatement of the reference path "
                                   f"({total:.1f} s); the reference itself (Numba CUDA) cannot run here: "
                                   "numba is not installed on this box"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _has_cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def run_gpu(args, w):
    import torch
    from gvom_gb300 import Gvom
    from gvom_gb300 import build as gb

    rank, world, lrank = env_rank()
    torch.cuda.set_device(lrank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    gb.build()
    nscan = min(100, max(1, args.steps + args.warmup))
    scans = make_scans(w, nscan, device="cuda")
    n_pts = [s.points.shape[0] for s in scans]

    stream = torch.cuda.current_stream()
    g = Gvom(*w.gvom_args())
    g.set_stream(stream.cuda_stream)
    dev_pts = [torch.from_numpy(s.points).cuda() for s in scans]
    X = w.xy_size
    outs = [torch.empty((X, X), dtype=d, device="cuda") for d in (torch.int32, torch.int32, torch.float64, torch.int32)]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    lib = g._l
    import ctypes as C

    from gvom_gb300._lib import GVOM_F32, check
    ego_c = [np.ascontiguousarray(np.asarray(s.ego, np.float64)) for s in scans]
    T_c = [np.ascontiguousarray(s.transform) for s in scans]
    tcode = GVOM_F32 if scans[0].transform.dtype == np.float32 else 1
    out_ptrs = [C.c_void_p(t.data_ptr()) for t in outs]
    origin = np.zeros(3)

    def step_device(i):
        s = i % nscan
        check(lib.gvom_process_device(g._h, C.c_void_p(dev_pts[s].data_ptr()), GVOM_F32, n_pts[s], 3,
                                      ego_c[s].ctypes.data_as(C.c_void_p), T_c[s].ctypes.data_as(C.c_void_p), tcode))
        check(lib.gvom_combine_device(g._h, origin.ctypes.data_as(C.c_void_p), *out_ptrs))

    for i in range(args.warmup):
        step_device(i)
    torch.cuda.synchronize()

    # ---- timed region (device-resident inputs) ----
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    g.set_stage_timing(True)
    clocks = Clocks(lrank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall0 = time.perf_counter()
    pts_total = 0
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        step_device(args.warmup + k)
        ends[k].record(stream)
        pts_total += n_pts[(args.warmup + k) % nscan]
    torch.cuda.synchronize()
    t_wall1 = time.perf_counter()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    stages = g.stage_times()
    g.set_stage_timing(False)
    t_dev = sum(step_ms) / 1e3
    if dist:
        t = torch.tensor([t_dev, float(pts_total)], dtype=torch.float64, device="cuda")
        tm = t.clone()
        dist.all_reduce(tm, op=dist.ReduceOp.MAX)
        ts = t.clone()
        dist.all_reduce(ts, op=dist.ReduceOp.SUM)
        t_dev_max, pts_all = float(tm[0]), float(ts[1])
    else:
        t_dev_max, pts_all = t_dev, float(pts_total)

    # state sizes for the roofline accounting (last step)
    C_sum = 0
    for sl in range(w.buffer_size):
        n = C.c_int64()
        check(lib.gvom_slot_count(g._h, sl, C.byref(n)))
        C_sum += max(0, n.value)
    _, last = g.ring_state()
    nl = C.c_int64()
    check(lib.gvom_slot_count(g._h, int(last), C.byref(nl)))
    ncc = C.c_int64()
    check(lib.gvom_combined_count(g._h, C.byref(ncc)))
    V = w.voxels
    Vext = (w.xy_size + 2) ** 2 * (w.z_size + 2)
    n_mean = float(np.mean(n_pts))
    dom = max(stages.items(), key=lambda kv: kv[1][0])
    dom_name, (dom_ms, dom_n) = dom
    per_launch_ms = dom_ms / max(dom_n, 1)
    alg = stage_bytes(dom_name, n_mean, V, Vext, X * X, nl.value, C_sum, ncc.value, ncc.value, w.buffer_size + 1)
    peak, peak_kind = measured_peak_hbm()
    achieved = alg / (per_launch_ms / 1e3) / 1e9
    traffic = profiled_traffic(dom_name, w.name)
    stage_tab = {}
    for name, (ms, cnt) in stages.items():
        if cnt:
            b = stage_bytes(name, n_mean, V, Vext, X * X, nl.value, C_sum, ncc.value, ncc.value, w.buffer_size + 1)
            stage_tab[name] = {"ms_per_launch": ms / cnt, "launches": cnt,
                               "alg_bytes": int(b), "gbs": b / (ms / cnt / 1e3) / 1e9}
    ray = g.last_process_stats()

    # ---- e2e through the public API with host buffers ----
    e2e_times = []
    g.set_stream(None)
    torch.cuda.synchronize()
    for i in range(min(args.warmup, 5)):
        s = scans[i % nscan]
        g.process_pointcloud(s.points, s.ego, s.transform)
        g.combine_maps()
    e2e_pts = 0
    for k in range(args.steps):
        s = scans[(args.warmup + k) % nscan]
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.process_pointcloud(s.points, s.ego, s.transform)
        g.combine_maps()
        e2e_times.append(time.perf_counter() - t0)
        e2e_pts += s.points.shape[0]
    e2e_t = sum(e2e_times)
    if dist:
        t = torch.tensor([e2e_t, float(e2e_pts)], dtype=torch.float64, device="cuda")
        tm = t.clone()
        dist.all_reduce(tm, op=dist.ReduceOp.MAX)
        ts = t.clone()
        dist.all_reduce(ts, op=dist.ReduceOp.SUM)
        e2e_t, e2e_pts = float(tm[0]), float(ts[1])
    h2d = int(n_mean * 12 + 16 * scans[0].transform.itemsize + 24)
    d2h = X * X * (4 + 4 + 8 + 4)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, scans[: min(len(scans), 8)])

    if rank == 0:
        line = {
            "metric": METRIC, "value": pts_all / t_dev_max, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_dev_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (int32 counts, f64 index/height math)",
            "data": "synthetic (seeded terrain / lidar / trajectory generator)",
            "config": {"workload": w.name, "grid": [w.xy_size, w.xy_size, w.z_size], "voxel_m": w.res,
                       "buffer_size": w.buffer_size, "points_per_scan": int(n_mean), "scans": nscan,
                       "l2": "flushed (256 MB write) before every step", "parallelism": f"replicas x{world}"},
            "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                           "e2e_p50": 1e3 * float(np.percentile(e2e_times, 50)),
                           "e2e_p99": 1e3 * float(np.percentile(e2e_times, 99))},
            "e2e": {"value": e2e_pts / e2e_t, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": 9 * args.steps,
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak,
                         "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "alg_bytes_per_launch": int(alg), "ms_per_launch": per_launch_ms,
                         "traffic": traffic},
            "stages": stage_tab,
            "ray": {"valid_points": ray["valid_points"], "hits": ray["hits"], "ray_steps": ray["ray_steps"]},
            "wall_s_timed": t_wall1 - t_wall0,
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    g.close()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gvom", choices=["gvom", "reference"])
    ap.add_argument("--workload", default="os1_64_veg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    from gvom_gb300.synthetic import WORKLOADS
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w)
    return run_gpu(args, w)


if __name__ == "__main__":
    sys.exit(main())
