#!/usr/bin/env python
"""Scan->map throughput of the GB300 G-VOM path (one JSON line on rank 0).

Forms (workloads from gvom_gb300.synthetic, seeded; the reference publishes
no dataset, so synthetic scans of the named shapes stand in for its logs):

  os1_64_veg (default headline, the plain form): OS1-64-shaped scans
      (64 x 1024 = 65,536 float32 points) plus world-fixed vegetation at 20
      points/m^2 inside the map footprint, along a seeded trajectory (0.4 m
      and up to 3 deg yaw per scan, float32 4x4 transforms); grid 256 x 256 x
      64 at 0.15 m, buffer 4.  One step = one scan through Process_pointcloud
      followed by combine_maps.
  batched_8 (the batched form): 8 sensors of 16,384-262,144 points before
      0-60 % seeded whole-beam dropout, on 4 mountings; grid 256 x 256 x 64 at
      0.15 m, buffer 16.  One step = the 8 scans of one vehicle pose through
      one process_batch (one set of launches over all scans) followed by
      combine_maps.
  served: two device-resident instances behind the request loop of
      gvom_gb300.serve, Poisson arrivals; p50 / p99 scan->map latency.
  ros: the reference ROS node's two ends on the headline workload: each step
      maps one lidar message from host bytes (process_pointcloud2 with the tf
      translation and quaternion) and reads back combine_maps' outputs and
      the five OccupancyGrid payloads (ros_grids), beside the host time of
      the conversions the node would run for the same message and maps.

Metric: points/sec = points ingested per step / step time.

  value    device-resident inputs (points already in HBM, maps written to
           device buffers), per-step CUDA events on the launching stream,
           L2 flushed (256 MB write) before every step outside the timed span
  e2e      the public API with host buffers: numpy points in, numpy maps out
           (host<->device copies inside the timed span), wall clock
  roofline per-kernel CUDA-event durations inside the timed region; the
           dominant kernel's algorithmic bytes / its mean launch time against
           the measured HBM copy bandwidth
  forms    the other forms measured the same way in the same run
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
import math
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
KERNELS_PER_STEP = 11  # 6 process kernels (all scans of a step in one set) + 5 combine kernels
# distinct steps the timed inputs cycle through: 200 plain scans (228 MB of
# points) and 48 batched steps (256 MB), more than the 129 MB of L2
HEAD_DISTINCT_STEPS = 200
FORM_DISTINCT_STEPS = 48


# per-stage algorithmic bytes of one launch (n = points of the launch, ns = scans
# of the launch); the per-unit figures follow the scan->map roofline accounting
def stage_bytes(name, n, ns, V, Vext, X2, C_new, C_sum, Cc, nsrc):
    if name == "k_voxelize_trace":
        return 12 * n + 64 * ns
    if name == "k_assign":  # cell and rank per point; per occupied cell its words, index word and record
        return 20 * n + 36 * C_new
    if name == "k_scatter":
        return 20 * n + 16 * n
    if name == "k_cell_moments":
        return 20 * n + 16 * n + 48 * C_new
    if name == "k_voxel_stats":
        return 52 * C_new + 27 * 56 * C_new
    if name == "k_cleanup":
        return 20 * n
    if name == "k_merge":
        return 4 * V * nsrc + 4 * V + 4 * Cc + 8 * X2 * ((V // X2 + 7) // 8)
    if name == "k_merge_counts":  # index words of the sources, hit / total / min height of their records
        return 4 * Cc + 4 * nsrc * Cc + 12 * (C_sum + Cc) + 12 * Cc
    if name == "k_merge_stats":
        return 4 * Cc + 4 * nsrc * Cc + 64 * (C_sum + Cc) + 64 * Cc
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

    def __init__(self, gpu_index, tag=""):
        self.p = None
        self.gpu = gpu_index
        # the raw samples go to $GVOM_CLOCKS_DIR (default: the temporary directory)
        import tempfile
        self.path = os.path.join(os.environ.get("GVOM_CLOCKS_DIR") or tempfile.gettempdir(),
                                 f"gvom_clocks_gpu{gpu_index}{tag}.csv")

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
        with open(self.path) as f:
            return summarize_clocks(f)


def summarize_clocks(lines):
    """Median SM clock, its maximum and the throttle reasons seen, from
    nvidia-smi CSV rows of Clocks.Q (no header, no units); None without rows."""
    rows = []
    for line in lines:
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


def _safe(fn):
    """fn() or None: an auxiliary figure never breaks the bench line."""
    try:
        return fn()
    except Exception:
        return None


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


# ---------------------------------------------------------------------------
# forms: what one step is
# ---------------------------------------------------------------------------

class Form:
    """A workload and its steps; each step is a list of scans that go through
    one process call (one scan for the plain form) and one combine."""

    def __init__(self, name, device, n_steps):
        from gvom_gb300 import synthetic as S
        self.name = name
        if name in S.WORKLOADS:
            self.w = S.WORKLOADS[name]
            self.kind = "plain"
            self.steps = [[s] for s in S.make_workload_scans(self.w, n_steps, device=device)]
        elif name in S.BATCHED:
            self.w = S.BATCHED[name]
            self.kind = "batched"
            self.steps = S.make_batched_steps(self.w, n_steps, device=device)
        else:
            raise SystemExit(f"unknown workload {name}")
        self.points = [sum(s.points.shape[0] for s in st) for st in self.steps]

    def __len__(self):
        return len(self.steps)

    def input_mb(self):
        return sum(s.points.nbytes for st in self.steps for s in st) / 1e6

    def config(self):
        w = self.w
        c = {"workload": w.name, "form": self.kind, "grid": [w.xy_size, w.xy_size, w.z_size], "voxel_m": w.res,
             "buffer_size": w.buffer_size, "scans_per_step": len(self.steps[0]),
             "points_per_step": int(np.mean(self.points)), "distinct_steps": len(self.steps)}
        if self.kind == "batched":
            c["sensors"] = [[s.beams, s.columns, s.dropout, s.mount] for s in w.sensors]
        return c

    def cpu_step(self, o, i):
        st = self.steps[i % len(self.steps)]
        for s in st:
            o.Process_pointcloud(s.points, s.ego, s.transform)
        o.combine_maps()
        return self.points[i % len(self.steps)]


def cpu_baseline(form, budget_s=12.0, threads=None):
    """Time the CPU oracle (all host threads) on a bounded sample of the workload."""
    from oracle.oracle import OracleGvom
    threads = threads or os.cpu_count() or 1
    o = OracleGvom(*form.w.gvom_args(), threads=threads)
    pts = 0
    steps = 0
    t0 = time.perf_counter()
    while True:
        pts += form.cpu_step(o, steps)
        steps += 1
        if time.perf_counter() - t0 >= budget_s and steps >= 3:
            break
    dt = time.perf_counter() - t0
    return {"value": pts / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} steps (process+combine) of {form.name}, {pts} points, {dt:.1f} s"}


def _has_cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    from gvom_gb300 import synthetic as S
    # the GPU arm's distinct steps, cycled the same way (step i = distinct step i mod len)
    n = FORM_DISTINCT_STEPS if args.workload in S.BATCHED else HEAD_DISTINCT_STEPS
    form = Form(args.workload, "cuda" if _has_cuda() else "cpu", n)
    from oracle.oracle import OracleGvom
    threads = os.cpu_count() or 1
    o = OracleGvom(*form.w.gvom_args(), threads=threads)
    tw = time.perf_counter()
    for i in range(max(1, args.warmup)):
        form.cpu_step(o, i)
    est = (time.perf_counter() - tw) / max(1, args.warmup)
    # bounded sample: at most ~60 s of CPU work whatever --steps asks for
    n_run = int(min(args.steps, max(3, 60.0 / max(est, 1e-3))))
    times = []
    pts = 0
    t_start = time.perf_counter()
    for k in range(n_run):
        t0 = time.perf_counter()
        pts += form.cpu_step(o, args.warmup + k)
        times.append(time.perf_counter() - t0)
    total = time.perf_counter() - t_start
    v = pts / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": n_run,
        "steps_requested": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (reference typing)", "data": "synthetic",
        "config": form.config(),
        "latency_ms": {"p50": 1e3 * float(np.percentile(times, 50)), "p99": 1e3 * float(np.percentile(times, 99))},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n_run} steps of {form.name} on the CPU restatement of the reference path "
                                   f"({total:.1f} s); the reference itself (Numba CUDA) cannot run here: "
                                   "numba is not installed on this box"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU measurement of one form
# ---------------------------------------------------------------------------

def step_roofline(n_pts, ns, V, X2, B, C_new, C_sum, Cc, hits, steps, peak_gbs, ms_per_step):
    """The whole step against HBM, with the per-unit work of the scan->map
    roofline accounting: process = 12N + 64 + 4V + 52C per scan, combine =
    4V (B + 1) + 4V + 52 sum(C_i) + 2 52 Cc + 20 X^2; int32 atomics = 2H + S
    per scan (H, S: means per scan over the timed steps)."""
    process = 12 * n_pts + ns * (64 + 4 * V) + 52 * C_new
    combine = 4 * V * (B + 1) + 4 * V + 52 * C_sum + 2 * 52 * Cc + 20 * X2
    b = process + combine
    t_hbm = b / (peak_gbs * 1e9)
    return {"bytes_per_step": int(b), "atomics_per_step": int(ns * (2 * hits + steps)),
            "hbm_bound_ms": 1e3 * t_hbm, "ms_per_step": ms_per_step,
            "frac_of_measured_hbm": t_hbm / (ms_per_step / 1e3)}


# Scattered 32-bit L2 reductions (atomicAdd without return to hashed words of
# a 16.8 MB int32 array, the headline slot's index map) sustained this rate on
# GB300 in a throughput probe (method in the design notes); the trace kernel's
# atomic ceiling.
RED32_SCATTERED_PER_S = 200e9


def trace_atomic_roofline(hits, steps, ms_per_launch, peak=RED32_SCATTERED_PER_S):
    """The ray-trace kernel against the L2 reduction rate: its int32 atomics
    per launch (2H + S, mean over the timed scans: a hit and a total per hit,
    one total per ray step) over its measured launch time."""
    atomics = 2 * hits + steps
    achieved = atomics / (ms_per_launch / 1e3)
    return {"bound": "l2_atomics", "atomics_per_launch": int(atomics), "achieved_per_s": achieved,
            "peak_per_s": peak, "frac": achieved / peak,
            "peak_source": "scattered 32-bit reduction throughput probe on GB300"}


def scan_counts(g, form, torch, indices):
    """Valid points, in-grid hits H and ray steps S of the distinct steps
    `indices` (each scan processed alone on `g`, untimed): the timed steps
    cycle through the distinct steps, so these give the timed scans' means."""
    per_step = {}
    for i in sorted(set(indices)):
        h = s_ = v = 0
        for s in form.steps[i]:
            g.Process_pointcloud(s.points, s.ego, s.transform)
            r = g.last_process_stats()
            h += r["hits"]
            s_ += r["ray_steps"]
            v += r["valid_points"]
        per_step[i] = (v, h, s_)
    torch.cuda.synchronize()
    return per_step


def _quat_xyzw(R):
    """Unit quaternion (x, y, z, w) of a rotation matrix (Shepperd's method)."""
    R = np.asarray(R, np.float64)
    tr = R[0, 0] + R[1, 1] + R[2, 2]
    if tr > 0.0:
        s = 2.0 * math.sqrt(tr + 1.0)
        return np.array([(R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s, 0.25 * s])
    i = int(np.argmax(np.diag(R)))
    j, k = (i + 1) % 3, (i + 2) % 3
    s = 2.0 * math.sqrt(1.0 + R[i, i] - R[j, j] - R[k, k])
    q = np.empty(4)
    q[i] = 0.25 * s
    q[j] = (R[j, i] + R[i, j]) / s
    q[k] = (R[k, i] + R[i, k]) / s
    q[3] = (R[k, j] - R[j, k]) / s
    return q


def lidar_message(points, rng, point_step=48):
    """A PointCloud2-style payload of `points`: float32 x, y, z at byte
    offsets 0, 4, 8 of each `point_step`-byte point, other fields random."""
    rows = rng.random((points.shape[0], point_step // 4), dtype=np.float32)
    rows[:, :3] = points
    return rows


def node_host_work(rows, maps, density_threshold=50, min_roughness=-10, max_roughness=0):
    """The host conversions the reference's ROS node runs for one message and
    one map (scripts/gvom_ros.py:108, 141-164), which process_pointcloud2 and
    ros_grids move to the device: the message's x, y, z fields to a float64
    (N, 3) array without non-finite rows, and the five int8 payloads."""
    import warnings
    xyz = np.empty((rows.shape[0], 3), np.float64)
    xyz[:, 0], xyz[:, 1], xyz[:, 2] = rows[:, 0], rows[:, 1], rows[:, 2]
    xyz = xyz[np.isfinite(xyz).all(axis=1)]
    _, obs, neg, rough, cert = maps
    F = lambda a: np.reshape(a, -1, order="F")  # noqa: E731
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        out = [F(np.maximum(100 * (obs > density_threshold), neg)).astype(np.int8),
               F(100 * (obs <= density_threshold) * (obs > 0)).astype(np.int8),
               F(cert * 100).astype(np.int8), F(neg).astype(np.int8),
               F(((np.maximum(np.minimum(rough, max_roughness), min_roughness) + min_roughness)
                  / (max_roughness - min_roughness)) * 100).astype(np.int8)]
    return xyz, out


def measure_ros(form, torch, n_steps=200, warmup=5):
    """The reference ROS node's two ends on the headline workload: each step
    maps one lidar message from host memory (process_pointcloud2: bytes,
    tf translation and quaternion) and reads back combine_maps' outputs and
    the five OccupancyGrid payloads (ros_grids).  Reported beside the host
    time of the conversions the node itself would run for the same message
    and maps."""
    from gvom_gb300 import Gvom
    rng = np.random.default_rng(5)
    msgs = []
    for st in form.steps[:24]:
        s = st[0]
        T = np.asarray(s.transform, np.float64)
        msgs.append((lidar_message(s.points, rng), s.points.shape[0], s.ego, T[:3, 3].copy(), _quat_xyzw(T[:3, :3])))
    g = Gvom(*form.w.gvom_args())
    t_in, t_comb, t_grid, t_dbg, pts, maps = [], [], [], [], 0, None
    for k in range(warmup + n_steps):
        rows, n, ego, t, q = msgs[k % len(msgs)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.process_pointcloud2(rows, n, 48, (0, 4, 8), ego, t, q)
        t1 = time.perf_counter()
        maps = g.combine_maps()
        t2 = time.perf_counter()
        g.ros_grids()
        t3 = time.perf_counter()
        if k >= warmup:
            t_in.append(t1 - t0)
            t_comb.append(t2 - t1)
            t_grid.append(t3 - t2)
            pts += n
        if k >= warmup and k % 10 == 0:  # the node's three debug clouds (scripts/gvom_ros.py:168-190)
            t4 = time.perf_counter()
            g.make_debug_voxel_map()
            g.make_debug_height_map()
            g.make_debug_inferred_height_map()
            t_dbg.append(time.perf_counter() - t4)
    g.close()
    host = []
    for k in range(20):
        t0 = time.perf_counter()
        node_host_work(msgs[k % len(msgs)][0], maps)
        host.append(time.perf_counter() - t0)
    us = lambda v: 1e6 * float(np.median(v))  # noqa: E731
    total = sum(t_in) + sum(t_comb) + sum(t_grid)
    return {"workload": form.name, "steps": n_steps, "point_step_bytes": 48,
            "points_per_s": pts / total,
            "entry": "process_pointcloud2 (host bytes, translation + quaternion), combine_maps, ros_grids",
            "us_p50": {"process_pointcloud2": us(t_in), "combine_maps": us(t_comb), "ros_grids": us(t_grid),
                       "debug_exports_all_three": us(t_dbg)},
            "node_host_conversions_us_p50": us(host)}


def _reduce_max_sum(torch, dist, t_val, pts):
    """(max over ranks of the timed seconds, sum over ranks of the points)."""
    if not dist:
        return t_val, float(pts)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([t_val, float(pts)], dtype=torch.float64, device=dev)
    tm = t.clone()
    dist.all_reduce(tm, op=dist.ReduceOp.MAX)
    ts = t.clone()
    dist.all_reduce(ts, op=dist.ReduceOp.SUM)
    return float(tm[0]), float(ts[1])


def measure_form(form, args, torch, dist, lrank, flush, headline, graphs=True):
    import ctypes as C

    from gvom_gb300 import Gvom
    from gvom_gb300._lib import GVOM_F32, GvomScan, check

    w = form.w
    X = w.xy_size
    # one explicit stream for the mapper, the L2 flush and the timing events
    # (the legacy default stream is not ordered with the mapper's own stream)
    stream = torch.cuda.Stream(priority=-1)
    torch.cuda.set_stream(stream)
    g = Gvom(*w.gvom_args())
    g.set_stream(stream.cuda_stream)
    lib = g._l
    # per-kernel stage times need direct launches; the timed steps replay CUDA graphs when `graphs`
    timing_pass = graphs
    outs = [torch.empty((X, X), dtype=d, device="cuda") for d in (torch.int32, torch.int32, torch.float64, torch.int32)]
    out_ptrs = [C.c_void_p(t.data_ptr()) for t in outs]
    origin = np.zeros(3)
    # device-resident inputs and the call arguments of every step, built outside the timed span
    keep = []
    calls = []
    for st in form.steps:
        arr = (GvomScan * len(st))()
        for j, s in enumerate(st):
            dp = torch.from_numpy(s.points).cuda()
            T = np.ascontiguousarray(s.transform)
            keep += [dp, T]
            arr[j].points = C.c_void_p(dp.data_ptr())
            arr[j].dtype = GVOM_F32
            arr[j].transform_dtype = GVOM_F32 if T.dtype == np.float32 else 1
            arr[j].n = s.points.shape[0]
            arr[j].row_stride = 3
            arr[j].ego[:] = [float(v) for v in s.ego]
            arr[j].transform = T.ctypes.data_as(C.c_void_p)
        calls.append(arr)

    # launch shapes for this workload (gvom_gb300.autotune, on a private mapper)
    from gvom_gb300.autotune import autotune
    dev_of = {id(s): keep[2 * j] for j, s in enumerate(x for st in form.steps for x in st)}
    tune_steps = [[(dev_of[id(s)], s.ego, s.transform) for s in st] for st in form.steps[:4]]
    tuning = autotune(g, tune_steps, reps=8, use_cache=False, save=False) if args.autotune else g.get_tuning()

    def step_device(i):
        # gvom_step: process_batch + combine_maps in one call (device outputs)
        arr = calls[i % len(calls)]
        check(lib.gvom_step(g._h, arr, len(arr), 1, origin.ctypes.data_as(C.c_void_p), *out_ptrs, 1))

    n_steps = args.steps if headline else max(10, min(args.steps, args.form_steps))
    # H and S of the distinct steps the timed steps use, on a private mapper (its state is not the timed one's)
    timed_idx = [(args.warmup + k) % len(form) for k in range(n_steps)]
    counts = scan_counts(Gvom(*w.gvom_args()), form, torch, timed_idx)

    for i in range(args.warmup):
        step_device(i)
    torch.cuda.synchronize()

    # ---- timed regions (device-resident inputs) ----

    def timed(n, use_graphs, stage_timing, clk_tag=None, back_to_back=False):
        """n steps.  back_to_back: submitted without a host wait or an L2 flush
        in between (a step's trace then runs beside the previous combine), one
        CUDA-event interval around all of them; the inputs cycle through the
        form's distinct steps, more bytes than L2 holds.  Otherwise each step
        is timed alone after a 256 MB write that flushes L2."""
        g.set_graphs(use_graphs)
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        for i in range(3):  # warm the graph executables / the timing events
            step_device(i)
        g.set_stage_timing(stage_timing)
        clocks = Clocks(lrank, clk_tag) if clk_tag is not None else None
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        t0 = time.perf_counter()
        pts = 0
        t_sub = None
        if back_to_back:
            starts[0].record(stream)
            for k in range(n):
                step_device(args.warmup + k)
                pts += form.points[(args.warmup + k) % len(form)]
            ends[0].record(stream)
            t_sub = time.perf_counter() - t0  # host time to submit the n steps
        else:
            for k in range(n):
                flush.zero_()
                starts[k].record(stream)
                step_device(args.warmup + k)
                ends[k].record(stream)
                pts += form.points[(args.warmup + k) % len(form)]
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        if dist:
            dist.barrier()
        clk = clocks.stop() if clocks else None
        if back_to_back:
            ms = [starts[0].elapsed_time(ends[0]) / n] * n
        else:
            ms = [x.elapsed_time(y) for x, y in zip(starts, ends)]
        st = g.stage_times() if stage_timing else None
        g.set_stage_timing(False)
        t, p = _reduce_max_sum(torch, dist, sum(ms) / 1e3, pts)
        timed.host_submit_s = t_sub
        return ms, t, p, wall, clk, st

    # the headline: steps back to back, CUDA-graph replay (or direct launches with graphs=False)
    _, t_dev_max, pts_all, wall_timed, clk, _ = timed(n_steps, graphs, False, "" if headline else "_" + form.name,
                                                      back_to_back=True)
    host_submit_s = timed.host_submit_s
    # mean H, S per step over the timed steps (steps warmup .. warmup + n_steps - 1)
    timed_counts = [counts[i] for i in timed_idx]
    H_mean = float(np.mean([c[1] for c in timed_counts]))
    S_mean = float(np.mean([c[2] for c in timed_counts]))
    # each step alone after an L2 flush (its latency), direct launches back to
    # back for comparison, and a pass with per-kernel CUDA events
    n_aux = max(10, min(n_steps, 300))
    # (one step at a time: no overlap with the neighbouring steps either)
    g.set_tuning(dict(tuning, step_pipeline=0))
    step_ms, t_flushed, pts_flushed, _, _, _ = timed(n_aux, graphs, False)
    g.set_tuning(tuning)
    ms_direct, t_direct, pts_direct, _, _, _ = timed(n_aux, False, False, back_to_back=True)
    _, _, _, _, _, stages = timed(n_aux, False, True)

    # state sizes for the roofline accounting (last step)
    C_sum = 0
    for sl in range(w.buffer_size):
        n = C.c_int64()
        check(lib.gvom_slot_count(g._h, sl, C.byref(n)))
        C_sum += max(0, n.value)
    ns = len(form.steps[0])
    bi, _ = g.ring_state()
    C_new = 0
    for j in range(ns):
        n = C.c_int64()
        check(lib.gvom_slot_count(g._h, int((bi - 1 - j) % w.buffer_size), C.byref(n)))
        C_new += max(0, n.value)
    ncc = C.c_int64()
    check(lib.gvom_combined_count(g._h, C.byref(ncc)))
    V = w.voxels
    Vext = (w.xy_size + 2) ** 2 * (w.z_size + 2)
    n_mean = float(np.mean(form.points))
    nsrc = w.buffer_size + 1
    stage_tab = {}
    for name, (ms, cnt) in stages.items():
        if cnt:
            b = stage_bytes(name, n_mean, ns, V, Vext, X * X, C_new, C_sum, ncc.value, nsrc)
            stage_tab[name] = {"ms_per_launch": ms / cnt, "launches": cnt,
                               "alg_bytes": int(b), "gbs": b / (ms / cnt / 1e3) / 1e9}
    dom_name = max(stage_tab.items(), key=lambda kv: kv[1]["ms_per_launch"])[0]
    dom = stage_tab[dom_name]
    peak, peak_kind = measured_peak_hbm()
    ray = g.last_process_stats()
    # the dominant kernel's roofline time: max(bytes / HBM, atomics / L2 reduction rate)
    t_bytes = dom["alg_bytes"] / (peak * 1e9)
    atomics = 2 * H_mean + S_mean if dom_name == "k_voxelize_trace" else 0.0
    t_atom = atomics / RED32_SCATTERED_PER_S
    t_roof = max(t_bytes, t_atom)

    # ---- e2e through the public API with host buffers ----
    e2e_times = []
    g.set_stream(None)
    g.set_graphs(graphs)
    torch.cuda.synchronize()

    def step_e2e(i):  # numpy in, numpy maps out: Gvom.step
        st = form.steps[i % len(form)]
        g.step([(s.points, s.ego, s.transform) for s in st])

    def step_ref_api(i):  # the reference's two calls: Process_pointcloud / process_batch, then combine_maps
        st = form.steps[i % len(form)]
        if form.kind == "plain":
            s = st[0]
            g.Process_pointcloud(s.points, s.ego, s.transform)
        else:
            g.process_batch([(s.points, s.ego, s.transform) for s in st])
        g.combine_maps()

    def timed_host(fn, n):
        for i in range(min(args.warmup, 5)):
            fn(i)
        times, pts = [], 0
        for k in range(n):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn(args.warmup + k)
            times.append(time.perf_counter() - t0)
            pts += form.points[(args.warmup + k) % len(form)]
        return times, pts

    e2e_times, e2e_pts = timed_host(step_e2e, n_steps)
    e2e_t, e2e_pts = _reduce_max_sum(torch, dist, sum(e2e_times), e2e_pts)
    ref_times, ref_pts = timed_host(step_ref_api, n_aux)
    ref_t, ref_pts = _reduce_max_sum(torch, dist, sum(ref_times), ref_pts)
    torch.cuda.synchronize()
    torch.cuda.set_stream(torch.cuda.default_stream())
    h2d = int(n_mean * 12 + ns * (16 * form.steps[0][0].transform.itemsize + 24))
    d2h = X * X * (4 + 4 + 8 + 4)
    g.close()
    return {
        "value": pts_all / t_dev_max, "ms_per_step": 1e3 * t_dev_max / n_steps, "steps": n_steps,
        "config": dict(form.config(), launch="cuda graphs" if graphs else "direct", tuning=tuning,
                       entry="gvom_step (process + combine, one call; device buffers), steps back to back",
                       l2=(f"no flush between back-to-back steps; inputs cycle through {form.input_mb():.0f} MB "
                           "of distinct steps (more than the 129 MB L2); each step alone after a 256 MB "
                           "flush: l2_flushed_per_step")),
        "direct_launches": {"value": pts_direct / t_direct, "ms_per_step": 1e3 * t_direct / n_aux, "steps": n_aux},
        "l2_flushed_per_step": {"value": pts_flushed / t_flushed, "ms_per_step": 1e3 * t_flushed / n_aux,
                                "steps": n_aux, "step_pipeline": 0},
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                       "e2e_p50": 1e3 * float(np.percentile(ref_times, 50)),
                       "e2e_p99": 1e3 * float(np.percentile(ref_times, 99))},
        "e2e": {"value": ref_pts / ref_t, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": n_aux, "entry": "Process_pointcloud / process_batch, then combine_maps (host numpy in and out)",
                "step_api": {"value": e2e_pts / e2e_t, "steps": n_steps,
                             "entry": "Gvom.step (gvom_step), host numpy in and out"}},
        "gpu_launches": KERNELS_PER_STEP * n_steps,
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": dom["gbs"], "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": dom["gbs"] / peak,
                     "alg_bytes_per_launch": dom["alg_bytes"], "ms_per_launch": dom["ms_per_launch"],
                     "traffic": profiled_traffic(dom_name, form.name),
                     # the scan->map accounting's two terms for this kernel: bytes / HBM and
                     # int32 atomics (2H + S, mean over the timed steps) / the L2 reduction rate
                     "atomics_per_launch": int(atomics), "atomic_peak_per_s": RED32_SCATTERED_PER_S,
                     "atomic_frac": (atomics / (dom["ms_per_launch"] / 1e3)) / RED32_SCATTERED_PER_S,
                     "t_roof_ms": 1e3 * t_roof, "t_roof_term": "atomics" if t_atom >= t_bytes else "hbm",
                     "frac_of_t_roof": 1e3 * t_roof / dom["ms_per_launch"]},
        "step_roofline": _safe(lambda: step_roofline(n_mean, ns, V, X * X, w.buffer_size, C_new, C_sum, ncc.value,
                                                     H_mean / ns, S_mean / ns, peak,
                                                     1e3 * t_dev_max / n_steps)),
        "trace_atomic_roofline": _safe(lambda: trace_atomic_roofline(
            H_mean, S_mean, stage_tab["k_voxelize_trace"]["ms_per_launch"])),
        "scan_counts_mean": {"hits": H_mean, "ray_steps": S_mean, "scans_per_step": ns},
        "stages": stage_tab,
        "ray_last_scan": ray,
        "wall_s_timed": wall_timed,
        # host time to submit the timed steps (no wait inside): when it is close to the device time the
        # host's calls, not the GPU, set the pace
        "host_submit_ms_per_step": 1e3 * host_submit_s / n_steps if host_submit_s else None,
        "clocks": clk,
    }


def measure_served(args, torch):
    """Served form: two device-resident map instances behind the request loop
    of gvom_gb300.serve -- 16 OS1-64 sensors at 10 Hz (Poisson arrivals) on a
    256 x 256 x 64 / 0.15 m map and 4 OS1-128x2048 sensors at 10 Hz on a
    512 x 512 x 96 / 0.1 m map.  Reports p50/p99 scan->map latency (submission
    to combine_maps outputs on the host) at that load, and the points/sec the
    loop sustains when every request of the window is queued at once."""
    from gvom_gb300 import serve
    from gvom_gb300 import synthetic as S

    duration = args.served_seconds
    specs = [  # (params, sensors, (beams, columns), rate)
        (S.WORKLOADS["os1_64_veg"].gvom_args()[:4] + (16,) + S.WORKLOADS["os1_64_veg"].gvom_args()[5:], 16, (64, 1024), 10.0),
        (S.WORKLOADS["os1_128_far"].gvom_args()[:4] + (8,) + S.WORKLOADS["os1_128_far"].gvom_args()[5:], 4, (128, 2048), 10.0),
    ]
    pools = []  # per instance, per sensor: a cycle of scans along the trajectory
    for params, n_sensors, (beams, cols), _ in specs:
        res, X = params[0], params[2]
        terrain = S.Terrain.make(S.SEED_TERRAIN, extent=X * res, path_len=4.0)
        poses = S.make_trajectory(4)
        per_sensor = []
        for k in range(n_sensors):
            mx, my, yaw, pitch = S.MOUNTS[k % 4]
            lid = S.Lidar(beams=beams, columns=cols, mount_x=mx, mount_y=my, mount_yaw_deg=yaw + 7.0 * (k // 4),
                          mount_pitch_deg=pitch)
            per_sensor.append([S.make_scan(terrain, lid, p, 1000 * k + i, device="cuda") for i, p in enumerate(poses)])
        pools.append(per_sensor)
    torch.cuda.synchronize()

    # one server for the three runs: instances, scratch and graph executables are set up once, as a
    # long-running loop has them (each instance reserves scratch for its largest batch at start-up)
    srv = serve.MapServer([sp[0] for sp in specs],
                          reserve_points=None)
    nxt = [[0] * len(p) for p in pools]

    def run(events, tag):
        reqs = []
        t0 = time.perf_counter()
        for t, (inst, k) in events:
            now = time.perf_counter() - t0
            if t > now:
                time.sleep(t - now)
            s = pools[inst][k][nxt[inst][k] % len(pools[inst][k])]
            nxt[inst][k] += 1
            reqs.append(srv.submit(inst, s.points, s.ego, s.transform))
        for r in reqs:
            r.done.wait(120)
        t_end = max(r.t_done for r in reqs)
        span = t_end - t0
        mine = {r.batch_id for r in reqs}
        out = {"requests": len(reqs), "span_s": span, "point_budget": srv.point_budget,
               "points_per_s": sum(r.points.shape[0] for r in reqs) / span, "instances": []}
        for i, sp in enumerate(specs):
            lat = [1e3 * r.latency for r in reqs if r.instance == i]
            nb = [len(seqs) for b, (inst, seqs) in enumerate(srv.batches) if inst == i and b in mine]
            out["instances"].append({"grid": [sp[0][2], sp[0][2], sp[0][3]], "voxel_m": sp[0][0],
                                     "sensors": sp[1], "rate_hz": sp[3],
                                     "points_per_scan": pools[i][0][0].points.shape[0],
                                     "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                                     "max_ms": float(np.max(lat)), "batches": len(nb),
                                     "mean_batch": float(np.mean(nb))})
        errors = [r.result for r in reqs if isinstance(r.result, Exception)]
        if errors:
            raise RuntimeError(f"served {tag}: {errors[0]}")
        return out

    rates = []
    for i, sp in enumerate(specs):
        rates += [(i, k, sp[3]) for k in range(sp[1])]
    arr = serve.poisson_arrivals([r for _, _, r in rates], duration, seed=S.SEED_ARRIVALS)
    events = [(t, (rates[j][0], rates[j][1])) for t, j in arr]
    run(events[: max(1, len(events) // 8)], "warm-up")
    run([(0.0, e[1]) for e in events[: max(1, len(events) // 8)]], "warm-up, queued at once")
    at_load = run(events, "at load")
    saturated = run([(0.0, e[1]) for e in events], "saturated")
    srv.close()
    return {"at_load": at_load, "saturated": saturated,
            "loop": f"pipelined: up to {serve.IN_FLIGHT} batches per instance in flight (gvom_step, device "
                    "outputs, asynchronous copies into pinned host memory); point budget from free HBM "
                    "(read at most every 50 ms); scratch reserved at start-up",
            "note": "latency = submission to combine_maps outputs on the host; the saturated run queues every "
                    "request of the window at once and reports the points/sec the loop sustains"}


def run_profile(args):
    """A short run for profilers: `--profile-steps` distinct steps of the
    workload through gvom_step (device inputs and outputs, direct launches,
    one stream, so each kernel is launched once per step in a fixed order:
    k_voxelize_trace, k_assign, k_scatter, k_cell_moments, k_voxel_stats,
    k_cleanup, k_merge, k_merge_counts, k_merge_stats, k_columns, k_maps2d)."""
    import torch

    from gvom_gb300 import Gvom
    from gvom_gb300 import build as gb
    gb.build()
    form = Form(args.workload, "cuda", args.profile_steps)
    g = Gvom(*form.w.gvom_args())
    g.set_tuning(dict(g.get_tuning(), step_pipeline=0))
    X = form.w.xy_size
    outs = [torch.empty((X, X), dtype=d, device="cuda") for d in (torch.int32, torch.int32, torch.float64, torch.int32)]
    dev = [[torch.from_numpy(s.points).cuda() for s in st] for st in form.steps]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k, st in enumerate(form.steps):
        g.step([(dev[k][j], s.ego, s.transform) for j, s in enumerate(st)], device_outputs=outs)
    g.synchronize()
    print(json.dumps({"profile_run": form.name, "steps": len(form.steps), "wall_s": time.perf_counter() - t0}))
    g.close()
    return 0


def run_gpu(args):
    import torch

    from gvom_gb300 import build as gb

    rank, world, lrank = env_rank()
    torch.cuda.set_device(lrank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    gb.build()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    head = Form(args.workload, "cuda", HEAD_DISTINCT_STEPS)
    res = measure_form(head, args, torch, dist, lrank, flush, headline=True)
    forms = {}
    for name in [f for f in args.forms.split(",") if f and f != args.workload]:
        if name == "served":
            if world == 1:
                forms[name] = measure_served(args, torch)
            continue
        if name == "ros":  # measured below, on the headline workload
            continue
        fm = Form(name, "cuda", FORM_DISTINCT_STEPS)
        forms[name] = measure_form(fm, args, torch, dist, lrank, flush, headline=False)
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            forms[name]["cpu_baseline"] = cpu_baseline(fm, budget_s=6.0)
    if world == 1 and "ros" in [f for f in args.forms.split(",")]:
        forms["ros"] = _safe(lambda: measure_ros(head, torch))
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(head)
    if rank == 0:
        line = {
            "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": world, "steps": res["steps"],
            "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (int32 counts, f64 index/height math)",
            "data": "synthetic (seeded terrain / lidar / trajectory generator)",
            "config": dict(res["config"], parallelism=f"replicas x{world}"),
            "latency_ms": res["latency_ms"], "e2e": res["e2e"], "gpu_launches": res["gpu_launches"],
            "roofline": res["roofline"], "step_roofline": res.get("step_roofline"),
            "trace_atomic_roofline": res.get("trace_atomic_roofline"), "stages": res["stages"],
            "ray_last_scan": res["ray_last_scan"], "scan_counts_mean": res.get("scan_counts_mean"),
            "direct_launches": res["direct_launches"], "l2_flushed_per_step": res["l2_flushed_per_step"],
            "wall_s_timed": res["wall_s_timed"], "host_submit_ms_per_step": res.get("host_submit_ms_per_step"), "clocks": res["clocks"], "cpu_baseline": cpu,
            "forms": forms,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gvom", choices=["gvom", "reference"])
    ap.add_argument("--workload", default="os1_64_veg", help="headline form")
    ap.add_argument("--forms", default="batched_8,served,ros",
                    help="comma-separated other forms measured in the same run")
    ap.add_argument("--served-seconds", type=float, default=6.0, help="arrival window of the served form")
    ap.add_argument("--form-steps", type=int, default=300, help="timed steps of each other form")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="default launch shapes instead of tuning them on the workload first")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="only run this many steps of --workload for a profiler (no JSON bench line)")
    args = ap.parse_args()
    if args.profile_steps > 0:
        return run_profile(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
