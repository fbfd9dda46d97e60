"""Timing recipe for the CPU baselines at the CPU-runnable size (measurement
infrastructure, not product code).

Workload: small_32x512 (gvom_gb300.synthetic), one 32 x 512 = 16,384-point
float32 scan over the seeded terrain, 0.2 m voxels, 128 x 128 x 32, buffer 2;
one step = one Process_pointcloud followed by combine_maps.

Rows measured:
  reference_shim  the reference's own scripts/gvom.py, unchanged, from the
                  checkout named by $GVOM_REFERENCE, executed by the sequential
                  numba stand-in in oracle/numba_shim on one core.  This is NOT
                  Numba's CUDA simulator (numba is not installed and there is
                  no network); the stand-in runs each CUDA thread of a launch
                  in turn in Python, as the simulator does.  Skipped when
                  $GVOM_REFERENCE is unset.
  oracle_1        the C oracle (oracle/gvom_oracle.c), 1 thread
  oracle_n        the C oracle, every host thread (OpenMP)

Prints one JSON line:  python oracle/time_reference.py [--oracle-steps N]
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)


def _scan():
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["small_32x512"]
    return w, make_workload_scans(w, 1)[0]


def time_reference_shim(w, s):
    ref = os.environ.get("GVOM_REFERENCE")
    if not ref:
        return None
    sys.path.insert(0, os.path.join(HERE, "numba_shim"))
    import numba  # the stand-in
    spec = importlib.util.spec_from_file_location("gvom_reference", os.path.join(ref, "scripts", "gvom.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.math = numba.math_proxy
    g = mod.Gvom(*w.gvom_args())
    t0 = time.perf_counter()
    g.Process_pointcloud(s.points.copy(), tuple(s.ego), s.transform.copy())
    t1 = time.perf_counter()
    out = g.combine_maps()
    t2 = time.perf_counter()
    assert out is not None
    n = int(s.points.shape[0])
    return {"value": n / (t2 - t0), "unit": "points/s", "cores": 1, "seconds_per_step": t2 - t0,
            "process_s": t1 - t0, "combine_s": t2 - t1,
            "sample": "1 step (Process_pointcloud + combine_maps) of small_32x512, "
                      f"{n} points; unchanged scripts/gvom.py under the sequential numba stand-in "
                      "(not the Numba CUDA simulator, which is not installed)"}


def time_oracle(w, s, threads, min_steps, budget_s=10.0):
    from oracle.oracle import OracleGvom
    o = OracleGvom(*w.gvom_args(), threads=threads)
    o.Process_pointcloud(s.points, s.ego, s.transform)  # warm-up
    o.combine_maps()
    steps = 0
    t0 = time.perf_counter()
    while steps < min_steps or time.perf_counter() - t0 < budget_s:
        o.Process_pointcloud(s.points, s.ego, s.transform)
        o.combine_maps()
        steps += 1
    dt = time.perf_counter() - t0
    n = int(s.points.shape[0])
    return {"value": steps * n / dt, "unit": "points/s", "cores": threads, "seconds_per_step": dt / steps,
            "sample": f"{steps} steps (process + combine) of small_32x512, {steps * n} points, {dt:.1f} s"}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--oracle-steps", type=int, default=5)
    a = ap.parse_args(argv)
    w, s = _scan()
    nproc = os.cpu_count() or 1
    line = {"workload": "small_32x512", "host": f"{platform.machine()}, {nproc} threads",
            "reference_shim": time_reference_shim(w, s),
            "oracle_1": time_oracle(w, s, 1, a.oracle_steps),
            "oracle_n": time_oracle(w, s, nproc, a.oracle_steps)}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
