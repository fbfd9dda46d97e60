"""Autotuner for the launch shapes of the GB300 mapper (GvomTuning).

Six choices, tuned one at a time (coordinate search) on sample steps of
the caller's workload:

  points_per_block         128 / 256   k_voxelize_trace, k_scatter, k_cell_moments, k_cleanup
  merge_planes_per_thread  4 / 8 / 16  k_merge, k_columns
  stats_blocks_per_sm      2 / 4 / 8   k_merge_stats
  step_overlap             0 / 1       gvom_step: the index merge beside the statistics kernels
  maps_tile_cells          64/128/224/256  k_maps2d (smaller tiles spread the float64 plane fits; 224 =
                                       14 x 16, two blocks on each of 152 SMs at 256 x 256)
  step_pipeline            0 / 1 / 2   gvom_step: ray tracing beside the previous step's combine (1),
                                       and the process + merge beside its columns and maps (2)

The others each affect their own kernels only and are timed with the
per-kernel CUDA events of the mapper's stage timer (direct launches); the
two overlap choices change how kernels share the GPU, so they are timed on
whole steps submitted back to back.
Candidates run on a private mapper of the same parameters, so the caller's
map state is untouched.  Results are cached in a JSON file keyed by
GPU name, grid and scans per step ($GVOM_TUNING_CACHE, default
~/.cache/gvom_gb300/tuning.json).  Tuning changes speed only: every choice
gives bit-identical maps.
"""
from __future__ import annotations

import json
import os

CHOICES = {
    "points_per_block": (128, 256),
    "merge_planes_per_thread": (4, 8, 16),
    "stats_blocks_per_sm": (2, 4, 8),
    "step_overlap": (0, 1),
    "maps_tile_cells": (64, 128, 224, 256),
    "step_pipeline": (0, 1, 2),
}
AFFECTS = {
    "points_per_block": ("k_voxelize_trace", "k_scatter", "k_cell_moments", "k_cleanup"),
    "merge_planes_per_thread": ("k_merge", "k_columns"),
    "stats_blocks_per_sm": ("k_merge_stats",),
    "step_overlap": None,  # whole steps
    "maps_tile_cells": ("k_maps2d",),
    "step_pipeline": None,  # whole steps
}
DEFAULT = {"points_per_block": 256, "merge_planes_per_thread": 8,
           "stats_blocks_per_sm": 4, "step_overlap": 1, "maps_tile_cells": 224, "step_pipeline": 2}


def cache_path() -> str:
    return os.environ.get("GVOM_TUNING_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "gvom_gb300",
                                                                "tuning.json")


def cache_key(params: tuple, scans_per_step: int, device_name: str) -> str:
    xy_res, z_res, X, Z, B = params[:5]
    exy, ez = params[12], params[13]
    return f"{device_name}|{X}x{X}x{Z}|B{B}|eig{exy},{ez}|scans{scans_per_step}"


def load_cache(path: str | None = None) -> dict:
    try:
        with open(path or cache_path()) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def save_cache(cache: dict, path: str | None = None) -> None:
    p = path or cache_path()
    os.makedirs(os.path.dirname(p) or ".", exist_ok=True)
    tmp = p + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def _run_step(mapper, step, outs):
    if len(step) == 1:
        mapper.Process_pointcloud(*step[0])
    else:
        mapper.process_batch(step)
    if outs is None:
        mapper.combine_maps()
    else:
        mapper.combine_maps_device(*outs)


def time_kernels(mapper, steps, reps: int, kernels, outs=None) -> float:
    """Mean summed duration (ms) of `kernels` per step over `reps` steps."""
    mapper.set_graphs(False)
    for i in range(2):
        _run_step(mapper, steps[i % len(steps)], outs)
    mapper.set_stage_timing(True)
    for i in range(reps):
        _run_step(mapper, steps[i % len(steps)], outs)
    st = mapper.stage_times()
    mapper.set_stage_timing(False)
    return sum(st[k][0] for k in kernels if k in st) / max(1, reps)


def time_steps(mapper, steps, reps: int) -> float:
    """Mean wall time (ms) of gvom_step over `reps` steps submitted back to
    back (device outputs, one wait at the end), graphs on."""
    import time
    outs = None
    try:
        import torch
        if torch.cuda.is_available():
            X = mapper.xy_size
            outs = [torch.empty((X, X), dtype=d, device="cuda")
                    for d in (torch.int32, torch.int32, torch.float64, torch.int32)]
    except ImportError:  # pragma: no cover
        pass
    mapper.set_graphs(True)
    for i in range(3):
        mapper.step(steps[i % len(steps)], device_outputs=outs)
    mapper.synchronize()
    t0 = time.perf_counter()
    for i in range(reps):
        mapper.step(steps[i % len(steps)], device_outputs=outs)
    mapper.synchronize()
    return 1e3 * (time.perf_counter() - t0) / max(1, reps)


def search(mapper, steps, reps: int = 10, outs=None, start: dict | None = None) -> tuple[dict, dict]:
    """Coordinate search over CHOICES; returns (best tuning, timings)."""
    best = dict(start or mapper.get_tuning())
    timings = {}
    for knob, values in CHOICES.items():
        t = {}
        for v in values:
            mapper.set_tuning(dict(best, **{knob: v}))
            if AFFECTS[knob] is None:
                t[v] = time_steps(mapper, steps, 3 * reps)
            else:
                t[v] = time_kernels(mapper, steps, reps, AFFECTS[knob], outs)
        best[knob] = min(t, key=t.get)
        timings[knob] = {str(k): v for k, v in t.items()}
    mapper.set_tuning(best)
    return best, timings


def autotune(mapper, steps, reps: int = 10, use_cache: bool = True, save: bool = True,
             cache_file: str | None = None, device_name: str | None = None) -> dict:
    """Pick the launch shapes for `mapper` (a gvom_gb300.Gvom) on sample
    `steps` (each a list of (points, ego, transform) processed together) and
    apply them; cached per GPU and workload shape."""
    from .gvom import Gvom
    if device_name is None:
        import torch
        device_name = torch.cuda.get_device_name()
    key = cache_key(mapper.params, len(steps[0]), device_name)
    cache = load_cache(cache_file) if use_cache else {}
    if key in cache:
        mapper.set_tuning(cache[key])
        return dict(cache[key])
    probe = Gvom(*mapper.params)
    try:
        best, _ = search(probe, steps, reps)
    finally:
        probe.close()
    mapper.set_tuning(best)
    if save:
        cache = load_cache(cache_file)
        cache[key] = best
        save_cache(cache, cache_file)
    return best
