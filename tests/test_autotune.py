"""Autotuner (gvom_gb300/autotune.py): the search and its cache on the CPU
with a stand-in mapper; on the GPU, every launch shape gives bit-identical
maps."""
import os

import numpy as np
import pytest

from gvom_gb300 import autotune as AT


class FakeMapper:
    """Stage times depend on the tuning: each knob has one best value."""

    BEST = {"points_per_block": 128, "merge_planes_per_thread": 4,
            "stats_blocks_per_sm": 8, "step_overlap": 0, "maps_tile_cells": 64, "step_pipeline": 0}

    def __init__(self, params=(0.15, 0.15, 256, 64, 4, 1, .5, .5, .3, 2, 4, 1, 1, 1)):
        self.params = params
        self.t = dict(AT.DEFAULT)
        self.timing = False
        self.acc = {}
        self.steps_run = 0

    def set_tuning(self, t):
        self.t = dict(self.t, **t)

    def get_tuning(self):
        return dict(self.t)

    def set_graphs(self, on):
        pass

    def set_stage_timing(self, on):
        self.timing = on
        self.acc = {}

    def stage_times(self):
        return {k: (v, 1) for k, v in self.acc.items()}

    def Process_pointcloud(self, *a):
        self._step()

    def process_batch(self, b):
        self._step()

    def combine_maps(self):
        pass

    def step(self, b, device_outputs=None):
        # whole-step wall time stands in for the overlap knob
        import time
        for knob in ("step_overlap", "step_pipeline"):
            if self.t[knob] != self.BEST[knob]:
                time.sleep(0.002)

    def synchronize(self):
        pass

    def _step(self):
        self.steps_run += 1
        if not self.timing:
            return
        for knob, kernels in AT.AFFECTS.items():
            if kernels is None:
                continue
            cost = 1.0 + (0 if self.t[knob] == self.BEST[knob] else 0.5)
            for k in kernels:
                self.acc[k] = self.acc.get(k, 0.0) + cost


def test_search_finds_each_best_choice():
    m = FakeMapper()
    best, timings = AT.search(m, [[(None, None, None)]], reps=3)
    assert best == FakeMapper.BEST
    assert m.get_tuning() == FakeMapper.BEST
    assert set(timings) == set(AT.CHOICES)


def test_cache_roundtrip_and_key(tmp_path, monkeypatch):
    p = str(tmp_path / "t.json")
    k1 = AT.cache_key((0.15, 0.15, 256, 64, 4, 1, .5, .5, .3, 2, 4, 1, 1, 1), 8, "GB300")
    k2 = AT.cache_key((0.15, 0.15, 256, 64, 16, 1, .5, .5, .3, 2, 4, 1, 1, 1), 8, "GB300")
    assert k1 != k2
    AT.save_cache({k1: FakeMapper.BEST}, p)
    assert AT.load_cache(p) == {k1: FakeMapper.BEST}
    assert AT.load_cache(str(tmp_path / "missing.json")) == {}
    monkeypatch.setenv("GVOM_TUNING_CACHE", p)
    assert AT.cache_path() == p


@pytest.mark.gpu
def test_every_launch_shape_gives_identical_maps(gpu_lib):
    from gvom_gb300 import Gvom
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    from oracle.canonical import canonical_state
    from replay import compare_slot
    w = WORKLOADS["small_32x512"]
    scans = make_workload_scans(w, 4)
    params = w.gvom_args()[:4] + (3,) + w.gvom_args()[5:]
    shapes = [dict(AT.DEFAULT),
              {"points_per_block": 128, "merge_planes_per_thread": 16,
               "stats_blocks_per_sm": 2, "step_overlap": 0, "maps_tile_cells": 64, "step_pipeline": 0},
              {"points_per_block": 256, "merge_planes_per_thread": 4,
               "stats_blocks_per_sm": 8, "step_overlap": 1, "maps_tile_cells": 128, "step_pipeline": 2},
              {"points_per_block": 128, "merge_planes_per_thread": 8,
               "stats_blocks_per_sm": 4, "step_overlap": 1, "maps_tile_cells": 224, "step_pipeline": 1}]
    results = []
    for t in shapes:
        g = Gvom(*params)
        g.set_tuning(t)
        assert g.get_tuning() == t
        outs = []
        g.Process_pointcloud(scans[0].points, scans[0].ego, scans[0].transform)
        outs.append(g.combine_maps())
        g.process_batch([(s.points, s.ego, s.transform) for s in scans[1:]])
        outs.append(g.combine_maps())
        results.append((outs, canonical_state(g.combined_state())))
        g.close()
    for outs, st in results[1:]:
        for a, b in zip(results[0][0], outs):
            for x, y in zip(a, b):
                np.testing.assert_array_equal(x, y)
        compare_slot(results[0][1], st, "combined")
