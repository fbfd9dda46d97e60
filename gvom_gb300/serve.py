"""Served form: a request loop over device-resident map instances.

Scans arrive as requests for one of several map instances (a vehicle's
sensors feed one instance).  Each instance has a worker thread and its own
CUDA stream: while the instance's previous batch is on the GPU, newly
arrived requests queue; when the worker is free it admits every queued
request that fits -- at most one ring slot per scan (the buffer size,
at most 16 per launch) and a point budget sized from free device memory at
start-up -- processes them in one `process_batch` launch set, runs
`combine_maps` and answers all of them with that map.  Instances run
concurrently, so their work overlaps on the device.  All map buffers stay
resident for the server's lifetime.

A request's result is the map after its batch; the batch composition is
recorded (`Request.batch_id`, `MapServer.batches`) so that any run can be
replayed alone, batch by batch, to the same outputs.

The reference has no server: its ROS node (scripts/gvom_ros.py:85-115) calls
Process_pointcloud from the lidar callback and combine_maps from a timer.
"""
from __future__ import annotations

import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .gvom import Gvom

# device bytes a queued point needs while its batch runs: staged xyz (12),
# per-point voxel fraction + cell (16), rank (4), grouped copy (16), cell
# moments (48)
BYTES_PER_POINT = 96


@dataclass
class Request:
    instance: int
    points: np.ndarray
    ego: tuple
    transform: np.ndarray | None
    t_submit: float = 0.0
    t_done: float = 0.0
    seq: int = -1
    batch_id: int = -1
    result: tuple | None = None
    done: threading.Event = field(default_factory=threading.Event)

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


def plan_batch(queue_points: list[int], max_scans: int, point_budget: int) -> int:
    """How many of the queued requests (oldest first, by point count) the next
    batch admits: as many as fit both limits, and always at least one (a scan
    larger than the budget runs alone)."""
    n = 0
    pts = 0
    for p in queue_points:
        if n >= max_scans or (n > 0 and pts + p > point_budget):
            break
        n += 1
        pts += p
    return n


class _Instance:
    def __init__(self, index: int, params: tuple, graphs: bool):
        import torch
        self.index = index
        self.params = params
        self.mapper = Gvom(*params)
        self.stream = torch.cuda.Stream()
        self.mapper.set_stream(self.stream.cuda_stream)
        self.mapper.set_graphs(graphs)
        self.max_scans = min(int(params[4]), 16)
        self.queue: deque[Request] = deque()
        self.cv = threading.Condition()
        self.thread: threading.Thread | None = None


class MapServer:
    """Continuous-batching request loop over map instances (one GB300)."""

    def __init__(self, instances: list[tuple], graphs: bool = True, mem_fraction: float = 0.25,
                 point_budget: int | None = None):
        import torch
        free, _ = torch.cuda.mem_get_info()
        self.instances: list[_Instance] = []
        for i, p in enumerate(instances):
            # gvom_create refuses (GvomError, out of memory) an instance whose
            # resident footprint does not fit in free device memory
            self.instances.append(_Instance(i, tuple(p), graphs))
        free_after, _ = torch.cuda.mem_get_info()
        budget = int(max(free_after, 0) * mem_fraction / BYTES_PER_POINT / max(1, len(instances)))
        self.point_budget = point_budget if point_budget is not None else max(1, budget)
        self.batches: list[tuple[int, list[int]]] = []  # (instance, request sequence numbers)
        self._seq = 0
        self._lock = threading.Lock()
        self._running = True
        self.free_at_start = free
        for inst in self.instances:
            inst.thread = threading.Thread(target=self._worker, args=(inst,), daemon=True)
            inst.thread.start()

    # ------------------------------------------------------------------
    def submit(self, instance: int, points: np.ndarray, ego, transform=None) -> Request:
        r = Request(instance, points, tuple(float(v) for v in ego), transform)
        inst = self.instances[instance]
        with inst.cv:
            r.t_submit = time.perf_counter()
            with self._lock:
                r.seq = self._seq
                self._seq += 1
            inst.queue.append(r)
            inst.cv.notify()
        return r

    def _worker(self, inst: _Instance):
        import torch
        torch.cuda.set_stream(inst.stream)
        while True:
            with inst.cv:
                while self._running and not inst.queue:
                    inst.cv.wait()
                if not self._running and not inst.queue:
                    return
                n = plan_batch([q.points.shape[0] for q in inst.queue], inst.max_scans, self.point_budget)
                batch = [inst.queue.popleft() for _ in range(n)]
            try:
                if len(batch) == 1:
                    r = batch[0]
                    inst.mapper.Process_pointcloud(r.points, r.ego, r.transform)
                else:
                    inst.mapper.process_batch([(r.points, r.ego, r.transform) for r in batch])
                out = inst.mapper.combine_maps()
                err = None
            except Exception as e:  # answer the batch with the error
                out, err = None, e
            t = time.perf_counter()
            with self._lock:
                bid = len(self.batches)
                self.batches.append((inst.index, [r.seq for r in batch]))
            for r in batch:
                r.result = out if err is None else err
                r.batch_id = bid
                r.t_done = t
                r.done.set()

    def close(self):
        self._running = False
        for inst in self.instances:
            with inst.cv:
                inst.cv.notify_all()
        for inst in self.instances:
            if inst.thread:
                inst.thread.join()
            inst.mapper.close()


def replay_alone(params: tuple, requests: list[Request], batches: list[tuple[int, list[int]]], instance: int):
    """Run one instance's recorded batches again on a fresh mapper, alone:
    returns the combine_maps outputs batch by batch."""
    by_seq = {r.seq: r for r in requests}
    g = Gvom(*params)
    outs = []
    for inst, seqs in batches:
        if inst != instance:
            continue
        rs = [by_seq[s] for s in seqs]
        if len(rs) == 1:
            g.Process_pointcloud(rs[0].points, rs[0].ego, rs[0].transform)
        else:
            g.process_batch([(r.points, r.ego, r.transform) for r in rs])
        outs.append(g.combine_maps())
    g.close()
    return outs


def poisson_arrivals(rates_hz: list[float], duration_s: float, seed: int = 4) -> list[tuple[float, int]]:
    """(time, sensor) pairs of independent Poisson arrival streams, sorted."""
    rng = np.random.default_rng(seed)
    ev = []
    for k, rate in enumerate(rates_hz):
        t = rng.exponential(1.0 / rate)
        while t < duration_s:
            ev.append((t, k))
            t += rng.exponential(1.0 / rate)
    ev.sort()
    return ev
