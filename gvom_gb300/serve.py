"""Served form: a request loop over device-resident map instances.

Scans arrive as requests for one of several map instances (a vehicle's
sensors feed one instance).  Each instance has its own CUDA stream and two
threads.  The submitter admits every queued request that fits -- at most one
ring slot per scan (the buffer size, at most 16 per launch) and a point
budget taken from the device's free memory (read at most every 50 ms) -- and submits
them as one step (`gvom_step`: one process launch set over the batch, then
the combine) with the maps written to a device output set, followed on the
same stream by an asynchronous copy into pinned host memory and an event.
It does not wait: while that batch is on the GPU it admits the next one into
another output set, and the mapper's step pipeline runs the next batch's ray
tracing beside the previous combine.  The completer waits for each batch's
event in order, answers its requests with host copies of the maps and
returns the output set.  Instances run concurrently, so their work overlaps
on the device.  All map buffers stay resident for the server's lifetime, and
each instance reserves its scratch at start-up (`Gvom.reserve`), so no
request waits for an allocation.

A request's result is the map after its batch; the batch composition is
recorded (`Request.batch_id`, `MapServer.batches`) so that any run can be
replayed alone, batch by batch, to the same outputs.

The reference has no server: its ROS node (scripts/gvom_ros.py:85-115) calls
Process_pointcloud from the lidar callback and combine_maps from a timer.
"""
from __future__ import annotations

import gc
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
IN_FLIGHT = 2  # batches of one instance on the GPU at once (output sets)


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


class OutputSet:
    """One batch's maps: device buffers the step writes, pinned host copies
    filled by an asynchronous copy on the instance stream, and the event that
    marks them complete."""

    def __init__(self, X: int):
        import torch
        dt = (torch.int32, torch.int32, torch.float64, torch.int32)
        self.dev = [torch.empty((X, X), dtype=d, device="cuda") for d in dt]
        self.host = [torch.empty((X, X), dtype=d, pin_memory=True) for d in dt]
        self.event = torch.cuda.Event()
        self.origin = None

    def submit(self, mapper, scans, stream):
        """Queue the step and the copy to host; returns without waiting."""
        self.origin = mapper.step(scans, device_outputs=self.dev)
        for h, d in zip(self.host, self.dev):
            h.copy_(d, non_blocking=True)
        self.event.record(stream)

    def result(self):
        """Waits for the batch; fresh host arrays (origin, pos, neg, roughness, visibility)."""
        self.event.synchronize()
        return (self.origin, *[h.numpy().copy() for h in self.host])


class _Instance:
    def __init__(self, index: int, params: tuple, graphs: bool, reserve_points: int):
        import torch
        self.index = index
        self.params = params
        self.mapper = Gvom(*params)
        self.stream = torch.cuda.Stream()
        self.mapper.set_stream(self.stream.cuda_stream)
        self.mapper.set_graphs(graphs)
        self.max_scans = min(int(params[4]), 16)
        if reserve_points > 0:
            self.mapper.reserve(self.max_scans, reserve_points)
        self.outs = [OutputSet(int(params[2])) for _ in range(IN_FLIGHT)]
        self.free_outs: deque[int] = deque(range(IN_FLIGHT))
        self.queue: deque[Request] = deque()
        self.inflight: deque = deque()  # (batch, output set, error)
        self.cv = threading.Condition()
        self.submitting = True
        self.threads: list[threading.Thread] = []


class MapServer:
    """Continuous-batching request loop over map instances (one GB300).

    `point_budget` fixes the points per batch; by default it is taken at each
    admission as `mem_fraction` of the device's free memory, shared by the
    instances.  `reserve_points`: points per batch whose scratch each instance
    allocates at start-up (default: `max_scans` scans of 262,144 points).
    `freeze_gc`: move every object alive at start-up into the garbage
    collector's permanent generation (gc.freeze), so that a full collection
    during serving does not traverse the whole start-up heap.  The free
    memory behind the budget is read at most every `free_refresh_s` seconds:
    the query runs with the interpreter lock held, so an occasional slow
    driver call would stall every thread of the loop."""

    def __init__(self, instances: list[tuple], graphs: bool = True, mem_fraction: float = 0.25,
                 point_budget: int | None = None, reserve_points: int | None = None, freeze_gc: bool = True,
                 free_refresh_s: float = 0.05):
        import torch
        free, _ = torch.cuda.mem_get_info()
        self.free_at_start = free
        self.free_refresh_s = free_refresh_s
        self._free, self._free_t = free, float("-inf")  # read again at the first admission
        self.mem_fraction = mem_fraction
        self.fixed_budget = point_budget
        self.instances: list[_Instance] = []
        for i, p in enumerate(instances):
            # gvom_create refuses (GvomError, out of memory) an instance whose
            # resident footprint does not fit in free device memory
            rp = reserve_points if reserve_points is not None else min(int(p[4]), 16) * 262144
            self.instances.append(_Instance(i, tuple(p), graphs, rp))
        self.batches: list[tuple[int, list[int]]] = []  # (instance, request sequence numbers)
        self.budgets: list[int] = []  # point budget of each admission
        self._seq = 0
        self._lock = threading.Lock()
        self._running = True
        if freeze_gc:
            gc.collect()
            gc.freeze()
        for inst in self.instances:
            inst.threads = [threading.Thread(target=self._submitter, args=(inst,), daemon=True),
                            threading.Thread(target=self._completer, args=(inst,), daemon=True)]
            for t in inst.threads:
                t.start()

    @property
    def point_budget(self) -> int:
        return self._budget()

    def _budget(self) -> int:
        """Points the next batch may hold: fixed, or from the free device memory now."""
        if self.fixed_budget is not None:
            return self.fixed_budget
        import torch
        with self._lock:
            now = time.perf_counter()
            if now - self._free_t >= self.free_refresh_s:
                self._free, _ = torch.cuda.mem_get_info()
                self._free_t = now
            free = self._free
        return max(1, int(free * self.mem_fraction / BYTES_PER_POINT / max(1, len(self.instances))))

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
            inst.cv.notify_all()
        return r

    def _submitter(self, inst: _Instance):
        import torch
        torch.cuda.set_stream(inst.stream)
        while True:
            with inst.cv:
                while self._running and not (inst.queue and inst.free_outs):
                    inst.cv.wait()
                if not inst.queue:  # closing, nothing left to admit
                    inst.submitting = False
                    inst.cv.notify_all()
                    return
                while not inst.free_outs:
                    inst.cv.wait()
                budget = self._budget()
                n = plan_batch([q.points.shape[0] for q in inst.queue], inst.max_scans, budget)
                batch = [inst.queue.popleft() for _ in range(n)]
                j = inst.free_outs.popleft()
                self.budgets.append(budget)
            err = None
            try:
                inst.outs[j].submit(inst.mapper, [(r.points, r.ego, r.transform) for r in batch], inst.stream)
            except Exception as e:  # the batch is answered with the error
                err = e
            with inst.cv:
                inst.inflight.append((batch, j, err))
                inst.cv.notify_all()

    def _completer(self, inst: _Instance):
        while True:
            with inst.cv:
                while not inst.inflight and inst.submitting:
                    inst.cv.wait()
                if not inst.inflight:
                    return
                batch, j, err = inst.inflight.popleft()
            out = None
            if err is None:
                try:
                    out = inst.outs[j].result()
                except Exception as e:
                    err = e
            t = time.perf_counter()
            with self._lock:
                bid = len(self.batches)
                self.batches.append((inst.index, [r.seq for r in batch]))
            for r in batch:
                r.result = out if err is None else err
                r.batch_id = bid
                r.t_done = t
                r.done.set()
            with inst.cv:
                inst.free_outs.append(j)
                inst.cv.notify_all()

    def close(self):
        self._running = False
        for inst in self.instances:
            with inst.cv:
                inst.cv.notify_all()
        for inst in self.instances:
            for t in inst.threads:
                t.join()
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
