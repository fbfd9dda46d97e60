"""Served form (gvom_gb300/serve.py): admission policy, arrival process and
the request loop (with a stand-in mapper) on the CPU; on the GPU, two instances served concurrently with continuous
batching give, batch by batch, the same maps as the same batches run alone."""
import numpy as np
import pytest

from gvom_gb300.serve import plan_batch, poisson_arrivals


def test_plan_batch_limits():
    assert plan_batch([], 16, 1000) == 0
    assert plan_batch([5000], 16, 1000) == 1          # a scan above the budget runs alone
    assert plan_batch([400, 400, 400], 16, 1000) == 2  # point budget
    assert plan_batch([1] * 40, 16, 10 ** 9) == 16     # ring slots / launch limit
    assert plan_batch([1] * 40, 4, 10 ** 9) == 4
    assert plan_batch([600, 100, 100], 16, 1000) == 3


def test_poisson_arrivals_seeded_and_rate():
    a = poisson_arrivals([10.0, 20.0], 50.0, seed=4)
    b = poisson_arrivals([10.0, 20.0], 50.0, seed=4)
    assert a == b
    assert all(a[i][0] <= a[i + 1][0] for i in range(len(a) - 1))
    n0 = sum(1 for _, k in a if k == 0)
    n1 = sum(1 for _, k in a if k == 1)
    assert 400 < n0 < 600 and 850 < n1 < 1150


@pytest.mark.gpu
def test_served_mix_equals_alone(gpu_lib):
    import threading
    import time

    from gvom_gb300.serve import MapServer, replay_alone
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans

    wa = WORKLOADS["small_32x512"]
    pa = wa.gvom_args()[:4] + (16,) + wa.gvom_args()[5:]  # a 16-slot ring: merges of up to 17 sources
    pb = (0.2, 0.2, 96, 24, 4, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    scans = make_workload_scans(wa, 12)
    srv = MapServer([pa, pb], point_budget=60000)
    reqs = []

    def feed(inst, order, gap):
        for i in order:
            s = scans[i]
            reqs.append(srv.submit(inst, s.points, s.ego, s.transform))
            time.sleep(gap)

    # bursts: while an instance's first batch runs, the rest of its requests queue
    ta = threading.Thread(target=feed, args=(0, list(range(12)), 0.0))
    tb = threading.Thread(target=feed, args=(1, list(range(11, -1, -1)), 0.0))
    ta.start(); tb.start(); ta.join(); tb.join()
    for r in reqs:
        assert r.done.wait(60)
        assert not isinstance(r.result, Exception), r.result
    srv.close()
    assert any(len(seqs) > 1 for _, seqs in srv.batches), "no batching happened"
    for inst, params in ((0, pa), (1, pb)):
        alone = replay_alone(params, reqs, srv.batches, inst)
        served = []
        for bid, (i, seqs) in enumerate(srv.batches):
            if i != inst:
                continue
            r = next(q for q in reqs if q.batch_id == bid)
            served.append(r.result)
        assert len(alone) == len(served)
        for a, b in zip(alone, served):
            for x, y in zip(a, b):
                np.testing.assert_array_equal(x, y)


class _FakeMapper:
    """Stands in for Gvom in the request loop (CPU): records the calls, blocks
    the first process call until released, numbers its combines."""
    gate = None
    entered = {}
    calls = []

    def __init__(self, *params):
        self.params = params
        self.combines = 0
        self.first = True

    def set_stream(self, s):
        pass

    def set_graphs(self, on):
        pass

    def _process(self, kind, scans):
        if self.first and _FakeMapper.gate is not None:
            self.first = False
            _FakeMapper.entered[self.params[4]].set()
            _FakeMapper.gate.wait(10)
        if any(np.isnan(p).any() for p, _, _ in scans):
            raise RuntimeError("bad scan")
        _FakeMapper.calls.append((self.params[4], kind, [p.shape[0] for p, _, _ in scans]))

    def Process_pointcloud(self, points, ego, transform=None):
        self._process("one", [(points, ego, transform)])

    def process_batch(self, scans):
        self._process("batch", scans)

    def combine_maps(self):
        self.combines += 1
        return ("map", self.params[4], self.combines)

    def step(self, scans, device_outputs=None):
        self._process("one" if len(scans) == 1 else "batch", scans)
        return self.combine_maps()

    def reserve(self, max_scans, max_points, max_row_bytes=12):
        _FakeMapper.reserved[self.params[4]] = (max_scans, max_points)

    def close(self):
        pass


class _FakeOutputSet:
    """Stands in for serve.OutputSet on the CPU: the step runs when submitted."""

    def __init__(self, X):
        self.out = None

    def submit(self, mapper, scans, stream):
        self.out = mapper.step(scans)

    def result(self):
        return self.out


def test_request_loop_batches_and_answers(monkeypatch):
    """Continuous batching on CPU with a stand-in mapper: while an instance's
    first scan is on the (fake) device, later requests queue and go out as one
    batch, within the ring-slot and point limits; every request is answered
    with the map of its own batch; a failing batch (a scan the mapper rejects)
    answers with its error and the loop goes on."""
    import threading
    import types

    import torch

    from gvom_gb300 import serve
    monkeypatch.setattr(serve, "Gvom", _FakeMapper)
    monkeypatch.setattr(serve, "OutputSet", _FakeOutputSet)
    fake_cuda = types.SimpleNamespace(Stream=lambda: types.SimpleNamespace(cuda_stream=0),
                                      mem_get_info=lambda: (8 << 30, 16 << 30), set_stream=lambda s: None)
    monkeypatch.setattr(torch, "cuda", fake_cuda)
    _FakeMapper.gate = threading.Event()
    _FakeMapper.entered = {4: threading.Event(), 2: threading.Event()}
    _FakeMapper.calls = []
    _FakeMapper.reserved = {}
    p4 = (0.2, 0.2, 32, 16, 4, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    p2 = p4[:4] + (2,) + p4[5:]
    srv = serve.MapServer([p4, p2], point_budget=1000, freeze_gc=False)
    pts = lambda n: np.zeros((n, 3), np.float32)  # noqa: E731
    first = srv.submit(0, pts(10), (0, 0, 0))
    assert _FakeMapper.entered[4].wait(10)  # the first scan is on the device alone
    queued = [srv.submit(0, pts(300), (0, 0, 0)) for _ in range(6)]  # 4 slots, 1000 points -> 3 + 3
    other = [srv.submit(1, pts(5), (0, 0, 0)) for _ in range(3)]
    _FakeMapper.gate.set()
    for r in [first] + queued + other:
        assert r.done.wait(10)
    bad = srv.submit(1, np.full((2, 3), np.nan, np.float32), (0, 0, 0))
    assert bad.done.wait(10)
    after = srv.submit(1, pts(5), (0, 0, 0))  # the loop goes on after a failed batch
    assert after.done.wait(10)
    srv.close()
    assert first.result == ("map", 4, 1)
    inst0 = [c for c in _FakeMapper.calls if c[0] == 4]
    assert inst0[0] == (4, "one", [10])
    assert [c[2] for c in inst0[1:]] == [[300, 300, 300], [300, 300, 300]]
    assert [r.result[2] for r in queued] == [2, 2, 2, 3, 3, 3]
    assert len({r.batch_id for r in queued}) == 2
    assert all(isinstance(r.result, tuple) and r.result[1] == 2 for r in other)
    assert isinstance(bad.result, RuntimeError)
    assert isinstance(after.result, tuple) and after.result[1] == 2
    seqs = sorted(s for _, b in srv.batches for s in b)
    assert seqs == list(range(12))
    assert _FakeMapper.reserved == {4: (4, 4 * 262144), 2: (2, 2 * 262144)}  # scratch reserved at start-up
    assert all(r.latency >= 0 for r in [first] + queued + other)


def test_submitter_runs_ahead_of_completion(monkeypatch):
    """The submitter does not wait for a batch's maps: with two output sets a
    second batch is submitted while the first is still on the (fake) device,
    and a third waits only for a free output set."""
    import threading
    import types

    import torch

    from gvom_gb300 import serve

    release = threading.Event()
    submitted = []

    class HeldOutputSet(_FakeOutputSet):
        def submit(self, mapper, scans, stream):
            submitted.append(len(scans))
            super().submit(mapper, scans, stream)

        def result(self):
            assert release.wait(10)
            return super().result()

    monkeypatch.setattr(serve, "Gvom", _FakeMapper)
    monkeypatch.setattr(serve, "OutputSet", HeldOutputSet)
    fake_cuda = types.SimpleNamespace(Stream=lambda: types.SimpleNamespace(cuda_stream=0),
                                      mem_get_info=lambda: (8 << 30, 16 << 30), set_stream=lambda s: None)
    monkeypatch.setattr(torch, "cuda", fake_cuda)
    _FakeMapper.gate = None
    _FakeMapper.calls = []
    _FakeMapper.reserved = {}
    p = (0.2, 0.2, 32, 16, 1, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)  # one slot: one scan per batch
    srv = serve.MapServer([p], point_budget=1000, reserve_points=0, freeze_gc=False)
    pts = np.zeros((10, 3), np.float32)
    reqs = [srv.submit(0, pts, (0, 0, 0)) for _ in range(3)]
    import time
    deadline = time.time() + 10
    while len(submitted) < 2 and time.time() < deadline:
        time.sleep(0.01)
    time.sleep(0.1)
    assert submitted == [1, 1]          # two batches in flight, none answered yet
    assert not any(r.done.is_set() for r in reqs)
    release.set()
    for r in reqs:
        assert r.done.wait(10)
    srv.close()
    assert submitted == [1, 1, 1]
    assert [r.result[2] for r in reqs] == [1, 2, 3]
    assert _FakeMapper.reserved == {}  # reserve_points=0: nothing reserved


@pytest.mark.gpu
def test_instance_refused_when_device_memory_is_short(gpu_lib):
    """gvom_create's admission check: an instance whose resident footprint
    exceeds the free device memory is refused with GVOM_ERR_OOM before any
    allocation (2.0e9 voxels need about 300 GB), and the server's constructor
    raises it; a fitting instance is still admitted afterwards."""
    import ctypes as C

    from gvom_gb300 import Gvom
    from gvom_gb300._lib import GVOM_ERR_OOM, GvomError, GvomParams
    big = (0.2, 0.2, 8192, 29, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    h = C.c_void_p()
    rc = gpu_lib.gvom_create(C.byref(GvomParams(*big)), C.byref(h))
    assert rc == GVOM_ERR_OOM, rc
    assert b"admission refused" in gpu_lib.gvom_last_error()
    with pytest.raises(GvomError):
        Gvom(*big)
    g = Gvom(0.2, 0.2, 64, 16, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    assert g.device_bytes() > 0


def test_point_budget_reads_free_memory_at_most_every_refresh(monkeypatch):
    """Without a fixed budget, the point budget follows the device's free
    memory, read at most every `free_refresh_s` (the query holds the
    interpreter lock, so it is not made at every admission)."""
    import time
    import types

    import torch

    from gvom_gb300 import serve
    monkeypatch.setattr(serve, "Gvom", _FakeMapper)
    monkeypatch.setattr(serve, "OutputSet", _FakeOutputSet)
    _FakeMapper.gate = None
    _FakeMapper.reserved = {}
    reads = []
    free = [8 << 30]

    def mem_get_info():
        reads.append(time.perf_counter())
        return free[0], 16 << 30

    fake_cuda = types.SimpleNamespace(Stream=lambda: types.SimpleNamespace(cuda_stream=0),
                                      mem_get_info=mem_get_info, set_stream=lambda s: None)
    monkeypatch.setattr(torch, "cuda", fake_cuda)
    p = (0.2, 0.2, 32, 16, 4, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    srv = serve.MapServer([p, p], mem_fraction=0.25, free_refresh_s=0.2, freeze_gc=False)
    try:
        n0 = len(reads)  # the start-up reading
        b1 = srv.point_budget  # the first admission reads again
        assert len(reads) == n0 + 1
        assert b1 == int((8 << 30) * 0.25 / serve.BYTES_PER_POINT / 2)
        free[0] = 4 << 30
        for _ in range(50):  # within the refresh interval: the cached reading
            assert srv.point_budget == b1
        assert len(reads) == n0 + 1
        time.sleep(0.25)
        b2 = srv.point_budget
        assert len(reads) == n0 + 2
        assert b2 == int((4 << 30) * 0.25 / serve.BYTES_PER_POINT / 2)
    finally:
        srv.close()
