"""Served form (gvom_gb300/serve.py): admission policy and arrival process on
the CPU; on the GPU, two instances served concurrently with continuous
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
    pa = wa.gvom_args()[:4] + (8,) + wa.gvom_args()[5:]
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
