"""Admission, continuous batching and cancellation of the SCD server, with a fake
engine (CPU): the host logic of serve.py without a GPU."""
import threading
import time

import numpy as np
import pytest

import serve


class FakeEngine:
    """Stands in for scd_gb300.Engine.  A converted graph of r records needs
    1 + r % 3 iterations; one resident step (1 ms) advances every running graph
    by one iteration, like the single CUDA-graph replay of the real set."""

    def __init__(self):
        self.graphs = None
        self.lock = threading.Lock()

    def batch_convert(self, graphs):
        time.sleep(0.001)
        self.graphs = [g.shape[0] for g in graphs]

    def resident_init(self, threshold, max_iters):
        self.max_iters = max_iters
        self.pending, self.live, self.next_id = [], {}, 0

    def resident_add(self, src):
        with self.lock:
            ids = list(range(self.next_id, self.next_id + len(src.graphs)))
            self.next_id += len(ids)
            self.pending += [(i, r) for i, r in zip(ids, src.graphs)]
        src.graphs = None
        return ids

    def resident_step(self):
        with self.lock:
            for i, r in self.pending:
                self.live[i] = {"records": r, "need": 1 + r % 3, "iters": 0, "done": False}
            self.pending = []
        running = [g for g in self.live.values() if not g["done"]]
        time.sleep(0.001)
        fin = 0
        for g in running:
            g["iters"] += 1
            if g["iters"] >= min(g["need"], self.max_iters):
                g["done"] = True
                fin += 1
        return len(running), fin

    def resident_take(self):
        out = []
        for i in [i for i, g in self.live.items() if g["done"]]:
            g = self.live.pop(i)
            st = -7 if g["need"] > self.max_iters else 0
            out.append((i, {"iterations": g["iters"], "records": g["records"]}, st,
                        np.full(g["records"], i, np.uint32)))
        return out

    def close(self):
        pass


def test_budget_fifo_and_coscheduling():
    srv = serve.Server(converters=2, budget_bytes=8 * (64e6 + 3000), max_batch=2, bytes_per_record=10,
                       engine_factory=FakeEngine)
    reqs = []
    for i in range(40):
        reqs.append(srv.submit(np.zeros((100 + 50 * (i % 5), 2), np.uint32)))
        if i % 4 == 3:
            time.sleep(0.002)   # arrivals while earlier requests iterate
    for r in reqs:
        res, lab = r.wait(10)
        assert res["records"] == r.records and lab.shape[0] == r.records
        assert res["iterations"] == 1 + r.records % 3
    srv.close()
    assert srv.peak_in_use <= srv.budget
    assert all(len_ <= 2 for len_, _ in srv.batches)
    assert sum(len_ for len_, _ in srv.batches) == 40
    starts = [r.started for r in reqs]
    assert starts == sorted(starts)          # admitted in arrival order
    assert srv.mean_coscheduled() > 1        # requests iterated in the same steps


def test_oversized_request_rejected():
    srv = serve.Server(converters=1, budget_bytes=65e6, bytes_per_record=1000, engine_factory=FakeEngine)
    r = srv.submit(np.zeros((10_000, 2), np.uint32))
    with pytest.raises(Exception, match="budget"):
        r.wait(1)
    ok = srv.submit(np.zeros((10, 2), np.uint32))
    ok.wait(5)
    srv.close()


def test_cancelled_requests():
    """A request cancelled while queued never converts and frees nothing it did
    not take; one cancelled after conversion has its result dropped; the others
    are unaffected and the budget returns to zero."""
    srv = serve.Server(converters=1, budget_bytes=2 * (64e6 + 10_000), max_batch=1, bytes_per_record=10,
                       engine_factory=FakeEngine)
    first = [srv.submit(np.zeros((500 + i, 2), np.uint32)) for i in range(6)]
    queued = first[-1]
    assert srv.cancel(queued)
    with pytest.raises(serve.Cancelled):
        queued.wait(5)
    assert queued.started is None                      # never converted
    late = srv.submit(np.zeros((300, 2), np.uint32))
    while late.started is None:                        # converted and in the set
        time.sleep(0.0005)
    srv.cancel(late)
    with pytest.raises(serve.Cancelled):
        late.wait(5)
    for r in first[:-1]:
        res, lab = r.wait(10)
        assert lab.shape[0] == r.records
    assert not srv.cancel(first[0])                    # already finished
    srv.close()
    assert abs(srv._in_use) < 1e-6


def test_failed_conversion_fails_its_batch_only():
    class Failing(FakeEngine):
        def batch_convert(self, graphs):
            if any(g.shape[0] == 13 for g in graphs):
                raise RuntimeError("SCD_ERR_OOM: simulated allocator failure")
            super().batch_convert(graphs)

    srv = serve.Server(converters=1, budget_bytes=1e12, max_batch=1, bytes_per_record=10, engine_factory=Failing)
    bad = srv.submit(np.zeros((13, 2), np.uint32))
    good = srv.submit(np.zeros((20, 2), np.uint32))
    with pytest.raises(RuntimeError, match="OOM"):
        bad.wait(5)
    assert good.wait(5)[0]["records"] == 20
    srv.close()
    assert abs(srv._in_use) < 1e-6


def test_percentile():
    assert serve.percentile([3, 1, 2], 50) == 2
    assert serve.percentile(list(range(101)), 99) == 99


def test_size_lanes():
    """Requests above the lane bound go to the second resident set; each lane's
    results are right and both lanes stepped."""
    srv = serve.Server(converters=2, budget_bytes=1e12, max_batch=4, bytes_per_record=10, engine_factory=FakeEngine,
                       lanes=(1000,))
    reqs = [srv.submit(np.zeros((300 if i % 3 else 4000 + i, 2), np.uint32)) for i in range(12)]
    for r in reqs:
        res, lab = r.wait(10)
        assert res["records"] == r.records and lab.shape[0] == r.records
    srv.close()
    assert srv.lane_of(300) == 0 and srv.lane_of(4000) == 1
    assert srv.lanes[0].steps > 0 and srv.lanes[1].steps > 0
    assert all(len({srv.lane_of(r.records) for r in reqs[i:i + 1]}) == 1 for i in range(12))
