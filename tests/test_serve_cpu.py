"""Admission and continuous batching of the SCD server, with a fake engine (CPU)."""
import threading
import time

import numpy as np

import serve


class FakeEngine:
    """Stands in for scd_gb300.Engine: a batch takes 2 ms per graph."""
    live = 0
    peak = 0
    lock = threading.Lock()

    def batch_convert(self, graphs):
        self.graphs = graphs

    def batch_run(self, threshold, max_iters):
        with FakeEngine.lock:
            FakeEngine.live += 1
            FakeEngine.peak = max(FakeEngine.peak, FakeEngine.live)
        time.sleep(0.002 * len(self.graphs))
        with FakeEngine.lock:
            FakeEngine.live -= 1
        return [{"iterations": 1, "records": g.shape[0]} for g in self.graphs], 0

    def batch_labels_all(self):
        return [np.full(p.shape[0], g, np.uint32) for g, p in enumerate(self.graphs)]

    def close(self):
        pass


def test_budget_fifo_and_overlap():
    FakeEngine.live = FakeEngine.peak = 0
    srv = serve.Server(workers=3, budget_bytes=8 * (64e6 + 3000), max_batch=2, bytes_per_record=10,
                       engine_factory=FakeEngine)
    reqs = [srv.submit(np.zeros((100 + 50 * (i % 5), 2), np.uint32)) for i in range(40)]
    for r in reqs:
        res, lab = r.wait(10)
        assert res["records"] == r.records and lab.shape[0] == r.records
    srv.close()
    assert srv.peak_in_use <= srv.budget
    assert all(len_ <= 2 for len_, _ in srv.batches)
    assert sum(len_ for len_, _ in srv.batches) == 40
    starts = [r.started for r in reqs]
    assert starts == sorted(starts)          # admitted in arrival order
    assert FakeEngine.peak >= 2              # batches overlapped


def test_oversized_request_rejected():
    srv = serve.Server(workers=1, budget_bytes=65e6, bytes_per_record=1000, engine_factory=FakeEngine)
    r = srv.submit(np.zeros((10_000, 2), np.uint32))
    try:
        r.wait(1)
        assert False, "expected rejection"
    except Exception as e:
        assert "budget" in str(e)
    ok = srv.submit(np.zeros((10, 2), np.uint32))
    ok.wait(5)
    srv.close()


def test_percentile():
    assert serve.percentile([3, 1, 2], 50) == 2
    assert serve.percentile(list(range(101)), 99) == 99
