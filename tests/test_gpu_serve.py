"""Served SCD on the GPU: every request's result in the mix equals the result alone."""
import threading
import time

import numpy as np
import pytest

import scd_gb300 as S
import scdgen
import serve

pytestmark = pytest.mark.gpu


def _requests(k, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(k):
        if rng.random() < 0.8:
            n = int(np.exp(rng.uniform(np.log(1000), np.log(20000))))
            out.append(scdgen.planted(n, 16.0 * 0.9, 0.1, 20, 100, seed=500 + i))
        else:
            out.append(scdgen.rmat(int(rng.integers(11, 14)), 16, seed=600 + i))
    return out


def test_results_identical_alone_and_in_the_mix():
    reqs_pairs = _requests(30, 5)
    with serve.Server(device=0, converters=2, max_batch=8) as srv:
        reqs = []
        for i, p in enumerate(reqs_pairs):
            reqs.append(srv.submit(p))
            if i >= 12:
                time.sleep(0.002)   # after a burst (batched), arrivals while earlier graphs iterate
        outs = [r.wait(120) for r in reqs]
        assert sum(b for b, _ in srv.batches) == len(reqs)
        assert max(b for b, _ in srv.batches) > 1   # batched conversion happened
        assert srv.mean_coscheduled() > 1           # graphs iterated in the same launches
    alone = S.Engine(0)
    for p, (res, lab) in zip(reqs_pairs, outs):
        alone.convert_edges(p)
        if alone.graph_info()[0] == 0:
            continue
        ra = alone.run(0.01, 1000)
        assert ra["iterations"] == res["iterations"]
        assert ra["best_wcc"] == res["best_wcc"]
        assert np.array_equal(alone.labels_from_device(), lab)
    alone.close()


def test_late_request_joins_running_iterations():
    """A request submitted while another request's graph is iterating is converted
    alongside and joins the running graph's launches (a step with both running,
    one replay's kernels for both); both results equal the results alone.  The
    step hook holds the iterations after the first request's first step until
    the second request has been converted and handed over, so the overlap does
    not depend on timing."""
    slow = scdgen.planted(20000, 16.0, 0.35, 20, 100, seed=77)   # several iterations
    late = scdgen.planted(1000, 14.0, 0.1, 20, 100, seed=78)
    gate, held = threading.Event(), threading.Event()

    def hook(lane, steps_done):
        if lane == 0 and steps_done == 1:   # after the slow request's first iteration
            held.set()
            assert gate.wait(60)

    with serve.Server(device=0, converters=1, max_batch=8, step_hook=hook) as srv:
        r1 = srv.submit(slow)
        assert held.wait(60)
        r2 = srv.submit(late)
        t0 = time.time()
        while srv.set.resident_info()["pending"] < 1:   # converted and handed over
            assert time.time() - t0 < 60
            time.sleep(0.001)
        gate.set()
        out1, out2 = r1.wait(120), r2.wait(120)
        info = srv.set.resident_info()
        assert srv.step_running[1] == 2                  # the step after the join: both graphs
        assert info["graph_steps"] > info["steps"]       # (test_gpu_resident counts the launches of such steps)
    alone = S.Engine(0)
    for p, (res, lab) in ((slow, out1), (late, out2)):
        alone.convert_edges(p)
        ra = alone.run(0.01, 1000)
        assert ra["iterations"] == res["iterations"]
        assert ra["best_wcc"] == res["best_wcc"]
        assert np.array_equal(alone.labels_from_device(), lab)
    alone.close()
