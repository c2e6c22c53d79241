"""Served SCD on the GPU: every request's result in the mix equals the result alone."""
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
    with serve.Server(device=0, workers=3, max_batch=8) as srv:
        reqs = []
        for i, p in enumerate(reqs_pairs):
            reqs.append(srv.submit(p))
            if i >= 12:
                time.sleep(0.002)   # after a burst (batched), arrivals while earlier batches run
        outs = [r.wait(120) for r in reqs]
        assert sum(b for b, _ in srv.batches) == len(reqs)
        assert max(b for b, _ in srv.batches) > 1   # batching happened
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
