"""The resident set on the GPU (continuous batching at the iteration level).

Graphs join a running set between iterations and iterate in the same launches
as the graphs already there; every graph's result (iteration count, best WCC
bit for bit, best labels) must equal the result of running it alone."""
import threading

import numpy as np
import pytest

import scd_gb300 as S
import scdgen

pytestmark = pytest.mark.gpu


def _alone(pairs, max_iters=1000):
    with S.Engine(0) as e:
        e.convert_edges(pairs)
        if e.graph_info()[0] == 0:
            return None
        try:
            r = e.run(0.01, max_iters)
        except S.ScdError as x:   # max_iters reached
            assert x.status == -7
            r = None
        lab = e.labels_from_device()
        return r, lab


def _check(pairs, res, lab, max_iters=1000):
    want = _alone(pairs, max_iters)
    if want is None:
        assert res["iterations"] == 0 and lab.size == 0
        return
    r, wl = want
    if r is not None:
        assert res["iterations"] == r["iterations"]
        assert res["best_wcc"] == r["best_wcc"]
        assert res["printed_communities"] == r["printed_communities"]
    assert np.array_equal(lab, wl)


def test_graph_joins_running_graph_in_the_same_launches():
    a = scdgen.planted(20000, 16.0, 0.3, 20, 100, seed=41)    # needs several iterations
    b = scdgen.rmat(13, 16, seed=42)
    with S.Engine(0) as rs, S.Engine(0) as stage:
        rs.resident_init(0.01, 1000)
        stage.convert_edges(a)
        [ia] = rs.resident_add(stage)
        assert rs.resident_step() == (1, 0)          # a's first iteration, alone
        stage.convert_edges(b)                       # converted while a is resident
        [ib] = rs.resident_add(stage)
        assert rs.resident_info()["pending"] == 1
        l0 = rs.kernel_launches()
        running, _ = rs.resident_step()              # b joins: one replay for both graphs
        info = rs.resident_info()
        assert info["pending"] == 0 and info["graphs"] == 2
        launched = rs.kernel_launches() - l0
        assert launched >= info["kernels_per_step"] > 0
        out = {}
        steps_both = 0
        while len(out) < 2:
            l1 = rs.kernel_launches()
            running, fin = rs.resident_step()
            if running == 2:
                steps_both += 1
                # two graphs iterated, one replay's launches (no per-graph launches)
                assert rs.kernel_launches() - l1 == rs.resident_info()["kernels_per_step"]
            for gid, res, st, lab in rs.resident_take():
                assert st == 0
                out[gid] = (res, lab)
        assert rs.resident_info()["graph_steps"] > rs.resident_info()["steps"]   # co-scheduled
    _check(a, *out[ia])
    _check(b, *out[ib])


def test_many_graphs_joining_from_another_thread_equal_alone():
    rng = np.random.default_rng(9)
    graphs = []
    for i in range(18):
        k = i % 3
        if k == 0:
            graphs.append(scdgen.planted(int(rng.integers(500, 8000)), float(rng.uniform(6, 20)),
                                         float(rng.uniform(0.05, 0.4)), 20, 100, seed=700 + i))
        elif k == 1:
            graphs.append(scdgen.rmat(int(rng.integers(8, 13)), 8, seed=800 + i))
        else:
            graphs.append(scdgen.chunglu(int(rng.integers(1000, 6000)), 2.1, 5.0, 400.0, 0.2, 10, 100, seed=900 + i))
    graphs.insert(5, np.zeros((0, 2), np.uint32))               # an empty graph
    graphs.insert(9, np.array([[0, 1], [1, 2], [0, 2]], np.uint32))   # a single triangle
    ids = {}
    with S.Engine(0) as rs:
        rs.resident_init(0.01, 1000)
        lock = threading.Lock()
        added = threading.Event()

        def feed():
            with S.Engine(0) as stage:
                for lo in range(0, len(graphs), 4):
                    stage.batch_convert(graphs[lo:lo + 4])
                    got = rs.resident_add(stage)
                    with lock:
                        for j, g in enumerate(got):
                            ids[g] = lo + j
            added.set()

        t = threading.Thread(target=feed)
        t.start()
        out = {}
        while not (added.is_set() and len(out) == len(graphs)):
            rs.resident_step()
            for gid, res, st, lab in rs.resident_take():
                assert st == 0
                out[gid] = (res, lab)
        t.join()
        info = rs.resident_info()
        rs.resident_step()                         # every graph taken: the union is dropped
        assert rs.resident_info()["graphs"] == 0 and rs.memory_usage() == 0
    assert len(out) == len(graphs)
    for gid, (res, lab) in out.items():
        _check(graphs[ids[gid]], res, lab)
    assert info["graph_steps"] > info["steps"]


def test_max_iters_stops_a_graph_with_its_best_labels():
    a = scdgen.planted(10000, 18.0, 0.1, 20, 100, seed=1)   # 9 iterations to converge
    with S.Engine(0) as rs, S.Engine(0) as stage:
        rs.resident_init(0.01, 2)
        stage.convert_edges(a)
        rs.resident_add(stage)
        out = []
        while not out:
            rs.resident_step()
            out = rs.resident_take()
    [(_, res, st, lab)] = out
    assert st == -7 and res["iterations"] == 2
    _check(a, res, lab, max_iters=2)


def test_resident_errors():
    with S.Engine(0) as e, S.Engine(0) as f:
        with pytest.raises(S.ScdError) as ex:
            e.resident_step()
        assert ex.value.status == -4                 # not a resident set
        e.resident_init(0.01, 10)
        with pytest.raises(S.ScdError):
            e.resident_init(0.01, 10)                # already one
        assert e.resident_step() == (0, 0)           # empty set
        assert S.lib().scd_resident_add(e._ctx, f._ctx, None) == -4   # f holds no graph
        assert e.resident_take() == []
