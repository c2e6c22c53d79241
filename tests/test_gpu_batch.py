"""Batched SCD (one block-diagonal union of many graphs) through the C ABI.

Each graph of a batch must give exactly what it gives alone: the converted
graph bit for bit (and equal to the reference's convert), p_ext, the
iteration count, the best labels and the WCC values bit for bit.
"""
import numpy as np
import pytest

import golden_data as G
import oracle as O
import scd_gb300 as S
import scdgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    e = S.Engine(0)
    yield e
    e.close()


def test_golden_fixtures_as_one_batch(engine):
    names = G.partition_cases()
    engine.batch_convert([G.pairs(n) for n in names])
    assert engine.batch_size() == len(names)
    for g, name in enumerate(names):
        assert engine.batch_graph_bytes(g) == G.graph_bytes(name), name
    results, rc = engine.batch_run(0.01, 1000)
    assert rc in (0, -7)
    for g, name in enumerate(names):
        tr = G.trace(name)
        n, m, cc = engine.batch_graph_info(g)
        if tr is None:          # empty graph: nothing to iterate
            assert n == 0
            continue
        assert cc == tr["p_ext"], name
        r = results[g]
        assert r["iterations"] == tr["iters"], name
        assert r["initial_communities"] == tr["num_comms"], name
        assert np.array_equal(engine.batch_labels(g), tr["best_labels"]), name
        assert abs(r["best_wcc"] - tr["best_wcc"]) <= 1e-6 * abs(tr["best_wcc"]), name
        assert r["printed_communities"] == tr["printed_comms"], name


def _random_graphs(k, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(k):
        kind = i % 3
        if kind == 0:
            n = int(np.exp(rng.uniform(np.log(300), np.log(6000))))
            out.append(scdgen.planted(n, float(rng.uniform(6, 24)), float(rng.uniform(0.05, 0.4)), 20, 100,
                                      seed=1000 + i))
        elif kind == 1:
            out.append(scdgen.rmat(int(rng.integers(8, 12)), 8, seed=2000 + i))
        else:
            out.append(scdgen.chunglu(int(rng.integers(1000, 5000)), 2.1, 5.0, 300.0, 0.2, 10, 100, seed=3000 + i))
    out.insert(k // 2, np.zeros((0, 2), np.uint32))            # an empty graph in the middle
    out.append(np.array([[0, 1], [1, 2], [0, 2]], np.uint32))   # a single triangle
    return out


@pytest.mark.parametrize("seed", [1, 2])
def test_each_graph_same_alone_and_in_the_batch(engine, seed):
    graphs = _random_graphs(24, seed)
    engine.batch_convert(graphs)
    results, rc = engine.batch_run(0.01, 500)
    assert rc == 0
    batch = []
    for g in range(len(graphs)):
        batch.append((engine.batch_graph_bytes(g), engine.batch_graph_info(g)[2], results[g],
                      engine.batch_labels(g)))
    alone = S.Engine(0)
    for g, pairs in enumerate(graphs):
        alone.convert_edges(pairs)
        gb, cc, r, lab = batch[g]
        assert alone.graph_bytes() == gb, g
        n = alone.graph_info()[0]
        if n == 0:
            continue
        assert alone.graph_info()[2] == cc or (np.isnan(cc) and np.isnan(alone.graph_info()[2]))
        ra = alone.run(0.01, 500)
        assert ra["iterations"] == r["iterations"], g
        assert ra["initial_wcc"] == r["initial_wcc"], g      # same summation shape: bit-identical
        assert ra["best_wcc"] == r["best_wcc"], g
        assert ra["printed_communities"] == r["printed_communities"], g
        assert np.array_equal(alone.labels_from_device(), lab), g
    alone.close()


def test_all_labels_at_once(engine):
    graphs = [scdgen.planted(500 + 300 * i, 8.0, 0.2, 20, 60, seed=70 + i) for i in range(6)]
    graphs.insert(3, np.zeros((0, 2), np.uint32))
    engine.batch_convert(graphs)
    engine.batch_run(0.01, 500)
    every = engine.batch_labels_all()
    assert len(every) == len(graphs)
    for g in range(len(graphs)):
        assert np.array_equal(every[g], engine.batch_labels(g)), g


def test_batch_against_oracle(engine):
    graphs = [scdgen.planted(2000 + 700 * i, 10.0 + i, 0.1 + 0.05 * i, 20, 100, seed=40 + i) for i in range(5)]
    engine.batch_convert(graphs)
    results, rc = engine.batch_run(0.01, 500)
    assert rc == 0
    for g, pairs in enumerate(graphs):
        ref, _ = O.convert(pairs)
        assert engine.batch_graph_bytes(g) == ref.to_bytes()
        r = O.run(ref, max_iters=500)
        assert results[g]["iterations"] == r["iters"]
        assert np.array_equal(engine.batch_labels(g), r["best_labels"])
        assert abs(results[g]["best_wcc"] - r["best_wcc"]) <= 1e-6 * r["best_wcc"]
