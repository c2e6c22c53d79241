"""GPU engine vs the reference (golden fixtures) and vs the oracle, through the C ABI.

Bar (from the task): the converted graph (CSR, tri, tri_deg) and the initial
partition bit-exact; per-iteration labels identical under the reference's
tie-breaking rule; WCC within 1e-6 relative (the engine sums per-vertex terms
in a fixed tree order, the reference in index order, so the last bits of the
sum may differ).  p_ext is summed in the reference's single-thread order and
must be bit-exact.
"""
import numpy as np
import pytest

import golden_data as G
import oracle as O
import scd_gb300 as S
import scdgen
from parity_log import log

pytestmark = pytest.mark.gpu
WCC_RTOL = 1e-6
CASES = G.cases()
TRACED = [c for c in G.partition_cases() if G.manifest()[c].get("iters")]
FROM_LABELS = [c for c in CASES if G.starts_from_labels(c)]


@pytest.fixture(scope="module")
def engine():
    e = S.Engine(0)
    yield e
    e.close()


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("name", CASES)
def test_convert_bit_exact_with_reference(engine, name):
    engine.convert_edges(G.pairs(name))
    assert engine.graph_bytes() == G.graph_bytes(name)


def _divergence_report(g, p_ext, labels, stats, got, want):
    bad = np.nonzero(got != want)[0]
    return f"{len(bad)} vertices differ, first {bad[:10].tolist()}: got {got[bad[:10]].tolist()} want {want[bad[:10]].tolist()}"


@pytest.mark.parametrize("name", TRACED)
def test_iterations_match_reference_trace(engine, name):
    g = O.Graph.from_bytes(G.graph_bytes(name))
    tr = G.trace(name)
    engine.transfer_graph(g)
    n, m, cc = engine.graph_info()
    assert (n, m) == (tr["n"], tr["m"])
    assert cc == tr["p_ext"], "p_ext must be the reference's single-thread sum"
    nc = engine.initial_partition()
    assert nc == tr["num_comms"]
    assert np.array_equal(engine.current_labels(), tr["initial_labels"])
    assert np.array_equal(np.stack(engine.community_stats()), tr["initial_stats"])
    w0 = engine.compute_wcc()
    assert rel(w0, tr["initial_wcc"]) < WCC_RTOL
    for i in range(tr["iters"]):
        w = engine.improve_labels()
        got = engine.current_labels()
        log(name, f"iteration {i + 1}", labels_equal=bool(np.array_equal(got, tr["labels"][i])), wcc=w.hex(),
            wcc_ref=tr["wcc"][i].hex(), wcc_rel=rel(w, tr["wcc"][i]))
        assert np.array_equal(got, tr["labels"][i]), f"iteration {i}: " + _divergence_report(
            g, cc, None, None, got, tr["labels"][i])
        assert np.array_equal(np.stack(engine.community_stats()), tr["stats"][i])
        assert rel(w, tr["wcc"][i]) < WCC_RTOL


@pytest.mark.parametrize("name", TRACED)
def test_run_loop_matches_reference(engine, name):
    g = O.Graph.from_bytes(G.graph_bytes(name))
    tr = G.trace(name)
    engine.transfer_graph(g)
    r = engine.run(0.01, 1000)
    assert r["iterations"] == tr["iters"]
    assert r["initial_communities"] == tr["num_comms"]
    assert rel(r["best_wcc"], tr["best_wcc"]) < WCC_RTOL
    assert np.array_equal(engine.labels_from_device(), tr["best_labels"])
    assert r["printed_communities"] == tr["printed_comms"]
    for a, b in zip(r["wcc"], tr["wcc"]):
        assert rel(a, b) < WCC_RTOL


@pytest.mark.parametrize("name", FROM_LABELS)
def test_iterations_from_given_labels_match_reference(engine, name):
    """wrap_windmill: a hub of degree 60,000 whose community has 50,001 members, so
    the int32 products d_in*(d_in-1), d_out*(d_out-1) and (r-1)*(r-2) of the gain
    model (src/scd.cpp:185-213) wrap; labels, statistics and WCC of every
    iteration against the reference's loop started from the same labels."""
    g = O.Graph.from_bytes(G.graph_bytes(name))
    tr = G.trace(name)
    engine.transfer_graph(g)
    assert engine.graph_info()[2] == tr["p_ext"]
    engine.labels_to_device(G.start_labels(name))
    assert np.array_equal(np.stack(engine.community_stats()), tr["initial_stats"])
    assert rel(engine.compute_wcc(), tr["initial_wcc"]) < WCC_RTOL
    for i in range(tr["iters"]):
        w = engine.improve_labels()
        got = engine.current_labels()
        log(name, f"iteration {i + 1} (from given labels)", labels_equal=bool(np.array_equal(got, tr["labels"][i])),
            wcc=w.hex(), wcc_ref=tr["wcc"][i].hex(), wcc_rel=rel(w, tr["wcc"][i]))
        assert np.array_equal(got, tr["labels"][i]), f"iteration {i}: " + _divergence_report(
            g, None, None, None, got, tr["labels"][i])
        assert np.array_equal(np.stack(engine.community_stats()), tr["stats"][i])
        assert rel(w, tr["wcc"][i]) < WCC_RTOL


@pytest.mark.parametrize("name", FROM_LABELS)
def test_run_loop_from_given_labels_matches_reference(engine, name):
    g = O.Graph.from_bytes(G.graph_bytes(name))
    tr = G.trace(name)
    engine.transfer_graph(g)
    engine.labels_to_device(G.start_labels(name))
    r = engine.run(0.01, 1000)
    assert r["iterations"] == tr["iters"]
    assert rel(r["best_wcc"], tr["best_wcc"]) < WCC_RTOL
    assert np.array_equal(engine.labels_from_device(), tr["best_labels"])
    assert r["printed_communities"] == tr["printed_comms"]


RANDOM_GRAPHS = [
    ("planted", lambda s: scdgen.planted(3000 + 500 * s, 10.0 + 2 * s, 0.05 + 0.07 * s, 20, 100, seed=100 + s)),
    ("rmat", lambda s: scdgen.rmat(10 + s % 4, 8 + 4 * (s % 3), seed=200 + s)),
    ("chunglu", lambda s: scdgen.chunglu(4000 + 1000 * s, 2.1, 5.0, 300.0 + 200 * s, 0.2, 10, 200, seed=300 + s)),
]


@pytest.mark.parametrize("kind,make", RANDOM_GRAPHS, ids=[k for k, _ in RANDOM_GRAPHS])
@pytest.mark.parametrize("seed", range(4))
def test_random_graphs_against_oracle(engine, kind, make, seed):
    pairs = make(seed)
    # shuffle the record order and flip some pairs: exercises first-appearance renumbering
    rng = np.random.default_rng(seed)
    pairs = pairs[rng.permutation(pairs.shape[0])]
    dup = pairs[rng.integers(0, pairs.shape[0], pairs.shape[0] // 20)]
    pairs = np.concatenate([pairs, dup, np.array([[7, 7], [3, 3]], np.uint32)])
    ref, _ = O.convert(pairs)
    engine.convert_edges(pairs)
    assert engine.graph_bytes() == ref.to_bytes()
    if ref.n == 0:
        return
    r = O.run(ref, max_iters=200)
    n, m, cc = engine.graph_info()
    assert cc == O.clustering_coef(ref)
    engine.initial_partition()
    assert np.array_equal(engine.current_labels(), r["initial_labels"])
    for i in range(len(r["wcc"])):
        w = engine.improve_labels()
        assert np.array_equal(engine.current_labels(), r["labels"][i]), f"iteration {i}"
        assert rel(w, r["wcc"][i]) < WCC_RTOL


def test_empty_and_degenerate_inputs(engine):
    engine.convert_edges(np.zeros((0, 2), np.uint32))
    assert engine.graph_info()[:2] == (0, 0)
    assert engine.graph_bytes() == O.convert(np.zeros((0, 2), np.uint32))[0].to_bytes()
    loops = np.array([[5, 5], [9, 9]], np.uint32)
    engine.convert_edges(loops)
    assert engine.graph_bytes() == O.convert(loops)[0].to_bytes()
    tri = np.array([[0, 1], [1, 2], [0, 2]], np.uint32)
    engine.convert_edges(tri)
    assert engine.graph_bytes() == O.convert(tri)[0].to_bytes()
    r = engine.run()
    assert r["iterations"] >= 1


def test_transferred_graph_with_isolated_vertices(engine):
    """A graph file may hold vertices without edges (convert never writes one): they keep
    their labels, count in their communities' sizes and add nothing to the WCC sum.  Their
    clustering coefficient is 0/0 (NaN), whose place in the reference's std::sort order is
    undefined, so the iterations start from the oracle's initial labels."""
    g = O.Graph.from_bytes(G.graph_bytes("planted_2k_mu03"))
    extra = 7
    ind = np.concatenate([g.indices, np.full(extra, g.indices[-1], np.uint32)])
    pad = np.zeros(extra, np.int32)
    gi = O.Graph(g.n + extra, g.m, ind, g.adj, np.concatenate([g.tri, pad]), np.concatenate([g.tri_deg, pad]))
    ref = O.run(gi, max_iters=200)
    engine.transfer_graph(gi)
    assert engine.graph_info()[2] == O.clustering_coef(gi)
    engine.labels_to_device(ref["initial_labels"])
    assert rel(engine.compute_wcc(), ref["initial_wcc"]) < WCC_RTOL
    for i in range(len(ref["wcc"])):
        w = engine.improve_labels()
        assert np.array_equal(engine.current_labels(), ref["labels"][i]), f"iteration {i}"
        assert rel(w, ref["wcc"][i]) < WCC_RTOL


def _compress_intended(labels):
    """compress_labels (src/scd.cpp:32-55) with its branch the way round it is meant."""
    out, seen, k = np.empty_like(labels), {}, 0
    for p, l in enumerate(labels.tolist()):
        if l == 0xFFFFFFFF:
            out[p] = k
            k += 1
        elif l not in seen:
            seen[l] = k
            out[p] = k
            k += 1
        else:
            out[p] = seen[l]
    return out, k


@pytest.mark.parametrize("name", ["planted_2k_mu03", "chunglu_20k", "rmat_12"])
def test_compressed_labels(engine, name):
    engine.transfer_graph(O.Graph.from_bytes(G.graph_bytes(name)))
    r = engine.run(0.01, 1000)
    best = engine.labels_from_device()
    got, k = engine.compressed_labels()
    want, kw = _compress_intended(best)
    assert k == kw and np.array_equal(got, want)
    assert k == r["distinct_communities"] + int((best == 0xFFFFFFFF).sum())


def test_call_order_and_argument_errors(engine):
    e = S.Engine(0)
    with pytest.raises(S.ScdError) as ex:
        e.improve_labels()
    assert ex.value.status == -4
    e.convert_edges(G.pairs("planted_2k_mu03"))
    with pytest.raises(S.ScdError) as ex:
        e.compute_wcc()
    assert ex.value.status == -4
    n = e.graph_info()[0]
    with pytest.raises(S.ScdError) as ex:
        e.labels_to_device(np.full(n, n + 5, np.uint32))
    assert ex.value.status == -1
    e.close()


def test_labels_to_device_roundtrip(engine):
    name = "planted_2k_mu03"
    g = O.Graph.from_bytes(G.graph_bytes(name))
    tr = G.trace(name)
    engine.transfer_graph(g)
    engine.labels_to_device(tr["labels"][2])
    st = np.stack(engine.community_stats())
    k = st.shape[1]
    assert np.array_equal(st, tr["stats"][2][:, :k]) and not tr["stats"][2][:, k:].any()
    engine.improve_labels()
    assert np.array_equal(engine.current_labels(), tr["labels"][3])


@pytest.mark.parametrize("scale", [16, 18])
def test_rmat_full_pipeline_against_oracle(engine, scale):
    # scale 18: n = 104k, 13 tiles of the exact p_ext sum, hubs of degree ~25k
    pairs = scdgen.rmat(scale, 16, seed=22)
    ref, _ = O.convert(pairs)
    engine.convert_edges(pairs)
    assert engine.graph_bytes() == ref.to_bytes()
    assert engine.graph_info()[2] == O.clustering_coef(ref)
    r = O.run(ref, max_iters=50)
    engine.initial_partition()
    assert np.array_equal(engine.current_labels(), r["initial_labels"])
    for i in range(len(r["wcc"])):
        w = engine.improve_labels()
        assert np.array_equal(engine.current_labels(), r["labels"][i])
        assert rel(w, r["wcc"][i]) < WCC_RTOL


@pytest.mark.parametrize("make", [lambda: scdgen.rmat(16, 16, seed=7),
                                  lambda: scdgen.chunglu(60_000, 2.1, 5.0, 5000.0, 0.2, 10, 200, seed=5)])
def test_in_list_units_agree_with_out_list_counting(engine, make):
    # the same triangles counted from the out-list tables only (no in-list centres)
    pairs = make()
    engine.convert_edges(pairs)
    e2 = S.Engine(0, flags=S.FLAG_TC_OUT_ONLY)
    try:
        e2.convert_edges(pairs)
        assert e2.graph_bytes() == engine.graph_bytes()
        r1, r2 = engine.run(0.01, 20), e2.run(0.01, 20)
        assert np.array_equal(r1["wcc"], r2["wcc"]) and r1["iterations"] == r2["iterations"]
        assert np.array_equal(engine.labels_from_device(), e2.labels_from_device())
    finally:
        e2.close()


def _dense_block(n=1600, p=0.8, seed=11):
    # out-degrees beyond 1024: centres of the second CTA bucket (1024, 8192]
    rng = np.random.default_rng(seed)
    iu, ju = np.triu_indices(n, 1)
    keep = rng.random(iu.size) < p
    return np.stack([iu[keep], ju[keep]], axis=1).astype(np.uint32)


@pytest.mark.parametrize("out_only", [False, True], ids=["in-lists", "out-only"])
@pytest.mark.parametrize("kind,make", [
    ("rmat16", lambda: scdgen.rmat(16, 16, seed=7)),
    ("rmat18", lambda: scdgen.rmat(18, 16, seed=9)),   # > 128K vertices: the split chosen from core sizes
    ("chunglu60k", lambda: scdgen.chunglu(60_000, 2.1, 5.0, 5000.0, 0.2, 10, 200, seed=5)),
    ("planted20k", lambda: scdgen.planted(20_000, 30.0, 0.3, 20, 400, seed=3)),
    ("dense1600", _dense_block),
], ids=lambda v: v if isinstance(v, str) else "")
def test_core_bitmap_kernel_agrees_with_hash_kernels(kind, make, out_only):
    # the exact core-bitmap CTA kernel (default) and the shared hash-table CTA
    # kernels count the same triangles: the same graph bytes
    pairs = make()
    base = S.FLAG_TC_OUT_ONLY if out_only else 0
    e1, e2 = S.Engine(0, flags=base), S.Engine(0, flags=base | S.FLAG_TC_HASH)
    try:
        e1.convert_edges(pairs)
        e2.convert_edges(pairs)
        assert e1.graph_bytes() == e2.graph_bytes()
    finally:
        e1.close()
        e2.close()


def test_core_bitmap_kernel_against_oracle_on_dense_block(engine):
    pairs = _dense_block()
    engine.convert_edges(pairs)
    assert engine.graph_bytes() == O.convert(pairs)[0].to_bytes()


def test_autotune_keeps_results():
    # every split the autotuner may pick counts the same triangles
    pairs = scdgen.chunglu(40_000, 2.1, 5.0, 3000.0, 0.2, 10, 200, seed=9)
    e = S.Engine(0)
    try:
        e.convert_edges(pairs)
        ref = e.graph_bytes()
        r0 = e.run(0.01, 20)
        t = e.autotune()
        assert t["small_max"] in (0, 16, 32) and t["warp_max"] in (16, 32, 64) and t["cta_max"] in (256, 512, 1024)
        assert t["in_list_min"] in (0, 16, 32) and t["in_list_min"] <= t["small_max"]
        assert len(t["report"]) > 20
        e.convert_edges(pairs)
        assert e.graph_bytes() == ref
        r1 = e.run(0.01, 20)
        assert np.array_equal(r1["wcc"], r0["wcc"])
    finally:
        e.close()
