"""The oracle (CPU restatement) against the reference's own outputs.

The golden fixtures were produced by the reference's convert binary and by a
driver linking the reference's scd.cpp/wcc.cpp/graph.cpp (tests/golden/make_golden.py);
the oracle must reproduce them bit for bit before it may check the GPU engine.
"""
import os

import numpy as np
import pytest

import golden_data as G
import oracle as O

CASES = G.cases()
TRACED = [c for c in G.partition_cases() if G.manifest()[c].get("iters")]
FROM_LABELS = [c for c in CASES if G.starts_from_labels(c)]


@pytest.mark.parametrize("name", CASES)
def test_convert_matches_reference_file(name):
    g, _ = O.convert(G.pairs(name))
    assert g.to_bytes() == G.graph_bytes(name)


@pytest.mark.parametrize("name", TRACED)
def test_refinement_trace_matches_reference(name):
    g = O.Graph.from_bytes(G.graph_bytes(name))
    tr = G.trace(name)
    assert O.clustering_coef(g) == tr["p_ext"]
    r = O.run(g, max_iters=1000)
    assert r["iters"] == tr["iters"]
    assert np.array_equal(r["initial_labels"], tr["initial_labels"])
    assert r["initial_wcc"] == tr["initial_wcc"]
    assert r["num_comms"] == tr["num_comms"]
    for i in range(tr["iters"]):
        assert np.array_equal(r["labels"][i], tr["labels"][i]), f"iteration {i}"
        assert r["wcc"][i] == tr["wcc"][i]
    assert np.array_equal(r["best_labels"], tr["best_labels"])
    assert r["best_wcc"] == tr["best_wcc"]
    assert r["printed_comms"] == tr["printed_comms"]


@pytest.mark.parametrize("name", TRACED + FROM_LABELS)
def test_statistics_match_reference(name):
    g = O.Graph.from_bytes(G.graph_bytes(name))
    tr = G.trace(name)
    nc = tr["num_comms"]
    s, e, i = O.collect_stats(g, tr["initial_labels"], nc)
    assert np.array_equal(np.stack([s, e, i]), tr["initial_stats"])
    for it in range(tr["iters"]):
        s, e, i = O.collect_stats(g, tr["labels"][it], nc)
        assert np.array_equal(np.stack([s, e, i]), tr["stats"][it])


@pytest.mark.parametrize("name", FROM_LABELS)
def test_loop_from_given_labels_matches_reference(name):
    """The reference's loop started from a given labelling (wrap_windmill: the
    int32 products of the gain model wrap for the hub and its community)."""
    g = O.Graph.from_bytes(G.graph_bytes(name))
    tr = G.trace(name)
    lab = G.start_labels(name)
    assert np.array_equal(lab, tr["initial_labels"])
    r = O.run_from_labels(g, lab, max_iters=1000)
    assert r["num_comms"] == tr["num_comms"]
    assert r["initial_wcc"] == tr["initial_wcc"]
    assert r["iters"] == tr["iters"]
    for i in range(tr["iters"]):
        assert np.array_equal(r["labels"][i], tr["labels"][i]), f"iteration {i}"
        assert r["wcc"][i] == tr["wcc"][i]
    assert np.array_equal(r["best_labels"], tr["best_labels"])
    assert r["best_wcc"] == tr["best_wcc"]
    assert r["printed_comms"] == tr["printed_comms"]


def test_windmill_reaches_the_int32_wrap():
    """The wrap_windmill labelling puts d_in*(d_in-1), d_out*(d_out-1) and
    (r-1)*(r-2) of src/scd.cpp:185-213 past 2^31 for the hub."""
    g = O.Graph.from_bytes(G.graph_bytes("wrap_windmill"))
    lab = G.start_labels("wrap_windmill")
    deg = int(g.indices[1] - g.indices[0])
    nb = lab[g.adj[g.indices[0]:g.indices[1]]]
    d_in0 = int((nb == 0).sum())
    r0 = int((lab == 0).sum()) - 1                 # own community, the hub taken out
    d_out1 = deg - int((nb == 1).sum())
    for x in (d_in0, r0 - 1, d_out1):
        assert x * (x - 1) > 2**31 - 1


def test_known_answer_triangle_pendant():
    # triangle 0-1-2 plus pendant 2-3: the pendant edge has no triangle
    g, _ = O.convert(G.pairs("triangle_pendant"))
    assert (g.n, g.m) == (3, 3)
    assert g.tri.tolist() == [2, 2, 2] and g.tri_deg.tolist() == [2, 2, 2]


def test_readme_example_is_empty():
    g, _ = O.convert(G.pairs("readme_example"))
    assert (g.n, g.m) == (0, 0)
    assert g.indices.tolist() == [0]


def test_compress_labels_inverted_branch():
    # a triangle in one community prints 2 communities (src/scd.cpp:44-48)
    cnt, lab = O.compress_labels(np.zeros(3, np.uint32))
    assert cnt == 2 and lab.tolist() == [0, 0, 1]
    cnt, _ = O.compress_labels(np.array([5, 0xFFFFFFFF, 5, 7], np.uint32))
    assert cnt == 4 - 2


def test_text_parser(tmp_path):
    p = tmp_path / "e.txt"
    p.write_text("# c\n\n  3 1\n2 2\n\t7 4 junk\n")
    assert O.read_text(str(p)).tolist() == [[1, 3], [2, 2], [4, 7]]
    p.write_text("1 2\nx 3\n")
    with pytest.raises(ValueError):
        O.read_text(str(p))


def test_gain_model_spot_values():
    # hand-evaluated corner cases of src/scd.cpp:173-219
    assert O.gain(0, 0, 0, 0, 0.0, 0.5) == 0.0
    g = O.gain(10, 3, 2, 7, 0.4, 0.3)
    assert np.isfinite(g)
    # int32 wrap-around of d_in*(d_in-1) is part of the model
    assert np.isfinite(O.gain(70000, 50000, 100, 5, 0.01, 0.2))


def test_oracle_thread_count_independent():
    import subprocess
    import sys
    code = ("import sys; sys.path[:0]=[%r,%r]; import golden_data as G, oracle as O;"
            "g=O.Graph.from_bytes(G.graph_bytes('planted_2k_mu03')); r=O.run(g);"
            "print(r['best_wcc'].hex(), int(r['best_labels'].sum()))") % (
        os.path.join(os.path.dirname(__file__)), os.path.join(os.path.dirname(__file__), "..", "oracle"))
    outs = set()
    for t in ("1", "3"):
        env = dict(os.environ, OMP_NUM_THREADS=t)
        outs.add(subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                                check=True).stdout)
    assert len(outs) == 1
