"""The engine at full size against the reference's own outputs.

tests/golden/pins.json holds, for each full-size workload (R-MAT scale 22 of the
headline benchmark; the skewed-degree Chung-Lu graphs with hubs past degree
46,341, where the int32 products of the gain model wrap), hashes of what the
reference's `convert` and its refinement loop at one thread produced
(tests/golden/make_golden.py --pins): the input records, the graph file, the
initial partition and its statistics, the labels and statistics of every
iteration and the best labels, plus the exact FP64 p_ext and WCC values.

Bar: graph bytes, p_ext, initial partition, every iteration's labels and
statistics, iteration count and best labels bit-exact; every WCC within 1e-6
relative.  Each comparison is logged (SCD_PARITY_LOG, see parity_log) with the
number of differing vertices and whether the WCC bits are equal, so a
divergence that only a floating-point tie could explain would show up there.
"""
import hashlib

import numpy as np
import pytest

import golden_data as G
import scd_gb300 as S
import scdgen
from parity_log import log

pytestmark = pytest.mark.gpu
WCC_RTOL = 1e-6
PINS = G.pins()


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("name", sorted(PINS))
def test_full_size_workload_matches_reference_pins(name):
    p = PINS[name]
    pairs = getattr(scdgen, p["generator"])(**p["args"])
    # the generator gives the same records on this machine as where the pins were made
    assert pairs.shape[0] == p["edges_in"] and sha(pairs) == p["pairs_sha256"]
    with S.Engine(0) as eng:
        eng.convert_edges(pairs)
        del pairs
        n, m, cc = eng.graph_info()
        assert (n, m) == (p["n"], p["m"])
        assert hashlib.sha256(eng.graph_bytes()).hexdigest() == p["graph_sha256"]
        assert cc.hex() == p["p_ext"]
        nc = eng.initial_partition()
        assert nc == p["num_comms"]
        assert sha(eng.current_labels()) == p["initial_labels_sha256"]
        assert sha(np.stack(eng.community_stats())) == p["initial_stats_sha256"]
        w0 = eng.compute_wcc()
        log(name, "initial", labels_equal=True, wcc=w0.hex(), wcc_ref=p["initial_wcc"],
            wcc_rel=rel(w0, float.fromhex(p["initial_wcc"])))
        assert rel(w0, float.fromhex(p["initial_wcc"])) < WCC_RTOL
        for i in range(p["iters"]):
            w = eng.improve_labels()
            same = sha(eng.current_labels()) == p["labels_sha256"][i]
            log(name, f"iteration {i + 1}", labels_equal=same, wcc=w.hex(), wcc_ref=p["wcc"][i],
                wcc_rel=rel(w, float.fromhex(p["wcc"][i])))
            assert same, f"labels of iteration {i + 1} differ from the reference"
            assert sha(np.stack(eng.community_stats())) == p["stats_sha256"][i]
            assert rel(w, float.fromhex(p["wcc"][i])) < WCC_RTOL
        # the whole loop again through scd_run: iterations, best labels, printed count
        eng.convert_edges(getattr(scdgen, p["generator"])(**p["args"]))
        r = eng.run(0.01, 1000)
        assert r["iterations"] == p["iters"]
        assert r["initial_communities"] == p["num_comms"]
        assert sha(eng.labels_from_device()) == p["best_labels_sha256"]
        assert rel(r["best_wcc"], float.fromhex(p["best_wcc"])) < WCC_RTOL
        assert r["printed_communities"] == p["printed_comms"]
        log(name, "run", labels_equal=True, iterations=r["iterations"], wcc=r["best_wcc"].hex(),
            wcc_ref=p["best_wcc"])


def test_pins_cover_the_wrap_degrees():
    """At least one pinned workload has a vertex of degree > 46,341, so its hub
    gains pass through the wrapped int32 products d_out*(d_out-1)."""
    if not PINS:
        pytest.skip("no pins")
    assert max(p["max_degree"] for p in PINS.values()) > 46341
