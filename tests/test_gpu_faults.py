"""Host-side failures on the GPU path, made without faulting the GPU: an allocation
that fails (a context memory cap stands in for a full device, SCD_ERR_OOM) and
the state the engine is left in afterwards."""
import numpy as np
import pytest

import golden_data as G
import scd_gb300 as S
import scdgen

pytestmark = pytest.mark.gpu


def test_memory_cap_fails_with_oom_and_the_context_recovers():
    pairs = G.pairs("planted_10k")
    with S.Engine(0) as e:
        e.set_memory_limit(1 << 20)              # the graph's arrays need more than 1 MB
        with pytest.raises(S.ScdError) as ex:
            e.convert_edges(pairs)
        assert ex.value.status == -3
        with pytest.raises(S.ScdError) as ex:    # nothing half-built is left to use
            e.initial_partition()
        assert ex.value.status == -4
        e.set_memory_limit(0)
        e.convert_edges(pairs)
        assert e.graph_bytes() == G.graph_bytes("planted_10k")
        r = e.run(0.01, 1000)
        assert r["iterations"] == G.manifest()["planted_10k"]["iters"]


def test_resident_set_over_its_cap_drops_its_graphs_and_stays_usable():
    a = scdgen.planted(5000, 14.0, 0.2, 20, 100, seed=61)
    b = scdgen.planted(60000, 14.0, 0.2, 20, 100, seed=62)
    with S.Engine(0) as rs, S.Engine(0) as stage:
        rs.resident_init(0.01, 1000)
        stage.convert_edges(a)
        rs.resident_add(stage)
        rs.resident_step()
        used = rs.memory_usage()
        rs.set_memory_limit(used + (1 << 20))    # room for a, not for a and b together
        stage.convert_edges(b)
        rs.resident_add(stage)
        with pytest.raises(S.ScdError) as ex:
            rs.resident_step()                   # merging b passes the cap
        assert ex.value.status == -3
        info = rs.resident_info()
        assert info["graphs"] == 0 and info["pending"] == 0 and rs.memory_usage() == 0
        rs.set_memory_limit(0)                   # usable again: a alone, same result as alone
        stage.convert_edges(a)
        [ia] = rs.resident_add(stage)
        out = []
        while not out:
            rs.resident_step()
            out = rs.resident_take()
        [(gid, res, st, lab)] = out
        assert gid == ia and st == 0
    with S.Engine(0) as e:
        e.convert_edges(a)
        r = e.run(0.01, 1000)
        assert r["iterations"] == res["iterations"] and r["best_wcc"] == res["best_wcc"]
        assert np.array_equal(e.labels_from_device(), lab)
