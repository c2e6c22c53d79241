"""scd_wcc_static: WCC without any device allocation by the library.

Some callers cannot let a library allocate device memory: a serving process
whose pool already holds the free HBM, a plugin host that accounts for every
allocation itself, or a loop that cannot take cudaFree's device-wide
synchronisation.  They own every buffer and call scd_wcc_static with device
pointers; its only scratch is a fixed array inside the library.

This file is collected last on purpose (other GPU tests run first in a run that
stops at the first failure).  It must pass alone in a fresh process and after
the other tests, so it builds all of its own state.
"""
import ctypes

import numpy as np
import pytest

import golden_data as G
import scd_gb300 as S

pytestmark = pytest.mark.gpu
RTOL = 1e-6   # the WCC tolerance of the parity tests


def _device(t, torch):
    return torch.from_numpy(np.ascontiguousarray(t)).cuda()


def _static_wcc(lib, torch, graph, labels, sizes, alpha=1.0):
    """Calls scd_wcc_static through the C ABI with caller-owned device buffers."""
    ind = _device(graph["indices"].view(np.int32), torch)
    adj = _device(graph["adj"].view(np.int32) if graph["adj"].size else np.zeros(1, np.int32), torch)
    tri = _device(graph["tri"], torch)
    tdg = _device(graph["tri_deg"], torch)
    lab = _device(labels.view(np.int32), torch)
    siz = _device(sizes if sizes.size else np.zeros(1, np.int32), torch)
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.scd_wcc_static(ind.data_ptr(), adj.data_ptr(), tri.data_ptr(), tdg.data_ptr(), lab.data_ptr(),
                            siz.data_ptr(), graph["n"], alpha, out.data_ptr(), stream)
    assert rc == S.OK, rc
    torch.cuda.synchronize()
    return float(out.item())


def _engine_pair(name):
    """The engine's WCC, labels and community sizes of the initial partition and
    of the first iteration of a golden case."""
    with S.Engine(0) as eng:
        eng.convert_edges(G.pairs(name))
        graph = eng.graph_download()
        eng.initial_partition()
        want = [eng.compute_wcc()]
        labels = [eng.current_labels()]
        sizes = [eng.community_stats()[0].copy()]
        want.append(eng.improve_labels())
        labels.append(eng.current_labels())
        sizes.append(eng.community_stats()[0].copy())
    return graph, want, labels, sizes


@pytest.mark.parametrize("name", ["planted_10k", "rmat_12", "chunglu_20k"])
def test_static_wcc_matches_engine_on_two_calls_in_a_row(name):
    """Same terms and the same summation order as scd_compute_wcc: equal bit for
    bit, on two calls in a row (the second sees the second labelling).  The
    R-MAT and Chung-Lu cases have hub rows; planted_10k ends in a partly full
    block of 2048 vertices."""
    torch = pytest.importorskip("torch")
    lib = S.lib()
    graph, want, labels, sizes = _engine_pair(name)
    got = [_static_wcc(lib, torch, graph, labels[k], sizes[k]) for k in range(2)]
    assert got == want, (got, want)
    assert abs(got[0] - want[0]) <= RTOL * abs(want[0])
    assert got[0] != got[1]


def test_static_wcc_skip_branches_match_engine():
    """A labelling with unlabelled vertices and communities of one and two
    vertices (the terms the reference skips: INVALID label, size <= 2)."""
    torch = pytest.importorskip("torch")
    lib = S.lib()
    with S.Engine(0) as eng:
        eng.convert_edges(G.pairs("planted_10k"))
        graph = eng.graph_download()
        eng.initial_partition()
        lab = eng.current_labels().copy()
        n = lab.size
        rng = np.random.default_rng(3)
        lab[rng.choice(n, n // 10, replace=False)] = S.INVALID_LABEL
        a, b = np.unique(lab[lab != S.INVALID_LABEL])[:2]   # two labels in use: a keeps 2 vertices, b one
        lab[(lab == a) | (lab == b)] = S.INVALID_LABEL
        lab[0] = lab[1] = a
        lab[2] = b
        eng.labels_to_device(lab)
        want = eng.compute_wcc()
        sizes = eng.community_stats()[0].copy()
    assert sizes[a] == 2 and sizes[b] == 1 and (lab == S.INVALID_LABEL).any()
    got = _static_wcc(lib, torch, graph, lab, sizes)
    assert got == want, (got, want)


def test_static_wcc_hubs_at_high_ids_match_engine():
    """Hub rows at ids beyond the first 131072 vertices (whose hub counts the
    library spreads over many CTAs) take the one-warp-per-vertex path: an R-MAT
    graph renumbered in reverse behind 100,000 isolated vertices puts its hubs
    there; the value still equals scd_compute_wcc's bit for bit."""
    torch = pytest.importorskip("torch")
    import oracle as O
    import scdgen
    lib = S.lib()
    with S.Engine(0) as eng:
        eng.convert_edges(scdgen.rmat(17, 16, seed=23))
        g = eng.graph_download()
    n0, pad = g["n"], 100000
    n = n0 + pad
    deg = np.diff(g["indices"].astype(np.int64))
    new_of = (n - 1 - np.arange(n0)).astype(np.uint32)          # old id v -> n-1-v: hubs last
    old_of = np.full(n, 0xFFFFFFFF, np.uint32)
    old_of[new_of] = np.arange(n0, dtype=np.uint32)
    ndeg = np.zeros(n, np.int64)
    ndeg[new_of] = deg
    ind = np.zeros(n + 1, np.uint32)
    ind[1:] = np.cumsum(ndeg)
    adj = np.empty_like(g["adj"])
    for v in range(n0):
        row = new_of[g["adj"][g["indices"][v]:g["indices"][v + 1]]]
        w = new_of[v]
        adj[ind[w]:ind[w + 1]] = np.sort(row)
    tri = np.zeros(n, np.int32)
    tdg = np.zeros(n, np.int32)
    tri[new_of] = g["tri"]
    tdg[new_of] = g["tri_deg"]
    assert int(new_of[0]) >= 131072 and deg[0] > 128            # the biggest hub lies beyond the hub slots
    graph = dict(n=n, m=g["m"], indices=ind, adj=adj, tri=tri, tri_deg=tdg)
    lab = np.full(n, S.INVALID_LABEL, np.uint32)
    lab[new_of] = (np.arange(n0) * 2654435761 % (n0 // 12)).astype(np.uint32)   # communities of ~12
    with S.Engine(0) as eng:
        eng.transfer_graph(O.Graph(n, g["m"], ind, adj, tri, tdg))
        eng.labels_to_device(lab)
        want = eng.compute_wcc()
        sizes = eng.community_stats()[0].copy()
    got = _static_wcc(lib, torch, graph, lab, sizes)
    assert got == want, (got, want)


def test_static_wcc_limits_and_arguments():
    lib = S.lib()
    dummy = ctypes.c_void_p(1)
    over = S.lib().scd_wcc_static(dummy, dummy, dummy, dummy, dummy, dummy, (1 << 24) + 1, 1.0, dummy, None)
    assert over == -7   # SCD_ERR_LIMIT, rejected before any GPU work
    assert lib.scd_wcc_static(None, None, None, None, None, None, 10, 1.0, None, None) == -1
