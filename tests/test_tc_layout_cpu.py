"""CPU checks of the facts the preprocessing kernels rest on (no GPU).

The core-bitmap triangle count (triangles.cu, k_tc_core) holds a centre's
out-list in a bitmap over the vertices of degree > T and ranks a member by a
per-word prefix plus a popcount; the ranking of the kept vertices
(preprocess.cu, k_kept_keys) sorts only the vertices that keep an edge, on
keys as wide as the largest tri_deg needs.  These tests restate each fact with
numpy on seeded graphs, so a change of the orientation rule or of the key
layout that breaks one fails here before it can reach the device.
"""
import numpy as np
import pytest

import scdgen


def _oriented(pairs):
    """Degree orientation of the de-duplicated graph as the preprocessing uses it:
    u -> v iff (deg v, v) > (deg u, u)."""
    u = pairs[:, 0].astype(np.int64)
    v = pairs[:, 1].astype(np.int64)
    n = int(pairs.max()) + 1
    deg = np.bincount(np.concatenate([u, v]), minlength=n)
    fwd = (deg[v] > deg[u]) | ((deg[v] == deg[u]) & (v > u))
    src = np.where(fwd, u, v)
    dst = np.where(fwd, v, u)
    return n, deg, src, dst


GRAPHS = [
    ("rmat14", lambda: scdgen.rmat(14, 16, seed=3)),
    ("chunglu30k", lambda: scdgen.chunglu(30_000, 2.1, 5.0, 3000.0, 0.2, 10, 200, seed=4)),
    ("planted8k", lambda: scdgen.planted(8_000, 30.0, 0.3, 20, 400, seed=5)),
]


@pytest.mark.parametrize("kind,make", GRAPHS, ids=[k for k, _ in GRAPHS])
@pytest.mark.parametrize("t", [64, 128, 256])
def test_out_lists_of_long_centres_lie_in_the_core(kind, make, t):
    # a centre of out-degree > t has degree > t, and each of its out-neighbours
    # has a degree at least its own: the whole out-list lies in {deg > t}
    n, deg, src, dst = _oriented(make())
    dplus = np.bincount(src, minlength=n)
    centre = dplus[src] > t
    assert np.all(deg[dst[centre]] > t)


def test_popcount_rank_is_the_list_position():
    # core numbers ascend with ids, so a sorted out-list in core numbers is
    # ascending: position = pre[first member's word] + popcount below the bit
    rng = np.random.default_rng(8)
    for _ in range(50):
        core_n = int(rng.integers(100, 5000))
        lst = np.sort(rng.choice(core_n, size=int(rng.integers(1, min(core_n, 1100))), replace=False))
        words = core_n // 32 + 1
        bm = np.zeros(words, np.uint64)
        pre = np.zeros(words, np.int64)
        for i, c in enumerate(lst):
            w = c >> 5
            if i == 0 or (lst[i - 1] >> 5) != w:
                pre[w] = i
            bm[w] |= np.uint64(1) << np.uint64(c & 31)
        for i, c in enumerate(lst):
            w, b = c >> 5, c & 31
            below = int(bm[w]) & ((1 << b) - 1)
            assert pre[w] + bin(below).count("1") == i


@pytest.mark.parametrize("seed", range(5))
def test_ranking_only_the_kept_vertices_keeps_their_order(seed):
    # all vertices on ((2^32-1 - tri_deg) << k) | (2^k-1 - v), or only those with
    # tri_deg > 0 on ((maxd - tri_deg) << k) | (2^k-1 - v): the kept vertices come
    # out in the same order (tri_deg 0 sorts after every kept vertex)
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1000, 20000))
    tri_deg = rng.integers(0, 300, n) * (rng.random(n) < 0.7)
    k = max(1, int(np.ceil(np.log2(max(n, 2)))))
    v = np.arange(n, dtype=np.uint64)
    vmax = np.uint64((1 << k) - 1)
    full = (np.uint64(0xFFFFFFFF) - tri_deg.astype(np.uint64)) << np.uint64(k) | (vmax - v)
    order_full = np.argsort(full, kind="stable")
    kept_full = order_full[tri_deg[order_full] > 0]
    kept = np.nonzero(tri_deg > 0)[0]
    maxd = np.uint64(tri_deg.max())
    narrow = (maxd - tri_deg[kept].astype(np.uint64)) << np.uint64(k) | (vmax - kept.astype(np.uint64))
    bits = k + int(np.ceil(np.log2(int(maxd) + 1)))
    assert int(narrow.max()) < (1 << bits)
    kept_narrow = kept[np.argsort(narrow, kind="stable")]
    assert np.array_equal(kept_full, kept_narrow)
