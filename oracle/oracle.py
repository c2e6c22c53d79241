"""ctypes binding of the oracle (oracle/scd_oracle.cpp) and a reader for the
reference traces written by oracle/ref_driver.cpp.

Test infrastructure only: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, always as the checker or the timed CPU baseline,
never as the thing measured or shipped.
"""
import ctypes
import gzip
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
U32P = ctypes.POINTER(ctypes.c_uint32)
I32P = ctypes.POINTER(ctypes.c_int32)
F64P = ctypes.POINTER(ctypes.c_double)


class _Graph(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("m", ctypes.c_uint32), ("indices", U32P),
                ("adj", U32P), ("tri", I32P), ("tri_deg", I32P)]


class Times(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in (
        "process_graph", "tc", "initial_partition", "initial_wcc", "iterations",
        "improve", "stats", "wcc")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(path)
        GP = ctypes.POINTER(_Graph)
        L.orc_convert.argtypes = [ctypes.c_void_p, ctypes.c_int64, GP, ctypes.POINTER(Times)]
        L.orc_read_text.argtypes = [ctypes.c_char_p, ctypes.POINTER(U32P),
                                    ctypes.POINTER(ctypes.c_int64), U32P]
        L.orc_write_graph.argtypes = [ctypes.c_char_p, GP]
        L.orc_read_graph.argtypes = [ctypes.c_char_p, GP]
        L.orc_free_graph.argtypes = [GP]
        L.orc_clustering_coef.argtypes = [GP]
        L.orc_clustering_coef.restype = ctypes.c_double
        L.orc_initial_partition.argtypes = [GP, ctypes.c_void_p]
        L.orc_initial_partition.restype = ctypes.c_uint32
        L.orc_collect_stats.argtypes = [GP, ctypes.c_void_p, ctypes.c_uint32,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_gain.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double] * 3
        L.orc_gain.restype = ctypes.c_double
        L.orc_improve.argtypes = [GP, ctypes.c_double, ctypes.c_double] + [ctypes.c_void_p] * 5
        L.orc_wcc.argtypes = [GP, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_wcc.restype = ctypes.c_double
        L.orc_compress_labels.argtypes = [ctypes.c_uint32, ctypes.c_void_p]
        L.orc_compress_labels.restype = ctypes.c_uint32
        L.orc_run.argtypes = [GP, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                              ctypes.c_void_p, F64P, U32P, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p, F64P, U32P, ctypes.POINTER(Times)]
        L.orc_run.restype = ctypes.c_int
        L.orc_free.argtypes = [ctypes.c_void_p]
        L.orc_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def _ptr(a):
    return a.ctypes.data if a is not None else None


class Graph:
    """CSR graph in the binary-format layout (src/graph.hpp:23-62)."""

    def __init__(self, n, m, indices, adj, tri, tri_deg):
        self.n, self.m = int(n), int(m)
        self.indices = np.ascontiguousarray(indices, dtype=np.uint32)
        self.adj = np.ascontiguousarray(adj, dtype=np.uint32)
        self.tri = np.ascontiguousarray(tri, dtype=np.int32)
        self.tri_deg = np.ascontiguousarray(tri_deg, dtype=np.int32)

    def _c(self):
        g = _Graph(self.n, self.m, self.indices.ctypes.data_as(U32P), self.adj.ctypes.data_as(U32P),
                   self.tri.ctypes.data_as(I32P), self.tri_deg.ctypes.data_as(I32P))
        g._keep = self
        return g

    @staticmethod
    def _from_c(g):
        n, m = g.n, g.m
        take = lambda p, k, dt: np.ctypeslib.as_array(p, shape=(max(k, 1),))[:k].astype(dt, copy=True)
        out = Graph(n, m, take(g.indices, n + 1, np.uint32), take(g.adj, 2 * m, np.uint32),
                    take(g.tri, n, np.int32), take(g.tri_deg, n, np.int32))
        lib().orc_free_graph(ctypes.byref(g))
        return out

    def to_bytes(self):
        hdr = np.array([self.n, self.m], dtype=np.uint32)
        return b"".join(a.tobytes() for a in (hdr, self.indices, self.adj, self.tri, self.tri_deg))

    @staticmethod
    def from_bytes(buf):
        hdr = np.frombuffer(buf, dtype=np.uint32, count=2)
        n, m = int(hdr[0]), int(hdr[1])
        want = 8 + 4 * (n + 1) + 8 * m + 8 * n
        if len(buf) != want:
            raise ValueError(f"graph file has {len(buf)} bytes, expected {want}")
        o = 8
        ind = np.frombuffer(buf, np.uint32, n + 1, o); o += 4 * (n + 1)
        adj = np.frombuffer(buf, np.uint32, 2 * m, o); o += 8 * m
        tri = np.frombuffer(buf, np.int32, n, o); o += 4 * n
        tdg = np.frombuffer(buf, np.int32, n, o)
        return Graph(n, m, ind, adj, tri, tdg)

    def degrees(self):
        return np.diff(self.indices.astype(np.int64))


def convert(pairs):
    """Oracle `convert` (src/convert.cpp:141-463) of (min,max) pairs in file order."""
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
    g = _Graph()
    t = Times()
    rc = lib().orc_convert(pairs.ctypes.data, pairs.shape[0], ctypes.byref(g), ctypes.byref(t))
    if rc != 0:
        raise RuntimeError("oracle convert failed")
    return Graph._from_c(g), t.as_dict()


def read_text(path):
    p = U32P()
    cnt = ctypes.c_int64()
    nn = ctypes.c_uint32()
    rc = lib().orc_read_text(os.fsencode(path), ctypes.byref(p), ctypes.byref(cnt), ctypes.byref(nn))
    if rc != 0:
        raise ValueError(f"read_text failed ({rc})")
    k = cnt.value
    arr = np.ctypeslib.as_array(p, shape=(max(2 * k, 1),))[: 2 * k].copy().reshape(k, 2)
    lib().orc_free(p)
    return arr


def clustering_coef(g):
    return lib().orc_clustering_coef(ctypes.byref(g._c()))


def initial_partition(g):
    labels = np.empty(g.n, dtype=np.uint32)
    nc = lib().orc_initial_partition(ctypes.byref(g._c()), _ptr(labels))
    return labels, int(nc)


def collect_stats(g, labels, nc):
    s = np.empty(max(nc, 1), np.int32); e = np.empty_like(s); i = np.empty_like(s)
    lib().orc_collect_stats(ctypes.byref(g._c()), _ptr(np.ascontiguousarray(labels, np.uint32)),
                            nc, _ptr(s), _ptr(e), _ptr(i))
    return s[:nc], e[:nc], i[:nc]


def gain(r, d_in, d_out, c_out, p_in, p_ext, alpha=1.0):
    return lib().orc_gain(r, d_in, d_out, c_out, p_in, p_ext, alpha)


def improve(g, p_ext, labels, sizes, ext, intl, alpha=1.0):
    out = np.empty(g.n, np.uint32)
    c = lambda a, dt: np.ascontiguousarray(a, dtype=dt)
    lib().orc_improve(ctypes.byref(g._c()), p_ext, alpha, _ptr(c(labels, np.uint32)),
                      _ptr(c(sizes, np.int32)), _ptr(c(ext, np.int32)), _ptr(c(intl, np.int32)),
                      _ptr(out))
    return out


def wcc(g, labels, sizes, alpha=1.0, per_vertex=False):
    pv = np.empty(g.n, np.float64) if per_vertex else None
    w = lib().orc_wcc(ctypes.byref(g._c()), alpha, _ptr(np.ascontiguousarray(labels, np.uint32)),
                      _ptr(np.ascontiguousarray(sizes, np.int32)), _ptr(pv))
    return (w, pv) if per_vertex else w


def compress_labels(labels):
    lab = np.array(labels, dtype=np.uint32, copy=True)
    cnt = lib().orc_compress_labels(lab.shape[0], _ptr(lab))
    return int(cnt), lab


def run(g, max_iters=200, alpha=1.0, threshold=0.01, keep_trace=True):
    """Oracle refinement loop (src/main.cpp:35-93)."""
    n = g.n
    lab0 = np.empty(n, np.uint32)
    tl = np.empty((max_iters, n), np.uint32) if keep_trace else None
    tw = np.empty(max_iters, np.float64)
    best = np.empty(n, np.uint32)
    w0, bw = ctypes.c_double(), ctypes.c_double()
    nc, pc = ctypes.c_uint32(), ctypes.c_uint32()
    t = Times()
    it = lib().orc_run(ctypes.byref(g._c()), alpha, threshold, max_iters, _ptr(lab0), ctypes.byref(w0),
                       ctypes.byref(nc), _ptr(tl), _ptr(tw), _ptr(best), ctypes.byref(bw),
                       ctypes.byref(pc), ctypes.byref(t))
    k = it if it >= 0 else max_iters
    return dict(iters=it, initial_labels=lab0, initial_wcc=w0.value, num_comms=nc.value,
                labels=(tl[:k] if keep_trace else None), wcc=tw[:k].copy(), best_labels=best,
                best_wcc=bw.value, printed_comms=pc.value, times=t.as_dict())


def run_from_labels(g, labels, max_iters=200, alpha=1.0, threshold=0.01):
    """The refinement loop of src/main.cpp:60-82 started from a given labelling
    (num_communities = largest label + 1, statistics by collect_stats), built
    from the oracle's collect_stats / improve / wcc restatements."""
    lab = np.ascontiguousarray(labels, np.uint32).copy()
    valid = lab[lab != 0xFFFFFFFF]
    nc = int(valid.max()) + 1 if valid.size else 0
    p_ext = clustering_coef(g)
    st = collect_stats(g, lab, nc)
    w0 = wcc(g, lab, st[0], alpha)
    best_wcc, best = w0, lab.copy()
    labs, wccs = [], []
    it = 0
    while it < max_iters:
        it += 1
        lab = improve(g, p_ext, lab, *st, alpha=alpha)
        st = collect_stats(g, lab, nc)
        w = wcc(g, lab, st[0], alpha)
        if w > best_wcc:
            best = lab.copy()
        labs.append(lab.copy())
        wccs.append(w)
        if w < best_wcc * (1 + threshold):
            break
        best_wcc = w
    printed, _ = compress_labels(best)
    return dict(iters=it, initial_labels=np.ascontiguousarray(labels, np.uint32), initial_wcc=w0, num_comms=nc,
                labels=labs, wcc=wccs, best_labels=best, best_wcc=best_wcc, printed_comms=printed)


def threads():
    return lib().orc_threads()


def read_trace(path):
    """Reads a trace written by oracle/ref_driver.cpp (optionally gzip-compressed)."""
    op = gzip.open if path.endswith(".gz") else open
    with op(path, "rb") as f:
        buf = f.read()
    if buf[:8] != b"SCDTRACE":
        raise ValueError("not a trace")
    o = 8
    n, m, nc, iters = np.frombuffer(buf, np.uint32, 4, o).tolist(); o += 16
    pext, wcc0, best_wcc = np.frombuffer(buf, np.float64, 3, o).tolist(); o += 24
    printed = int(np.frombuffer(buf, np.uint32, 1, o)[0]); o += 4
    lab0 = np.frombuffer(buf, np.uint32, n, o); o += 4 * n
    st0 = np.frombuffer(buf, np.int32, 3 * nc, o).reshape(3, nc); o += 12 * nc
    wccs, labs, stats = [], [], []
    for _ in range(iters):
        wccs.append(float(np.frombuffer(buf, np.float64, 1, o)[0])); o += 8
        labs.append(np.frombuffer(buf, np.uint32, n, o)); o += 4 * n
        stats.append(np.frombuffer(buf, np.int32, 3 * nc, o).reshape(3, nc)); o += 12 * nc
    best = np.frombuffer(buf, np.uint32, n, o); o += 4 * n
    assert o == len(buf), "trailing bytes in trace"
    return dict(n=n, m=m, num_comms=nc, iters=iters, p_ext=pext, initial_wcc=wcc0,
                best_wcc=best_wcc, printed_comms=printed, initial_labels=lab0,
                initial_stats=st0, wcc=wccs, labels=labs, stats=stats, best_labels=best)
