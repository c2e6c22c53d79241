"""Python binding of the C ABI in include/scd_gb300.h (libscd_gb300.so).

Mirrors the reference's GPU backend interface (src/cuda.hpp:23-28) one call per
function, plus the device-side preprocessing of `convert` and the full run
loop.  Every call goes straight to the CUDA library; there is no CPU path, and
constructing an Engine fails loudly when the library or a GPU is missing.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libscd_gb300.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "scd_gb300.h")
_LIB = None

OK = 0
ERRORS = {-1: "SCD_ERR_ARG", -2: "SCD_ERR_CUDA", -3: "SCD_ERR_OOM", -4: "SCD_ERR_STATE",
          -5: "SCD_ERR_FORMAT", -6: "SCD_ERR_TIMEOUT", -7: "SCD_ERR_LIMIT"}
INVALID_LABEL = 0xFFFFFFFF
FLAG_PROFILE, FLAG_PEXT_TREE, FLAG_NO_GRAPHS, FLAG_TC_OUT_ONLY, FLAG_PRIORITY, FLAG_TC_HASH = 1, 2, 4, 8, 16, 32
PHASES = ("parse", "convert", "tc", "partition", "improve", "stats", "wcc_tc", "wcc")


class ScdError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{ERRORS.get(status, status)}: {msg}")
        self.status = status


class Result(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("initial_wcc", ctypes.c_double),
                ("best_wcc", ctypes.c_double), ("initial_communities", ctypes.c_uint32),
                ("printed_communities", ctypes.c_uint32), ("distinct_communities", ctypes.c_uint32),
                ("ms_partition", ctypes.c_double), ("ms_iterations", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: the CUDA engine was not built "
                               "(run __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        u32, u64, i32, dbl = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_double
        sig = {
            "scd_create": ([ctypes.POINTER(P), i32, i32, ctypes.c_uint], i32),
            "scd_destroy": ([P], None),
            "scd_last_error": ([P], ctypes.c_char_p),
            "scd_convert_edges": ([P, P, u64, i32], i32),
            "scd_transfer_graph": ([P, u32, u32, P, P, P, P, dbl], i32),
            "scd_graph_info": ([P, ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(dbl)], i32),
            "scd_graph_download": ([P, P, P, P, P], i32),
            "scd_initial_partition": ([P, ctypes.POINTER(u32)], i32),
            "scd_labels_to_device": ([P, P], i32),
            "scd_compute_wcc": ([P, ctypes.POINTER(dbl)], i32),
            "scd_improve_labels": ([P, ctypes.POINTER(dbl)], i32),
            "scd_store_labels": ([P], i32),
            "scd_labels_from_device": ([P, P], i32),
            "scd_current_labels": ([P, P], i32),
            "scd_community_stats": ([P, P, P, P, ctypes.POINTER(u32)], i32),
            "scd_run": ([P, dbl, i32, P, ctypes.POINTER(Result)], i32),
            "scd_memory_usage": ([P, ctypes.POINTER(u64)], i32),
            "scd_kernel_launches": ([P, ctypes.POINTER(u64)], i32),
            "scd_stream": ([P, ctypes.POINTER(P)], i32),
            "scd_profile_get": ([P, ctypes.c_char_p, ctypes.POINTER(dbl), ctypes.POINTER(u64)], i32),
            "scd_profile_reset": ([P], i32),
            "scd_wcc_static": ([P, P, P, P, P, P, u32, dbl, P, P], i32),
            "scd_batch_convert": ([P, P, P, u32, i32], i32),
            "scd_batch_size": ([P, ctypes.POINTER(u32)], i32),
            "scd_batch_graph_info": ([P, u32, ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(dbl)], i32),
            "scd_batch_graph_download": ([P, u32, P, P, P, P], i32),
            "scd_batch_run": ([P, dbl, i32, P], i32),
            "scd_batch_labels": ([P, u32, P], i32),
            "scd_batch_convert_lists": ([P, P, P, u32], i32),
            "scd_convert_text": ([P, ctypes.c_char_p, u64, i32], i32),
            "scd_compressed_labels": ([P, P, ctypes.POINTER(u32)], i32),
            "scd_parse_text": ([P, ctypes.c_char_p, u64, i32, P, ctypes.POINTER(u64)], i32),
            "scd_batch_labels_all": ([P, P, P], i32),
            "scd_autotune": ([P, ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(dbl),
                              ctypes.c_char_p, u64], i32),
            "scd_load_graph_file": ([P, ctypes.c_char_p, dbl], i32),
            "scd_transfer_graph_bytes": ([P, ctypes.c_char_p, u64, dbl], i32),
            "scd_set_memory_limit": ([P, u64], i32),
            "scd_resident_init": ([P, dbl, i32], i32),
            "scd_resident_add": ([P, P, P], i32),
            "scd_resident_step": ([P, ctypes.POINTER(u32), ctypes.POINTER(u32)], i32),
            "scd_resident_take": ([P, u32, P, P, P, P, u64, P, ctypes.POINTER(u32)], i32),
            "scd_resident_info": ([P, ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(u32),
                                   ctypes.POINTER(u64), ctypes.POINTER(u64), ctypes.POINTER(u64)], i32),
            "scd_resident_timing": ([P, ctypes.POINTER(dbl), ctypes.POINTER(dbl), ctypes.POINTER(dbl),
                                     ctypes.POINTER(u64)], i32),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


def chosen_in_list_min(report, small_max, warp_max, cta_max):
    """The in-list split of the autotuner's choice: not an ABI output, it is read from the
    report line (the fastest among the lines of the chosen three splits)."""
    head = f"small<={small_max} warp<={warp_max} cta<={cta_max} in-list>"
    lines = [ln for ln in report if ln.startswith(head)]
    if not lines:
        return None
    best = min(lines, key=lambda ln: float(ln.rsplit(":", 1)[1].split()[0]))
    return int(best[len(head):].split(":")[0])


def header_symbols():
    """Names of the functions include/scd_gb300.h declares."""
    import re
    text = open(HEADER_PATH).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(scd_\w+)\s*\(", text, re.M)))


def _p(a):
    return None if a is None else a.ctypes.data


class Engine:
    """One SCD context (one graph) on one GPU."""

    def __init__(self, device=0, work_group_size=256, flags=0):
        self._ctx = ctypes.c_void_p()
        rc = lib().scd_create(ctypes.byref(self._ctx), device, work_group_size, flags)
        if rc != OK:
            raise ScdError(rc, f"cannot open CUDA device {device}")

    def _check(self, rc):
        if rc != OK:
            raise ScdError(rc, lib().scd_last_error(self._ctx).decode())

    def close(self):
        if self._ctx:
            lib().scd_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- graph -------------------------------------------------------------
    def convert_edges(self, pairs=None, device_ptr=None, count=None):
        """Device preprocessing (convert) of (min,max) pairs in file order."""
        if device_ptr is not None:
            self._check(lib().scd_convert_edges(self._ctx, device_ptr, count, 1))
            return
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        self._check(lib().scd_convert_edges(self._ctx, _p(pairs), pairs.shape[0], 0))

    def convert_text(self, text):
        """Device parse of an edge-list text (bytes) and device preprocessing."""
        text = bytes(text)
        self._check(lib().scd_convert_text(self._ctx, text, len(text), 0))

    def parse_text(self, text):
        """The (min, max) records of an edge-list text, parsed on the device."""
        text = bytes(text)
        cnt = ctypes.c_uint64()
        self._check(lib().scd_parse_text(self._ctx, text, len(text), 0, None, ctypes.byref(cnt)))
        out = np.empty((max(cnt.value, 1), 2), np.uint32)
        self._check(lib().scd_parse_text(self._ctx, text, len(text), 0, _p(out), ctypes.byref(cnt)))
        return out[: cnt.value]

    def transfer_graph(self, g, alpha=1.0):
        arrs = [np.ascontiguousarray(getattr(g, k), dtype=t) for k, t in
                (("indices", np.uint32), ("adj", np.uint32), ("tri", np.int32), ("tri_deg", np.int32))]
        self._check(lib().scd_transfer_graph(self._ctx, g.n, g.m, *[_p(a) for a in arrs], alpha))

    def load_graph_file(self, path, alpha=1.0):
        """A binary-format graph file straight to the device (pinned pieces)."""
        self._check(lib().scd_load_graph_file(self._ctx, os.fsencode(path), alpha))

    def transfer_graph_bytes(self, data, alpha=1.0):
        """A graph file's full contents (bytes) to the device."""
        self._check(lib().scd_transfer_graph_bytes(self._ctx, bytes(data), len(data), alpha))

    def graph_info(self):
        n, m, cc = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
        self._check(lib().scd_graph_info(self._ctx, ctypes.byref(n), ctypes.byref(m), ctypes.byref(cc)))
        return n.value, m.value, cc.value

    def graph_download(self):
        n, m, _ = self.graph_info()
        ind = np.empty(n + 1, np.uint32)
        adj = np.empty(2 * m, np.uint32)
        tri = np.empty(n, np.int32)
        tdg = np.empty(n, np.int32)
        self._check(lib().scd_graph_download(self._ctx, _p(ind), _p(adj), _p(tri), _p(tdg)))
        return dict(n=n, m=m, indices=ind, adj=adj, tri=tri, tri_deg=tdg)

    def graph_bytes(self):
        d = self.graph_download()
        hdr = np.array([d["n"], d["m"]], np.uint32)
        return b"".join(a.tobytes() for a in (hdr, d["indices"], d["adj"], d["tri"], d["tri_deg"]))

    # --- partition ----------------------------------------------------------
    def initial_partition(self):
        nc = ctypes.c_uint32()
        self._check(lib().scd_initial_partition(self._ctx, ctypes.byref(nc)))
        return nc.value

    def labels_to_device(self, labels):
        labels = np.ascontiguousarray(labels, dtype=np.uint32)
        self._check(lib().scd_labels_to_device(self._ctx, _p(labels)))

    def compute_wcc(self):
        w = ctypes.c_double()
        self._check(lib().scd_compute_wcc(self._ctx, ctypes.byref(w)))
        return w.value

    def improve_labels(self):
        w = ctypes.c_double()
        self._check(lib().scd_improve_labels(self._ctx, ctypes.byref(w)))
        return w.value

    def store_labels(self):
        self._check(lib().scd_store_labels(self._ctx))

    def labels_from_device(self):
        n = self.graph_info()[0]
        out = np.empty(n, np.uint32)
        self._check(lib().scd_labels_from_device(self._ctx, _p(out)))
        return out

    def compressed_labels(self):
        """The best labels renumbered as compress_labels intends; returns (labels, count)."""
        n = self.graph_info()[0]
        out = np.empty(max(n, 1), np.uint32)
        k = ctypes.c_uint32()
        self._check(lib().scd_compressed_labels(self._ctx, _p(out), ctypes.byref(k)))
        return out[:n], k.value

    def current_labels(self):
        n = self.graph_info()[0]
        out = np.empty(n, np.uint32)
        self._check(lib().scd_current_labels(self._ctx, _p(out)))
        return out

    def community_stats(self):
        nc = ctypes.c_uint32()
        self._check(lib().scd_community_stats(self._ctx, None, None, None, ctypes.byref(nc)))
        k = nc.value
        s, e, i = (np.empty(max(k, 1), np.int32) for _ in range(3))
        self._check(lib().scd_community_stats(self._ctx, _p(s), _p(e), _p(i), ctypes.byref(nc)))
        return s[:k], e[:k], i[:k]

    def run(self, threshold=0.01, max_iters=1000):
        trace = np.zeros(max_iters, np.float64)
        r = Result()
        self._check(lib().scd_run(self._ctx, threshold, max_iters, _p(trace), ctypes.byref(r)))
        d = r.as_dict()
        d["wcc"] = trace[: r.iterations].copy()
        return d

    def set_memory_limit(self, nbytes):
        self._check(lib().scd_set_memory_limit(self._ctx, int(nbytes)))

    def memory_usage(self):
        b = ctypes.c_uint64()
        self._check(lib().scd_memory_usage(self._ctx, ctypes.byref(b)))
        return b.value

    # --- batches -------------------------------------------------------------
    def batch_convert(self, graphs):
        """Device preprocessing of a list of edge lists ((E_g, 2) uint32 each)."""
        arrs = [np.ascontiguousarray(p, dtype=np.uint32).reshape(-1, 2) for p in graphs]
        ptrs = (ctypes.c_void_p * max(len(arrs), 1))(*[a.ctypes.data for a in arrs])
        counts = np.array([a.shape[0] for a in arrs], np.uint64)
        self._check(lib().scd_batch_convert_lists(self._ctx, ptrs, _p(counts), len(arrs)))

    def batch_convert_device(self, dev_ptr, record_offsets):
        off = np.ascontiguousarray(record_offsets, dtype=np.uint64)
        self._check(lib().scd_batch_convert(self._ctx, dev_ptr, _p(off), len(off) - 1, 1))

    def batch_size(self):
        g = ctypes.c_uint32()
        self._check(lib().scd_batch_size(self._ctx, ctypes.byref(g)))
        return g.value

    def batch_graph_info(self, g):
        n, m, cc = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
        self._check(lib().scd_batch_graph_info(self._ctx, g, ctypes.byref(n), ctypes.byref(m), ctypes.byref(cc)))
        return n.value, m.value, cc.value

    def batch_graph_bytes(self, g):
        n, m, _ = self.batch_graph_info(g)
        ind = np.empty(n + 1, np.uint32)
        adj = np.empty(max(2 * m, 1), np.uint32)
        tri = np.empty(max(n, 1), np.int32)
        tdg = np.empty(max(n, 1), np.int32)
        self._check(lib().scd_batch_graph_download(self._ctx, g, _p(ind), _p(adj), _p(tri), _p(tdg)))
        hdr = np.array([n, m], np.uint32)
        return b"".join(a.tobytes() for a in (hdr, ind, adj[: 2 * m], tri[:n], tdg[:n]))

    def batch_run(self, threshold=0.01, max_iters=1000):
        G = self.batch_size()
        res = (Result * G)()
        rc = lib().scd_batch_run(self._ctx, threshold, max_iters, res)
        if rc not in (OK, -7):
            self._check(rc)
        return [r.as_dict() for r in res], rc

    def batch_labels(self, g):
        n = self.batch_graph_info(g)[0]
        out = np.empty(max(n, 1), np.uint32)
        self._check(lib().scd_batch_labels(self._ctx, g, _p(out)))
        return out[:n]

    def batch_labels_all(self, out=None):
        """Best labels of every graph (own numbering), one array per graph; out
        (optional): a uint32 array of at least the batch's vertex count to copy
        into (pinned memory makes the copy a plain DMA)."""
        G = self.batch_size()
        off = np.zeros(G + 1, np.uint64)
        self._check(lib().scd_batch_labels_all(self._ctx, None, _p(off)))
        if out is None or out.size < int(off[-1]):
            out = np.empty(max(int(off[-1]), 1), np.uint32)
        self._check(lib().scd_batch_labels_all(self._ctx, _p(out), None))
        return [out[int(off[g]):int(off[g + 1])] for g in range(G)]

    def autotune(self):
        sm, w, c, ms = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
        buf = ctypes.create_string_buffer(8192)
        self._check(lib().scd_autotune(self._ctx, ctypes.byref(sm), ctypes.byref(w), ctypes.byref(c),
                                       ctypes.byref(ms), buf, 8192))
        report = buf.value.decode().splitlines()
        return dict(small_max=sm.value, warp_max=w.value, cta_max=c.value,
                    in_list_min=chosen_in_list_min(report, sm.value, w.value, c.value), best_ms=ms.value,
                    report=report)

    def stream(self):
        p = ctypes.c_void_p()
        self._check(lib().scd_stream(self._ctx, ctypes.byref(p)))
        return p.value

    def profile(self, phase):
        ms, cnt = ctypes.c_double(), ctypes.c_uint64()
        self._check(lib().scd_profile_get(self._ctx, phase.encode(), ctypes.byref(ms), ctypes.byref(cnt)))
        return ms.value, cnt.value

    def profile_reset(self):
        self._check(lib().scd_profile_reset(self._ctx))

    # --- resident set (continuous batching) ---------------------------------
    def resident_init(self, threshold=0.01, max_iters=1000):
        """Makes this engine an empty resident set (scd_resident_init)."""
        self._check(lib().scd_resident_init(self._ctx, threshold, max_iters))

    def resident_add(self, src):
        """Moves every graph resident in engine `src` into this set; returns their ids."""
        G = src.batch_size() if src.has_graph() else 0
        ids = np.zeros(max(G, 1), np.uint64)
        self._check(lib().scd_resident_add(self._ctx, src._ctx, _p(ids)))
        return [int(i) for i in ids[:G]]

    def resident_step(self):
        """One iteration of every running graph (graphs waiting to join are merged
        in first); returns (graphs that iterated, graphs that stopped in this step)."""
        run, fin = ctypes.c_uint32(), ctypes.c_uint32()
        self._check(lib().scd_resident_step(self._ctx, ctypes.byref(run), ctypes.byref(fin)))
        return run.value, fin.value

    def resident_take(self, cap=1 << 16, labels_cap=1 << 26):
        """Stopped graphs with their results: a list of (id, result dict, status, labels)."""
        ids = np.zeros(cap, np.uint64)
        res = (Result * cap)()
        status = np.zeros(cap, np.int32)
        labels = np.empty(max(labels_cap, 1), np.uint32)
        off = np.zeros(cap + 1, np.uint64)
        cnt = ctypes.c_uint32()
        self._check(lib().scd_resident_take(self._ctx, cap, _p(ids), res, _p(status), _p(labels), labels_cap,
                                            _p(off), ctypes.byref(cnt)))
        return [(int(ids[k]), res[k].as_dict(), int(status[k]), labels[int(off[k]):int(off[k + 1])].copy())
                for k in range(cnt.value)]

    def resident_info(self):
        g, r, p = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        st, gs, kp = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        self._check(lib().scd_resident_info(self._ctx, ctypes.byref(g), ctypes.byref(r), ctypes.byref(p),
                                            ctypes.byref(st), ctypes.byref(gs), ctypes.byref(kp)))
        return dict(graphs=g.value, running=r.value, pending=p.value, steps=st.value, graph_steps=gs.value,
                    kernels_per_step=kp.value)

    def resident_timing(self):
        a, b, c, r = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
        self._check(lib().scd_resident_timing(self._ctx, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                              ctypes.byref(r)))
        return dict(ms_steps=a.value, ms_rebuild=b.value, ms_capture=c.value, rebuilds=r.value)

    def has_graph(self):
        return lib().scd_batch_size(self._ctx, ctypes.byref(ctypes.c_uint32())) == OK

    def kernel_launches(self):
        b = ctypes.c_uint64()
        self._check(lib().scd_kernel_launches(self._ctx, ctypes.byref(b)))
        return b.value
