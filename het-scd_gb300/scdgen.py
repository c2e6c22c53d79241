"""Seeded synthetic graph generators (ctypes binding of gen/scdgen.c).

Every generator returns the undirected edge list as an (E, 2) uint32 array of
sorted, de-duplicated, self-loop-free pairs (u < v): the canonical text order
that the `convert` tool reads.  The graphs stand in for the reference's SNAP
inputs, which are not available offline; the named workloads below follow the
shapes the benchmark is quoted on.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "libscdgen.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} missing: run __graft_entry__.build() first")
        lib = ctypes.CDLL(path)
        p32 = ctypes.POINTER(ctypes.POINTER(ctypes.c_uint32))
        lib.scdgen_planted.argtypes = [ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, p32]
        lib.scdgen_planted.restype = ctypes.c_int64
        lib.scdgen_rmat.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_uint64, p32]
        lib.scdgen_rmat.restype = ctypes.c_int64
        lib.scdgen_chunglu.argtypes = [ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_uint64, p32]
        lib.scdgen_chunglu.restype = ctypes.c_int64
        lib.scdgen_free.argtypes = [ctypes.c_void_p]
        lib.scdgen_write_text.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64]
        lib.scdgen_write_text.restype = ctypes.c_int
        _LIB = lib
    return _LIB


def _take(fn, *args):
    out = ctypes.POINTER(ctypes.c_uint32)()
    count = fn(*args, ctypes.byref(out))
    if count < 0:
        raise RuntimeError("generator failed")
    arr = np.ctypeslib.as_array(out, shape=(max(count, 1) * 2,))[: count * 2].copy()
    _lib().scdgen_free(out)
    return arr.reshape(count, 2)


def planted(n, k_in=18.0, mu=0.1, smin=20, smax=100, seed=1):
    """Planted partition: communities with P(s) ∝ 1/s on [smin, smax], mean
    internal degree k_in (capped at s-1), n*k_in*mu/(1-mu)/2 uniform external edges."""
    return _take(_lib().scdgen_planted, n, float(k_in), float(mu), smin, smax, seed)


def rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=22):
    """R-MAT with 2^scale * edge_factor samples, symmetrised and de-duplicated."""
    return _take(_lib().scdgen_rmat, scale, edge_factor, a, b, c, seed)


def chunglu(n, gamma=2.1, wmin=5.0, wmax=200000.0, mu=0.2, smin=10, smax=500, seed=3):
    """Chung-Lu with power-law expected degrees and planted communities."""
    return _take(_lib().scdgen_chunglu, n, gamma, wmin, wmax, mu, smin, smax, seed)


def write_text(path, pairs):
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32)
    rc = _lib().scdgen_write_text(os.fsencode(path), pairs.ctypes.data, pairs.shape[0])
    if rc != 0:
        raise OSError(f"could not write {path}")


# The named workloads (sizes of the benchmark configurations).
def workload(name, **override):
    if name == "planted-10k":        # n=10,000, mean internal degree 18, mu=0.1
        return planted(10000, 18.0, 0.1, 20, 100, override.get("seed", 1))
    if name.startswith("rmat-"):     # rmat-22: scale 22, edge factor 16
        return rmat(int(name.split("-")[1]), 16, 0.57, 0.19, 0.19, override.get("seed", 22))
    if name == "chunglu-8m":         # 8M vertices, exponent 2.1 in [5, 200000], mu=0.2
        return chunglu(8_000_000, 2.1, 5.0, 200000.0, 0.2, 10, 500, override.get("seed", 3))
    raise KeyError(name)
