"""Loader for the golden fixtures (reference outputs) in tests/golden."""
import gzip
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def cases():
    return sorted(manifest().keys())


def pairs(name):
    with gzip.open(os.path.join(GOLDEN, name + ".pairs.npy.gz"), "rb") as f:
        return np.load(f)


def graph_bytes(name):
    with gzip.open(os.path.join(GOLDEN, name + ".graph.gz"), "rb") as f:
        return f.read()


def trace(name):
    import oracle
    p = os.path.join(GOLDEN, name + ".trace.gz")
    return oracle.read_trace(p) if os.path.exists(p) else None
