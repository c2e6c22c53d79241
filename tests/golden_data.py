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


def starts_from_labels(name):
    """True if the case's trace starts from a given labelling (start_labels)
    instead of the reference's initial partition."""
    return bool(manifest()[name].get("start_labels"))


def partition_cases():
    """Cases whose trace starts from the initial partition (or that have none)."""
    return [c for c in cases() if not starts_from_labels(c)]


def start_labels(name):
    with gzip.open(os.path.join(GOLDEN, name + ".labels.npy.gz"), "rb") as f:
        return np.load(f)


def pins():
    """Compact pins of the full-size workloads (tests/golden/pins.json)."""
    p = os.path.join(GOLDEN, "pins.json")
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f)
