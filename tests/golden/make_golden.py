"""Generates the golden fixtures in this directory from the REFERENCE itself.

For every case: the input edge list (as the reference's read_edges stores it,
(min,max) pairs in file order), the binary graph written by the reference's
own `convert` (built unmodified from its sources by oracle/build_ref.sh), and
the trace of the reference's refinement loop (oracle/ref_driver.cpp linked
against the reference's graph.cpp/scd.cpp/wcc.cpp, OMP_NUM_THREADS=1).

Run in the development container, where the reference sources exist:
    python tests/golden/make_golden.py
"""
import gzip
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "het-scd_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
REF = os.path.join(ROOT, "oracle", "_ref")

# hand-written text inputs (edge-case coverage of the text parser and convert)
TEXT_CASES = {
    # one triangle plus a pendant vertex: n=3, m=3, tri=[2,2,2], tri_deg=[2,2,2]
    "triangle_pendant": "0 1\n1 2\n2 0\n2 3\n",
    # the example of the reference README: no triangle, so 0 vertices and 0 edges
    "readme_example": "1 2\n2 3\n3 5\n1 5\n",
    # comments, blank lines, leading blanks, reversed / repeated pairs, self-loops,
    # sparse large ids (renumbering by first appearance) and a two-triangle fan
    "messy_text": ("# comment line\n\n   7000000 12\n12 7000000\n12 12\n  99 12\n99 7000000\n"
                   "\t5 99\n5 12\n5 5\n5 7000000\n# trailing comment\n8 9\n9 10\n10 8\n10 8\n11 10\n"),
}


def generated_cases():
    import scdgen
    return {
        "planted_10k": scdgen.planted(10000, 18.0, 0.1, 20, 100, seed=1),    # the plain-SCD config
        "planted_2k_mu03": scdgen.planted(2000, 12.0, 0.3, 20, 100, seed=8),
        "planted_5k_mu04": scdgen.planted(5000, 20.0, 0.4, 20, 100, seed=9),
        "rmat_12": scdgen.rmat(12, 16, 0.57, 0.19, 0.19, seed=5),
        "chunglu_20k": scdgen.chunglu(20000, 2.1, 5.0, 2000.0, 0.2, 10, 500, seed=7),
    }


def text_to_pairs(text):
    import oracle as O
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write(text)
        p = f.name
    try:
        return O.read_text(p)
    finally:
        os.unlink(p)


def run_case(name, text_path, pairs, manifest, trace=True):
    import oracle as O
    gpath = os.path.join(HERE, name + ".graph")
    r = subprocess.run([os.path.join(REF, "convert"), text_path, gpath], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    graph = open(gpath, "rb").read()
    os.unlink(gpath)
    with gzip.open(gpath + ".gz", "wb", compresslevel=9) as f:
        f.write(graph)
    with gzip.open(os.path.join(HERE, name + ".pairs.npy.gz"), "wb", compresslevel=9) as f:
        np.save(f, pairs.astype(np.uint32))
    entry = {"edges_in": int(pairs.shape[0]), "graph_bytes": len(graph)}
    g = O.Graph.from_bytes(graph)
    entry.update(n=g.n, m=g.m)
    if trace and g.n > 0:
        tpath = os.path.join(HERE, name + ".trace")
        with tempfile.NamedTemporaryFile(suffix=".graph", delete=False) as f:
            f.write(graph)
            tmpg = f.name
        env = dict(os.environ, OMP_NUM_THREADS="1")
        r = subprocess.run([os.path.join(REF, "ref_driver"), tmpg, tpath, "1000"], capture_output=True,
                           text=True, env=env)
        os.unlink(tmpg)
        if r.returncode != 0:
            raise RuntimeError(r.stderr)
        raw = open(tpath, "rb").read()
        os.unlink(tpath)
        with gzip.open(tpath + ".gz", "wb", compresslevel=9) as f:
            f.write(raw)
        tr = O.read_trace(tpath + ".gz")
        entry.update(iters=tr["iters"], num_comms=tr["num_comms"], p_ext=tr["p_ext"].hex(),
                     initial_wcc=tr["initial_wcc"].hex(), wcc=[w.hex() for w in tr["wcc"]],
                     best_wcc=tr["best_wcc"].hex(), printed_comms=tr["printed_comms"])
    manifest[name] = entry


def main():
    if not os.path.exists(os.path.join(REF, "ref_driver")):
        subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    import scdgen
    manifest = {}
    tmpdir = tempfile.mkdtemp()
    for name, text in TEXT_CASES.items():
        p = os.path.join(tmpdir, name + ".txt")
        open(p, "w").write(text)
        run_case(name, p, text_to_pairs(text), manifest)
    for name, pairs in generated_cases().items():
        p = os.path.join(tmpdir, name + ".txt")
        scdgen.write_text(p, pairs)
        run_case(name, p, pairs, manifest)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print(json.dumps({k: {kk: v[kk] for kk in ("n", "m", "edges_in") if kk in v} | {"iters": v.get("iters")}
                      for k, v in manifest.items()}, indent=1))


if __name__ == "__main__":
    main()
