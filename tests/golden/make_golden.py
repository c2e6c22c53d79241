"""Generates the golden fixtures in this directory from the REFERENCE itself.

For every case: the input edge list (as the reference's read_edges stores it,
(min,max) pairs in file order), the binary graph written by the reference's
own `convert` (built unmodified from its sources by oracle/build_ref.sh), and
the trace of the reference's refinement loop (oracle/ref_driver.cpp linked
against the reference's graph.cpp/scd.cpp/wcc.cpp, OMP_NUM_THREADS=1).

A case may start from a given labelling instead of the initial partition
(oracle/ref_driver.cpp's labels argument): wrap_windmill does, to put the int32
products of the gain model (src/scd.cpp:185-213) past 2^31.

The full-size workloads (R-MAT scale 22, a Chung-Lu graph with hubs of degree
> 46,341) are too large to commit; for them `--pins` records compact pins in
pins.json instead: sha256 of the input records, of the reference's graph file
and of every labelling of its trace, and the exact FP64 values.

Run in the development container, where the reference sources exist:
    python tests/golden/make_golden.py            # fixtures + manifest.json
    python tests/golden/make_golden.py --pins     # pins.json (reference runs of many minutes)
    python tests/golden/make_golden.py --cli      # the reference CLIs' stdout lines, into manifest.json
"""
import hashlib
import time
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


def windmill_text(blades):
    """A hub joined to `blades` disjoint triangles (hub, a, b): every edge lies on a
    triangle, the hub's degree is 2 * blades."""
    out = []
    for i in range(blades):
        a, b = 2 * i + 1, 2 * i + 2
        out.append(f"0 {a}\n0 {b}\n{a} {b}\n")
    return "".join(out)


WINDMILL_BLADES = 30000                          # hub degree 60,000
WINDMILL_SPLIT = (25000, 29000)                  # blades in community 0 / 1 / unlabelled


def windmill_labels(graph):
    """The hub (final id 0) and the leaves of the first 25,000 blades in
    community 0 (size 50,001: the hub's d_in = 50,000, so d_in*(d_in-1) and
    (r-1)*(r-2) wrap), the next 4,000 blades in community 1 (the hub's d_out for
    it is 52,000: d_out*(d_out-1) wraps), the last 1,000 blades unlabelled."""
    import oracle as O
    g = O.Graph.from_bytes(graph)
    ind, adj = g.indices, g.adj
    assert ind[1] - ind[0] == 2 * WINDMILL_BLADES
    lab = np.full(g.n, 0xFFFFFFFF, np.uint32)
    lab[0] = 0
    k = 0
    done = set()
    for v in range(1, g.n):
        if lab[v] != 0xFFFFFFFF or v in done:
            continue
        row = adj[ind[v]:ind[v + 1]]
        w = int(row[row != 0][0])
        c = 0 if k < WINDMILL_SPLIT[0] else 1 if k < WINDMILL_SPLIT[1] else None
        if c is not None:
            lab[v] = lab[w] = c
        done.update((v, w))
        k += 1
    return lab


def generated_cases():
    import scdgen
    return {
        "planted_10k": lambda: scdgen.planted(10000, 18.0, 0.1, 20, 100, seed=1),    # the plain-SCD config
        "planted_2k_mu03": lambda: scdgen.planted(2000, 12.0, 0.3, 20, 100, seed=8),
        "planted_5k_mu04": lambda: scdgen.planted(5000, 20.0, 0.4, 20, 100, seed=9),
        "rmat_12": lambda: scdgen.rmat(12, 16, 0.57, 0.19, 0.19, seed=5),
        "chunglu_20k": lambda: scdgen.chunglu(20000, 2.1, 5.0, 2000.0, 0.2, 10, 500, seed=7),
    }


def gz_write(path):
    """gzip writer with a fixed header time, so regenerated fixtures are byte-stable."""
    return gzip.GzipFile(path, "wb", compresslevel=9, mtime=0)


def text_to_pairs(text):
    import oracle as O
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write(text)
        p = f.name
    try:
        return O.read_text(p)
    finally:
        os.unlink(p)


def run_case(name, text_path, pairs, manifest, trace=True, start_labels=None):
    """start_labels (graph bytes -> labels): the trace starts from that labelling."""
    import oracle as O
    gpath = os.path.join(HERE, name + ".graph")
    r = subprocess.run([os.path.join(REF, "convert"), text_path, gpath], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    graph = open(gpath, "rb").read()
    os.unlink(gpath)
    with gz_write(gpath + ".gz") as f:
        f.write(graph)
    with gz_write(os.path.join(HERE, name + ".pairs.npy.gz")) as f:
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
        cmd = [os.path.join(REF, "ref_driver"), tmpg, tpath, "1000"]
        if start_labels is not None:
            lab = start_labels(graph)
            lpath = tmpg + ".labels"
            lab.astype("<u4").tofile(lpath)
            cmd.append(lpath)
            with gz_write(os.path.join(HERE, name + ".labels.npy.gz")) as f:
                np.save(f, lab)
            entry["start_labels"] = True
        r = subprocess.run(cmd, capture_output=True, text=True, env=env)
        os.unlink(tmpg)
        if start_labels is not None:
            os.unlink(lpath)
        if r.returncode != 0:
            raise RuntimeError(r.stderr)
        raw = open(tpath, "rb").read()
        os.unlink(tpath)
        with gz_write(tpath + ".gz") as f:
            f.write(raw)
        tr = O.read_trace(tpath + ".gz")
        entry.update(iters=tr["iters"], num_comms=tr["num_comms"], p_ext=tr["p_ext"].hex(),
                     initial_wcc=tr["initial_wcc"].hex(), wcc=[w.hex() for w in tr["wcc"]],
                     best_wcc=tr["best_wcc"].hex(), printed_comms=tr["printed_comms"])
    manifest[name] = entry


# Full-size workloads pinned by hashes (pins.json): the R-MAT graph of the headline
# benchmark (scale 22) and the skewed-degree Chung-Lu stress graph (8M vertices).
# Both have vertices of degree > 46,341, where the int32 products of the gain
# model wrap (max degree 160,369 and 79,126).
PIN_WORKLOADS = {
    "rmat_22": ("rmat", dict(scale=22, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=22)),
    "chunglu_8m": ("chunglu", dict(n=8_000_000, gamma=2.1, wmin=5.0, wmax=200000.0, mu=0.2, smin=10, smax=500,
                                   seed=3)),
}


def sha256(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_pins(names):
    """Runs the reference's convert (all host threads; its output is integer and
    thread-count independent) and ref_driver (one thread: the canonical sums) on
    each workload and records hashes of everything they produce."""
    import oracle as O
    import scdgen
    path = os.path.join(HERE, "pins.json")
    pins = json.load(open(path)) if os.path.exists(path) else {}
    tmpdir = tempfile.mkdtemp()
    for name in names:
        gen, args = PIN_WORKLOADS[name]
        pairs = getattr(scdgen, gen)(**args)
        txt = os.path.join(tmpdir, name + ".txt")
        scdgen.write_text(txt, pairs)
        gpath = os.path.join(tmpdir, name + ".graph")
        t0 = time.time()
        r = subprocess.run([os.path.join(REF, "convert"), txt, gpath], capture_output=True, text=True,
                           env=dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count())))
        if r.returncode != 0:
            raise RuntimeError(r.stderr)
        convert_s = time.time() - t0
        os.unlink(txt)
        graph = open(gpath, "rb").read()
        g = O.Graph.from_bytes(graph)
        deg = np.diff(g.indices.astype(np.int64))
        tpath = os.path.join(tmpdir, name + ".trace")
        t0 = time.time()
        r2 = subprocess.run([os.path.join(REF, "ref_driver"), gpath, tpath, "1000"], capture_output=True, text=True,
                            env=dict(os.environ, OMP_NUM_THREADS="1"))
        if r2.returncode != 0:
            raise RuntimeError(r2.stderr)
        driver_s = time.time() - t0
        tr = O.read_trace(tpath)
        os.unlink(gpath)
        os.unlink(tpath)
        pins[name] = {
            "generator": gen, "args": args, "edges_in": int(pairs.shape[0]), "pairs_sha256": sha256(pairs),
            "n": g.n, "m": g.m, "max_degree": int(deg.max()) if g.n else 0, "graph_bytes": len(graph),
            "graph_sha256": hashlib.sha256(graph).hexdigest(),
            "p_ext": tr["p_ext"].hex(), "num_comms": tr["num_comms"],
            "initial_labels_sha256": sha256(tr["initial_labels"]),
            "initial_stats_sha256": sha256(tr["initial_stats"]), "initial_wcc": tr["initial_wcc"].hex(),
            "iters": tr["iters"], "wcc": [w.hex() for w in tr["wcc"]],
            "labels_sha256": [sha256(l) for l in tr["labels"]],
            "stats_sha256": [sha256(st) for st in tr["stats"]],
            "best_labels_sha256": sha256(tr["best_labels"]), "best_wcc": tr["best_wcc"].hex(),
            "printed_comms": tr["printed_comms"],
            "reference_seconds": {"convert": round(convert_s, 1), "convert_threads": os.cpu_count(),
                                  "ref_driver_1_thread": round(driver_s, 1)},
            "reference_convert_stdout": [l for l in r.stdout.splitlines() if "lines read" not in l],
        }
        with open(path, "w") as f:
            json.dump(pins, f, indent=1, sort_keys=True)
        print(name, json.dumps({k: pins[name][k] for k in ("n", "m", "max_degree", "iters", "reference_seconds")}))


def is_timer(line):
    return line.endswith(" ms") or "lines read so far" in line


def record_cli_lines(manifest):
    """The stdout lines (timer lines dropped) of the reference's `convert` on each
    case's text and of its `main` (one thread: the canonical WCC sums) on the
    resulting graph, for the command-line drop-in test."""
    import scdgen
    tmpdir = tempfile.mkdtemp()
    texts = dict(TEXT_CASES)
    for name, make in generated_cases().items():
        p = os.path.join(tmpdir, name + ".txt")
        scdgen.write_text(p, make())
        texts[name] = p
    for name in manifest:
        if name not in texts:
            continue
        src = texts[name]
        if not os.path.exists(src):
            p = os.path.join(tmpdir, name + ".txt")
            open(p, "w").write(src)
            src = p
        gpath = os.path.join(tmpdir, name + ".graph")
        conv = subprocess.run([os.path.join(REF, "convert"), src, gpath], capture_output=True, text=True, check=True)
        lines = [l.replace(src, "<input>").replace(gpath, "<output>") for l in conv.stdout.splitlines()]
        manifest[name]["ref_convert_lines"] = [l for l in lines if not is_timer(l)]
        if manifest[name]["n"] > 0:
            main = subprocess.run([os.path.join(REF, "main"), gpath], capture_output=True, text=True, check=True,
                                  env=dict(os.environ, OMP_NUM_THREADS="1"))
            manifest[name]["ref_main_lines"] = [l for l in main.stdout.splitlines() if l and not is_timer(l)]
        os.unlink(gpath)


def main():
    if "--cli" in sys.argv:
        mpath = os.path.join(HERE, "manifest.json")
        manifest = json.load(open(mpath))
        record_cli_lines(manifest)
        with open(mpath, "w") as f:
            json.dump(manifest, f, indent=1, sort_keys=True)
        return
    if "--pins" in sys.argv:
        names = [a for a in sys.argv[1:] if not a.startswith("--")] or list(PIN_WORKLOADS)
        if not os.path.exists(os.path.join(REF, "ref_driver")):
            subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
        return make_pins(names)
    if not os.path.exists(os.path.join(REF, "ref_driver")):
        subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    import scdgen
    only = [a for a in sys.argv[1:] if not a.startswith("--")]   # regenerate just these cases
    mpath = os.path.join(HERE, "manifest.json")
    manifest = json.load(open(mpath)) if only else {}
    tmpdir = tempfile.mkdtemp()
    for name, text in TEXT_CASES.items():
        if only and name not in only:
            continue
        p = os.path.join(tmpdir, name + ".txt")
        open(p, "w").write(text)
        run_case(name, p, text_to_pairs(text), manifest)
    for name, make in generated_cases().items():
        if only and name not in only:
            continue
        pairs = make()
        p = os.path.join(tmpdir, name + ".txt")
        scdgen.write_text(p, pairs)
        run_case(name, p, pairs, manifest)
    if not only or "wrap_windmill" in only:
        text = windmill_text(WINDMILL_BLADES)
        p = os.path.join(tmpdir, "wrap_windmill.txt")
        open(p, "w").write(text)
        run_case("wrap_windmill", p, text_to_pairs(text), manifest, start_labels=windmill_labels)
    with open(mpath, "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print(json.dumps({k: {kk: v[kk] for kk in ("n", "m", "edges_in") if kk in v} | {"iters": v.get("iters")}
                      for k, v in manifest.items()}, indent=1))


if __name__ == "__main__":
    main()
