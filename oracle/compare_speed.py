"""Times the oracle restatement (the CPU "port" that bench.py's CPU legs run) beside
the reference's own CPU binaries (oracle/_ref/convert and oracle/_ref/main, built
unmodified from the reference's sources by build_ref.sh) on the same R-MAT
graphs with the same thread count, using the reference's own timers:

  T = convert's "process graph" + main's "create initial partition"
      + the initial "compute WCC" + the sum of its "iteration" timers

(the CPU time of bench.py's cpu_baseline).  Prints a Markdown table and every
timer line both sides printed.  Test and measurement infrastructure only: it
needs oracle/_ref, which exists where the reference's sources were present.

usage: python oracle/compare_speed.py [--threads T] [--scales 18 20] [--repeat R]
With R > 1 the two sides run alternately R times and each column is the median
(the runs share the machine with whatever else runs there).
"""
import argparse
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF = os.path.join(HERE, "_ref")


def timer_lines(text):
    return [(m.group(1), float(m.group(2))) for m in re.finditer(r"^([^:\n]+): ([0-9.eE+-]+) ms$", text, re.M)]


def reference_run(txt, graph, threads):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    conv = subprocess.run([os.path.join(REF, "convert"), txt, graph], capture_output=True, text=True, env=env,
                          check=True).stdout
    main = subprocess.run([os.path.join(REF, "main"), graph], capture_output=True, text=True, env=env,
                          check=True).stdout
    ct, mt = timer_lines(conv), timer_lines(main)
    pg = sum(v for k, v in ct if k == "process graph")
    part = sum(v for k, v in mt if k == "create initial partition")
    wcc0 = next(v for k, v in mt if k == "compute WCC")   # the first one: the initial WCC
    iters = [v for k, v in mt if k == "iteration"]
    return {"process_graph": pg, "initial_partition": part, "initial_wcc": wcc0, "iterations": sum(iters),
            "n_iterations": len(iters), "total": pg + part + wcc0 + sum(iters),
            "lines": [f"{k}: {v:.1f} ms" for k, v in ct if k != "write output" and "read" not in k] +
                     [f"{k}: {v:.1f} ms" for k, v in mt if k != "load graph"]}


def port_run(scale, threads):
    """The restatement in a child process (its OpenMP thread count is fixed at load)."""
    code = (f"import sys, json; sys.path[:0] = [{os.path.join(ROOT, 'het-scd_gb300')!r}, {HERE!r}]\n"
            "import oracle, scdgen\n"
            f"p = scdgen.rmat({scale}, 16, 0.57, 0.19, 0.19, seed=22)\n"
            "g, tm = oracle.convert(p)\n"
            "r = oracle.run(g, max_iters=1000, keep_trace=False)\n"
            "print(json.dumps({'convert': tm, 'run': r['times'], 'iters': r['iters'], 'threads': oracle.threads()}))\n")
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    out = json.loads(subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                                    check=True).stdout.strip().splitlines()[-1])
    t = out["run"]
    pg = out["convert"]["process_graph"]
    return {"process_graph": pg, "initial_partition": t["initial_partition"], "initial_wcc": t["initial_wcc"],
            "iterations": t["iterations"], "n_iterations": out["iters"],
            "total": pg + t["initial_partition"] + t["initial_wcc"] + t["iterations"], "threads": out["threads"],
            "timers": {"convert": out["convert"], "run": t}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--scales", type=int, nargs="+", default=[18, 20])
    ap.add_argument("--repeat", type=int, default=1)
    a = ap.parse_args()
    sys.path[:0] = [os.path.join(ROOT, "het-scd_gb300"), HERE]
    import scdgen
    rows, details = [], []
    tmp = tempfile.mkdtemp()
    for s in a.scales:
        pairs = scdgen.rmat(s, 16, 0.57, 0.19, 0.19, seed=22)
        txt, graph = os.path.join(tmp, f"r{s}.txt"), os.path.join(tmp, f"r{s}.graph")
        scdgen.write_text(txt, pairs)
        refs, ports = [], []
        for _ in range(a.repeat):
            refs.append(reference_run(txt, graph, a.threads))
            ports.append(port_run(s, a.threads))
        ref = sorted(refs, key=lambda r: r["total"])[len(refs) // 2]
        port = sorted(ports, key=lambda r: r["total"])[len(ports) // 2]
        os.unlink(txt)
        os.unlink(graph)
        rows.append(f"| R-MAT {s} ({pairs.shape[0]:,} edges) | {a.threads} | {a.repeat} | "
                    f"{ref['process_graph']:.0f} / {port['process_graph']:.0f} | "
                    f"{ref['initial_partition'] + ref['initial_wcc']:.0f} / "
                    f"{port['initial_partition'] + port['initial_wcc']:.0f} | "
                    f"{ref['iterations']:.0f} ({ref['n_iterations']}) / {port['iterations']:.0f} ({port['n_iterations']}) | "
                    f"{ref['total']:.0f} / {port['total']:.0f} | {port['total'] / ref['total']:.2f} |")
        details.append((s, ref, port))
    print("| graph | threads | runs (median) | process graph ms (reference / port) | partition + initial WCC ms | "
          "iterations ms (count) | T ms | port / reference |")
    print("|---|---|---|---|---|---|---|---|")
    print("\n".join(rows))
    for s, ref, port in details:
        print(f"\nR-MAT {s}, reference timer lines:")
        print("\n".join("    " + l for l in ref["lines"]))
        print(f"R-MAT {s}, port timers: " + json.dumps(port["timers"]))


if __name__ == "__main__":
    main()
