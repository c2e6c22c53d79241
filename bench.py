"""Benchmark of the GB300 SCD engine: plain SCD on R-MAT scale 22 (edge factor
16, a/b/c/d = .57/.19/.19/.05), one step = the whole pipeline of `convert` +
`main-gpu` on one graph: device preprocessing (renumbering, sort/dedup,
triangle counting, triangle filter, degree relabel, CSR), initial partition,
initial WCC and refinement iterations until convergence, best labels ready.

  value     E_in / step time with the edge list already resident in HBM
            (CUDA events on the engine's stream)
  e2e       the same through the C ABI with HOST buffers: pinned edge list
            H2D inside the timed region, best labels D2H at the end
  roofline  the dominant kernel (triangle counting) against measured HBM peak
  cpu_baseline  the CPU oracle (restatement of the reference's CPU path, with
            all host threads) on the full workload, once: the reference's own
            timers (convert's "process graph" + initial partition + initial WCC +
            iterations); its labels are compared with the engine's.  The R-MAT
            scale 18 sample of the reference arm is reported beside it
            (cpu_baseline_sample)

`--impl reference` times the reference's CPU implementation instead (its own
binaries when they were built from its sources, else the oracle restatement),
each step a bounded sample of the same workload.  Single graph, so more GPUs
run independent replicas (weak scaling, no collective).
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _sub in ("het-scd_gb300", "oracle"):
    sys.path.insert(0, os.path.join(ROOT, _sub))

METRIC = "SCD edges/s end-to-end"
UNIT = "edges/s"
CPU_SAMPLE_SCALE = 18


def algorithmic_tc_bytes(indices, adj):
    """B_tc = 4*[(n+1) + m + sum over oriented edges u->v of (d+(u) + d+(v))] + 8n,
    orientation from the larger to the smaller final id (degree-descending ids)."""
    import numpy as np
    n = len(indices) - 1
    deg = np.diff(indices.astype(np.int64))
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    out = adj.astype(np.int64) < src
    dplus = np.bincount(src[out], minlength=n)
    m = int(out.sum())
    s = int(dplus[src[out]].sum() + dplus[adj[out].astype(np.int64)].sum())
    return 4 * ((n + 1) + m + s) + 8 * n, dict(n=n, m=m, merge_items=s)


def iteration_bytes(indices, adj, labels):
    """B_it = 4*[3(n+1) + 6*(2m) + 12n] + 12*P + B_int for one refinement iteration
    under `labels`: P = distinct (vertex, neighbour label) pairs, B_int = 4 * sum over
    internal edges u<v of (d_int(u) + d_int(v)).  Counted on the GPU with torch."""
    import torch
    dev = torch.device("cuda")
    ind = torch.from_numpy(indices.astype("int64")).to(dev)
    nbr = torch.from_numpy(adj.astype("int64")).to(dev)
    lab = torch.from_numpy(labels.astype("int64")).to(dev)
    n = ind.numel() - 1
    deg = ind[1:] - ind[:-1]
    src = torch.repeat_interleave(torch.arange(n, device=dev), deg)
    lu, lv = lab[src], lab[nbr]
    valid = lv != 0xFFFFFFFF
    p_pairs = torch.unique(src[valid] * (1 << 32) + lv[valid]).numel()
    same = valid & (lu == lv)
    d_int = torch.bincount(src[same], minlength=n)
    up = same & (src < nbr)
    b_int = 4 * int((d_int[src[up]] + d_int[nbr[up]]).sum())
    m2 = nbr.numel()
    return 4 * (3 * (n + 1) + 6 * m2 + 12 * n) + 12 * p_pairs + b_int, dict(P=p_pairs, B_int=b_int)


class ClockSampler:
    def __init__(self):
        self.rows, self.proc = [], None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = sorted(float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit())
        mx = max((float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()), default=None)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for k, name in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(dist, values, device):
    """Each value's maximum over all ranks (replicas: the slowest one sets the job's
    time); the values unchanged on one process (dist None)."""
    if not dist:
        return list(values)
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def job_throughput(world, units_per_replica, ms):
    """Whole-job rate of N independent replicas timed together: all the units over
    the slowest replica's time."""
    return world * units_per_replica / (ms / 1e3)


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_traffic(kernel, scale):
    """DRAM bytes (read + write) of one launch from the committed ncu summary
    (profiles/traffic.json), scaled to R-MAT `scale` by the algorithmic bytes."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        rec = json.load(f).get(kernel, {})
    return rec.get(f"rmat{scale}_bytes_per_launch")


def cpu_sample_run(threads=None):
    """The CPU path on the bounded sample: T = convert's "process graph" + initial
    partition + initial WCC + sum of iteration timers (the reference's own timers)."""
    import oracle
    import scdgen
    pairs = scdgen.rmat(CPU_SAMPLE_SCALE, 16, 0.57, 0.19, 0.19, seed=22)
    ref_bin = os.path.join(ROOT, "oracle", "_ref")
    g, tm = oracle.convert(pairs)
    r = oracle.run(g, max_iters=1000, keep_trace=False)
    t_ms = tm["process_graph"] + r["times"]["initial_partition"] + r["times"]["initial_wcc"] + r["times"]["iterations"]
    return pairs.shape[0] / (t_ms / 1e3), t_ms, pairs.shape[0], "port"


def time_wcc_static(S, eng, gd):
    """scd_wcc_static (no device allocation) on the resident graph and its current
    labels: CUDA-event time per call (3 calls after one warm-up) and equality with
    scd_compute_wcc.  Not part of the step."""
    import numpy as np
    import torch
    lab = eng.current_labels()
    sizes = eng.community_stats()[0]
    want = eng.compute_wcc()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()
    ind, adj, tri, tdg = dev(gd["indices"]), dev(gd["adj"]), dev(gd["tri"]), dev(gd["tri_deg"])
    lb, sz = dev(lab), dev(sizes if sizes.size else np.zeros(1, np.int32))
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    call = lambda: S.lib().scd_wcc_static(ind.data_ptr(), adj.data_ptr(), tri.data_ptr(), tdg.data_ptr(),
                                          lb.data_ptr(), sz.data_ptr(), int(lab.size), 1.0, out.data_ptr(),
                                          st.cuda_stream)
    assert call() == S.OK
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(3):
        assert call() == S.OK
    e1.record(st)
    torch.cuda.synchronize()
    return {"ms_per_call": e0.elapsed_time(e1) / 3, "equal_to_scd_compute_wcc": float(out.item()) == want,
            "n": int(lab.size)}


def cpu_model():
    """The host CPU's model name (lscpu on Arm, /proc/cpuinfo elsewhere)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


def cpu_full_run(pairs):
    """The CPU path on the full workload, once (T as in cpu_sample_run).  Returns
    edges/s, T in ms, the per-timer split and the best labels."""
    import oracle
    g, tm = oracle.convert(pairs)
    r = oracle.run(g, max_iters=1000, keep_trace=False)
    t = r["times"]
    split = {"process_graph": tm["process_graph"], "initial_partition": t["initial_partition"],
             "initial_wcc": t["initial_wcc"], "iterations": t["iterations"]}
    t_ms = sum(split.values())
    return pairs.shape[0] / (t_ms / 1e3), t_ms, split, r


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    cores = oracle.threads()
    W, K = args.warmup, args.steps
    vals = []
    for i in range(W + K):
        v, t_ms, e, kind = cpu_sample_run()
        if i >= W:
            vals.append((v, t_ms))
    v = sorted(x[0] for x in vals)[len(vals) // 2]
    ms = sorted(x[1] for x in vals)[len(vals) // 2]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": K, "warmup": W, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32+f64", "data": "synthetic",
            "config": {"workload": f"rmat-{args.scale}", "edge_factor": 16, "abcd": [0.57, 0.19, 0.19, 0.05],
                       "parallelism": f"host cores ({cores} threads)",
                       "sample": f"each step: R-MAT scale {CPU_SAMPLE_SCALE} of the same generator ({e} edges)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"R-MAT scale {CPU_SAMPLE_SCALE} (same generator and a,b,c,d), "
                                       "reference timers: process graph + initial partition + initial WCC + iterations"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_config(S, device, workload, pairs, steps, warmup):
    """Another named configuration through the same two paths as the headline:
    edges/s with the edge list resident in HBM (CUDA events) and end to end with
    pinned host pairs in and labels out, plus the preprocessing triangle count
    against the measured HBM peak (algorithmic bytes B_tc)."""
    import numpy as np
    import torch
    E = pairs.shape[0]
    dev_pairs = torch.from_numpy(pairs.view(np.int32)).cuda()
    host_pairs = torch.from_numpy(pairs.view(np.int32)).pin_memory()
    eng = S.Engine(device, flags=S.FLAG_PROFILE)
    stream = torch.cuda.ExternalStream(eng.stream())

    def step_device():
        eng.convert_edges(device_ptr=dev_pairs.data_ptr(), count=E)
        return eng.run(0.01, 1000)

    for _ in range(warmup):
        step_device()
    torch.cuda.synchronize()
    eng.profile_reset()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        r = step_device()
    ev1.record(stream)
    torch.cuda.synchronize()
    dev_ms = ev0.elapsed_time(ev1) / steps
    tc_ms, tc_n = eng.profile("tc")
    t = time.perf_counter()
    for _ in range(steps):
        eng._check(S.lib().scd_convert_edges(eng._ctx, host_pairs.data_ptr(), E, 0))
        r = eng.run(0.01, 1000)
        lab = eng.labels_from_device()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t) * 1e3 / steps
    n, m, _ = eng.graph_info()
    gd = eng.graph_download()
    eng.close()
    b_tc, _ = algorithmic_tc_bytes(gd["indices"], gd["adj"])
    tc_avg = tc_ms / max(tc_n, 1)
    peak, kind = measured_peak_gbs()
    return {"workload": workload, "edges_in": E, "n": n, "m": m, "iterations": r["iterations"],
            "value": E / (dev_ms / 1e3), "unit": UNIT, "ms_per_step": dev_ms, "steps": steps, "warmup": warmup,
            "e2e": {"value": E / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": E * 8,
                    "d2h_bytes_per_step": 4 * int(lab.size)},
            "triangle_count": {"ms": tc_avg, "bytes": b_tc, "gbs": b_tc / (tc_avg / 1e3) / 1e9,
                               "frac": b_tc / (tc_avg / 1e3) / 1e9 / peak, "peak": peak, "peak_kind": kind}}


def c4_specs(k):
    """Batched workload: planted-partition graphs, n log-uniform in [1000, 200000],
    mean degree D uniform in [8, 40], mixing mu uniform in [0.05, 0.4], internal
    degree D*(1-mu), community sizes 20..100 (P(s) ~ 1/s), graph i seeded 4+i."""
    import numpy as np
    out = []
    for i in range(k):
        rng = np.random.default_rng(4 + i)
        n = int(np.exp(rng.uniform(np.log(1000), np.log(200000))))
        d = float(rng.uniform(8, 40))
        mu = float(rng.uniform(0.05, 0.4))
        out.append((n, d * (1 - mu), mu, 4 + i))
    return out


def _gen_planted(spec):
    import scdgen
    n, k_in, mu, seed = spec
    return scdgen.planted(n, k_in, mu, 20, 100, seed=seed)


def generate(fn, specs, threads=8):
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(threads) as ex:
        return list(ex.map(fn, specs))


def split_batches(sizes, cap):
    """Consecutive runs of graphs with at most `cap` edge records each."""
    out, cur, tot = [], [], 0
    for i, e in enumerate(sizes):
        if cur and tot + e > cap:
            out.append(cur)
            cur, tot = [], 0
        cur.append(i)
        tot += e
    if cur:
        out.append(cur)
    return out


def bench_batched(S, device, args):
    """4096 planted graphs: block-diagonal batches (each batch one union graph whose
    kernels run every graph's work together, iterations replayed from CUDA graphs)
    against a per-graph loop of the plain engine, both through the public API from
    host edge lists to host labels.  The loop is timed on an evenly spaced sample
    of the same graphs (the graphs are i.i.d.), and its results are compared with
    the batched ones for that sample."""
    import numpy as np
    import torch
    k = args.batch_graphs
    t0 = time.time()
    graphs = generate(_gen_planted, c4_specs(k))
    gen_s = time.time() - t0
    sizes = [g.shape[0] for g in graphs]
    records = int(sum(sizes))
    groups = split_batches(sizes, args.batch_records)
    host = pin_lists(graphs)   # both arms read the edge lists from pinned memory
    labels_out = torch.empty(records, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    eng = S.Engine(device)
    eng.batch_convert([graphs[i] for i in groups[0]])
    tune = eng.autotune() if not args.no_autotune else {"small_max": None, "warp_max": None, "cta_max": None,
                                                         "in_list_min": None}

    phase = {"convert_s": 0.0, "run_s": 0.0, "labels_s": 0.0}

    def run_group(ids):
        t0 = time.perf_counter()
        eng.batch_convert([graphs[i] for i in ids])        # H2D of the host lists + device preprocessing
        t1 = time.perf_counter()
        res, rc = eng.batch_run(0.01, 1000)                 # initial partition + iterations to convergence
        t2 = time.perf_counter()
        labs = [x.copy() for x in eng.batch_labels_all(labels_out)]   # best labels D2H (pinned), kept
        t3 = time.perf_counter()
        phase["convert_s"] += t1 - t0
        phase["run_s"] += t2 - t1
        phase["labels_s"] += t3 - t2
        return res, rc, labs

    run_group(groups[0])                    # warm-up (allocator, module load)
    torch.cuda.synchronize()
    for key in phase:
        phase[key] = 0.0
    launches0 = eng.kernel_launches()
    t = time.perf_counter()
    results, not_converged = {}, 0
    for ids in groups:
        res, rc, labs = run_group(ids)
        not_converged += rc != 0
        for j, i in enumerate(ids):
            results[i] = (res[j]["iterations"], res[j]["best_wcc"], labs[j])
    torch.cuda.synchronize()
    batch_s = time.perf_counter() - t
    launches = eng.kernel_launches() - launches0
    mem = eng.memory_usage()
    eng.close()

    if args.loop_sample <= 0:
        return {"graphs": k, "edges_in": records, "batches": len(groups), "graphs_per_s": k / batch_s,
                "edges_per_s": records / batch_s, "seconds": batch_s, "gpu_launches": launches,
                "phases_s": {key: round(v, 4) for key, v in phase.items()}}
    step = max(1, k // args.loop_sample)
    sample = list(range(0, k, step))[: args.loop_sample]
    plain = S.Engine(device)
    plain.convert_edges(graphs[sample[0]])
    plain.run(0.01, 1000)
    torch.cuda.synchronize()
    t = time.perf_counter()
    same = True
    loop_records = 0
    for i in sample:
        plain.convert_edges(graphs[i])
        r = plain.run(0.01, 1000)
        lab = plain.labels_from_device()
        loop_records += sizes[i]
        it, w, bl = results[i]
        same &= r["iterations"] == it and r["best_wcc"] == w and np.array_equal(lab, bl)
    torch.cuda.synchronize()
    loop_s = time.perf_counter() - t
    plain.close()
    b_gps = k / batch_s
    l_gps = len(sample) / loop_s
    return {"workload": f"{k} planted-partition graphs, n log-uniform [1000,200000], mean degree U[8,40], "
                        "mu U[0.05,0.4], seeds 4..",
            "graphs": k, "edges_in": records, "batches": len(groups), "max_records_per_batch": args.batch_records,
            "graphs_per_s": b_gps, "edges_per_s": records / batch_s, "seconds": batch_s,
            "gpu_launches": launches, "peak_engine_bytes": mem, "not_converged_batches": not_converged,
            "phases_s": {key: round(v, 4) for key, v in phase.items()},
            "per_graph_loop": {"graphs_per_s": l_gps, "edges_per_s": loop_records / loop_s, "sample_graphs": len(sample),
                               "seconds": loop_s},
            "speedup_vs_loop": b_gps / l_gps, "identical_on_sample": bool(same),
            "autotune": {"small_max": tune["small_max"], "warp_max": tune["warp_max"], "cta_max": tune["cta_max"],
                         "in_list_min": tune["in_list_min"]},
            "timing": "host wall clock, host edge lists (pinned) in, host labels out", "generate_s": round(gen_s, 1)}


def c5_specs(count, seed=5):
    """Served workload: 80% planted partition, n log-uniform in [1000, 50000],
    mean degree 16 (internal 14.4), mu 0.1; 20% R-MAT scale 19..21, edge factor 16."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        if rng.uniform() < 0.8:
            out.append(("planted", int(np.exp(rng.uniform(np.log(1000), np.log(50000)))), 1000 + i))
        else:
            out.append(("rmat", int(rng.integers(19, 22)), 5000 + i))
    return out


def _gen_request(spec):
    import scdgen
    kind, size, seed = spec
    if kind == "planted":
        return scdgen.planted(size, 14.4, 0.1, 20, 100, seed=seed)
    return scdgen.rmat(size, 16, 0.57, 0.19, 0.19, seed=seed)


def pin_lists(graphs):
    """Moves the (E, 2) uint32 edge lists into one pinned host buffer, as a serving
    host's request buffer would hold them, and replaces them by views into it: the
    device then copies them with DMA at full speed.  (From pageable memory the device
    reads them through address translation, whose speed drifted down run after run:
    0.64 -> 0.99 s for the same 14.5 GB in one process, and served capacity fell by
    half over a sequence of processes on one box.)  Returns the buffer (keep it alive)."""
    import numpy as np
    import torch
    records = int(sum(g.shape[0] for g in graphs))
    host = torch.empty(max(2 * records, 1), dtype=torch.int32, pin_memory=True)
    hv = host.numpy().view(np.uint32)
    off = 0
    for i, g in enumerate(graphs):
        n2 = 2 * g.shape[0]
        hv[off:off + n2] = g.reshape(-1)
        graphs[i] = hv[off:off + n2].reshape(-1, 2)
        off += n2
    return host


def per_graph_loop(S, device, graphs):
    """The plain per-graph loop: one engine, each graph converted, run to
    convergence and its labels copied out before the next (the reference's one
    graph per main-gpu process, src/main-gpu.cpp:43-110, without process start-up).
    Returns the total seconds and (iterations, best WCC, labels, seconds) per graph."""
    import numpy as np
    import torch
    plain = S.Engine(device)
    plain.convert_edges(graphs[0])
    plain.run(0.01, 1000)
    torch.cuda.synchronize()
    out = []
    t = time.perf_counter()
    for p in graphs:
        t0 = time.perf_counter()
        plain.convert_edges(p)
        if plain.graph_info()[0] == 0:
            out.append((0, 0.0, np.zeros(0, np.uint32), time.perf_counter() - t0))
            continue
        r = plain.run(0.01, 1000)
        out.append((r["iterations"], r["best_wcc"], plain.labels_from_device(), time.perf_counter() - t0))
    torch.cuda.synchronize()
    secs = time.perf_counter() - t
    plain.close()
    return secs, out


def bench_served(S, device, args):
    """The continuous-batching server (120 GB admission budget; requests convert on
    staging engines and join the resident set's iterations): its capacity with all
    requests submitted at once, then open-loop Poisson arrivals at a fixed offered
    rate (by default 75% of that capacity); latency = submission to labels on the
    host.  Beside it, the plain per-graph loop over the same requests, whose
    results every served result must equal."""
    import numpy as np
    import serve
    specs = c5_specs(args.serve_requests)
    t0 = time.time()
    reqs = generate(_gen_request, specs)
    gen_s = time.time() - t0
    pinned = pin_lists(reqs)   # requests arrive in a pinned receive buffer, for the loop and the server
    loop_s, loop_out = per_graph_loop(S, device, reqs)
    srv = serve.Server(device, converters=args.serve_converters, budget_bytes=120e9, max_batch=64)
    for r in [srv.submit(reqs[i]) for i in range(min(8, len(reqs)))]:   # warm-up
        r.wait(600)
    # capacity: every request submitted at once (closed loop)
    for ln in srv.lanes:
        ln.step_running.clear()
    t = time.perf_counter()
    handles = [srv.submit(p) for p in reqs]
    for h in handles:
        h.wait(1200)
    capacity = len(reqs) / (max(h.finished for h in handles) - t)
    cap_cosched = srv.mean_coscheduled()
    same = all(h.result["iterations"] == it and h.result["best_wcc"] == w and np.array_equal(h.labels, lab)
               for h, (it, w, lab, _) in zip(handles, loop_out) if it > 0)
    rate = args.serve_rate if args.serve_rate > 0 else 0.75 * capacity
    rng = np.random.default_rng(55)
    gaps = rng.exponential(1.0 / rate, size=len(reqs))
    srv.batches.clear()
    for ln in srv.lanes:
        ln.step_running.clear()
    srv.peak_in_use = 0.0
    handles = []
    t = time.perf_counter()
    nxt = t
    for i, pairs in enumerate(reqs):
        nxt += gaps[i]
        d = nxt - time.perf_counter()
        if d > 0:
            time.sleep(d)
        handles.append(srv.submit(pairs))
    for h in handles:
        h.wait(1200)
    end = max(h.finished for h in handles)
    same = same and all(h.result["iterations"] == it and np.array_equal(h.labels, lab)
                        for h, (it, w, lab, _) in zip(handles, loop_out) if it > 0)
    lanes = [{"max_records": (srv.bounds[k] if k < len(srv.bounds) else None), "steps": len(ln.step_running),
              "mean_coscheduled": float(np.mean(ln.step_running)) if ln.step_running else 0.0,
              **{k2: round(v, 1) if isinstance(v, float) else v for k2, v in ln.set.resident_timing().items()}}
             for k, ln in enumerate(srv.lanes)]
    conv_ms = [b[1] * 1e3 for b in srv.batches]
    srv.close()
    del pinned   # the request buffer outlives the loop and the server
    lat = [h.latency * 1e3 for h in handles]
    span = end - t
    sizes = [b[0] for b in srv.batches]
    loop_gps = len(reqs) / loop_s
    # where the loop's time goes: requests of the first lane (<= 2^21 records, the planted
    # graphs) and the rest (the R-MAT graphs); the large ones are already one graph per
    # launch-filling pipeline, so co-scheduling cannot take the loop below their share
    big = [x[3] for p, x in zip(reqs, loop_out) if p.shape[0] > (1 << 21)]
    small = [x[3] for p, x in zip(reqs, loop_out) if p.shape[0] <= (1 << 21)]
    return {"workload": "Poisson arrivals; 80% planted n log-uniform [1000,50000] degree 16 mu 0.1, "
                        "20% R-MAT scale 19-21 edge factor 16",
            "requests": len(reqs), "capacity_graphs_per_s": capacity, "offered_per_s": rate,
            "graphs_per_s": len(reqs) / span,
            "edges_per_s": sum(p.shape[0] for p in reqs) / span,
            "p50_ms": serve.percentile(lat, 50), "p99_ms": serve.percentile(lat, 99), "max_ms": max(lat),
            "per_graph_loop": {"graphs_per_s": loop_gps, "seconds": loop_s,
                               "seconds_requests_le_2e21_records": round(sum(small), 4), "count_small": len(small),
                               "seconds_requests_gt_2e21_records": round(sum(big), 4), "count_large": len(big),
                               "speedup_bound_if_small_ones_were_free": loop_s / max(sum(big), 1e-9)},
            "speedup_vs_loop": capacity / loop_gps, "identical_to_loop": bool(same),
            "mean_coscheduled_graphs": {"capacity_run": cap_cosched, "poisson_run": srv.mean_coscheduled()},
            "converters": args.serve_converters, "budget_gb": 120, "peak_admitted_gb": srv.peak_in_use / 1e9,
            "conversion_batches": len(sizes), "mean_conversion_batch": float(np.mean(sizes)) if sizes else 0.0,
            "conversion_ms_p50": serve.percentile(conv_ms, 50), "lanes": lanes,
            "timing": "host wall clock, requests in a pinned host buffer, labels out to the host",
            "generate_s": round(gen_s, 1)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine")
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-full", dest="cpu_full", action="store_true", default=True,
                    help="CPU baseline on the full workload (default)")
    ap.add_argument("--cpu-sample-only", dest="cpu_full", action="store_false",
                    help="CPU baseline on the scale-18 sample only")
    ap.add_argument("--no-plain", action="store_true", help="skip the R-MAT line (profiling the other sections)")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the planted-10k and Chung-Lu 8M lines")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--batch-graphs", type=int, default=4096)
    ap.add_argument("--no-autotune", action="store_true", help="batched section: keep the default split")
    ap.add_argument("--batch-records", type=int, default=1 << 28)
    ap.add_argument("--loop-sample", type=int, default=256)
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-rate", type=float, default=0.0, help="requests/s; 0: 75%% of the measured capacity")
    ap.add_argument("--serve-converters", type=int, default=2)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch

    import scd_gb300 as S

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    line = {} if args.no_plain else bench_plain(S, args, world, rank, local, dist)
    if not args.no_configs:
        import scdgen
        line["c1"] = bench_config(S, local, "planted partition n=10000, mean internal degree 18, mu 0.1, seed 1",
                                  scdgen.workload("planted-10k"), max(args.steps, 10), max(args.warmup, 3))
        line["c3"] = bench_config(S, local, "Chung-Lu n=8M, exponent 2.1 in [5, 200000], planted communities "
                                  "10..500, mu 0.2, seed 3", scdgen.workload("chunglu-8m"), min(args.steps, 5),
                                  min(args.warmup, 3))
    if not args.no_batched:
        line["batched"] = bench_batched(S, local, args)
    if not args.no_served:
        line["served"] = bench_served(S, local, args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def bench_plain(S, args, world, rank, local, dist):
    """The headline: plain SCD on one R-MAT graph, device-resident and end to end."""
    import numpy as np
    import torch

    import scdgen

    t0 = time.time()
    pairs = scdgen.rmat(args.scale, 16, 0.57, 0.19, 0.19, seed=22)
    gen_s = time.time() - t0
    E = pairs.shape[0]
    dev_pairs = torch.from_numpy(pairs.view(np.int32)).cuda()
    host_pairs = torch.from_numpy(pairs.view(np.int32)).pin_memory()

    # timed engine: CUDA events around the preprocessing phases (the triangle-counting
    # phase gives the roofline), iterations replayed from captured CUDA graphs
    eng = S.Engine(local, flags=S.FLAG_PROFILE)
    stream = torch.cuda.ExternalStream(eng.stream())

    def step_device():
        eng.convert_edges(device_ptr=dev_pairs.data_ptr(), count=E)
        return eng.run(0.01, 1000)

    def step_e2e():
        rc = S.lib().scd_convert_edges(eng._ctx, host_pairs.data_ptr(), E, 0)
        eng._check(rc)
        r = eng.run(0.01, 1000)
        lab = eng.labels_from_device()
        return r, lab

    for _ in range(args.warmup):
        r = step_device()
    torch.cuda.synchronize()
    eng.profile_reset()
    launches0 = eng.kernel_launches()
    clocks = ClockSampler()
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        r = step_device()
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    dev_ms = ev0.elapsed_time(ev1) / args.steps
    launches = eng.kernel_launches() - launches0
    tc_ms, tc_n = eng.profile("tc")
    ck = clocks.stop()
    # e2e through the public API with host buffers
    for _ in range(1):
        step_e2e()
    torch.cuda.synchronize()
    t = time.perf_counter()
    e_ev0, e_ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_ev0.record(stream)
    for _ in range(args.steps):
        r2, lab = step_e2e()
    e_ev1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t) * 1e3 / args.steps
    n, m, cc = eng.graph_info()
    # end to end from the edge-list TEXT in host memory (device parse, as read_edges + convert + main-gpu)
    import tempfile
    with tempfile.NamedTemporaryFile(suffix=".txt", delete=False) as f:
        tpath = f.name
    scdgen.write_text(tpath, pairs)
    with open(tpath, "rb") as f:
        text = f.read()
    os.unlink(tpath)
    # the text in pinned host memory (as the pairs of the e2e step): read by DMA at full speed
    text_pin = torch.from_numpy(np.frombuffer(text, dtype=np.uint8).copy()).pin_memory()
    text_ptr = ctypes.cast(text_pin.data_ptr(), ctypes.c_char_p)

    def step_text():
        eng._check(S.lib().scd_convert_text(eng._ctx, text_ptr, len(text), 0))
        r = eng.run(0.01, 1000)
        return r, eng.labels_from_device()

    step_text()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(args.steps):
        step_text()
    torch.cuda.synchronize()
    text_ms = (time.perf_counter() - t) * 1e3 / args.steps

    dev_ms, e2e_ms = max_over_ranks(dist, [dev_ms, e2e_ms], "cuda")

    # roofline of the dominant kernel: preprocessing triangle counting
    gd = eng.graph_download()
    b_tc, tcinfo = algorithmic_tc_bytes(gd["indices"], gd["adj"])
    tc_avg = tc_ms / max(tc_n, 1)
    # phase breakdown: a separate engine launching the iterations kernel by kernel
    peng = S.Engine(local, flags=S.FLAG_PROFILE | S.FLAG_NO_GRAPHS)
    for i in range(2):
        if i == 1:
            torch.cuda.synchronize()
            peng.profile_reset()
        peng.convert_edges(device_ptr=dev_pairs.data_ptr(), count=E)
        peng.run(0.01, 1000)
    torch.cuda.synchronize()
    prof = {p: peng.profile(p) for p in S.PHASES}
    peng.close()
    peak, peak_kind = measured_peak_gbs()
    achieved = b_tc / (tc_avg / 1e3) / 1e9
    traffic = measured_traffic("tc", args.scale)
    # the other stages against the same peak (phase times of the kernel-by-kernel run)
    b_pre = 16 * E + 4 * (n + 1) + 8 * m
    pre_ms = prof["convert"][0] - prof["tc"][0]
    b_it, itinfo = iteration_bytes(gd["indices"], gd["adj"], eng.labels_from_device())
    it_ms = sum(prof[k][0] / max(prof[k][1], 1) for k in ("improve", "stats", "wcc"))   # one call of each
    stages = {"preprocess_sort_csr": {"bytes": b_pre, "ms": pre_ms, "gbs": b_pre / pre_ms / 1e6},
              "triangle_count": {"bytes": b_tc, "ms": tc_avg, "gbs": achieved},
              "iteration": {"bytes": b_it, "ms": it_ms, "gbs": b_it / it_ms / 1e6, **itinfo,
                            "labels": "best labels of the run"}}
    for v in stages.values():
        v["frac"] = v["gbs"] / peak

    line = {"metric": METRIC, "value": job_throughput(world, E, dev_ms), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64", "data": "synthetic",
            "config": {"workload": f"rmat-{args.scale}", "edge_factor": 16, "abcd": [0.57, 0.19, 0.19, 0.05],
                       "edges_in": E, "n": n, "m": m, "iterations": r["iterations"], "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2 (edge list %d MB)" % (E * 8 >> 20)},
            "e2e": {"value": job_throughput(world, E, e2e_ms), "unit": UNIT, "h2d_bytes_per_step": E * 8,
                    "d2h_bytes_per_step": n * 4 + 8 * (r2["iterations"] + 1)},
            "e2e_text": {"value": world * E / (text_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": len(text),
                         "d2h_bytes_per_step": n * 4 + 8 * (r2["iterations"] + 1),
                         "note": "from the edge-list text in pinned host memory: device parse + preprocessing + SCD + labels"},
            "gpu_launches": launches,
            "phases_ms": {p: round(v[0], 3) for p, v in prof.items()},
            "roofline": {"kernel": "k_tc_core + k_tc_cta + k_tc_warp + k_tc_small (preprocessing triangle counting)",
                         "bound": "hbm",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "algorithmic_bytes": b_tc, "ms_per_launch": tc_avg,
                         "traffic": traffic},
            "stages": stages,
            "clocks": ck, "generate_s": round(gen_s, 2)}
    best_labels = eng.labels_from_device()
    line["wcc_static"] = time_wcc_static(S, eng, gd)
    eng.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        model = cpu_model()
        if args.cpu_full:
            t0 = time.time()
            v, t_ms, split, r_cpu = cpu_full_run(pairs)
            line["cpu_baseline"] = {
                "value": v, "unit": UNIT, "cores": oracle.threads(), "kind": "port", "cpu_model": model,
                "sample": f"the full workload (R-MAT scale {args.scale}, {E} edges), one run; reference timers: "
                          "process graph + initial partition + initial WCC + iterations",
                "ms": t_ms, "ms_split": split, "iterations": r_cpu["iters"],
                "labels_identical_to_engine": bool(np.array_equal(r_cpu["best_labels"], best_labels)),
                "wall_s": round(time.time() - t0, 1)}
            line["speedup_vs_cpu"] = {"e2e": line["e2e"]["value"] / v, "device_resident": line["value"] / v,
                                      "note": "same workload, same host: engine e2e vs the CPU path of the line's cpu_baseline"}
        vs, ts, es, kind = cpu_sample_run()
        key = "cpu_baseline_sample" if args.cpu_full else "cpu_baseline"
        line[key] = {"value": vs, "unit": UNIT, "cores": oracle.threads(), "kind": kind, "cpu_model": model,
                     "sample": f"R-MAT scale {CPU_SAMPLE_SCALE} ({es} edges), same generator; "
                               f"{ts:.0f} ms of reference-timer CPU work (the reference arm's per-step sample)"}
    return line


if __name__ == "__main__":
    main()
