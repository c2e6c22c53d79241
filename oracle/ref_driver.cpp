/*
 * ref_driver — runs the REFERENCE implementation (its graph.cpp, scd.cpp,
 * wcc.cpp and common.cpp, compiled unmodified by oracle/build_ref.sh) through
 * the refinement loop of src/main.cpp:42-93 and dumps everything the reference
 * `main` only prints or keeps in memory: p_ext, the initial partition and its
 * statistics, per-iteration labels/statistics/WCC, the best labels and the
 * printed community count.  Test infrastructure: it pins the oracle
 * restatement and produces the golden traces; it is never part of the product.
 *
 * usage: ref_driver <graph file> <trace out> [max iterations] [labels file]
 * With a labels file (u32[n], SCD_INVALID_LABEL for none) the loop starts from
 * that labelling instead of create_initial_partition: the Partition gets those
 * labels, num_communities = largest label + 1, and the reference's own
 * collect_stats fills its statistics (what cuda_labels_to_device and the
 * engine's scd_labels_to_device do).
 * Trace layout (little-endian): "SCDTRACE", u32 n, m, num_comms, iters,
 * f64 p_ext, initial_wcc, best_wcc, u32 printed_comms, u32 labels0[n],
 * i32 sizes0/ext0/int0[num_comms], then per iteration f64 wcc, u32 labels[n],
 * i32 sizes/ext/int[num_comms], and finally u32 best_labels[n].
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "graph.hpp"
#include "scd.hpp"
#include "wcc.hpp"

static void put(FILE *f, const void *p, size_t bytes) {
    if (bytes && fwrite(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "write failed\n");
        exit(2);
    }
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s <graph> <trace out> [max iterations]\n", argv[0]);
        return 1;
    }
    int max_iters = argc > 3 ? atoi(argv[3]) : 1000;
    const double alpha = 1.0, threshold = 0.01;
    const Graph *g = Graph::read(argv[1]);
    if (!g) return 1;
    const unsigned n = g->n;

    Partition *p = nullptr;
    if (argc > 4) {
        FILE *lf = fopen(argv[4], "rb");
        if (!lf) return 1;
        p = new Partition;
        p->labels = new unsigned int[n];
        if (fread(p->labels, 4, n, lf) != n) {
            fprintf(stderr, "short labels file\n");
            return 1;
        }
        fclose(lf);
        unsigned nc = 0;
        for (unsigned v = 0; v < n; v++)
            if (p->labels[v] != INVALID_LABEL && p->labels[v] + 1 > nc) nc = p->labels[v] + 1;
        p->num_communities = nc;
        p->sizes = new int[n];
        p->ext_edges = new int[n];
        p->int_edges = new int[n];
        collect_stats(g, p);
    } else {
        p = create_initial_partition(g);
    }
    double best_wcc = compute_wcc(g, p, alpha);
    const unsigned nc = p->num_communities;

    std::vector<unsigned> labels0(p->labels, p->labels + n), best(p->labels, p->labels + n);
    std::vector<int> stats0;
    stats0.insert(stats0.end(), p->sizes, p->sizes + nc);
    stats0.insert(stats0.end(), p->ext_edges, p->ext_edges + nc);
    stats0.insert(stats0.end(), p->int_edges, p->int_edges + nc);
    const double wcc0 = best_wcc;

    std::vector<double> wccs;
    std::vector<unsigned> trace_labels;
    std::vector<int> trace_stats;
    int iters = 0;
    while (iters < max_iters) {
        iters++;
        improve_partition(g, p, alpha);
        collect_stats(g, p);
        double wcc = compute_wcc(g, p, alpha);
        if (wcc > best_wcc) best.assign(p->labels, p->labels + n);
        wccs.push_back(wcc);
        trace_labels.insert(trace_labels.end(), p->labels, p->labels + n);
        trace_stats.insert(trace_stats.end(), p->sizes, p->sizes + nc);
        trace_stats.insert(trace_stats.end(), p->ext_edges, p->ext_edges + nc);
        trace_stats.insert(trace_stats.end(), p->int_edges, p->int_edges + nc);
        if (wcc < best_wcc * (1 + threshold)) break;
        best_wcc = wcc;
    }
    std::vector<unsigned> best_copy = best;
    unsigned printed = 0;
    compress_labels(g, best_copy.data(), &printed);

    FILE *f = fopen(argv[2], "wb");
    if (!f) return 1;
    put(f, "SCDTRACE", 8);
    unsigned hdr[4] = {n, g->m, nc, (unsigned)iters};
    put(f, hdr, sizeof hdr);
    double dd[3] = {g->clustering_coef, wcc0, best_wcc};
    put(f, dd, sizeof dd);
    put(f, &printed, 4);
    put(f, labels0.data(), 4 * (size_t)n);
    put(f, stats0.data(), 4 * stats0.size());
    for (int i = 0; i < iters; i++) {
        put(f, &wccs[i], 8);
        put(f, trace_labels.data() + (size_t)i * n, 4 * (size_t)n);
        put(f, trace_stats.data() + (size_t)i * 3 * nc, 4 * 3 * (size_t)nc);
    }
    put(f, best.data(), 4 * (size_t)n);
    return fclose(f) == 0 ? 0 : 1;
}
