// main-gpu <filename> <device> [group size]
//
// Drop-in for the reference's `main-gpu` (src/main-gpu.cpp:30-113): the same
// argv and the same stdout lines, with every stage on the GPU through the C ABI
// (the reference computes the initial partition and the initial WCC on the CPU,
// src/main-gpu.cpp:54-55).  The refinement loop below is the reference's loop
// with cuda_* calls replaced by their scd_* equivalents.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>

#include "graph_io.hpp"
#include "scd_gb300.h"

using namespace std;

static int fail(scd_ctx *ctx, const char *what) {
    cerr << what << ": " << (ctx ? scd_last_error(ctx) : "") << endl;
    if (ctx) scd_destroy(ctx);
    return EXIT_FAILURE;
}

int main(int argc, char *argv[]) {
    if (argc < 2) {
        cerr << "usage: " << argv[0] << " <filename> <device> [group size]" << endl;
        return EXIT_FAILURE;
    }
    const double threshold = 0.01, alpha = 1.0;
    const int work_group_size = argc >= 4 ? atoi(argv[3]) : 256;
    const int device = argc >= 3 ? atoi(argv[2]) : -1;

    scd_ctx *ctx = nullptr;
    if (scd_create(&ctx, device, work_group_size, 0) != SCD_OK) {
        cerr << "Please select a CUDA-enabled device" << endl;
        return EXIT_FAILURE;
    }
    cout << "selected device: " << device << endl;

    double t = scdio::wall_ms();
    scdio::HostGraph g;
    string err = scdio::read_graph(argv[1], g);
    if (!err.empty()) {
        cerr << err << endl;
        scd_destroy(ctx);
        return EXIT_FAILURE;
    }
    cout << "load graph: " << scdio::wall_ms() - t << " ms" << endl;

    t = scdio::wall_ms();
    if (scd_transfer_graph(ctx, g.n, g.m, g.indices.data(), g.adj.data(), g.tri.data(), g.tri_deg.data(), alpha))
        return fail(ctx, "transfer graph to device");
    cout << "transfer graph to device: " << scdio::wall_ms() - t << " ms" << endl;

    t = scdio::wall_ms();
    uint32_t initial_comms = 0;
    if (scd_initial_partition(ctx, &initial_comms)) return fail(ctx, "create initial partition");
    cout << "create initial partition: " << scdio::wall_ms() - t << " ms" << endl;
    t = scdio::wall_ms();
    double best_wcc = 0;
    if (scd_compute_wcc(ctx, &best_wcc)) return fail(ctx, "compute WCC");
    cout << "compute WCC: " << scdio::wall_ms() - t << " ms" << endl;
    double cc = 0;
    scd_graph_info(ctx, nullptr, nullptr, &cc);

    cout << endl;
    cout << "nodes: " << g.n << endl;
    cout << "edges: " << g.m << endl;
    cout << "avg. cc: " << cc << endl;
    cout << "initial WCC: " << best_wcc << endl;
    cout << "work group size: " << work_group_size << endl;
    cout << endl;

    double before = scdio::wall_ms();
    int iters = 0;
    while (1) {
        iters++;
        t = scdio::wall_ms();
        double wcc = 0;
        if (scd_improve_labels(ctx, &wcc)) return fail(ctx, "improve labels");
        if (wcc > best_wcc && scd_store_labels(ctx)) return fail(ctx, "store labels");
        cout << "iteration: " << scdio::wall_ms() - t << " ms" << endl;
        cout << "WCC: " << wcc << endl;
        cout << endl;
        if (wcc < best_wcc * (1 + threshold)) break;   // src/main-gpu.cpp:89-92
        best_wcc = wcc;
        if (g.n == 0) break;   // the reference loops forever here (WCC stays 0)
    }
    double after = scdio::wall_ms();

    t = scdio::wall_ms();
    vector<uint32_t> best_labels(g.n);
    if (scd_labels_from_device(ctx, best_labels.data())) return fail(ctx, "transfer labels back");
    cout << "transfer labels back: " << scdio::wall_ms() - t << " ms" << endl;

    // compress_labels (src/scd.cpp:32-55) prints n minus the number of distinct
    // valid labels because of its inverted branch; reproduced for parity.
    vector<char> seen(initial_comms + 1, 0);
    uint32_t distinct = 0;
    for (uint32_t l : best_labels)
        if (l != SCD_INVALID_LABEL && l < initial_comms && !seen[l]) {
            seen[l] = 1;
            distinct++;
        }
    if (getenv("SCD_LABELS_OUT")) {
        FILE *f = fopen(getenv("SCD_LABELS_OUT"), "wb");
        if (f) {
            fwrite(best_labels.data(), 4, best_labels.size(), f);
            fclose(f);
        }
    }
    cout << "----------------------------------------" << endl;
    cout << "num. communities: " << g.n - distinct << endl;
    cout << "WCC: " << best_wcc << endl;
    cout << "iterations: " << iters << endl;
    cout << "time per iteration: " << (after - before) / iters << " ms" << endl;
    cout << "----------------------------------------" << endl;
    scd_destroy(ctx);
    return EXIT_SUCCESS;
}
