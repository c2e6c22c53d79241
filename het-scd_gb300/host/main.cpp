// main <filename>
//
// Drop-in for the reference's CPU driver `main` (src/main.cpp:29-94): the same
// argv and stdout layout, with the whole run on GPU 0 through scd_run (initial
// partition, initial WCC and the refinement loop on the device).  There is no
// CPU code path: "num. threads" reports the one host thread driving the GPU.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>

#include "graph_io.hpp"
#include "scd_gb300.h"

using namespace std;

int main(int argc, char *argv[]) {
    if (argc < 2) {
        cerr << "usage: " << argv[0] << " <filename>" << endl;
        return EXIT_FAILURE;
    }
    const double alpha = 1.0, threshold = 0.01;
    double t = scdio::wall_ms();
    scdio::HostGraph g;
    string err = scdio::read_graph(argv[1], g);
    if (!err.empty()) {
        cerr << err << endl;
        return EXIT_FAILURE;
    }
    cout << "load graph: " << scdio::wall_ms() - t << " ms" << endl;
    scd_ctx *ctx = nullptr;
    if (scd_create(&ctx, 0, 256, 0) != SCD_OK) {
        cerr << "no CUDA device" << endl;
        return EXIT_FAILURE;
    }
    if (scd_transfer_graph(ctx, g.n, g.m, g.indices.data(), g.adj.data(), g.tri.data(), g.tri_deg.data(), alpha)) {
        cerr << scd_last_error(ctx) << endl;
        scd_destroy(ctx);
        return EXIT_FAILURE;
    }
    const int max_iters = 100000;
    vector<double> trace(max_iters);
    scd_result r;
    int rc = g.n ? scd_run(ctx, threshold, max_iters, trace.data(), &r) : SCD_ERR_LIMIT;
    if (rc != SCD_OK) {
        cerr << (g.n ? scd_last_error(ctx) : "empty graph: the WCC stays 0 and the loop would not end") << endl;
        scd_destroy(ctx);
        return EXIT_FAILURE;
    }
    double cc = 0;
    scd_graph_info(ctx, nullptr, nullptr, &cc);
    cout << "create initial partition + compute WCC: " << r.ms_partition << " ms" << endl;
    cout << endl;
    cout << "nodes: " << g.n << endl;
    cout << "edges: " << g.m << endl;
    cout << "avg. cc: " << cc << endl;
    cout << "initial WCC: " << r.initial_wcc << endl;
    cout << "num. threads: 1" << endl;
    cout << endl;
    for (int i = 0; i < r.iterations; i++) {
        cout << "WCC: " << trace[i] << endl;
        cout << endl;
    }
    cout << "----------------------------------------" << endl;
    cout << "num. communities: " << r.printed_communities << endl;
    cout << "WCC: " << r.best_wcc << endl;
    cout << "iterations: " << r.iterations << endl;
    cout << "time per iteration: " << r.ms_iterations / r.iterations << " ms" << endl;
    cout << "----------------------------------------" << endl;
    scd_destroy(ctx);
    return EXIT_SUCCESS;
}
