// convert <input file> <output file>
//
// Drop-in for the reference's `convert` (src/convert.cpp:466-537): reads the
// text edge list on the host, runs the preprocessing on the GPU through the C
// ABI (scd_convert_edges) and writes the binary graph format.
// Optional third argument: CUDA device ordinal (default 0).
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "graph_io.hpp"
#include "scd_gb300.h"

using namespace std;

int main(int argc, char **argv) {
    if (argc < 3) {
        cerr << "usage: " << argv[0] << " <input file> <output file>" << endl;
        return -1;
    }
    const int device = argc > 3 ? atoi(argv[3]) : 0;
    double t0 = scdio::wall_ms();
    cout << "reading graph from file " << argv[1] << endl;
    vector<uint32_t> pairs;
    uint32_t num_nodes = 0;
    string err = scdio::read_edge_text(argv[1], pairs, num_nodes);
    if (!err.empty()) {
        cerr << err << endl;
        return -1;
    }
    cout << "found " << num_nodes << " nodes and " << pairs.size() / 2 << " edges" << endl;
    cout << "read input: " << scdio::wall_ms() - t0 << " ms" << endl;

    scd_ctx *ctx = nullptr;
    int rc = scd_create(&ctx, device, 256, 0);
    if (rc != SCD_OK) {
        cerr << "could not open CUDA device " << device << " (status " << rc << ")" << endl;
        return -1;
    }
    double t1 = scdio::wall_ms();
    rc = scd_convert_edges(ctx, pairs.data(), pairs.size() / 2, 0);
    if (rc != SCD_OK) {
        cerr << "preprocessing failed: " << scd_last_error(ctx) << endl;
        scd_destroy(ctx);
        return -1;
    }
    cout << "process graph: " << scdio::wall_ms() - t1 << " ms" << endl;

    scdio::HostGraph g;
    scd_graph_info(ctx, &g.n, &g.m, nullptr);
    g.indices.resize((size_t)g.n + 1);
    g.adj.resize(2 * (size_t)g.m);
    g.tri.resize(g.n);
    g.tri_deg.resize(g.n);
    rc = scd_graph_download(ctx, g.indices.data(), g.adj.data(), g.tri.data(), g.tri_deg.data());
    scd_destroy(ctx);
    if (rc != SCD_OK) {
        cerr << "could not copy the graph back" << endl;
        return -1;
    }
    cout << "final graph has " << g.n << " nodes and " << g.m << " edges" << endl;
    cout << "writing final graph to " << argv[2] << endl;
    double t2 = scdio::wall_ms();
    err = scdio::write_graph(argv[2], g);
    if (!err.empty()) {
        cerr << err << endl;
        return -1;
    }
    cout << "write output: " << scdio::wall_ms() - t2 << " ms" << endl;
    return 0;
}
