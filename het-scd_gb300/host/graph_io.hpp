// Host-side file formats of the SCD tools: the text edge list `convert` reads
// (src/convert.cpp:74-138) and the binary graph format it writes and
// main/main-gpu read (src/convert.cpp:430-455, src/graph.cpp:86-134).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace scdio {

struct HostGraph {
    uint32_t n = 0, m = 0;
    std::vector<uint32_t> indices, adj;
    std::vector<int32_t> tri, tri_deg;
};

// Text edge list: one "a b" pair per line, leading blanks skipped, empty lines
// and lines starting with '#' ignored, order of the two ids irrelevant.
// Appends (min, max) per line in file order; num_nodes = max id + 1.
// Returns "" on success, else an error message (the reference prints it and
// exits, src/convert.cpp:92-95,108-111,132-135).
std::string read_edge_text(const std::string &path, std::vector<uint32_t> &pairs, uint32_t &num_nodes);

// Binary graph: u32 n | u32 m | u32 indices[n+1] | u32 adj[2m] | i32 tri[n] |
// i32 tri_deg[n], and nothing after (the reader checks end of file).
std::string write_graph(const std::string &path, const HostGraph &g);
std::string read_graph(const std::string &path, HostGraph &g);

double wall_ms();

}  // namespace scdio
