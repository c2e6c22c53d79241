#include "graph_io.hpp"

#include <sys/time.h>

#include <cstdio>
#include <cstring>

namespace scdio {

double wall_ms() {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return tv.tv_sec * 1000.0 + tv.tv_usec / 1000.0;
}

static inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }
static inline bool is_digit(char c) { return c >= '0' && c <= '9'; }

std::string read_edge_text(const std::string &path, std::vector<uint32_t> &pairs, uint32_t &num_nodes) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return "could not open " + path;
    num_nodes = 0;
    std::vector<char> buf(1 << 22);
    std::string carry;
    size_t line_no = 0;
    std::string err;
    auto parse_line = [&](const char *s, size_t len) -> bool {
        line_no++;
        if (len > 1023) {
            err = "an error occured while reading input file";
            return false;
        }
        size_t k = 0;
        while (k < len && is_space(s[k])) k++;
        if (k == len || s[k] == '#') return true;
        if (!is_digit(s[k])) {
            err = "line " + std::to_string(line_no) + " is corrupt";
            return false;
        }
        uint32_t a = 0, b = 0;
        while (k < len && is_digit(s[k])) a = 10u * a + (uint32_t)(s[k++] - '0');
        while (k < len && is_space(s[k])) k++;
        if (k == len || !is_digit(s[k])) {
            err = "line " + std::to_string(line_no) + " is corrupt";
            return false;
        }
        while (k < len && is_digit(s[k])) b = 10u * b + (uint32_t)(s[k++] - '0');
        pairs.push_back(a < b ? a : b);
        pairs.push_back(a < b ? b : a);
        uint32_t hi = (a > b ? a : b) + 1;
        if (hi > num_nodes) num_nodes = hi;
        return true;
    };
    bool ok = true;
    size_t got;
    while (ok && (got = fread(buf.data(), 1, buf.size(), f)) > 0) {
        size_t start = 0;
        for (size_t i = 0; i < got && ok; i++) {
            if (buf[i] != '\n') continue;
            if (!carry.empty()) {
                carry.append(buf.data() + start, i - start);
                ok = parse_line(carry.data(), carry.size());
                carry.clear();
            } else {
                ok = parse_line(buf.data() + start, i - start);
            }
            start = i + 1;
        }
        if (ok) carry.append(buf.data() + start, got - start);
    }
    if (ok && !carry.empty()) ok = parse_line(carry.data(), carry.size());
    if (ferror(f)) {
        ok = false;
        err = "an error occured while reading input file";
    }
    fclose(f);
    return ok ? "" : err;
}

std::string write_graph(const std::string &path, const HostGraph &g) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return "an error occured while writing output file";
    bool ok = fwrite(&g.n, 4, 1, f) == 1 && fwrite(&g.m, 4, 1, f) == 1 &&
              fwrite(g.indices.data(), 4, (size_t)g.n + 1, f) == (size_t)g.n + 1 &&
              fwrite(g.adj.data(), 4, 2 * (size_t)g.m, f) == 2 * (size_t)g.m &&
              fwrite(g.tri.data(), 4, g.n, f) == g.n && fwrite(g.tri_deg.data(), 4, g.n, f) == g.n;
    ok = (fclose(f) == 0) && ok;
    return ok ? "" : "an error occured while writing output file";
}

std::string read_graph(const std::string &path, HostGraph &g) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return "failed to open " + path;
    uint32_t hdr[2];
    std::string err = "error while reading " + path;
    if (fread(hdr, 4, 2, f) != 2) {
        fclose(f);
        return err;
    }
    g.n = hdr[0];
    g.m = hdr[1];
    g.indices.resize((size_t)g.n + 1);
    g.adj.resize(2 * (size_t)g.m);
    g.tri.resize(g.n);
    g.tri_deg.resize(g.n);
    bool ok = fread(g.indices.data(), 4, (size_t)g.n + 1, f) == (size_t)g.n + 1 &&
              fread(g.adj.data(), 4, 2 * (size_t)g.m, f) == 2 * (size_t)g.m &&
              fread(g.tri.data(), 4, g.n, f) == g.n && fread(g.tri_deg.data(), 4, g.n, f) == g.n;
    ok = ok && fgetc(f) == EOF;
    fclose(f);
    return ok ? "" : err;
}

}  // namespace scdio
