/*
 * CPU restatement of the reference SCD path (test infrastructure only: the
 * parity checker and the timed CPU baseline; never linked into the product).
 * Each function cites the reference lines it follows.  The parallel structure
 * (OpenMP loops, atomics, per-thread sorts) follows the reference's so that the
 * timed baseline does the same work; all floating-point sums are index-ordered,
 * which equals the reference at OMP_NUM_THREADS=1.
 */
#include "scd_oracle.h"

#include <omp.h>
#include <sys/time.h>

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <utility>
#include <vector>

typedef std::pair<uint32_t, uint32_t> Edge;

static double now_ms() {
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return tv.tv_sec * 1000.0 + tv.tv_usec / 1000.0;
}

/* Parallel sort with the reference's shape (src/convert.cpp:33-65): every thread
 * sorts one contiguous slice, then slices are merged pairwise in log2(T) rounds.
 * Equal elements are identical values, so the result equals any correct sort. */
template <typename It, typename Cmp>
static void slice_merge_sort(It first, It last, Cmp cmp) {
    const size_t len = (size_t)(last - first);
    const int T = omp_get_max_threads();
#pragma omp parallel num_threads(T)
    {
        const size_t t = (size_t)omp_get_thread_num();
        std::sort(first + len * t / T, first + len * (t + 1) / T, cmp);
    }
    for (size_t width = 1; width < (size_t)T; width *= 2) {
#pragma omp parallel num_threads(T)
        {
            const size_t t = (size_t)omp_get_thread_num();
            const size_t lo = std::min(len * (2 * t) * width / T, len);
            const size_t mid = std::min(len * (2 * t + 1) * width / T, len);
            const size_t hi = std::min(len * (2 * t + 2) * width / T, len);
            if (mid != hi) std::inplace_merge(first + lo, first + mid, first + hi, cmp);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* convert                                                                   */

extern "C" int orc_read_text(const char *path, uint32_t **pairs_out, int64_t *count,
                             uint32_t *num_nodes) {
    /* src/convert.cpp:74-138: lines of at most 1023 characters; leading blanks
     * skipped; empty and '#' lines ignored; two unsigned decimal fields. */
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    std::vector<uint32_t> out;
    uint32_t nn = 0;
    char line[1024];
    int rc = 0;
    while (fgets(line, sizeof line, f)) {
        size_t k = 0;
        while (isspace((unsigned char)line[k])) k++;
        if (line[k] == '\0' || line[k] == '#') continue;
        if (!isdigit((unsigned char)line[k])) { rc = -2; break; }
        uint32_t a = 0, b = 0;
        while (isdigit((unsigned char)line[k])) a = 10u * a + (uint32_t)(line[k++] - '0');
        while (isspace((unsigned char)line[k])) k++;
        if (!isdigit((unsigned char)line[k])) { rc = -2; break; }
        while (isdigit((unsigned char)line[k])) b = 10u * b + (uint32_t)(line[k++] - '0');
        out.push_back(std::min(a, b));
        out.push_back(std::max(a, b));
        nn = std::max(std::max(a, b) + 1, nn);
    }
    fclose(f);
    if (rc) return rc;
    uint32_t *p = (uint32_t *)malloc(std::max<size_t>(out.size(), 1) * sizeof(uint32_t));
    if (!out.empty()) memcpy(p, out.data(), out.size() * sizeof(uint32_t));
    *pairs_out = p;
    *count = (int64_t)(out.size() / 2);
    *num_nodes = nn;
    return 0;
}

extern "C" int orc_convert(const uint32_t *pairs, int64_t count, orc_graph *out, orc_times *tm) {
    double t0 = now_ms();
    std::vector<Edge> edges((size_t)count);
    uint32_t max_id = 0;
    for (int64_t i = 0; i < count; i++) {
        edges[(size_t)i] = Edge(pairs[2 * i], pairs[2 * i + 1]);
        max_id = std::max(max_id, std::max(pairs[2 * i], pairs[2 * i + 1]));
    }
    uint32_t n = count ? max_id + 1 : 0;

    /* src/convert.cpp:141-170: renumber by first appearance, scanning each pair's
     * first then second component in file order */
    {
        std::vector<uint32_t> rename(n, ORC_INVALID);
        uint32_t next = 0;
        for (size_t i = 0; i < edges.size(); i++) {
            uint32_t a = edges[i].first, b = edges[i].second;
            if (rename[a] == ORC_INVALID) rename[a] = next++;
            if (rename[b] == ORC_INVALID) rename[b] = next++;
            edges[i] = Edge(std::min(rename[a], rename[b]), std::max(rename[a], rename[b]));
        }
        n = next;
    }

    /* src/convert.cpp:500-509 + 252-268: lexicographic sort, drop loops and repeats */
    slice_merge_sort(edges.begin(), edges.end(), std::less<Edge>());
    {
        size_t w = 0;
        for (size_t i = 0; i < edges.size(); i++)
            if (edges[i].first != edges[i].second && (i == 0 || edges[i] != edges[i - 1]))
                edges[w++] = edges[i];
        edges.resize(w);
    }

    /* src/convert.cpp:271-351: per-edge triangle counts over the id-oriented list */
    double t1 = now_ms();
    const size_t E = edges.size();
    std::vector<int32_t> tri(n, 0), tri_deg(n, 0);
    {
        std::vector<uint32_t> row(n + 1, 0);
        for (size_t i = 0; i < E; i++) row[edges[i].first + 1]++;
        for (uint32_t v = 0; v < n; v++) row[v + 1] += row[v];
        std::vector<int32_t> t(E, 0);
#pragma omp parallel for schedule(guided)
        for (size_t e = 0; e < E; e++) {
            uint32_t a = row[edges[e].first], a_end = row[edges[e].first + 1];
            uint32_t b = row[edges[e].second], b_end = row[edges[e].second + 1];
            /* branches, not a branch-free a += x <= y: the merge runs ahead on the
             * branch predictor instead of waiting for each comparison, as the
             * reference's loop does (a branch-free form ran at half its speed) */
            while (a < a_end && b < b_end) {
                uint32_t x = edges[a].second, y = edges[b].second;
                if (x == y) {
#pragma omp atomic
                    t[e]++;
#pragma omp atomic
                    t[a]++;
#pragma omp atomic
                    t[b]++;
                }
                if (x <= y) a++;
                if (x >= y) b++;
            }
        }
#pragma omp parallel for schedule(guided)
        for (size_t e = 0; e < E; e++) {
            int32_t c = t[e];
            if (c > 0) {
                uint32_t p = edges[e].first, q = edges[e].second;
#pragma omp atomic
                tri_deg[p]++;
#pragma omp atomic
                tri_deg[q]++;
                /* int32 wrap like the reference's int accumulators */
#pragma omp atomic
                tri[p] += c;
#pragma omp atomic
                tri[q] += c;
            }
        }
        size_t w = 0;
        for (size_t e = 0; e < E; e++)
            if (t[e] > 0) edges[w++] = edges[e];
        edges.resize(w);
    }
    double t2 = now_ms();

    /* src/convert.cpp:354-414: rank vertices by (degree, id) descending, drop
     * degree-0 vertices (they rank last) */
    {
        const size_t F = edges.size();
        std::vector<uint32_t> deg(n, 0);
#pragma omp parallel for schedule(guided)
        for (size_t e = 0; e < F; e++) {
#pragma omp atomic
            deg[edges[e].first]++;
#pragma omp atomic
            deg[edges[e].second]++;
        }
        std::vector<Edge> order(n);
#pragma omp parallel for schedule(guided)
        for (uint32_t v = 0; v < n; v++) order[v] = Edge(deg[v], v);
        slice_merge_sort(order.begin(), order.end(), std::greater<Edge>());
        std::vector<uint32_t> rank(n);
        std::vector<int32_t> tri2(n), tri_deg2(n);
#pragma omp parallel for schedule(guided)
        for (uint32_t r = 0; r < n; r++) {
            uint32_t old = order[r].second;
            rank[old] = r;
            tri2[r] = tri[old];
            tri_deg2[r] = tri_deg[old];
        }
        uint32_t nn = 0;
#pragma omp parallel for schedule(guided) reduction(max : nn)
        for (size_t e = 0; e < F; e++) {
            edges[e].first = rank[edges[e].first];
            edges[e].second = rank[edges[e].second];
            nn = std::max(nn, std::max(edges[e].first, edges[e].second) + 1);
        }
        n = nn;
        tri.swap(tri2);
        tri_deg.swap(tri_deg2);
    }
    double t3 = now_ms();

    /* src/convert.cpp:417-463: both directions, sorted, as CSR */
    const size_t F = edges.size();
    edges.resize(2 * F);
#pragma omp parallel for
    for (size_t e = 0; e < F; e++) edges[F + e] = Edge(edges[e].second, edges[e].first);
    slice_merge_sort(edges.begin(), edges.end(), std::less<Edge>());

    out->n = n;
    out->m = (uint32_t)F;
    out->indices = (uint32_t *)malloc(((size_t)n + 1) * sizeof(uint32_t));
    out->adj = (uint32_t *)malloc(std::max<size_t>(2 * F, 1) * sizeof(uint32_t));
    out->tri = (int32_t *)malloc(std::max<size_t>(n, 1) * sizeof(int32_t));
    out->tri_deg = (int32_t *)malloc(std::max<size_t>(n, 1) * sizeof(int32_t));
    std::fill(out->indices, out->indices + n + 1, 0u);
    for (size_t i = 0; i < 2 * F; i++) {
        out->indices[edges[i].first + 1]++;
        out->adj[i] = edges[i].second;
    }
    for (uint32_t v = 0; v < n; v++) out->indices[v + 1] += out->indices[v];
    if (n) {
        memcpy(out->tri, tri.data(), n * sizeof(int32_t));
        memcpy(out->tri_deg, tri_deg.data(), n * sizeof(int32_t));
    }
    if (tm) {
        tm->process_graph = t3 - t0;
        tm->tc = t2 - t1;
    }
    return 0;
}

extern "C" int orc_write_graph(const char *path, const orc_graph *g) {
    FILE *f = fopen(path, "wb");
    if (!f) return -1;
    size_t ok = 0, want = 0;
    ok += fwrite(&g->n, 4, 1, f); want += 1;
    ok += fwrite(&g->m, 4, 1, f); want += 1;
    ok += fwrite(g->indices, 4, (size_t)g->n + 1, f); want += (size_t)g->n + 1;
    ok += fwrite(g->adj, 4, 2 * (size_t)g->m, f); want += 2 * (size_t)g->m;
    ok += fwrite(g->tri, 4, g->n, f); want += g->n;
    ok += fwrite(g->tri_deg, 4, g->n, f); want += g->n;
    int rc = fclose(f);
    return (ok == want && rc == 0) ? 0 : -1;
}

extern "C" int orc_read_graph(const char *path, orc_graph *g) {
    /* src/graph.cpp:86-134: header, four arrays, then exactly end of file */
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    uint32_t hdr[2];
    if (fread(hdr, 4, 2, f) != 2) { fclose(f); return -2; }
    g->n = hdr[0];
    g->m = hdr[1];
    g->indices = (uint32_t *)malloc(((size_t)g->n + 1) * 4);
    g->adj = (uint32_t *)malloc(std::max<size_t>(2 * (size_t)g->m, 1) * 4);
    g->tri = (int32_t *)malloc(std::max<size_t>(g->n, 1) * 4);
    g->tri_deg = (int32_t *)malloc(std::max<size_t>(g->n, 1) * 4);
    bool ok = fread(g->indices, 4, (size_t)g->n + 1, f) == (size_t)g->n + 1 &&
              fread(g->adj, 4, 2 * (size_t)g->m, f) == 2 * (size_t)g->m &&
              fread(g->tri, 4, g->n, f) == g->n && fread(g->tri_deg, 4, g->n, f) == g->n;
    ok = ok && fgetc(f) == EOF;
    fclose(f);
    if (!ok) { orc_free_graph(g); return -2; }
    return 0;
}

extern "C" void orc_free_graph(orc_graph *g) {
    free(g->indices); free(g->adj); free(g->tri); free(g->tri_deg);
    g->indices = g->adj = NULL;
    g->tri = g->tri_deg = NULL;
}

/* ------------------------------------------------------------------------ */
/* SCD                                                                       */

static inline uint32_t degree(const orc_graph *g, uint32_t v) { return g->indices[v + 1] - g->indices[v]; }

extern "C" double orc_clustering_coef(const orc_graph *g) {
    /* src/graph.cpp:57-68: (1/n) sum over deg>1 of tri/(deg*(deg-1.0)) */
    std::vector<double> term(g->n, 0.0);
#pragma omp parallel for schedule(static, 16)
    for (uint32_t p = 0; p < g->n; p++) {
        uint32_t d = degree(g, p);
        if (d > 1) term[p] = g->tri[p] / (d * (d - 1.0));
    }
    double cc = 0.0;
    for (uint32_t p = 0; p < g->n; p++)
        if (degree(g, p) > 1) cc += term[p];
    return cc / g->n;
}

extern "C" uint32_t orc_initial_partition(const orc_graph *g, uint32_t *labels) {
    /* src/scd.cpp:113-157: order by ((cc, deg), id) descending, then each
     * still-unlabelled vertex opens a label and claims its unlabelled neighbours */
    const uint32_t n = g->n;
    typedef std::pair<std::pair<double, int>, uint32_t> Key;
    std::vector<Key> order(n);
    for (uint32_t p = 0; p < n; p++) {
        uint32_t d = degree(g, p);
        double cc = g->tri[p] / (d * (d - 1.0));
        order[p] = Key(std::make_pair(cc, (int)d), p);
    }
    std::sort(order.begin(), order.end(), std::greater<Key>());
    std::fill(labels, labels + n, ORC_INVALID);
    uint32_t next = 0;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t p = order[i].second;
        if (labels[p] != ORC_INVALID) continue;
        for (uint32_t j = g->indices[p]; j != g->indices[p + 1]; j++)
            if (labels[g->adj[j]] == ORC_INVALID) labels[g->adj[j]] = next;
        labels[p] = next++;
    }
    return next;
}

extern "C" void orc_collect_stats(const orc_graph *g, const uint32_t *labels, uint32_t num_comms,
                                  int32_t *sizes, int32_t *ext_edges, int32_t *int_edges) {
    /* src/scd.cpp:57-111 */
    std::fill(sizes, sizes + num_comms, 0);
    std::fill(ext_edges, ext_edges + num_comms, 0);
    std::fill(int_edges, int_edges + num_comms, 0);
#pragma omp parallel for schedule(dynamic, 512)
    for (uint32_t p = 0; p < g->n; p++) {
        uint32_t l = labels[p];
        if (l == ORC_INVALID) continue;
        int32_t same = 0, other = 0;
        for (uint32_t j = g->indices[p]; j != g->indices[p + 1]; j++) {
            if (labels[g->adj[j]] == l) same++;
            else other++;
        }
#pragma omp atomic
        sizes[l]++;
        if (other) {
#pragma omp atomic
            ext_edges[l] += other;
        }
        if (same) {
#pragma omp atomic
            int_edges[l] += same;
        }
    }
}

/* int products wrap in two's complement, as the reference's int arithmetic does */
static inline int imul(int a, int b) { return (int)((uint32_t)a * (uint32_t)b); }

extern "C" double orc_gain(int r, int d_in, int d_out, int c_out, double p_in, double p_ext,
                           double alpha) {
    /* src/scd.cpp:173-219, operation by operation */
    double t = r > 0 ? (c_out - d_in) / (double)r : 0.0;
    double A = 0.0, denom;
    denom = ((double)imul(d_in, d_in - 1) * p_in + (double)imul(d_out, d_out - 1) * p_ext) +
            (double)imul(d_out, d_in) * p_ext;
    denom *= (double)(d_in + d_out) + alpha * (double)(r - 1 - d_in);
    if (denom != 0.0) A = (((double)imul(d_in, d_in - 1) * p_in) * (double)(d_in + d_out)) / denom;

    const double rr = (double)imul(r - 1, r - 2) * p_in * p_in * p_in;
    const double q = (double)(r - 1) * p_in;
    double B = 0.0;
    denom = rr + (double)(2 * (d_in - 1)) * p_in + t * (double)(r - 1) * p_in * p_ext +
            t * (t - 1) * p_ext + (double)d_out * p_ext;
    denom *= q + 1 + t + alpha * ((double)r - q - 1);
    if (denom != 0.0) B = ((double)(2 * (d_in - 1)) * p_in) * (q + 1 + t) / denom;

    double C = 0.0;
    denom = rr + t * (t - 1) * p_ext + t * (double)(r - 1) * p_in * p_ext;
    denom *= q + t + alpha * ((double)r - q);
    denom *= q + t + alpha * ((double)r - q - 1);
    if (denom != 0.0 && (r + t) > 0 && ((r - 1) + t) > 0) C = -rr * (q + t) * alpha / denom;

    return A + d_in * B + (r - d_in) * C;
}

extern "C" void orc_improve(const orc_graph *g, double p_ext, double alpha, const uint32_t *labels,
                            const int32_t *sizes, const int32_t *ext_edges,
                            const int32_t *int_edges, uint32_t *new_labels) {
    /* src/scd.cpp:221-341: Jacobi update from the previous labels */
#pragma omp parallel
    {
        std::vector<uint32_t> buf;
#pragma omp for schedule(dynamic, 512)
        for (uint32_t p = 0; p < g->n; p++) {
            const uint32_t deg = degree(g, p), mine = labels[p];
            buf.resize(deg);
            for (uint32_t i = 0; i < deg; i++) buf[i] = labels[g->adj[g->indices[p] + i]];
            std::sort(buf.begin(), buf.end());   /* unsigned: INVALID sorts last */

            double remove_gain = 0.0, best_gain = 0.0;
            uint32_t best_label = 0;
            for (uint32_t i = 0; i < deg;) {
                const uint32_t l = buf[i];
                if (l == ORC_INVALID) { i++; continue; }
                uint32_t freq = 1;
                while (i + freq < deg && buf[i + freq] == l) freq++;
                int size = sizes[l], ext = ext_edges[l], in = int_edges[l] / 2;
                if (l == mine) {
                    size--;
                    ext += (int)(freq - (deg - freq));
                    in -= (int)freq;
                }
                double p_in = size > 1 ? (2.0 * in) / (size * (size - 1.0)) : 0.0;
                double gain = orc_gain(size, (int)freq, (int)deg - (int)freq, ext, p_in, p_ext, alpha);
                if (l == mine) remove_gain = -gain;
                if (gain > best_gain) { best_gain = gain; best_label = l; }
                i += freq;
            }
            const double insert_gain = best_gain + remove_gain;
            uint32_t next;
            if (insert_gain > remove_gain && insert_gain > 0.0) next = best_label;
            else if (remove_gain > 0) next = ORC_INVALID;
            else next = mine;
            new_labels[p] = next;
        }
    }
}

extern "C" double orc_wcc(const orc_graph *g, double alpha, const uint32_t *labels,
                          const int32_t *sizes, double *per_vertex) {
    /* src/wcc.cpp:31-141: per vertex, its same-label neighbours N, and for each
     * q in N the size of N ∩ adj(q) (merge), giving internal triangles */
    const uint32_t n = g->n;
    std::vector<double> term(n, 0.0);
#pragma omp parallel
    {
        std::vector<uint32_t> inner;
#pragma omp for schedule(dynamic, 32)
        for (uint32_t p = 0; p < n; p++) {
            const uint32_t l = labels[p];
            if (l == ORC_INVALID) continue;
            const int tri = g->tri[p], tdeg = g->tri_deg[p], size = sizes[l];
            if (size <= 2 || tdeg == 0) continue;
            inner.clear();
            for (uint32_t j = g->indices[p]; j != g->indices[p + 1]; j++)
                if (labels[g->adj[j]] == l) inner.push_back(g->adj[j]);
            int itri = 0, itdeg = 0;
            for (size_t k = 0; k < inner.size(); k++) {
                const uint32_t q = inner[k];
                size_t a = 0;
                uint32_t b = g->indices[q];
                const uint32_t b_end = g->indices[q + 1];
                bool hit = false;
                while (a != inner.size() && b != b_end) {   /* branches, as in orc_convert */
                    uint32_t x = inner[a], y = g->adj[b];
                    if (x == y) { hit = true; itri++; }
                    if (x <= y) a++;
                    if (x >= y) b++;
                }
                itdeg += hit;
            }
            double nom = (double)imul(itri, tdeg);
            double denom = tri * (tdeg + alpha * (size - 1 - itdeg));
            if (denom != 0.0) term[p] = nom / denom;
        }
    }
    double sum = 0.0;
    for (uint32_t p = 0; p < n; p++) sum += term[p];
    if (per_vertex) std::copy(term.begin(), term.end(), per_vertex);
    return n > 0 ? sum / n : 0;
}

extern "C" uint32_t orc_compress_labels(uint32_t n, uint32_t *labels) {
    /* src/scd.cpp:32-55 as written: a label's first occurrence maps to 0 and
     * every later occurrence to a fresh number, so the count printed is
     * n - (number of distinct valid labels). */
    std::map<uint32_t, uint32_t> seen;
    uint32_t next = 0;
    for (uint32_t p = 0; p < n; p++) {
        uint32_t l = labels[p];
        if (l == ORC_INVALID) l = next++;
        else if (seen.count(l)) l = seen[l] = next++;
        else l = seen[l];
        labels[p] = l;
    }
    return next;
}

extern "C" int orc_run(const orc_graph *g, double alpha, double threshold, int max_iters,
                       uint32_t *initial_labels, double *initial_wcc, uint32_t *num_comms_out,
                       uint32_t *trace_labels, double *trace_wcc, uint32_t *best_labels,
                       double *best_wcc_out, uint32_t *printed_comms, orc_times *tm) {
    /* src/main.cpp:35-93 */
    const uint32_t n = g->n;
    const double p_ext = orc_clustering_coef(g);
    std::vector<uint32_t> labels(n), next(n), best(n);
    double t0 = now_ms();
    const uint32_t nc = orc_initial_partition(g, labels.data());
    std::vector<int32_t> sizes(std::max<uint32_t>(nc, 1)), ext(std::max<uint32_t>(nc, 1)),
        in(std::max<uint32_t>(nc, 1));
    orc_collect_stats(g, labels.data(), nc, sizes.data(), ext.data(), in.data());
    double t1 = now_ms();
    double best_wcc = orc_wcc(g, alpha, labels.data(), sizes.data(), NULL);
    double t2 = now_ms();
    best = labels;
    if (initial_labels) std::copy(labels.begin(), labels.end(), initial_labels);
    if (initial_wcc) *initial_wcc = best_wcc;
    if (num_comms_out) *num_comms_out = nc;

    double t_imp = 0, t_stats = 0, t_wcc = 0, t_iter = 0;
    int iters = 0;
    bool capped = true;
    while (iters < max_iters) {
        double a = now_ms();
        orc_improve(g, p_ext, alpha, labels.data(), sizes.data(), ext.data(), in.data(), next.data());
        labels.swap(next);
        double b = now_ms();
        orc_collect_stats(g, labels.data(), nc, sizes.data(), ext.data(), in.data());
        double c = now_ms();
        double wcc = orc_wcc(g, alpha, labels.data(), sizes.data(), NULL);
        if (wcc > best_wcc) best = labels;
        double d = now_ms();
        t_imp += b - a; t_stats += c - b; t_wcc += d - c; t_iter += d - a;
        if (trace_labels) std::copy(labels.begin(), labels.end(), trace_labels + (size_t)iters * n);
        if (trace_wcc) trace_wcc[iters] = wcc;
        iters++;
        if (wcc < best_wcc * (1 + threshold)) { capped = false; break; }
        best_wcc = wcc;
    }
    if (best_labels) std::copy(best.begin(), best.end(), best_labels);
    if (best_wcc_out) *best_wcc_out = best_wcc;
    if (printed_comms) *printed_comms = orc_compress_labels(n, best.data());
    if (tm) {
        tm->initial_partition = t1 - t0;
        tm->initial_wcc = t2 - t1;
        tm->iterations = t_iter;
        tm->improve = t_imp;
        tm->stats = t_stats;
        tm->wcc = t_wcc;
    }
    return capped ? -1 : iters;
}

extern "C" void orc_free(void *p) { free(p); }
extern "C" int orc_threads(void) { return omp_get_max_threads(); }
