/*
 * scd_oracle — CPU restatement of the reference's SCD path, used ONLY as test
 * infrastructure: the parity checker for the GPU engine (tests/, the smoke
 * check) and the timed CPU baseline in bench.py.  The product never links it.
 *
 * Parity: pinned against the reference itself (its convert/main sources built
 * unmodified into oracle/_ref by oracle/build_ref.sh, plus oracle/ref_driver.cpp
 * which links the reference's graph.cpp/scd.cpp/wcc.cpp to dump labels);
 * tests/golden holds the reference outputs for the committed fixtures.
 *
 * Canonical floating-point order: the reference sums p_ext and WCC with an
 * OpenMP reduction whose rounding depends on the thread count
 * (src/graph.cpp:59-68, src/wcc.cpp:49).  This restatement always uses the
 * single-thread (index-ordered) summation, so its results equal the reference
 * run with OMP_NUM_THREADS=1 at any thread count here.  Built with
 * -ffp-contract=off, like the reference oracle build.
 */
#ifndef SCD_ORACLE_H
#define SCD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_INVALID 0xffffffffu

typedef struct {
    uint32_t n, m;          /* vertices, undirected edges            */
    uint32_t *indices;      /* n+1                                   */
    uint32_t *adj;          /* 2m, rows ascending                    */
    int32_t *tri;           /* n: 2 x triangles per vertex           */
    int32_t *tri_deg;       /* n: incident edges lying on a triangle */
} orc_graph;

/* wall-clock ms of the reference's timer regions (src/convert.cpp:485-526,
 * src/main.cpp:42-84) */
typedef struct {
    double process_graph;   /* convert: reindex .. sort on degree     */
    double tc;              /* convert: removing edges w/o triangles  */
    double initial_partition;
    double initial_wcc;
    double iterations;      /* sum of "iteration" timers              */
    double improve, stats, wcc;
} orc_times;

/* src/convert.cpp:74-138 read_edges: parses "a b" lines into (min,max) pairs in
 * file order.  Returns 0, or -1 (unreadable) / -2 (corrupt line).  *pairs is malloc'd. */
int orc_read_text(const char *path, uint32_t **pairs, int64_t *count, uint32_t *num_nodes);

/* src/convert.cpp:141-414: renumber, sort, dedup, triangle filter, degree relabel;
 * src/convert.cpp:417-463 symmetrised CSR.  pairs are (min,max) in file order. */
int orc_convert(const uint32_t *pairs, int64_t count, orc_graph *out, orc_times *t);

int orc_write_graph(const char *path, const orc_graph *g);   /* src/convert.cpp:417-463 */
int orc_read_graph(const char *path, orc_graph *g);          /* src/graph.cpp:86-134    */
void orc_free_graph(orc_graph *g);

double orc_clustering_coef(const orc_graph *g);              /* src/graph.cpp:57-68 */

/* src/scd.cpp:113-171 (labels only; returns the number of communities) */
uint32_t orc_initial_partition(const orc_graph *g, uint32_t *labels);
/* src/scd.cpp:57-111 */
void orc_collect_stats(const orc_graph *g, const uint32_t *labels, uint32_t num_comms,
                       int32_t *sizes, int32_t *ext_edges, int32_t *int_edges);
/* src/scd.cpp:173-219 */
double orc_gain(int r, int d_in, int d_out, int c_out, double p_in, double p_ext, double alpha);
/* src/scd.cpp:221-341 */
void orc_improve(const orc_graph *g, double p_ext, double alpha, const uint32_t *labels,
                 const int32_t *sizes, const int32_t *ext_edges, const int32_t *int_edges,
                 uint32_t *new_labels);
/* src/wcc.cpp:31-141; per_vertex (nullable) receives each vertex's term */
double orc_wcc(const orc_graph *g, double alpha, const uint32_t *labels, const int32_t *sizes,
               double *per_vertex);
/* src/scd.cpp:32-55, including its inverted branch: returns the printed count */
uint32_t orc_compress_labels(uint32_t n, uint32_t *labels);

/*
 * src/main.cpp:35-93: initial partition, initial WCC, refinement loop until
 * wcc < best*(1+threshold).  trace_labels (nullable) receives max_iters*n labels
 * (iteration i at offset i*n), trace_wcc (nullable) max_iters values.
 * Returns the number of iterations, or -1 if max_iters was reached (the
 * reference loops forever on a graph whose WCC stays 0).
 */
int orc_run(const orc_graph *g, double alpha, double threshold, int max_iters,
            uint32_t *initial_labels, double *initial_wcc, uint32_t *num_comms,
            uint32_t *trace_labels, double *trace_wcc,
            uint32_t *best_labels, double *best_wcc, uint32_t *printed_comms, orc_times *t);

void orc_free(void *p);
int orc_threads(void);

#ifdef __cplusplus
}
#endif
#endif
