/*
 * scd_gb300 — C ABI of the GB300-native SCD engine (libscd_gb300.so).
 *
 * Drop-in for the reference's single-GPU backend (src/cuda.hpp:23-28, driven
 * by src/main-gpu.cpp) plus the preprocessing of the `convert` tool
 * (src/convert.cpp:141-463), which the reference runs on the CPU only.
 *
 * Conventions (differences from the reference are deliberate):
 *  - every entry point takes an opaque scd_ctx* instead of module globals
 *    (src/cuda.cu:29-52), so several graphs can live in one process;
 *  - every entry point returns an int status (SCD_OK or an SCD_ERR_* code)
 *    instead of calling exit() (src/cuda-common.cuh:67-77); the message of the
 *    last failure is available from scd_last_error();
 *  - host buffers are owned by the caller; device memory by the context;
 *  - one host thread per context; calls on a context are stream-ordered.
 *  - labels are uint32 with SCD_INVALID_LABEL (src/scd.hpp:23) for "no community".
 */
#ifndef SCD_GB300_H
#define SCD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCD_OK 0
#define SCD_ERR_ARG (-1)      /* invalid argument                          */
#define SCD_ERR_CUDA (-2)     /* CUDA runtime error                        */
#define SCD_ERR_OOM (-3)      /* device allocation failed / over budget    */
#define SCD_ERR_STATE (-4)    /* call out of order (no graph, no labels)   */
#define SCD_ERR_FORMAT (-5)   /* malformed graph or edge input             */
#define SCD_ERR_TIMEOUT (-6)  /* a bounded device-side wait gave up        */
#define SCD_ERR_LIMIT (-7)    /* input beyond a documented size limit      */

#define SCD_INVALID_LABEL 0xffffffffu

/* scd_create flags */
#define SCD_FLAG_PROFILE 1u       /* record per-phase CUDA-event timers (scd_profile_get), the
                                     counterpart of the event timers of src/cuda.cu:351-360 */
#define SCD_FLAG_PEXT_TREE 2u     /* p_ext by a parallel tree sum instead of the canonical
                                     index-ordered sum (faster; may differ in the last bits) */
#define SCD_FLAG_NO_GRAPHS 4u     /* launch every improvement iteration kernel by kernel instead
                                     of replaying a captured CUDA graph; with SCD_FLAG_PROFILE
                                     this times the iteration phases (captured iterations are
                                     not split into phases) */
#define SCD_FLAG_TC_OUT_ONLY 8u   /* count every triangle from the out-list table of its
                                     lowest-ordered vertex (no in-list units); same results,
                                     slower on skewed graphs */
#define SCD_FLAG_PRIORITY 16u     /* the context's streams get the device's highest priority:
                                     their pending thread blocks are scheduled before those of
                                     other contexts (latency-sensitive work beside bulk work) */
#define SCD_FLAG_TC_HASH 32u      /* preprocessing triangle count of long out-lists by the
                                     shared hash-table kernels instead of the exact core-bitmap
                                     kernel; same results */

typedef struct scd_ctx scd_ctx;

/* Replaces cuda_init(device_id, work_group_size, profile) (src/cuda.hpp:23,
 * src/cuda.cu:55-82).  work_group_size is kept for argv compatibility
 * (src/main-gpu.cpp:38); kernels choose their own launch shapes. */
int scd_create(scd_ctx **ctx, int device_id, int work_group_size, unsigned flags);
void scd_destroy(scd_ctx *ctx);
const char *scd_last_error(const scd_ctx *ctx);

/* Preprocessing on the device: the work of `convert` between reading the text
 * and writing the file (src/convert.cpp:487-525: first-appearance renumbering,
 * sort, de-duplication, loop removal, triangle counting, removal of
 * triangle-free edges, degree relabelling) followed by the symmetric CSR of
 * write_edges (src/convert.cpp:417-463).  pairs holds count (a, b) records as
 * read_edges stores them ((min, max) of each text line, in file order,
 * src/convert.cpp:120-123).  pairs_on_device != 0 means pairs is a device
 * pointer.  The resulting graph stays resident in the context. */
int scd_convert_edges(scd_ctx *ctx, const uint32_t *pairs, uint64_t count, int pairs_on_device);

/* Replaces read_edges (src/convert.cpp:74-138) followed by the processing of
 * scd_convert_edges: the edge-list text (bytes characters; a device pointer if
 * text_on_device) is parsed on the device with the reference's line rules
 * ('\n'-separated lines of at most 1023 characters, leading blanks skipped,
 * empty and '#' lines ignored, two unsigned decimal numbers, the record is
 * (min, max)) and converted.  SCD_ERR_FORMAT with the reference's message for
 * the first failing line ("line i is corrupt", or a line longer than 1023
 * characters). */
int scd_convert_text(scd_ctx *ctx, const char *text, uint64_t bytes, int text_on_device);
/* The parse alone: *count receives the number of records and, if pairs (host)
 * is not NULL, pairs receives them (2 * count words, file order). */
int scd_parse_text(scd_ctx *ctx, const char *text, uint64_t bytes, int text_on_device, uint32_t *pairs,
                   uint64_t *count);

/* Replaces cuda_transfer_graph(const Graph*, alpha) (src/cuda.hpp:24,
 * src/cuda.cu:84-148): uploads a graph in the binary-format layout
 * (src/graph.cpp:86-134).  The clustering coefficient p_ext
 * (src/graph.cpp:57-68) is computed on the device. */
int scd_transfer_graph(scd_ctx *ctx, uint32_t n, uint32_t m, const uint32_t *indices,
                       const uint32_t *adj, const int32_t *tri, const int32_t *tri_deg,
                       double alpha);

/* The binary-format fast path: Graph::read (src/graph.cpp:273-321) and
 * cuda_transfer_graph in one call.  The file goes to the device in 64 MB pieces
 * through two pinned buffers (reading one piece overlaps copying the other), with
 * no pageable host copy of the graph; p_ext on the device.  SCD_ERR_ARG if the
 * file cannot be opened, SCD_ERR_FORMAT ("error while reading <path>") if it is
 * short, long or inconsistent. */
int scd_load_graph_file(scd_ctx *ctx, const char *path, double alpha);

/* The same for a graph file already in host memory (bytes: its full contents;
 * pinned memory makes the copy asynchronous). */
int scd_transfer_graph_bytes(scd_ctx *ctx, const void *bytes, uint64_t size, double alpha);

/* Graph sizes and p_ext of the resident graph (src/graph.hpp:25-27). */
int scd_graph_info(scd_ctx *ctx, uint32_t *n, uint32_t *m, double *clustering_coef);

/* Copies the resident graph out in the binary-format layout; any pointer may
 * be NULL (what `convert` writes, src/convert.cpp:430-455). */
int scd_graph_download(scd_ctx *ctx, uint32_t *indices, uint32_t *adj, int32_t *tri,
                       int32_t *tri_deg);

/* create_initial_partition (src/scd.cpp:113-171) on the device, including its
 * collect_stats; leaves the labels as both current and best labels. */
int scd_initial_partition(scd_ctx *ctx, uint32_t *num_communities);

/* Replaces cuda_labels_to_device(labels) (src/cuda.hpp:25, src/cuda.cu:150-174):
 * sets current and best labels (n entries) and collects community statistics. */
int scd_labels_to_device(scd_ctx *ctx, const uint32_t *labels);

/* compute_wcc (src/wcc.cpp:31-141) of the current labels. */
int scd_compute_wcc(scd_ctx *ctx, double *wcc);

/* Replaces cuda_improve_labels(&wcc) (src/cuda.hpp:26, src/cuda.cu:176-361):
 * one refinement iteration — improve_partition (src/scd.cpp:221-341),
 * collect_stats (src/scd.cpp:57-111), compute_wcc — returning the new WCC. */
int scd_improve_labels(scd_ctx *ctx, double *wcc);

/* Replaces cuda_store_labels() (src/cuda.hpp:27): best labels := current labels. */
int scd_store_labels(scd_ctx *ctx);

/* Replaces cuda_labels_from_device(labels) (src/cuda.hpp:28): copies the best labels out. */
int scd_labels_from_device(scd_ctx *ctx, uint32_t *labels);

/* Current (not best) labels and the community statistics of the current
 * labels (sizes, ext_edges, int_edges of src/scd.hpp:25-31); any pointer may be
 * NULL; arrays hold *num_communities entries.  Statistics are for a single graph
 * (SCD_ERR_STATE on a batch: converged graphs of a batch stop updating theirs). */
int scd_current_labels(scd_ctx *ctx, uint32_t *labels);
/* compress_labels (src/scd.cpp:32-55) as its code intends, without the inverted
 * branch: the best labels renumbered in vertex order (an unlabelled vertex or the
 * first vertex of a label opens the next id, later vertices of the label take it);
 * labels (nullable) receives n entries, *num_communities the number of ids.
 * Single-graph contexts. */
int scd_compressed_labels(scd_ctx *ctx, uint32_t *labels, uint32_t *num_communities);
int scd_community_stats(scd_ctx *ctx, int32_t *sizes, int32_t *ext_edges, int32_t *int_edges,
                        uint32_t *num_communities);

typedef struct {
    int32_t iterations;            /* src/main-gpu.cpp:72-75 iters              */
    double initial_wcc;            /* src/main-gpu.cpp:55                       */
    double best_wcc;               /* the "WCC:" of the final block             */
    uint32_t initial_communities;  /* communities of the initial partition      */
    uint32_t printed_communities;  /* "num. communities:" as the reference prints
                                      it (src/scd.cpp:32-55, inverted branch)    */
    uint32_t distinct_communities; /* true number of distinct valid best labels */
    double ms_partition;           /* initial partition + initial WCC           */
    double ms_iterations;          /* refinement loop                           */
} scd_result;

/* The whole refinement loop of src/main-gpu.cpp:54-110 after the graph is
 * resident: initial partition (unless labels were already set), initial WCC,
 * iterations until wcc < best*(1+threshold) or max_iters, best-label
 * tracking.  wcc_trace (nullable) receives up to max_iters per-iteration WCCs.
 * Returns SCD_ERR_LIMIT if max_iters was reached without convergence (the
 * reference loops forever when the WCC stays 0, src/main.cpp:77). */
int scd_run(scd_ctx *ctx, double threshold, int max_iters, double *wcc_trace, scd_result *res);

/* Device memory currently held by the context (bytes). */
int scd_memory_usage(scd_ctx *ctx, uint64_t *bytes);
/* A cap on the device memory the context holds for its graphs (0: none): an
 * allocation that would pass it fails with SCD_ERR_OOM, as a failed cudaMalloc
 * does, and the context stays usable (the next call starts from a clean state).
 * Stream-ordered temporaries of a single call are not counted.  No counterpart
 * in the reference (whose allocation failures exit the process,
 * src/cuda-common.cuh:67-77). */
int scd_set_memory_limit(scd_ctx *ctx, uint64_t bytes);

/* Number of kernels this context launched so far (for launch accounting). */
int scd_kernel_launches(scd_ctx *ctx, uint64_t *count);

/* The CUDA stream (cudaStream_t) all work of the context is ordered on. */
int scd_stream(scd_ctx *ctx, void **stream);

/* Phase timers (CUDA events on the context's stream, recorded only when the
 * context was created with SCD_FLAG_PROFILE): accumulated milliseconds and
 * number of timed launches of a phase.  Phases: "convert", "tc" (triangle
 * counting kernel of the preprocessing), "partition", "improve", "stats",
 * "wcc_tc" (internal-triangle kernel), "wcc".  scd_profile_reset clears them. */
int scd_profile_get(scd_ctx *ctx, const char *phase, double *total_ms, uint64_t *count);
int scd_profile_reset(scd_ctx *ctx);

/* ---- Batched SCD ---------------------------------------------------------
 * Many independent graphs in one context.  They are processed together as one
 * block-diagonal union graph: every preprocessing, partition and refinement
 * stage is one launch over all graphs (work units drawn from all of them), and
 * each refinement iteration is one CUDA-graph replay for all graphs still
 * running.  Per graph, the arithmetic and the results are identical to
 * processing that graph alone (convert output, p_ext, labels of every
 * iteration, WCC bit for bit, iteration count). */

/* Preprocessing (as scd_convert_edges) of num_graphs graphs: the records of
 * graph g are pairs[2*record_offsets[g] .. 2*record_offsets[g+1]), each graph
 * numbered in its own id space.  record_offsets is a host array of
 * num_graphs+1 entries; pairs is a device pointer if pairs_on_device != 0.
 * Limits: fewer than 2^31 records and 2^32-1 distinct ids in total. */
int scd_batch_convert(scd_ctx *ctx, const uint32_t *pairs, const uint64_t *record_offsets,
                      uint32_t num_graphs, int pairs_on_device);
/* As scd_batch_convert from host memory, with each graph's records in its own
 * array: counts[g] pairs at pairs[g], so callers need not concatenate them. */
int scd_batch_convert_lists(scd_ctx *ctx, const uint32_t *const *pairs, const uint64_t *counts,
                            uint32_t num_graphs);
int scd_batch_size(scd_ctx *ctx, uint32_t *num_graphs);
/* Sizes and p_ext of graph g of the batch. */
int scd_batch_graph_info(scd_ctx *ctx, uint32_t g, uint32_t *n, uint32_t *m, double *clustering_coef);
/* Graph g in the binary-format layout with its own ids (what `convert` writes
 * for that graph alone); any pointer may be NULL. */
int scd_batch_graph_download(scd_ctx *ctx, uint32_t g, uint32_t *indices, uint32_t *adj, int32_t *tri,
                             int32_t *tri_deg);
/* The refinement loop of every graph (as scd_run); results holds num_graphs
 * entries.  Returns SCD_ERR_LIMIT if some graph was still improving after
 * max_iters (its results are those of the last iteration). */
int scd_batch_run(scd_ctx *ctx, double threshold, int max_iters, scd_result *results);
/* Best labels of graph g (n_g entries) in that graph's own label numbering. */
int scd_batch_labels(scd_ctx *ctx, uint32_t g, uint32_t *labels);
/* Best labels of all graphs in one copy: graph g's n_g labels (own numbering)
 * at labels[vertex_offsets[g] .. vertex_offsets[g+1]).  labels (nullable) holds
 * sum n_g entries; vertex_offsets (nullable) num_graphs+1 entries. */
int scd_batch_labels_all(scd_ctx *ctx, uint32_t *labels, uint64_t *vertex_offsets);

/* Autotuner: times the triangle-counting work split on the resident graph over
 * a small grid and keeps the fastest for this context's later conversions and
 * WCC passes (the current split stays unless another is at least 5 % faster).
 * The split is by out-list length: up to small_max (0, 16 or 32) a group of 16
 * or 32 lanes intersects in registers; up to warp_max a warp takes 32 list
 * entries at a time against a shared-memory hash table; up to cta_max a
 * 128-thread CTA does, longer lists go to 256-thread CTAs.  A fourth dimension,
 * the out-list length (0, 16 or 32) above which an edge may be counted at its
 * higher endpoint's table, is reported in the report line of the chosen split
 * ("in-list>N").  report (nullable, report_cap bytes) receives one line per
 * candidate. */
int scd_autotune(scd_ctx *ctx, uint32_t *small_max, uint32_t *warp_max, uint32_t *cta_max, double *best_ms,
                 char *report, uint64_t report_cap);

/* ---- Resident set (continuous batching) ---------------------------------
 * No counterpart in the reference (one graph per process there).  A context
 * made a resident set keeps graphs resident on the device and advances every
 * one of them that is still iterating with the same launches: one step is one
 * refinement iteration (improve, collect_stats, compute_wcc and the per-graph
 * loop control of src/main-gpu.cpp:71-95) of all running graphs, replayed from
 * one captured CUDA graph.  Graphs join between steps: another context converts
 * them (scd_convert_edges, scd_batch_convert*, or any context with a resident
 * graph) on its own stream, possibly on another host thread while steps run,
 * and hands them over with scd_resident_add.  Graphs that stop (converged, or
 * max_iters reached) leave with scd_resident_take.  Per graph, every result
 * (labels of every iteration, WCC, iteration count) is identical to running
 * that graph alone with scd_run; it does not depend on the other graphs or on
 * when the graph joined. */

/* Makes ctx (its resident graph, if any, is dropped) an empty resident set whose
 * graphs iterate until wcc < best*(1+threshold) or max_iters iterations. */
int scd_resident_init(scd_ctx *ctx, double threshold, int max_iters);
/* Moves every graph resident in src (a plain context or a batch, with or
 * without labels) into set: src runs the loop's prologue on its own stream
 * (initial partition unless labels were set, initial WCC), then its device
 * arrays move to the set, where its graphs join at the next scd_resident_step;
 * src is left empty and reusable.  ids (nullable) receives one id per graph
 * (the batch order of src).  May be called from another host thread than the
 * one stepping the set (one thread per src). */
int scd_resident_add(scd_ctx *set, scd_ctx *src, uint64_t *ids);
/* One step: graphs waiting to join are merged in (the union is re-formed, and
 * also when taken graphs hold more than a quarter of it), then one iteration of
 * every running graph.  running / finished (nullable): graphs that iterated in
 * this step (0 if none was running) / graphs that stopped in this step (their
 * results wait for scd_resident_take; joining empty graphs stop at once). */
int scd_resident_step(scd_ctx *set, uint32_t *running, uint32_t *finished);
/* Takes up to cap stopped graphs out of the set: ids[k], results[k] (as
 * scd_run's, ms_iterations = time since it was handed over) and status[k]
 * (SCD_OK, or SCD_ERR_LIMIT if max_iters stopped it); labels (nullable) receives
 * their best labels in their own numbering, graph k at
 * labels[label_offsets[k] .. label_offsets[k+1]) (label_offsets: cap+1 entries);
 * graphs are taken while their labels fit in labels_cap entries.  *count: graphs
 * taken.  Any array but count may be NULL. */
int scd_resident_take(scd_ctx *set, uint32_t cap, uint64_t *ids, scd_result *results, int32_t *status,
                      uint32_t *labels, uint64_t labels_cap, uint64_t *label_offsets, uint32_t *count);
/* graphs held (not yet taken), running, waiting to join; steps made, the sum of
 * running graphs over the steps (graph-iterations), kernels of the last step. */
int scd_resident_info(scd_ctx *set, uint32_t *graphs, uint32_t *running, uint32_t *pending, uint64_t *steps,
                      uint64_t *graph_steps, uint64_t *kernels_per_step);
/* Host wall time spent in scd_resident_step so far (all of it, re-forming the
 * union, capturing the iteration) and the number of re-formings. */
int scd_resident_timing(scd_ctx *set, double *ms_steps, double *ms_rebuild, double *ms_capture, uint64_t *rebuilds);

/* WCC of a labelling without any device allocation.  It has no counterpart in
 * the reference: it exists for callers that cannot let a library call
 * cudaMalloc/cudaFree — a serving process whose memory pool already holds the
 * free device memory, a plugin host that accounts for every allocation itself,
 * or a latency-critical loop that cannot take the device-wide synchronisation
 * of cudaFree.  The caller passes device pointers to the graph in the
 * binary-format layout (indices[n+1], adj, tri[n], tri_deg[n]), the labels[n]
 * and the size of every community its labels use (sizes[label]), and a device
 * pointer wcc that receives one double; work is queued on stream (a
 * cudaStream_t, NULL for the default stream) of the current device and the
 * call returns without waiting.  The value equals scd_compute_wcc's for the
 * same graph and labels.
 * Scratch: two fixed arrays inside the library, allocated when the library is
 * loaded and held by every GPU that uses it until the process exits: the block
 * partials of the sum (SCD_WCC_STATIC_MAX_VERTICES/2048 doubles, 64 KB) and the
 * internal-triangle counts of hub rows (the first 131072 vertices of degree > 128,
 * 1 MB; convert's ids are degree ranks, so those are its hubs; a hub beyond them
 * takes a slower path to the same value).  n above SCD_WCC_STATIC_MAX_VERTICES
 * returns SCD_ERR_LIMIT.  All calls share the arrays: calls that may overlap on
 * the GPU (different streams without ordering) race and must be ordered by the
 * caller.  The first call on a device looks up the array's device address
 * and must come before any stream capture (a first call made while its stream
 * is being captured returns SCD_ERR_STATE).  Every later call made outside a
 * capture looks the address up again, so a device reset or a new primary
 * context (which reloads the library's device code and moves the array) is
 * picked up; a call made during a capture reuses the address of the last call
 * outside one, so a device reset between that call and the capture leaves it
 * stale: make one uncaptured call after a reset before capturing again.
 * An error already pending on the calling thread (cudaPeekAtLastError) is left
 * in place and reported as SCD_ERR_CUDA before anything is launched.
 * Returns SCD_OK, SCD_ERR_ARG (NULL pointer), SCD_ERR_LIMIT, SCD_ERR_STATE or
 * SCD_ERR_CUDA. */
#define SCD_WCC_STATIC_MAX_VERTICES (1u << 24)
int scd_wcc_static(const uint32_t *indices, const uint32_t *adj, const int32_t *tri,
                   const int32_t *tri_deg, const uint32_t *labels, const int32_t *sizes, uint32_t n,
                   double alpha, double *wcc, void *stream);

#ifdef __cplusplus
}
#endif
#endif
