// Engine state shared by the translation units of libscd_gb300.
//
// HBM layout of one resident graph (all 32-bit words, n vertices, m undirected
// edges, ids are degree-descending ranks as written by `convert`):
//   indices[n+1], adj[2m]       symmetric CSR, rows ascending (binary format)
//   tri[n], tri_deg[n]          2 x triangles per vertex, triangle degree
//   nlow[n]                     neighbours with a smaller id = the out-list of
//                               the degree orientation, a prefix of each row
// Partition state:
//   labels / labels_next / best [n]
//   stats[2] x {sizes, ext_edges, int_edges}[n]   (current / next)
//   slot_cnt[2m]                internal-triangle counters per out-slot
//   itri[n], itdeg[n]           internal triangles / triangle degree
//   wcc_part[], wcc_sum         fixed-order WCC reduction
#pragma once

#include <string>
#include <vector>

#include "primitives.cuh"

namespace scd {

// vertex lists by degree: (0,8], (8,16], (16,32], (32,256], (256,2048], (2048,8192], > 8192
struct DegreeClasses {
    static constexpr int K = 8;
    static constexpr uint32_t upper[K] = {8, 16, 32, 256, 1024, 2048, 4096, 0xffffffffu};
    uint32_t *list[K] = {};   // class 0 also holds the isolated vertices (degree 0)
    uint32_t count[K] = {};
};

// Rows longer than CHUNK cut into CHUNK-entry pieces: per-row kernels (statistics,
// internal degrees) take one warp per short row in id order and one warp per
// piece of a long row, so hub rows run alongside the rest instead of in a tail.
struct RowWork {
    static constexpr uint32_t CHUNK = 256;
    const uint32_t *llong = nullptr;       // vertices of degree > CHUNK
    const uint32_t *chunk_off = nullptr;   // first piece of each (nlong + 1 entries)
    uint32_t nlong = 0, nchunks = 0;
};

struct Graph {
    uint32_t n = 0, m = 0;
    uint32_t *indices = nullptr, *adj = nullptr, *nlow = nullptr;
    int32_t *tri = nullptr, *tri_deg = nullptr;
    double p_ext = 0.0;   // of graph 0 (the only graph of a plain context)
    uint32_t max_deg = 0;
    // degree buckets of the improve kernels, built once per graph
    DegreeClasses cls;
    RowWork rows;
    uint64_t *big_table_off = nullptr;   // hash-table offsets of the last bucket
    uint64_t big_table_words = 0;
};

struct Stats {
    int32_t *sizes = nullptr, *ext = nullptr, *intl = nullptr;
};

// The graphs of a context.  A batch of G independent graphs is held as one
// block-diagonal union graph: graph g owns the vertex range
// [fin_off[g], fin_off[g+1]) and the label range [comm_off[g], comm_off[g+1]),
// so every kernel runs once over all graphs, while everything that is defined
// per graph (p_ext, the WCC and its summation order, the convergence test) is
// kept per graph.  A plain context is a batch with G = 1.
struct Batch {
    uint32_t G = 1;
    uint32_t *fin_off = nullptr;          // device, G+1
    std::vector<uint32_t> h_fin_off;      // host copy
    std::vector<uint32_t> h_m;            // undirected edges per graph
    uint32_t *gid = nullptr;              // device, n: graph of each vertex (nullptr if G == 1)
    double *p_ext = nullptr;              // device, G
    float2 *pe32 = nullptr;               // device, G: FP32 enclosure of p_ext
    std::vector<double> h_p_ext;
    uint32_t *comm_off = nullptr;         // device, G+1 (labels of the initial partition)
    std::vector<uint32_t> h_comm_off;
    uint32_t *blk_off = nullptr;          // device, G+1: WCC partial blocks of each graph
    uint32_t *blk_gid = nullptr;          // device, #blocks: graph of each WCC block
    uint32_t blocks = 0;
    double *wcc = nullptr;                // device, G: WCC of the current labels
    double *best_wcc = nullptr;           // device, G
    uint8_t *active = nullptr;            // device, G: still iterating
    uint8_t *improved = nullptr;          // device, G: last iteration beat the best
    int32_t *iters = nullptr;             // device, G
    uint32_t *n_active = nullptr;         // device, 1
};

// CUDA-event phase timers (active with SCD_FLAG_PROFILE)
struct PhaseTimers {
    struct Phase {
        double ms = 0;
        uint64_t count = 0;
    };
    std::vector<std::string> names;
    std::vector<Phase> phases;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::vector<cudaEvent_t> pool;
    int index(const char *name);
    cudaEvent_t get_event();
    void flush();   // waits for pending events and accumulates them
    void reset();
    void destroy();
};

// triangles.cu: oriented triangle counting (per out-slot counters)
struct Oriented {
    const uint32_t *beg;   // out-list of u starts at beg[u]
    const uint32_t *len;   // and has len[u] entries (sorted ascending by id)
    const uint32_t *adj;
    uint32_t n;
    // in-lists (the v with u in out(v)): iadj[ibeg[u], ibeg[u] + ilen[u]); without
    // ibeg, beg is the offset array of a symmetric CSR whose rows hold the
    // out-list first and the in-list after it
    const uint32_t *ibeg = nullptr, *ilen = nullptr, *iadj = nullptr;
    __device__ __forceinline__ uint32_t in_beg(uint32_t u) const { return ibeg ? ibeg[u] : beg[u] + len[u]; }
    __device__ __forceinline__ uint32_t in_len(uint32_t u) const {
        return ibeg ? ilen[u] : beg[u + 1] - beg[u] - len[u];
    }
    __device__ __forceinline__ const uint32_t *in_adj() const { return ibeg ? iadj : adj; }
};
// Label mode of triangle counting: only triangles whose three vertices carry
// the same valid label count; with `active`, vertices of graphs of a batch that
// stopped iterating are skipped (their WCC is no longer read).
struct LabelFilter {
    const uint32_t *labels = nullptr;   // nullptr: count every triangle
    const uint32_t *gid = nullptr;
    const uint8_t *active = nullptr;
    __device__ __forceinline__ bool frozen(uint32_t v) const { return active && !active[gid[v]]; }
};
// out-degree buckets and their work-unit offsets (built once per oriented graph)
// Bucket k lists its out-list centres first (nfwd[k] of them) and, for the CTA
// buckets, then the in-list centres: a vertex b whose edges a -> b with
// d+(a) < d+(b) (b-centric edges, below) are counted from b's table.
struct TcPlan {
    static constexpr int K = 7;
    uint32_t *verts[K] = {};
    uint32_t *unit_off[K] = {};
    uint32_t nverts[K] = {};
    uint32_t nfwd[K] = {};
    uint32_t dir_lo = 0, dir_hi = 0, dir_amin = 0;   // b-centric iff d+(a) < d+(b),
                                                      // dir_lo < d+(b) <= dir_hi, d+(a) > dir_amin
    DevBuf<uint32_t> tmp[2 * K];   // storage when the plan is temporary
    // Core map of the upper CTA bucket (tc_core_map): the vertices of degree >
    // cta_hi, numbered 0..core_n-1 in id order.  core_adj holds every out-list
    // in core numbers (core_n for a vertex outside the core), v's list at
    // core_adj[core_beg[v]..], each list starting on a 16-byte boundary and
    // padded with core_n to a multiple of 4 entries.  Every out-list of a centre
    // of that bucket lies in the core, so a bitmap of core_n bits holds it
    // exactly.  core_n == 0: no map (the hash-table kernels run); core_lcap:
    // the bucket's largest out-degree (rounded up to even).
    const uint32_t *core_adj = nullptr, *core_beg = nullptr;
    uint32_t core_n = 0, core_lcap = 0;
    uint32_t cta_lo = 0, cta_hi = 0;   // out-degree range (cta_lo, cta_hi] of the first CTA bucket
    DevBuf<uint32_t> core_buf, core_beg_buf;
};
struct Ctx;
// in_lists: also in-list centres (b-centric edges) in the CTA buckets
// core_from > 0: the upper CTA bucket starts at that out-degree (the core-bitmap
// kernel's split, for a plan that gets a core map) instead of tc_b1
void tc_plan(Ctx &c, const Oriented &o, TcPlan &plan, cudaStream_t s, bool owned, bool in_lists,
             uint32_t core_from = 0);
// builds the core map of the upper CTA bucket (from plan.cta_hi) for out-lists
// o.adj[0..slots) (symmetric degree of v = o.len[v] + o.in_len(v)); core_n: the
// core's size, lcap: the bucket's longest out-list (both counted beforehand)
void tc_core_map(Ctx &c, const Oriented &o, uint64_t slots, TcPlan &plan, uint32_t core_n, uint32_t lcap,
                 cudaStream_t s);
// the plan of a full count (preprocessing) over out-lists o.adj[0..slots) with in-list
// centres: the core split and its core map, or the hash kernels' split
void tc_plan_counting(Ctx &c, const Oriented &o, uint64_t slots, TcPlan &plan, cudaStream_t s);
// tcount[v] += triangles at v; flag[slot] = 1 for out-slots on a triangle.
// With labels: internal triangles only.  tcount and flag must be zeroed.
// Sorts every row of a CSR (offsets off[nrows+1], values vals) ascending in place;
// with dedup, repeated values of a row become INVALID and udeg[r] receives the
// number of distinct values of row r.
void sort_rows(Ctx &c, const uint32_t *off, uint32_t nrows, uint32_t *vals, bool dedup, uint32_t *udeg,
               cudaStream_t s);
void count_triangles(Ctx &c, const Oriented &o, const TcPlan &plan, LabelFilter labels, uint32_t *tcount,
                     uint8_t *flag, cudaStream_t s, const char *phase = nullptr);
// times the triangle-counting bucket splits on the resident graph, keeps the fastest
double autotune_tc(Ctx &c, std::vector<std::string> *report);
// set kernel attributes (dynamic shared memory) once per device, outside any capture
void prepare_tc_kernels();
void prepare_improve_kernels();

struct Ctx;
// records [start, end) of a phase on the context's stream when profiling
struct PhaseScope {
    Ctx *c;
    int idx;
    cudaEvent_t start = nullptr;
    PhaseScope(Ctx &ctx, const char *name);
    ~PhaseScope();
};

struct ResidentSet;   // resident.cu: graphs that join and leave between iterations

struct Ctx {
    int device = 0;
    int work_group_size = 256;
    unsigned flags = 0;
    double alpha = 1.0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;
    cudaStream_t aux = nullptr;                        // improve: the hub kernel beside the other classes
    cudaEvent_t aux_fork = nullptr, aux_join = nullptr;
    std::string err;
    uint64_t launches = 0;
    uint32_t tc_small = 32, tc_b0 = 64, tc_b1 = 1024;   // triangle-counting bucket splits (autotuned)
    uint32_t tc_amin = 0;   // b-centric edges need d+(a) > tc_amin (autotuned; at most tc_small)

    Graph g;
    Batch b;
    bool has_graph = false;
    bool capturing = false;           // inside a CUDA-graph capture: no host syncs, no timers
    cudaEvent_t pext_ready = nullptr;  // p_ext (side stream) done
    bool pext_join_pending = false;    // the main stream has not waited for it yet
    bool pext_host_valid = false;      // b.h_p_ext / g.p_ext hold it

    // partition state
    uint32_t *labels = nullptr, *labels_next = nullptr, *best = nullptr;
    Stats st[2];
    int cur = 0;
    uint32_t num_comms = 0;
    bool has_labels = false;
    uint8_t *slot_flag = nullptr;     // internal-triangle flag per adjacency position
    uint32_t *itcount = nullptr;      // internal triangles per vertex
    int32_t *itdeg = nullptr;         // edges on an internal triangle per vertex
    uint32_t *int_len = nullptr;      // label-mode count: internal out-list lengths (n)
    uint32_t *int_adj = nullptr;      // and the internal out-lists at the CSR offsets (2m)
    TcPlan wplan;                     // triangle-counting plan of the resident graph
    double *wcc_part = nullptr, *wcc_host = nullptr;
    uint32_t *host_u32 = nullptr;     // pinned: the active-graph count of an iteration [0, 2), planning words [2, 32)
    char *io_buf[2] = {};             // pinned pieces of a graph file on its way to the device
    cudaEvent_t io_done[2] = {};
    uint32_t *big_tables = nullptr;   // global hash tables of the last degree bucket
    double *pin64 = nullptr;          // per-community p_in of the current statistics
    int4 *civ = nullptr;              // size, external edges and the FP32 enclosure of p_in (bits)
    uint32_t *work_counter = nullptr; // dynamic work distribution

    ResidentSet *res = nullptr;       // set by scd_resident_init
    bool resident = false;            // every iteration skips the graphs that stopped

    PhaseTimers timers;
    std::vector<void *> owned;        // device allocations freed with the graph
    uint64_t bytes = 0;

    // graph-lifetime device arrays: stream-ordered from the device's memory pool, which
    // keeps freed memory cached (release threshold raised at scd_create), so a new graph
    // reuses the previous one's memory without cudaMalloc/cudaFree synchronisation
    uint64_t mem_limit = 0;           // scd_set_memory_limit (0: none)

    template <typename T>
    T *alloc(size_t count) {
        void *p = nullptr;
        if (count == 0) count = 1;
        if (mem_limit && bytes + count * sizeof(T) > mem_limit)
            throw Error(SCD_ERR_OOM, "device memory limit of the context reached");
        CK(cudaMallocAsync(&p, count * sizeof(T), stream));
        owned.push_back(p);
        bytes += count * sizeof(T);
        return (T *)p;
    }
    void free_all();
};

// preprocess.cu
// rec_off (host, G+1 entries, nullable): records of graph g are [rec_off[g], rec_off[g+1]),
// each graph with its own vertex ids; the graphs become one block-diagonal union.
void convert_edges(Ctx &c, const uint32_t *pairs_dev, uint64_t count, const std::vector<uint64_t> *rec_off = nullptr);
// read_edges on the device: (min, max) records of the text in file order into out
uint64_t parse_edge_text(Ctx &c, const char *text, uint64_t bytes, DevBuf<uint32_t> &out);
// empty graph arrays of n vertices and m edges in place of the resident graph
void alloc_graph(Ctx &c, uint32_t n, uint32_t m);
void upload_graph(Ctx &c, uint32_t n, uint32_t m, const uint32_t *indices, const uint32_t *adj,
                  const int32_t *tri, const int32_t *tri_deg);
void finish_graph(Ctx &c);   // nlow, p_ext, degree classes, partition buffers
// the derived structure of the union graph (see engine.cu); always_gid: a graph-id
// array even for one graph
void build_union_structure(Ctx &c, bool always_gid);
// engine.cu: one refinement iteration of every running graph without host
// synchronisation (capturable); kernel nodes of a captured CUDA graph
void iterate_async(Ctx &c, double threshold, double *trace, int max_trace);
uint64_t kernel_nodes(cudaGraph_t gr);
// resident.cu
void resident_destroy(Ctx &c);


// partition.cu
void initial_partition(Ctx &c);

// refine.cu
void collect_stats(Ctx &c, const uint32_t *labels, Stats &st, bool frozen_graphs = false);
double compute_wcc(Ctx &c, const uint32_t *labels, const Stats &st);
// frozen_graphs: vertices of graphs whose loop has ended keep their labels
void improve(Ctx &c, const uint32_t *labels, const Stats &st, uint32_t *next, bool frozen_graphs = false);
// per-graph WCC in c.b.wcc (device); frozen_graphs: skip the graphs of a batch that stopped iterating
void launch_wcc(Ctx &c, const uint32_t *labels, const Stats &st, bool frozen_graphs = false);
void compute_p_ext(Ctx &c);   // launches on the side stream
void join_p_ext(Ctx &c);      // main stream waits for p_ext (outside captures)
void host_p_ext(Ctx &c);      // host copies of p_ext (b.h_p_ext, g.p_ext)
// per-graph loop control after a WCC (src/main.cpp:68-81): iteration count,
// best WCC, best labels, convergence; *n_active receives the graphs still running
void batch_step(Ctx &c, double threshold, double *trace = nullptr, int max_trace = 0);
void batch_reset(Ctx &c);   // best := current WCC, all non-empty graphs active

}  // namespace scd

// the opaque handle of the C ABI
struct scd_ctx {
    scd::Ctx c;
};
