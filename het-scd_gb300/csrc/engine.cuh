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
    static constexpr int K = 7;
    static constexpr uint32_t upper[K] = {8, 16, 32, 256, 2048, 8192, 0xffffffffu};
    uint32_t *list[K] = {};
    uint32_t count[K] = {};
};

struct Graph {
    uint32_t n = 0, m = 0;
    uint32_t *indices = nullptr, *adj = nullptr, *nlow = nullptr;
    int32_t *tri = nullptr, *tri_deg = nullptr;
    double p_ext = 0.0;
    double *p_ext_dev = nullptr;
    uint32_t max_deg = 0;
    // degree buckets of the improve kernels, built once per graph
    DegreeClasses cls;
    uint64_t *big_table_off = nullptr;   // hash-table offsets of the last bucket
    uint64_t big_table_words = 0;
};

struct Stats {
    int32_t *sizes = nullptr, *ext = nullptr, *intl = nullptr;
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
};
// out-degree buckets and their work-unit offsets (built once per oriented graph)
struct TcPlan {
    static constexpr int K = 4;
    uint32_t *verts[K] = {};
    uint32_t *unit_off[K] = {};
    uint32_t nverts[K] = {};
    DevBuf<uint32_t> tmp[2 * K];   // storage when the plan is temporary
};
struct Ctx;
void tc_plan(Ctx &c, const Oriented &o, TcPlan &plan, cudaStream_t s, bool owned);
// tcount[v] += triangles at v; flag[slot] = 1 for out-slots on a triangle.
// With labels: internal triangles only.  tcount and flag must be zeroed.
void count_triangles(Ctx &c, const Oriented &o, const TcPlan &plan, const uint32_t *labels, uint32_t *tcount,
                     uint8_t *flag, cudaStream_t s);

struct Ctx;
// records [start, end) of a phase on the context's stream when profiling
struct PhaseScope {
    Ctx *c;
    int idx;
    cudaEvent_t start = nullptr;
    PhaseScope(Ctx &ctx, const char *name);
    ~PhaseScope();
};

struct Ctx {
    int device = 0;
    int work_group_size = 256;
    unsigned flags = 0;
    double alpha = 1.0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;
    std::string err;
    uint64_t launches = 0;

    Graph g;
    bool has_graph = false;

    // partition state
    uint32_t *labels = nullptr, *labels_next = nullptr, *best = nullptr;
    Stats st[2];
    int cur = 0;
    uint32_t num_comms = 0;
    bool has_labels = false;
    uint8_t *slot_flag = nullptr;     // internal-triangle flag per adjacency position
    uint32_t *itcount = nullptr;      // internal triangles per vertex
    int32_t *itdeg = nullptr;         // edges on an internal triangle per vertex
    TcPlan wplan;                     // triangle-counting plan of the resident graph
    double *wcc_part = nullptr, *wcc_sum = nullptr, *wcc_host = nullptr;
    uint32_t *big_tables = nullptr;   // global hash tables of the last degree bucket
    double *pin64 = nullptr;          // per-community p_in of the current statistics
    float2 *pin32 = nullptr;          // and its FP32 enclosure
    uint32_t *work_counter = nullptr; // dynamic work distribution

    PhaseTimers timers;
    std::vector<void *> owned;        // device allocations freed with the graph
    uint64_t bytes = 0;

    template <typename T>
    T *alloc(size_t count) {
        void *p = nullptr;
        if (count == 0) count = 1;
        CK(cudaMalloc(&p, count * sizeof(T)));
        owned.push_back(p);
        bytes += count * sizeof(T);
        return (T *)p;
    }
    void free_all();
};

// preprocess.cu
void convert_edges(Ctx &c, const uint32_t *pairs_dev, uint64_t count);
void upload_graph(Ctx &c, uint32_t n, uint32_t m, const uint32_t *indices, const uint32_t *adj,
                  const int32_t *tri, const int32_t *tri_deg);
void finish_graph(Ctx &c);   // nlow, p_ext, degree classes, partition buffers


// partition.cu
void initial_partition(Ctx &c);

// refine.cu
void collect_stats(Ctx &c, const uint32_t *labels, Stats &st);
double compute_wcc(Ctx &c, const uint32_t *labels, const Stats &st);
void improve(Ctx &c, const uint32_t *labels, const Stats &st, uint32_t *next);
void launch_wcc(Ctx &c, const uint32_t *labels, const Stats &st);   // result in c.wcc_sum (device)
void compute_p_ext(Ctx &c);

}  // namespace scd
