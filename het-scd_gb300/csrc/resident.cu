// Resident set: graphs that join and leave a running union between iterations.
//
// A context made a resident set (scd_resident_init) holds its graphs as one
// block-diagonal union graph, exactly like a batch, and advances all graphs
// that are still iterating with one CUDA-graph replay per step (improve,
// statistics, WCC and per-graph loop control of every graph in the same
// launches).  Other contexts convert new graphs meanwhile, on their own
// streams, and hand them over with scd_resident_add; at the next step the set
// re-forms its union from the graphs it keeps and the new ones:
//
//   * every array of a kept graph (CSR, tri, tri_deg, current and best labels,
//     the statistics of its label range, p_ext, WCC, best WCC, the active flag
//     and the iteration count) is gathered into the new union by one launch per
//     array, with its vertex, adjacency and label offsets shifted;
//   * the derived structure of the union (degree classes, row work, hash-table
//     offsets, triangle-counting plan, WCC blocks) is rebuilt;
//   * the captured iteration is captured again for the new union.
//
// Graphs that stopped (converged or reached max_iters) are frozen in place
// (every kernel skips them) until scd_resident_take copies their labels out;
// their memory is reclaimed at the next re-forming of the union, which happens
// when graphs are waiting to join or when taken graphs hold more than a quarter
// of the union's vertices.  Per graph, the arithmetic is the one of running it
// alone: a graph's result does not depend on its position in the union, on the
// other graphs, or on when it joined.
#include <chrono>
#include <cstring>
#include <deque>
#include <mutex>
#include <type_traits>

#include "engine.cuh"

namespace scd {

namespace {

constexpr unsigned TPB = 256;

// One contiguous piece of an array gathered into a new union:
// dst[dst_off + i] = src[src_off + i] + add for i < len (INVALID kept as is
// when the kernel is told to).
struct Seg {
    const void *src;
    uint64_t src_off, dst_off, len;
    int64_t add;
};

template <typename T>
__global__ void k_gather(const Seg *__restrict__ segs, uint32_t nseg, uint64_t total, T *__restrict__ dst,
                         bool keep_invalid) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = nseg;   // last segment with dst_off <= i
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (segs[mid].dst_off <= i) lo = mid;
            else hi = mid;
        }
        const Seg sg = segs[lo];
        T v = ((const T *)sg.src)[sg.src_off + (i - sg.dst_off)];
        if constexpr (std::is_integral<T>::value) {
            if (sg.add != 0 && !(keep_invalid && (uint64_t)v == (uint64_t)(T)INVALID))
                v = (T)((int64_t)v + sg.add);
        }
        dst[i] = v;
    }
}

// Host data of several small uploads gathered into one pinned buffer (pageable
// copies can wait for the driver's staging buffer, which waits for the device).
struct Uploads {
    std::vector<char> host;
    std::vector<std::pair<size_t, std::pair<void *, size_t>>> items;   // (offset in host, (device dst, bytes))
    size_t put(void *dst, const void *src, size_t bytes) {
        const size_t at = (host.size() + 15) & ~(size_t)15;
        host.resize(at + bytes);
        if (bytes) memcpy(host.data() + at, src, bytes);
        items.push_back({at, {dst, bytes}});
        return at;
    }
};

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// the arrays of a (source or current) union that a graph is gathered from
struct UnionArrays {
    const uint32_t *indices, *adj, *labels, *best;
    const int32_t *tri, *tri_deg;
    Stats st;
    const double *p_ext, *wcc, *best_wcc;
    const float2 *pe32;
    const uint8_t *active;
    const int32_t *iters;
};

UnionArrays arrays_of(const Ctx &c) {
    return UnionArrays{c.g.indices, c.g.adj, c.labels, c.best, c.g.tri, c.g.tri_deg, c.st[c.cur],
                       c.b.p_ext, c.b.wcc, c.b.best_wcc, c.b.pe32, c.b.active, c.b.iters};
}

// The vertex lists of a union's structure, each sorted by vertex id (so each
// graph's entries are one contiguous piece): the degree classes, the long rows,
// the WCC triangle-counting buckets; with the offset array that goes with some
// of them (table words of the last class, pieces of the long rows, work units of
// the buckets).
constexpr int NCLS = DegreeClasses::K, LONG = NCLS, BUCKET0 = NCLS + 1, NL = NCLS + 1 + TcPlan::K;
struct UnionLists {
    const uint32_t *list[NL];
    uint32_t count[NL];
    const void *off[NL];   // nullptr, or count+1 offsets (u64 for the table words)
    bool off64[NL];
};

UnionLists lists_of(const Ctx &c) {
    UnionLists L{};
    for (int k = 0; k < NCLS; k++) {
        L.list[k] = c.g.cls.list[k];
        L.count[k] = c.g.cls.count[k];
    }
    L.off[NCLS - 1] = c.g.big_table_off;
    L.off64[NCLS - 1] = true;
    L.list[LONG] = c.g.rows.llong;
    L.count[LONG] = c.g.rows.nlong;
    L.off[LONG] = c.g.rows.chunk_off;
    for (int k = 0; k < TcPlan::K; k++) {
        L.list[BUCKET0 + k] = c.wplan.verts[k];
        L.count[BUCKET0 + k] = c.wplan.nverts[k];
        L.off[BUCKET0 + k] = c.wplan.unit_off[k];
    }
    return L;
}

// A graph's share of each list: entries, and the span of the offsets (table
// words, long-row pieces, work units) they cover.
struct GraphLists {
    uint32_t cnt[NL] = {};
    uint64_t span[NL] = {};
};

// pos/off of the first entry of every graph g (vertex >= fin_off[g]) in every list
__global__ void k_list_bounds(UnionLists L, const uint32_t *__restrict__ fin_off, uint32_t G, uint64_t *out) {
    const uint32_t total = NL * (G + 1);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const uint32_t l = i / (G + 1), g = i % (G + 1);
        const uint32_t pos = L.count[l] ? lower_bound(L.list[l], L.count[l], fin_off[g]) : 0u;
        uint64_t ov = 0;
        if (L.off[l]) ov = L.off64[l] ? ((const uint64_t *)L.off[l])[pos] : ((const uint32_t *)L.off[l])[pos];
        out[2 * i] = pos;
        out[2 * i + 1] = ov;
    }
}

// every graph's GraphLists from the union's lists (one host read)
std::vector<GraphLists> graph_lists(Ctx &c) {
    const uint32_t G = c.b.G;
    cudaStream_t s = c.stream;
    std::vector<uint64_t> h(2 * (size_t)NL * (G + 1));
    DevBuf<uint64_t> d(h.size(), s);
    k_list_bounds<<<grid_for((uint64_t)NL * (G + 1), 256), 256, 0, s>>>(lists_of(c), c.b.fin_off, G, d.get());
    CK_LAUNCH("k_list_bounds");
    c.launches++;
    CK(cudaMemcpyAsync(h.data(), d.get(), 8 * h.size(), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::vector<GraphLists> out(G);
    for (int l = 0; l < NL; l++)
        for (uint32_t g = 0; g < G; g++) {
            const size_t a = 2 * ((size_t)l * (G + 1) + g), b = a + 2;
            out[g].cnt[l] = (uint32_t)(h[b] - h[a]);
            out[g].span[l] = h[b + 1] - h[a + 1];
        }
    return out;
}

__global__ void k_graph_ids(uint32_t n, uint32_t G, const uint32_t *__restrict__ fin_off, uint32_t *gid) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = G + 1;   // last g with fin_off[g] <= v
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (fin_off[mid] <= v) lo = mid + 1;
            else hi = mid;
        }
        gid[v] = lo - 1;
    }
}

}  // namespace

// Graphs converted by another context, waiting to join (their device arrays
// move with them and are freed once the union has gathered them).
struct ResidentSource {
    std::vector<void *> owned;
    uint64_t bytes = 0;
    UnionArrays a{};
    std::vector<uint32_t> fin_off, comm_off, m;   // per graph of the source union
    UnionLists lists{};
    const uint32_t *nlow = nullptr;
    std::vector<GraphLists> gl;                  // per graph of the source union
    std::vector<uint64_t> ids;
    std::vector<double> wcc0;
    cudaEvent_t ready = nullptr;   // the source's stream has finished its work
    double t_added = 0;
};

struct ResidentGraph {
    uint64_t id = 0;
    uint32_t n = 0, m = 0, nc = 0;   // vertices, undirected edges, label range
    uint32_t v0 = 0, c0 = 0;         // vertex and label offset in the union
    uint64_t e0 = 0;                 // adjacency offset in the union
    double wcc0 = 0, t_join = 0;
    bool finished = false, taken = false, limit = false;
    int32_t iters = 0;
    double best_wcc = 0;
    GraphLists gl;                   // its share of the union's structure lists
};

struct ResidentSet {
    std::mutex lock;                     // pending and next_id (scd_resident_add may run on other threads)
    std::deque<ResidentSource *> pending;
    uint64_t next_id = 0;
    double threshold = 0.01;
    int max_iters = 1000;
    std::vector<ResidentGraph> graphs;   // union order
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    uint64_t exec_kernels[2] = {0, 0};
    uint8_t *h_active = nullptr;         // pinned mirrors of the per-graph loop state
    int32_t *h_iters = nullptr;
    double *h_best = nullptr;
    size_t h_cap = 0;
    uint32_t *h_labels = nullptr;        // pinned staging of taken labels
    size_t h_labels_cap = 0;
    char *h_up = nullptr;                // pinned staging of a re-forming's uploads
    size_t h_up_cap = 0;
    cudaEvent_t up_done = nullptr;       // its copies have been made
    // copies u to the device through h_up: waits for the previous re-forming's copies
    // (long done, normally) before reusing the buffer
    void upload(const Uploads &u, cudaStream_t s) {
        if (u.items.empty()) return;
        if (up_done) CK(cudaEventSynchronize(up_done));
        else CK(cudaEventCreateWithFlags(&up_done, cudaEventDisableTiming));
        if (u.host.size() > h_up_cap) {
            if (h_up) cudaFreeHost(h_up);
            h_up = nullptr;
            h_up_cap = 0;
            const size_t cap = u.host.size() * 2 + 4096;
            CK(cudaMallocHost((void **)&h_up, cap));
            h_up_cap = cap;
        }
        memcpy(h_up, u.host.data(), u.host.size());
        for (const auto &it : u.items)
            if (it.second.second)
                CK(cudaMemcpyAsync(it.second.first, h_up + it.first, it.second.second, cudaMemcpyHostToDevice, s));
        CK(cudaEventRecord(up_done, s));
    }
    uint64_t steps = 0, graph_steps = 0, rebuilds = 0, last_kernels = 0;
    uint32_t stable = 0;                 // steps since the union was last re-formed
    uint32_t split[4] = {};              // triangle-counting split of the set (its buckets' bounds)
    double ms_rebuild = 0, ms_capture = 0, ms_step = 0;   // host wall time spent in each part of the steps

    void drop_exec() {
        for (int k = 0; k < 2; k++) {
            if (exec[k]) cudaGraphExecDestroy(exec[k]);
            exec[k] = nullptr;
            exec_kernels[k] = 0;
        }
    }
};

namespace {

void free_source(ResidentSource *ps, cudaStream_t s) {
    if (ps->ready) {
        cudaStreamWaitEvent(s, ps->ready, 0);
        cudaEventDestroy(ps->ready);
    }
    for (void *p : ps->owned) cudaFreeAsync(p, s);
    delete ps;
}

void ensure_host_mirrors(ResidentSet &R, size_t G) {
    if (G <= R.h_cap) return;
    size_t cap = R.h_cap ? R.h_cap : 64;
    while (cap < G) cap *= 2;
    if (R.h_active) cudaFreeHost(R.h_active);
    if (R.h_iters) cudaFreeHost(R.h_iters);
    if (R.h_best) cudaFreeHost(R.h_best);
    R.h_active = nullptr;
    R.h_iters = nullptr;
    R.h_best = nullptr;
    R.h_cap = 0;
    CK(cudaMallocHost((void **)&R.h_active, cap));
    CK(cudaMallocHost((void **)&R.h_iters, cap * 4));
    CK(cudaMallocHost((void **)&R.h_best, cap * 8));
    R.h_cap = cap;
}

// Gathers of several arrays with one upload of all their segment tables.
struct Gathers {
    enum Kind { U32, I32, F64, F2, U8, U64 };
    struct Job {
        size_t first, count;
        uint64_t total;
        void *dst;
        Kind kind;
        bool keep_invalid;
    };
    std::vector<Seg> segs;
    std::vector<Job> jobs;
    template <typename T>
    void add(const std::vector<Seg> &in, uint64_t total, T *dst, bool keep_invalid) {
        Kind k = std::is_same<T, uint32_t>::value   ? U32
                 : std::is_same<T, int32_t>::value  ? I32
                 : std::is_same<T, double>::value   ? F64
                 : std::is_same<T, float2>::value   ? F2
                 : std::is_same<T, uint64_t>::value ? U64
                                                    : U8;
        const size_t first = segs.size();
        for (const Seg &x : in)
            if (x.len) segs.push_back(x);
        if (total) jobs.push_back(Job{first, segs.size() - first, total, (void *)dst, k, keep_invalid});
    }
    // launches every job with the segment tables at dev (segs already copied there)
    void launch(Ctx &c, const Seg *dev) {
        cudaStream_t s = c.stream;
        for (const Job &j : jobs) {
            const Seg *t = dev + j.first;
            const uint32_t ns = (uint32_t)j.count;
            const unsigned grid = grid_for(j.total, TPB, 152 * 16);
            switch (j.kind) {
            case U32: k_gather<uint32_t><<<grid, TPB, 0, s>>>(t, ns, j.total, (uint32_t *)j.dst, j.keep_invalid); break;
            case I32: k_gather<int32_t><<<grid, TPB, 0, s>>>(t, ns, j.total, (int32_t *)j.dst, j.keep_invalid); break;
            case F64: k_gather<double><<<grid, TPB, 0, s>>>(t, ns, j.total, (double *)j.dst, false); break;
            case F2: k_gather<float2><<<grid, TPB, 0, s>>>(t, ns, j.total, (float2 *)j.dst, false); break;
            case U8: k_gather<uint8_t><<<grid, TPB, 0, s>>>(t, ns, j.total, (uint8_t *)j.dst, false); break;
            case U64: k_gather<uint64_t><<<grid, TPB, 0, s>>>(t, ns, j.total, (uint64_t *)j.dst, false); break;
            }
            CK_LAUNCH("k_gather");
            c.launches++;
        }
    }
    void run(Ctx &c) {   // with its own (pageable) upload of the tables
        if (jobs.empty()) return;
        DevBuf<Seg> d(segs.size(), c.stream);
        CK(cudaMemcpyAsync(d.get(), segs.data(), sizeof(Seg) * segs.size(), cudaMemcpyHostToDevice, c.stream));
        launch(c, d.get());
    }
};

// A graph of the new union and where its state comes from.
struct Move {
    UnionArrays a;
    uint32_t sg;             // graph index in its source union
    uint32_t v0, c0;         // offsets in the source union
    uint64_t e0;
    ResidentGraph info;      // offsets set to the new union's
    const UnionLists *lists = nullptr;   // its source's structure lists
    const uint32_t *nlow = nullptr;
    uint64_t lpos[NL] = {}, lbase[NL] = {};   // its first entry and offset in them
};

// Re-forms the union: the kept graphs (not taken) of the current union, then the
// graphs of the pending sources, gathered into fresh arrays.  The structure lists
// are concatenated from every graph's share (counts known on the host), so the
// whole re-forming is queued without waiting for the device.
// Returns the number of joining graphs that have nothing to iterate (empty graphs).
uint32_t rebuild(Ctx &c, ResidentSet &R, std::vector<ResidentSource *> &srcs) {
    cudaStream_t s = c.stream;
    std::vector<Move> mv;
    uint32_t joined_done = 0;
    const UnionArrays cur = arrays_of(c);
    const UnionLists cur_lists = lists_of(c);
    {
        uint64_t pos[NL] = {}, base[NL] = {};
        for (uint32_t k = 0; k < R.graphs.size(); k++) {
            const ResidentGraph &g = R.graphs[k];
            if (!g.taken) {
                Move m{cur, k, g.v0, g.c0, g.e0, g, &cur_lists, c.g.nlow};
                for (int l = 0; l < NL; l++) {
                    m.lpos[l] = pos[l];
                    m.lbase[l] = base[l];
                }
                mv.push_back(m);
            }
            for (int l = 0; l < NL; l++) {
                pos[l] += g.gl.cnt[l];
                base[l] += g.gl.span[l];
            }
        }
    }
    for (ResidentSource *ps : srcs) {
        CK(cudaStreamWaitEvent(s, ps->ready, 0));
        uint64_t e0 = 0, pos[NL] = {}, base[NL] = {};
        for (uint32_t k = 0; k + 1 < ps->fin_off.size(); k++) {
            ResidentGraph g;
            g.id = ps->ids[k];
            g.n = ps->fin_off[k + 1] - ps->fin_off[k];
            g.m = ps->m[k];
            g.nc = ps->comm_off[k + 1] - ps->comm_off[k];
            g.wcc0 = ps->wcc0[k];
            g.best_wcc = ps->wcc0[k];
            g.t_join = ps->t_added;
            g.gl = ps->gl[k];
            g.finished = g.n == 0;   // nothing to iterate (active is 0 for it already)
            joined_done += g.finished;
            Move m{ps->a, k, ps->fin_off[k], ps->comm_off[k], e0, g, &ps->lists, ps->nlow};
            for (int l = 0; l < NL; l++) {
                m.lpos[l] = pos[l];
                m.lbase[l] = base[l];
                pos[l] += g.gl.cnt[l];
                base[l] += g.gl.span[l];
            }
            mv.push_back(m);
            e0 += 2 * (uint64_t)g.m;
        }
    }
    // new offsets
    const uint32_t G = (uint32_t)mv.size();
    uint64_t N = 0, M2 = 0, NC = 0, lcnt[NL] = {}, lspan[NL] = {};
    for (Move &x : mv) {
        x.info.v0 = (uint32_t)N;
        x.info.e0 = M2;
        x.info.c0 = (uint32_t)NC;
        N += x.info.n;
        M2 += 2 * (uint64_t)x.info.m;
        NC += x.info.nc;
        for (int l = 0; l < NL; l++) {
            lcnt[l] += x.info.gl.cnt[l];
            lspan[l] += x.info.gl.span[l];
        }
    }
    if (N >= 0xffffffffull || M2 >= 0xffffffffull) throw Error(SCD_ERR_LIMIT, "resident set beyond 2^32-1 entries");
    std::vector<void *> old_owned = std::move(c.owned);
    c.owned.clear();
    c.bytes = 0;
    R.drop_exec();
    c.g = Graph();
    c.b = Batch();
    c.wplan = TcPlan();
    c.has_graph = c.has_labels = false;
    c.pext_join_pending = false;
    c.pext_host_valid = false;
    c.resident = true;
    if (G == 0) {
        for (void *p : old_owned) cudaFreeAsync(p, s);
        for (ResidentSource *ps : srcs) free_source(ps, s);
        srcs.clear();
        R.graphs.clear();
        c.labels = c.labels_next = c.best = nullptr;
        c.st[0] = c.st[1] = Stats();
        c.num_comms = 0;
        return joined_done;
    }
    try {
        Graph &g = c.g;
        Batch &b = c.b;
        g.n = (uint32_t)N;
        g.m = (uint32_t)(M2 / 2);
        b.G = G;
        g.indices = c.alloc<uint32_t>(N + 1);
        g.adj = c.alloc<uint32_t>(M2);
        g.tri = c.alloc<int32_t>(N);
        g.tri_deg = c.alloc<int32_t>(N);
        g.nlow = c.alloc<uint32_t>(N);
        c.labels = c.alloc<uint32_t>(N);
        c.labels_next = c.alloc<uint32_t>(N);
        c.best = c.alloc<uint32_t>(N);
        for (int k = 0; k < 2; k++) {
            c.st[k].sizes = c.alloc<int32_t>(N);
            c.st[k].ext = c.alloc<int32_t>(N);
            c.st[k].intl = c.alloc<int32_t>(N);
        }
        c.cur = 0;
        c.num_comms = (uint32_t)NC;
        b.fin_off = c.alloc<uint32_t>(G + 1);
        b.comm_off = c.alloc<uint32_t>(G + 1);
        b.gid = c.alloc<uint32_t>(N);
        b.p_ext = c.alloc<double>(G);
        b.pe32 = c.alloc<float2>(G);
        b.wcc = c.alloc<double>(G);
        b.best_wcc = c.alloc<double>(G);
        b.active = c.alloc<uint8_t>(G);
        b.improved = c.alloc<uint8_t>(G);
        b.iters = c.alloc<int32_t>(G);
        b.n_active = c.alloc<uint32_t>(1);
        // the structure: lists and their offset arrays (the last offset, the total, from the host)
        uint32_t *list[NL];
        void *off[NL] = {};
        for (int l = 0; l < NL; l++) list[l] = c.alloc<uint32_t>(lcnt[l]);
        off[NCLS - 1] = c.alloc<uint64_t>(lcnt[NCLS - 1] + 1);
        off[LONG] = c.alloc<uint32_t>(lcnt[LONG] + 1);
        for (int k = 0; k < TcPlan::K; k++) off[BUCKET0 + k] = c.alloc<uint32_t>(lcnt[BUCKET0 + k] + 1);
        for (int k = 0; k < NCLS; k++) {
            g.cls.list[k] = list[k];
            g.cls.count[k] = (uint32_t)lcnt[k];
        }
        g.big_table_off = (uint64_t *)off[NCLS - 1];
        g.big_table_words = lspan[NCLS - 1];
        c.big_tables = lspan[NCLS - 1] ? c.alloc<uint32_t>(lspan[NCLS - 1]) : nullptr;
        g.rows.llong = list[LONG];
        g.rows.nlong = (uint32_t)lcnt[LONG];
        g.rows.chunk_off = (uint32_t *)off[LONG];
        g.rows.nchunks = (uint32_t)lspan[LONG];
        TcPlan &pl = c.wplan;
        for (int k = 0; k < TcPlan::K; k++) {
            pl.verts[k] = list[BUCKET0 + k];
            pl.unit_off[k] = (uint32_t *)off[BUCKET0 + k];
            pl.nverts[k] = pl.nfwd[k] = (uint32_t)lcnt[BUCKET0 + k];
        }
        pl.dir_lo = pl.dir_hi = 0;   // out-list centres only, as tc_plan builds the WCC plan
        pl.dir_amin = c.tc_amin < c.tc_small ? c.tc_amin : c.tc_small;
        // scratch of the iteration
        c.pin64 = c.alloc<double>(N);
        c.civ = c.alloc<int4>(N);
        c.slot_flag = c.alloc<uint8_t>(M2);
        c.itcount = c.alloc<uint32_t>(N);
        c.itdeg = c.alloc<int32_t>(N);
        c.int_len = c.alloc<uint32_t>(N);
        c.int_adj = c.alloc<uint32_t>(M2);

        std::vector<Seg> ind, adj, tri, tdg, nlw, lab, bst, sz, ex, in, pe, pe2, wc, bw, ac, it;
        std::vector<Seg> lseg[NL], oseg[NL];
        uint64_t npos[NL] = {}, nbase[NL] = {};
        for (uint32_t j = 0; j < G; j++) {
            const Move &x = mv[j];
            const ResidentGraph &ni = x.info;
            const bool last = j + 1 == G;   // the last graph also supplies indices[N]
            const int64_t dv = (int64_t)ni.v0 - (int64_t)x.v0;
            ind.push_back(Seg{x.a.indices, x.v0, ni.v0, ni.n + (last ? 1u : 0u), (int64_t)ni.e0 - (int64_t)x.e0});
            adj.push_back(Seg{x.a.adj, x.e0, ni.e0, 2 * (uint64_t)ni.m, dv});
            tri.push_back(Seg{x.a.tri, x.v0, ni.v0, ni.n, 0});
            tdg.push_back(Seg{x.a.tri_deg, x.v0, ni.v0, ni.n, 0});
            nlw.push_back(Seg{x.nlow, x.v0, ni.v0, ni.n, 0});
            lab.push_back(Seg{x.a.labels, x.v0, ni.v0, ni.n, (int64_t)ni.c0 - (int64_t)x.c0});
            bst.push_back(Seg{x.a.best, x.v0, ni.v0, ni.n, (int64_t)ni.c0 - (int64_t)x.c0});
            sz.push_back(Seg{x.a.st.sizes, x.c0, ni.c0, ni.nc, 0});
            ex.push_back(Seg{x.a.st.ext, x.c0, ni.c0, ni.nc, 0});
            in.push_back(Seg{x.a.st.intl, x.c0, ni.c0, ni.nc, 0});
            pe.push_back(Seg{x.a.p_ext, x.sg, j, 1, 0});
            pe2.push_back(Seg{x.a.pe32, x.sg, j, 1, 0});
            wc.push_back(Seg{x.a.wcc, x.sg, j, 1, 0});
            bw.push_back(Seg{x.a.best_wcc, x.sg, j, 1, 0});
            ac.push_back(Seg{x.a.active, x.sg, j, 1, 0});
            it.push_back(Seg{x.a.iters, x.sg, j, 1, 0});
            for (int l = 0; l < NL; l++) {
                const uint32_t cn = ni.gl.cnt[l];
                lseg[l].push_back(Seg{x.lists->list[l], x.lpos[l], npos[l], cn, dv});
                if (off[l]) oseg[l].push_back(Seg{x.lists->off[l], x.lpos[l], npos[l], cn,
                                                  (int64_t)nbase[l] - (int64_t)x.lbase[l]});
                npos[l] += cn;
                nbase[l] += ni.gl.span[l];
            }
        }
        if (N == 0) CK(cudaMemsetAsync(g.indices, 0, 4, s));
        Gathers ga;
        ga.add<uint32_t>(ind, N + 1, g.indices, false);
        ga.add<uint32_t>(adj, M2, g.adj, false);
        ga.add<int32_t>(tri, N, g.tri, false);
        ga.add<int32_t>(tdg, N, g.tri_deg, false);
        ga.add<uint32_t>(nlw, N, g.nlow, false);
        ga.add<uint32_t>(lab, N, c.labels, true);
        ga.add<uint32_t>(bst, N, c.best, true);
        ga.add<int32_t>(sz, NC, c.st[0].sizes, false);
        ga.add<int32_t>(ex, NC, c.st[0].ext, false);
        ga.add<int32_t>(in, NC, c.st[0].intl, false);
        ga.add<double>(pe, G, b.p_ext, false);
        ga.add<float2>(pe2, G, b.pe32, false);
        ga.add<double>(wc, G, b.wcc, false);
        ga.add<double>(bw, G, b.best_wcc, false);
        ga.add<uint8_t>(ac, G, b.active, false);
        ga.add<int32_t>(it, G, b.iters, false);
        for (int l = 0; l < NL; l++) {
            ga.add<uint32_t>(lseg[l], lcnt[l], list[l], false);
            if (l == NCLS - 1) ga.add<uint64_t>(oseg[l], lcnt[l], (uint64_t *)off[l], false);
            else if (off[l]) ga.add<uint32_t>(oseg[l], lcnt[l], (uint32_t *)off[l], false);
        }
        // every small upload of the re-forming in one pinned copy-out, then the gathers
        Uploads up;
        DevBuf<Seg> dsegs(ga.segs.size() ? ga.segs.size() : 1, s);
        up.put(dsegs.get(), ga.segs.data(), sizeof(Seg) * ga.segs.size());
        for (int l = 0; l < NL; l++) {   // the offset arrays' totals
            if (!off[l]) continue;
            if (l == NCLS - 1) {
                up.put((uint64_t *)off[l] + lcnt[l], &lspan[l], 8);
            } else {
                const uint32_t t = (uint32_t)lspan[l];
                up.put((uint32_t *)off[l] + lcnt[l], &t, 4);
            }
        }
        b.h_fin_off.assign(G + 1, 0);
        b.h_comm_off.assign(G + 1, 0);
        b.h_m.assign(G, 0);
        R.graphs.clear();
        for (uint32_t j = 0; j < G; j++) {
            b.h_fin_off[j] = mv[j].info.v0;
            b.h_comm_off[j] = mv[j].info.c0;
            b.h_m[j] = mv[j].info.m;
            R.graphs.push_back(mv[j].info);
        }
        b.h_fin_off[G] = (uint32_t)N;
        b.h_comm_off[G] = (uint32_t)NC;
        up.put(b.fin_off, b.h_fin_off.data(), 4 * (G + 1));
        up.put(b.comm_off, b.h_comm_off.data(), 4 * (G + 1));
        {   // graph-aligned WCC blocks (host-computed)
            std::vector<uint32_t> blk_off(G + 1, 0), blk_gid;
            for (uint32_t k = 0; k < G; k++) {
                const uint32_t parts = (mv[k].info.n + 2047) / 2048;
                blk_off[k + 1] = blk_off[k] + parts;
                blk_gid.insert(blk_gid.end(), parts, k);
            }
            b.blocks = blk_off[G];
            b.blk_off = c.alloc<uint32_t>(G + 1);
            b.blk_gid = c.alloc<uint32_t>(b.blocks);
            up.put(b.blk_off, blk_off.data(), 4 * (G + 1));
            up.put(b.blk_gid, blk_gid.data(), 4 * (size_t)b.blocks);
        }
        R.upload(up, s);
        ga.launch(c, dsegs.get());
        if (N) {
            k_graph_ids<<<grid_for(N, TPB), TPB, 0, s>>>((uint32_t)N, G, b.fin_off, b.gid);
            CK_LAUNCH("k_graph_ids");
            c.launches++;
        }
        c.wcc_part = c.alloc<double>(b.blocks + 1);
        prepare_tc_kernels();
        prepare_improve_kernels();
        c.has_graph = c.has_labels = true;
        for (void *p : old_owned) cudaFreeAsync(p, s);
        for (ResidentSource *ps : srcs) free_source(ps, s);
        srcs.clear();
    } catch (...) {
        // an allocation or launch failed half-way: the set drops everything (old and
        // new arrays, the joining graphs) and stays usable, empty
        cudaStreamSynchronize(s);
        for (void *p : c.owned) cudaFreeAsync(p, s);
        c.owned.clear();
        c.bytes = 0;
        for (void *p : old_owned) cudaFreeAsync(p, s);
        for (ResidentSource *ps : srcs) free_source(ps, s);
        srcs.clear();
        R.graphs.clear();
        c.g = Graph();
        c.b = Batch();
        c.wplan = TcPlan();
        c.labels = c.labels_next = c.best = nullptr;
        c.st[0] = c.st[1] = Stats();
        c.num_comms = 0;
        c.has_graph = c.has_labels = false;
        throw;
    }
    R.rebuilds++;
    return joined_done;
}

ResidentSet &require_set(Ctx &c) {
    if (!c.res) throw Error(SCD_ERR_STATE, "the context is not a resident set (scd_resident_init)");
    return *c.res;
}

}  // namespace

void resident_destroy(Ctx &c) {
    if (!c.res) return;
    ResidentSet *R = c.res;
    c.res = nullptr;
    R->drop_exec();
    for (ResidentSource *ps : R->pending) free_source(ps, c.stream);
    R->pending.clear();
    if (R->h_active) cudaFreeHost(R->h_active);
    if (R->h_iters) cudaFreeHost(R->h_iters);
    if (R->h_best) cudaFreeHost(R->h_best);
    if (R->h_labels) cudaFreeHost(R->h_labels);
    if (R->h_up) cudaFreeHost(R->h_up);
    if (R->up_done) cudaEventDestroy(R->up_done);
    delete R;
}

}  // namespace scd

using namespace scd;

namespace {

template <typename F>
int guarded_res(scd_ctx *ctx, F &&f) {
    if (!ctx) return SCD_ERR_ARG;
    try {
        CK(cudaSetDevice(ctx->c.device));
        f(ctx->c);
        ctx->c.err.clear();
        return SCD_OK;
    } catch (const Error &e) {
        ctx->c.err = e.what();
        return e.status;
    } catch (const std::bad_alloc &) {
        ctx->c.err = "host allocation failed";
        return SCD_ERR_OOM;
    } catch (const std::exception &e) {
        ctx->c.err = e.what();
        return SCD_ERR_CUDA;
    }
}

}  // namespace

extern "C" {

int scd_resident_init(scd_ctx *ctx, double threshold, int max_iters) {
    return guarded_res(ctx, [&](Ctx &c) {
        if (c.res) throw Error(SCD_ERR_STATE, "already a resident set");
        if (max_iters < 1) throw Error(SCD_ERR_ARG, "max_iters < 1");
        c.free_all();
        c.res = new ResidentSet();
        c.res->threshold = threshold;
        c.res->max_iters = max_iters;
        const uint32_t sp[4] = {c.tc_small, c.tc_b0, c.tc_b1, c.tc_amin};
        memcpy(c.res->split, sp, sizeof sp);
        c.resident = true;
    });
}

int scd_resident_add(scd_ctx *set, scd_ctx *src, uint64_t *ids) {
    if (!set || !src || set == src) return SCD_ERR_ARG;
    ResidentSet *R = set->c.res;
    if (!R) return SCD_ERR_STATE;
    const int dev = set->c.device;
    return guarded_res(src, [&](Ctx &s) {
        if (!s.has_graph) throw Error(SCD_ERR_STATE, "no graph on the device");
        if (s.res) throw Error(SCD_ERR_ARG, "the source is itself a resident set");
        if (s.device != dev) throw Error(SCD_ERR_ARG, "the source is on another device");
        // the prologue of the refinement loop (src/main-gpu.cpp:54-70), on the source's stream
        if (!s.has_labels) initial_partition(s);
        launch_wcc(s, s.labels, s.st[s.cur]);
        join_p_ext(s);
        batch_reset(s);
        auto *ps = new ResidentSource();
        const uint32_t G = s.b.G;
        ps->wcc0.resize(G);
        CK(cudaMemcpyAsync(ps->wcc0.data(), s.b.wcc, 8 * G, cudaMemcpyDeviceToHost, s.stream));
        CK(cudaStreamSynchronize(s.stream));
        // the WCC's triangle-counting plan under the set's split, so every graph's
        // buckets mean the same in the union; then each graph's share of the lists
        const uint32_t *sp = R->split;
        if (s.tc_small != sp[0] || s.tc_b0 != sp[1] || s.tc_b1 != sp[2] || s.tc_amin != sp[3]) {
            s.tc_small = sp[0];
            s.tc_b0 = sp[1];
            s.tc_b1 = sp[2];
            s.tc_amin = sp[3];
            s.wplan = TcPlan();
            if (s.g.n) tc_plan(s, Oriented{s.g.indices, s.g.nlow, s.g.adj, s.g.n}, s.wplan, s.stream, true, false);
        }
        ps->lists = lists_of(s);
        ps->nlow = s.g.nlow;
        ps->gl = graph_lists(s);
        ps->a = arrays_of(s);
        ps->fin_off = s.b.h_fin_off;
        ps->comm_off = s.b.h_comm_off;
        ps->m = s.b.h_m;
        ps->owned = std::move(s.owned);
        ps->bytes = s.bytes;
        ps->t_added = now_ms();
        s.owned.clear();
        CK(cudaEventCreateWithFlags(&ps->ready, cudaEventDisableTiming));
        CK(cudaEventRecord(ps->ready, s.stream));
        s.free_all();   // nothing left to free: the arrays moved with the graphs
        std::lock_guard<std::mutex> hold(R->lock);
        for (uint32_t k = 0; k < G; k++) ps->ids.push_back(R->next_id++);
        if (ids)
            for (uint32_t k = 0; k < G; k++) ids[k] = ps->ids[k];
        R->pending.push_back(ps);
    });
}

int scd_resident_step(scd_ctx *ctx, uint32_t *running, uint32_t *finished) {
    return guarded_res(ctx, [&](Ctx &c) {
        ResidentSet &R = require_set(c);
        cudaStream_t s = c.stream;
        std::vector<ResidentSource *> srcs;
        {
            std::lock_guard<std::mutex> hold(R.lock);
            srcs.assign(R.pending.begin(), R.pending.end());
            R.pending.clear();
        }
        uint64_t taken_v = 0, kept = 0;
        for (const ResidentGraph &g : R.graphs) {
            if (g.taken) taken_v += g.n;
            else kept++;
        }
        const bool any_taken = kept < R.graphs.size();
        uint32_t run = 0, fin = 0;
        const double t_step = now_ms();
        if (!srcs.empty() || (any_taken && (kept == 0 || 4 * taken_v > c.g.n))) {
            R.stable = 0;
            try {
                const double t0 = now_ms();
                fin += rebuild(c, R, srcs);
                R.ms_rebuild += now_ms() - t0;
            } catch (...) {
                for (ResidentSource *ps : srcs) free_source(ps, s);
                throw;
            }
        }
        for (ResidentGraph &g : R.graphs)
            if (!g.finished) run++;
        if (run) {
            const int par = c.cur;
            // a union that changes every few steps is launched kernel by kernel: capturing and
            // instantiating a CUDA graph costs more than the launches it saves for one replay
            const bool replay = R.exec[par] || R.stable >= 6;
            R.stable++;
            if (!replay) {
                const uint64_t l0 = c.launches;
                iterate_async(c, R.threshold, nullptr, 0);
                R.last_kernels = c.launches - l0;
            } else if (!R.exec[par]) {
                const double t0 = now_ms();
                cudaGraph_t gr = nullptr;
                CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                c.capturing = true;
                try {
                    iterate_async(c, R.threshold, nullptr, 0);
                } catch (...) {
                    c.capturing = false;
                    cudaStreamEndCapture(s, &gr);
                    if (gr) cudaGraphDestroy(gr);
                    throw;
                }
                c.capturing = false;
                CK(cudaStreamEndCapture(s, &gr));
                R.exec_kernels[par] = kernel_nodes(gr);
                const cudaError_t e = cudaGraphInstantiate(&R.exec[par], gr, 0);
                cudaGraphDestroy(gr);
                CK(e);
                R.ms_capture += now_ms() - t0;
            } else {   // replaying advances the state as the captured host code did
                uint32_t *t = c.labels;
                c.labels = c.labels_next;
                c.labels_next = t;
                c.cur ^= 1;
            }
            if (replay) {
                CK(cudaGraphLaunch(R.exec[par], s));
                c.launches += R.exec_kernels[par];
                R.last_kernels = R.exec_kernels[par];
            }
            R.steps++;
            R.graph_steps += run;
            const uint32_t G = c.b.G;
            ensure_host_mirrors(R, G);
            CK(cudaMemcpyAsync(R.h_active, c.b.active, G, cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(R.h_iters, c.b.iters, 4 * (size_t)G, cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(R.h_best, c.b.best_wcc, 8 * (size_t)G, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            for (uint32_t j = 0; j < G; j++) {
                ResidentGraph &g = R.graphs[j];
                if (g.finished) continue;
                g.iters = R.h_iters[j];
                g.best_wcc = R.h_best[j];
                if (!R.h_active[j]) {
                    g.finished = true;
                } else if (g.iters >= R.max_iters) {   // stop it: every kernel skips it from now on
                    CK(cudaMemsetAsync(c.b.active + j, 0, 1, s));
                    g.finished = true;
                    g.limit = true;
                }
                fin += g.finished;
            }
        }
        R.ms_step += now_ms() - t_step;
        if (running) *running = run;
        if (finished) *finished = fin;
    });
}

int scd_resident_take(scd_ctx *ctx, uint32_t cap, uint64_t *ids, scd_result *results, int32_t *status,
                      uint32_t *labels, uint64_t labels_cap, uint64_t *label_offsets, uint32_t *count) {
    return guarded_res(ctx, [&](Ctx &c) {
        ResidentSet &R = require_set(c);
        if (!count) throw Error(SCD_ERR_ARG, "count is NULL");
        cudaStream_t s = c.stream;
        std::vector<uint32_t> pick;
        uint64_t total = 0;
        for (uint32_t j = 0; j < R.graphs.size() && pick.size() < cap; j++) {
            const ResidentGraph &g = R.graphs[j];
            if (!g.finished || g.taken) continue;
            if (labels && total + g.n > labels_cap) break;
            pick.push_back(j);
            total += g.n;
        }
        *count = (uint32_t)pick.size();
        if (pick.empty()) return;
        if (labels && total) {
            std::vector<Seg> segs;
            uint64_t off = 0;
            for (uint32_t j : pick) {
                const ResidentGraph &g = R.graphs[j];
                segs.push_back(Seg{c.best, g.v0, off, g.n, -(int64_t)g.c0});
                off += g.n;
            }
            DevBuf<uint32_t> tmp(total, s);
            Gathers ga;
            ga.add<uint32_t>(segs, total, tmp.get(), true);
            ga.run(c);
            if (total > R.h_labels_cap) {
                if (R.h_labels) cudaFreeHost(R.h_labels);
                R.h_labels = nullptr;
                R.h_labels_cap = 0;
                CK(cudaMallocHost((void **)&R.h_labels, 4 * total));
                R.h_labels_cap = total;
            }
            CK(cudaMemcpyAsync(R.h_labels, tmp.get(), 4 * total, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            memcpy(labels, R.h_labels, 4 * total);
        }
        const double t = now_ms();
        uint64_t off = 0;
        for (uint32_t k = 0; k < pick.size(); k++) {
            ResidentGraph &g = R.graphs[pick[k]];
            if (ids) ids[k] = g.id;
            if (label_offsets) label_offsets[k] = off;
            if (status) status[k] = g.limit ? SCD_ERR_LIMIT : SCD_OK;
            if (results) {
                scd_result &r = results[k];
                memset(&r, 0, sizeof r);
                r.iterations = g.iters;
                r.initial_wcc = g.wcc0;
                r.best_wcc = g.best_wcc;
                r.initial_communities = g.nc;
                if (labels) {   // distinct valid labels (compress_labels prints n minus that)
                    std::vector<uint8_t> seen(g.nc ? g.nc : 1, 0);
                    uint32_t d = 0;
                    for (uint32_t v = 0; v < g.n; v++) {
                        const uint32_t l = labels[off + v];
                        if (l != INVALID && l < g.nc && !seen[l]) {
                            seen[l] = 1;
                            d++;
                        }
                    }
                    r.distinct_communities = d;
                    r.printed_communities = g.n - d;
                }
                r.ms_iterations = t - g.t_join;
            }
            off += g.n;
            g.taken = true;
        }
        if (label_offsets) label_offsets[pick.size()] = off;
    });
}

int scd_resident_info(scd_ctx *ctx, uint32_t *graphs, uint32_t *running, uint32_t *pending, uint64_t *steps,
                      uint64_t *graph_steps, uint64_t *kernels_per_step) {
    return guarded_res(ctx, [&](Ctx &c) {
        ResidentSet &R = require_set(c);
        uint32_t run = 0, kept = 0;
        for (const ResidentGraph &g : R.graphs) {
            run += !g.finished;
            kept += !g.taken;
        }
        if (graphs) *graphs = kept;
        if (running) *running = run;
        if (pending) {
            std::lock_guard<std::mutex> hold(R.lock);
            uint32_t p = 0;
            for (ResidentSource *ps : R.pending) p += (uint32_t)ps->ids.size();
            *pending = p;
        }
        if (steps) *steps = R.steps;
        if (graph_steps) *graph_steps = R.graph_steps;
        if (kernels_per_step) *kernels_per_step = R.last_kernels;
    });
}

int scd_resident_timing(scd_ctx *ctx, double *ms_steps, double *ms_rebuild, double *ms_capture, uint64_t *rebuilds) {
    return guarded_res(ctx, [&](Ctx &c) {
        ResidentSet &R = require_set(c);
        if (ms_steps) *ms_steps = R.ms_step;
        if (ms_rebuild) *ms_rebuild = R.ms_rebuild;
        if (ms_capture) *ms_capture = R.ms_capture;
        if (rebuilds) *rebuilds = R.rebuilds;
    });
}

}  // extern "C"
