// Context management, per-graph setup and the C ABI (include/scd_gb300.h).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <new>

#include "engine.cuh"

namespace scd {

namespace {

constexpr unsigned TPB = 256;

// neighbours with a smaller id: the out-list of the degree orientation
__global__ void k_nlow(uint32_t n, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ adj,
                       uint32_t *nlow) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t beg = indices[v];
        nlow[v] = lower_bound(adj + beg, indices[v + 1] - beg, v);
    }
}

struct ChunksOf {   // RowWork chunks of a long row
    const uint32_t *verts, *indices;
    __device__ uint32_t operator[](size_t i) const {
        const uint32_t v = verts[i];
        return (indices[v + 1] - indices[v] + RowWork::CHUNK - 1) / RowWork::CHUNK;
    }
};

struct InClass {
    const uint32_t *indices;
    uint32_t lo, hi;   // lo <= deg <= hi
    __device__ uint32_t operator[](size_t v) const {
        const uint32_t d = indices[v + 1] - indices[v];
        return d >= lo && d <= hi;
    }
};

__global__ void k_class_scatter(uint32_t n, InClass f, const uint32_t *__restrict__ pos, uint32_t *out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (f[v]) out[pos[v]] = v;
}

struct TableWords {
    const uint32_t *verts, *indices;
    __device__ uint64_t operator[](size_t i) const {
        const uint32_t v = verts[i];
        const uint64_t d = indices[v + 1] - indices[v];
        uint64_t cap = 64;
        while (cap < 2 * d) cap <<= 1;
        return 3 * cap;   // keys, counts, occupied-entry list
    }
};

__global__ void k_seen_labels(uint32_t n, const uint32_t *__restrict__ labels, uint32_t nc, uint32_t *seen) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t l = labels[v];
        if (l != INVALID && l < nc) seen[l] = 1;
    }
}

// compress_labels as intended (src/scd.cpp:32-55 without the inverted branch):
// in vertex order, an unlabelled vertex or the first vertex of a label opens the
// next community id; later vertices of a label take its id
__global__ void k_first_of_label(uint32_t n, const uint32_t *__restrict__ labels, uint32_t *first) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t l = labels[v];
        if (l != INVALID) atomicMin(first + l, v);
    }
}

struct OpensCommunity {
    const uint32_t *labels, *first;
    __device__ uint32_t operator[](size_t v) const {
        const uint32_t l = labels[v];
        return l == INVALID || first[l] == (uint32_t)v;
    }
};

__global__ void k_compressed(uint32_t n, const uint32_t *__restrict__ labels, const uint32_t *__restrict__ first,
                             const uint32_t *__restrict__ rank, uint32_t *out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t l = labels[v];
        out[v] = rank[l == INVALID ? v : first[l]];
    }
}

__global__ void k_distinct_per_graph(uint32_t G, const uint32_t *__restrict__ comm_off, const uint32_t *__restrict__ scan,
                                     uint32_t *out) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < G; g += gridDim.x * blockDim.x)
        out[g] = scan[comm_off[g + 1]] - scan[comm_off[g]];
}

__global__ void k_local_graph(uint32_t n_g, uint32_t m2_g, uint32_t v0, const uint32_t *__restrict__ indices,
                              const uint32_t *__restrict__ adj, uint32_t *ind_out, uint32_t *adj_out) {
    const uint32_t e0 = indices[v0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= n_g; i += gridDim.x * blockDim.x)
        ind_out[i] = indices[v0 + i] - e0;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < m2_g; j += gridDim.x * blockDim.x)
        adj_out[j] = adj[e0 + j] - v0;
}

__global__ void k_local_labels(uint32_t n_g, uint32_t v0, uint32_t l0, const uint32_t *__restrict__ labels,
                               uint32_t *out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_g; i += gridDim.x * blockDim.x) {
        const uint32_t l = labels[v0 + i];
        out[i] = l == INVALID ? INVALID : l - l0;
    }
}

// every graph's labels in its own numbering: l - comm_off[gid[v]]
__global__ void k_local_labels_all(uint32_t n, const uint32_t *__restrict__ gid, const uint32_t *__restrict__ comm_off,
                                   const uint32_t *__restrict__ labels, uint32_t *out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t l = labels[v];
        out[v] = l == INVALID ? INVALID : l - comm_off[gid ? gid[v] : 0u];
    }
}

__global__ void k_gather_indices(uint32_t G, const uint32_t *__restrict__ fin_off, const uint32_t *__restrict__ indices,
                                 uint32_t *out) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += gridDim.x * blockDim.x)
        out[g] = indices[fin_off[g]];
}

__global__ void k_fill_gid(uint32_t n, uint32_t G, const uint32_t *__restrict__ fin_off, uint32_t *gid) {
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

__global__ void k_max_label(uint32_t n, const uint32_t *__restrict__ labels, uint32_t *out) {
    uint32_t m = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t l = labels[v];
        if (l != INVALID && l + 1 > m) m = l + 1;
    }
    m = __reduce_max_sync(FULL, m);
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// the vertex lists of K degree ranges (lo[k], hi[k]] with one host read for all counts
void class_lists(Ctx &c, int K, const uint32_t *lo, const uint32_t *hi, uint32_t **out, uint32_t *cnt) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    std::vector<DevBuf<uint32_t>> pos(K);
    DevBuf<uint32_t> counts(K, s);
    for (int k = 0; k < K; k++) {
        pos[k].alloc((size_t)g.n + 1, s);
        scan_exclusive<uint32_t>(InClass{g.indices, lo[k], hi[k]}, pos[k].get(), g.n, s);
        CK(cudaMemcpyAsync(counts.get() + k, pos[k].get() + g.n, 4, cudaMemcpyDeviceToDevice, s));
    }
    CK(cudaMemcpyAsync(cnt, counts.get(), 4 * K, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int k = 0; k < K; k++) {
        out[k] = c.alloc<uint32_t>(cnt[k]);
        if (cnt[k]) {
            k_class_scatter<<<grid_for(g.n, TPB), TPB, 0, s>>>(g.n, InClass{g.indices, lo[k], hi[k]}, pos[k].get(),
                                                               out[k]);
            CK_LAUNCH("k_class_scatter");
        }
    }
}

}  // namespace

int PhaseTimers::index(const char *name) {
    for (size_t i = 0; i < names.size(); i++)
        if (names[i] == name) return (int)i;
    names.push_back(name);
    phases.push_back(Phase());
    return (int)names.size() - 1;
}

cudaEvent_t PhaseTimers::get_event() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    return e;
}

void PhaseTimers::flush() {
    for (auto &p : pending) {
        CK(cudaEventSynchronize(p.second.second));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, p.second.first, p.second.second));
        phases[p.first].ms += ms;
        phases[p.first].count++;
        pool.push_back(p.second.first);
        pool.push_back(p.second.second);
    }
    pending.clear();
}

void PhaseTimers::reset() {
    flush();
    for (auto &p : phases) p = Phase();
}

void PhaseTimers::destroy() {
    for (auto &p : pending) {
        cudaEventDestroy(p.second.first);
        cudaEventDestroy(p.second.second);
    }
    for (auto e : pool) cudaEventDestroy(e);
    pending.clear();
    pool.clear();
}

PhaseScope::PhaseScope(Ctx &ctx, const char *name) : c(&ctx), idx(-1) {
    if (!(ctx.flags & SCD_FLAG_PROFILE) || ctx.capturing) return;
    idx = ctx.timers.index(name);
    start = ctx.timers.get_event();
    CK(cudaEventRecord(start, ctx.stream));
}

PhaseScope::~PhaseScope() {
    if (idx < 0) return;
    cudaEvent_t end = nullptr;
    try {
        end = c->timers.get_event();
    } catch (...) {
        return;
    }
    cudaEventRecord(end, c->stream);
    c->timers.pending.push_back({idx, {start, end}});
}

void Ctx::free_all() {
    if (stream) cudaStreamSynchronize(stream);
    if (side) cudaStreamSynchronize(side);
    pext_join_pending = false;
    pext_host_valid = false;
    for (void *p : owned) cudaFreeAsync(p, stream);
    owned.clear();
    bytes = 0;
    g = Graph();
    has_graph = has_labels = false;
    labels = labels_next = best = nullptr;
    st[0] = st[1] = Stats();
    slot_flag = nullptr;
    itcount = nullptr;
    itdeg = nullptr;
    int_len = nullptr;
    int_adj = nullptr;
    wplan = TcPlan();
    wcc_part = nullptr;
    b = Batch();
    big_tables = nullptr;
    pin64 = nullptr;
    civ = nullptr;
    num_comms = 0;
}

// The derived structure of the (union) graph: nlow, the graph of each vertex,
// the graph-aligned WCC blocks, degree classes, row work, the global hash tables,
// the iteration's scratch arrays and the triangle-counting plan.  Needs
// g.indices/adj, b.G, b.h_fin_off and b.fin_off; always_gid: a graph-id array even
// for one graph (resident sets run every kernel in the skip-converged-graphs mode).
void build_union_structure(Ctx &c, bool always_gid) {
    Graph &g = c.g;
    Batch &b = c.b;
    cudaStream_t s = c.stream;
    const uint32_t n = g.n;
    g.nlow = c.alloc<uint32_t>(n);
    prepare_tc_kernels();
    prepare_improve_kernels();
    if (b.G > 1 || always_gid) {
        b.gid = c.alloc<uint32_t>(n);
        if (n) {
            k_fill_gid<<<grid_for(n, TPB), TPB, 0, s>>>(n, b.G, b.fin_off, b.gid);
            CK_LAUNCH("k_fill_gid");
        }
    }
    {
        std::vector<uint32_t> blk_off(b.G + 1, 0), blk_gid;
        for (uint32_t k = 0; k < b.G; k++) {
            const uint32_t nk = b.h_fin_off[k + 1] - b.h_fin_off[k];
            const uint32_t parts = (nk + 2047) / 2048;
            blk_off[k + 1] = blk_off[k] + parts;
            blk_gid.insert(blk_gid.end(), parts, k);
        }
        b.blocks = blk_off[b.G];
        b.blk_off = c.alloc<uint32_t>(b.G + 1);
        b.blk_gid = c.alloc<uint32_t>(b.blocks);
        // (copies from pageable memory are staged before the calls return: no wait needed)
        CK(cudaMemcpyAsync(b.blk_off, blk_off.data(), 4 * (b.G + 1), cudaMemcpyHostToDevice, s));
        if (b.blocks) CK(cudaMemcpyAsync(b.blk_gid, blk_gid.data(), 4 * b.blocks, cudaMemcpyHostToDevice, s));
    }
    if (n) {
        k_nlow<<<grid_for(n, TPB), TPB, 0, s>>>(n, g.indices, g.adj, g.nlow);
        CK_LAUNCH("k_nlow");
    }
    {   // the degree classes and the long rows; class 0 includes degree 0 (possible in a
        // transferred graph; convert never keeps one)
        constexpr int K = DegreeClasses::K;
        uint32_t lo[K + 1], hi[K + 1], cnt[K + 1];
        uint32_t *lists[K + 1];
        for (int k = 0; k < K; k++) {
            lo[k] = k ? DegreeClasses::upper[k - 1] + 1 : 0u;
            hi[k] = DegreeClasses::upper[k];
        }
        lo[K] = RowWork::CHUNK + 1;
        hi[K] = 0xffffffffu;
        class_lists(c, K + 1, lo, hi, lists, cnt);
        for (int k = 0; k < K; k++) {
            g.cls.list[k] = lists[k];
            g.cls.count[k] = cnt[k];
        }
        g.rows.llong = lists[K];
        g.rows.nlong = cnt[K];
    }
    {
        RowWork &rw = g.rows;
        const uint32_t *llong = rw.llong;
        uint32_t *coff = c.alloc<uint32_t>((size_t)rw.nlong + 1);
        scan_exclusive<uint32_t>(ChunksOf{llong, g.indices}, coff, rw.nlong, s);
        CK(cudaMemcpyAsync(&rw.nchunks, coff + rw.nlong, 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        rw.chunk_off = coff;
    }
    const uint32_t n_big = g.cls.count[DegreeClasses::K - 1];
    g.big_table_off = c.alloc<uint64_t>((size_t)n_big + 1);
    g.big_table_words = 0;
    c.big_tables = nullptr;
    if (n_big) {
        scan_exclusive<uint64_t>(TableWords{g.cls.list[DegreeClasses::K - 1], g.indices}, g.big_table_off, n_big, s);
        CK(cudaMemcpyAsync(&g.big_table_words, g.big_table_off + n_big, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        c.big_tables = c.alloc<uint32_t>(g.big_table_words);
    }
    c.pin64 = c.alloc<double>(n);
    c.civ = c.alloc<int4>(n);
    c.slot_flag = c.alloc<uint8_t>(2 * (size_t)g.m);
    c.itcount = c.alloc<uint32_t>(n);
    c.itdeg = c.alloc<int32_t>(n);
    c.int_len = c.alloc<uint32_t>(n);
    c.int_adj = c.alloc<uint32_t>(2 * (size_t)g.m);
    c.wplan = TcPlan();
    if (n) tc_plan(c, Oriented{g.indices, g.nlow, g.adj, n}, c.wplan, s, true, false);
    c.wcc_part = c.alloc<double>(b.blocks + 1);
    c.launches += 3;
}

void finish_graph(Ctx &c) {
    Graph &g = c.g;
    cudaStream_t s = c.stream;
    const uint32_t n = g.n;
    // per-graph bookkeeping of the (possibly one-graph) batch
    Batch &b = c.b;
    if (!b.fin_off) {
        b.fin_off = c.alloc<uint32_t>(b.G + 1);
        CK(cudaMemcpyAsync(b.fin_off, b.h_fin_off.data(), 4 * (b.G + 1), cudaMemcpyHostToDevice, s));
    }
    CK(cudaStreamSynchronize(s));   // h_fin_off is complete
    {
        std::vector<uint32_t> ind_at(b.G + 1);
        DevBuf<uint32_t> tmp(b.G + 1, s);
        k_gather_indices<<<grid_for(b.G + 1, TPB), TPB, 0, s>>>(b.G, b.fin_off, g.indices, tmp.get());
        CK_LAUNCH("k_gather_indices");
        CK(cudaMemcpyAsync(ind_at.data(), tmp.get(), 4 * (b.G + 1), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        b.h_m.resize(b.G);
        for (uint32_t k = 0; k < b.G; k++) b.h_m[k] = (ind_at[k + 1] - ind_at[k]) / 2;
    }
    b.p_ext = c.alloc<double>(b.G);
    b.pe32 = c.alloc<float2>(b.G);
    b.comm_off = c.alloc<uint32_t>(b.G + 1);
    b.wcc = c.alloc<double>(b.G);
    b.best_wcc = c.alloc<double>(b.G);
    b.active = c.alloc<uint8_t>(b.G);
    b.improved = c.alloc<uint8_t>(b.G);
    b.iters = c.alloc<int32_t>(b.G);
    b.n_active = c.alloc<uint32_t>(1);
    c.labels = c.alloc<uint32_t>(n);
    c.labels_next = c.alloc<uint32_t>(n);
    c.best = c.alloc<uint32_t>(n);
    for (int k = 0; k < 2; k++) {
        c.st[k].sizes = c.alloc<int32_t>(n);
        c.st[k].ext = c.alloc<int32_t>(n);
        c.st[k].intl = c.alloc<int32_t>(n);
    }
    build_union_structure(c, false);
    compute_p_ext(c);
    c.launches++;
}

// One refinement iteration for every graph still running, without host
// synchronisation (so it can be captured in a CUDA graph): improve, statistics,
// WCC, per-graph loop control.
void iterate_async(Ctx &c, double threshold, double *trace, int max_trace) {
    // converged graphs of a batch or a resident set keep their labels; their statistics
    // and WCC are not needed any more
    const bool frozen = c.b.G > 1 || c.resident;
    improve(c, c.labels, c.st[c.cur], c.labels_next, frozen);
    uint32_t *t = c.labels;
    c.labels = c.labels_next;
    c.labels_next = t;
    c.cur ^= 1;
    collect_stats(c, c.labels, c.st[c.cur], frozen);
    launch_wcc(c, c.labels, c.st[c.cur], frozen);
    batch_step(c, threshold, trace, max_trace);
}

// Kernel nodes of a captured graph (the launches one replay makes).
uint64_t kernel_nodes(cudaGraph_t gr) {
    size_t n = 0;
    CK(cudaGraphGetNodes(gr, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) CK(cudaGraphGetNodes(gr, nodes.data(), &n));
    uint64_t k = 0;
    for (size_t i = 0; i < n; i++) {
        cudaGraphNodeType t;
        CK(cudaGraphNodeGetType(nodes[i], &t));
        k += t == cudaGraphNodeTypeKernel;
    }
    return k;
}

}  // namespace scd

using namespace scd;

namespace {

template <typename F>
int guarded(scd_ctx *ctx, F &&f) {
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

void require_graph(Ctx &c) {
    if (!c.has_graph) throw Error(SCD_ERR_STATE, "no graph on the device");
}
void require_labels(Ctx &c) {
    require_graph(c);
    if (!c.has_labels) throw Error(SCD_ERR_STATE, "no labels on the device");
}

void set_labels(Ctx &c, const uint32_t *host_labels) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    if (g.n) CK(cudaMemcpyAsync(c.labels, host_labels, (size_t)g.n * 4, cudaMemcpyHostToDevice, s));
    DevBuf<uint32_t> mx(1, s);
    CK(cudaMemsetAsync(mx.get(), 0, 4, s));
    if (g.n) {
        k_max_label<<<grid_for(g.n, TPB), TPB, 0, s>>>(g.n, c.labels, mx.get());
        CK_LAUNCH("k_max_label");
    }
    uint32_t nc = 0;
    CK(cudaMemcpyAsync(&nc, mx.get(), 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (nc > g.n) throw Error(SCD_ERR_ARG, "labels must be < n or SCD_INVALID_LABEL");
    c.num_comms = nc;
    c.b.h_comm_off.assign(c.b.G + 1, nc);
    c.b.h_comm_off[0] = 0;
    CK(cudaMemcpyAsync(c.b.comm_off, c.b.h_comm_off.data(), 4 * (c.b.G + 1), cudaMemcpyHostToDevice, s));
    c.cur = 0;
    collect_stats(c, c.labels, c.st[0]);
    if (g.n) CK(cudaMemcpyAsync(c.best, c.labels, (size_t)g.n * 4, cudaMemcpyDeviceToDevice, s));
    c.has_labels = true;
}

double iterate(Ctx &c) {
    // improve (old labels -> labels_next), statistics and WCC of the new labels
    join_p_ext(c);
    improve(c, c.labels, c.st[c.cur], c.labels_next);
    uint32_t *t = c.labels;
    c.labels = c.labels_next;
    c.labels_next = t;
    c.cur ^= 1;
    collect_stats(c, c.labels, c.st[c.cur]);
    return compute_wcc(c, c.labels, c.st[c.cur]);
}

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct RunOut {
    std::vector<double> wcc0, best;
    std::vector<int32_t> iters;
    std::vector<uint8_t> active;
    std::vector<uint32_t> distinct;
    double ms_partition = 0, ms_iterations = 0;
};

// number of distinct valid labels of each graph (compress_labels prints n - that)
std::vector<uint32_t> distinct_per_graph(Ctx &c, const uint32_t *labels) {
    Batch &b = c.b;
    cudaStream_t s = c.stream;
    std::vector<uint32_t> out(b.G, 0);
    if (c.g.n == 0 || c.num_comms == 0) return out;
    DevBuf<uint32_t> seen(c.num_comms, s), scan((size_t)c.num_comms + 1, s), dg(b.G, s);
    CK(cudaMemsetAsync(seen.get(), 0, (size_t)c.num_comms * 4, s));
    k_seen_labels<<<grid_for(c.g.n, TPB), TPB, 0, s>>>(c.g.n, labels, c.num_comms, seen.get());
    CK_LAUNCH("k_seen_labels");
    scan_exclusive<uint32_t>((const uint32_t *)seen.get(), scan.get(), c.num_comms, s);
    k_distinct_per_graph<<<grid_for(b.G, TPB), TPB, 0, s>>>(b.G, b.comm_off, scan.get(), dg.get());
    CK_LAUNCH("k_distinct_per_graph");
    CK(cudaMemcpyAsync(out.data(), dg.get(), 4 * b.G, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    c.launches += 3;
    return out;
}

// The loop of src/main-gpu.cpp:54-95 for every graph of the context at once;
// each iteration is replayed from a captured CUDA graph (two graphs, one per
// parity of the label double buffer), with one host read per iteration.
void run_loop(Ctx &c, double threshold, int max_iters, double *trace_dev, int max_trace, RunOut &out) {
    Batch &b = c.b;
    cudaStream_t s = c.stream;
    const double t0 = now_ms();
    if (!c.has_labels) initial_partition(c);
    launch_wcc(c, c.labels, c.st[c.cur]);
    join_p_ext(c);   // p_ext (side stream) is needed from the first improvement on
    batch_reset(c);
    out.wcc0.resize(b.G);
    CK(cudaMemcpyAsync(out.wcc0.data(), b.wcc, 8 * b.G, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const double t1 = now_ms();
    const bool graphs = !(c.flags & SCD_FLAG_NO_GRAPHS) && c.g.n > 0;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    uint64_t kernels[2] = {0, 0};
    try {
        for (int it = 0; it < max_iters; it++) {
            if (graphs) {
                const int par = c.cur;
                if (!exec[par]) {
                    cudaGraph_t gr = nullptr;
                    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                    c.capturing = true;
                    try {
                        iterate_async(c, threshold, trace_dev, max_trace);
                    } catch (...) {
                        c.capturing = false;
                        cudaStreamEndCapture(s, &gr);
                        if (gr) cudaGraphDestroy(gr);
                        throw;
                    }
                    c.capturing = false;
                    CK(cudaStreamEndCapture(s, &gr));
                    kernels[par] = kernel_nodes(gr);
                    const cudaError_t e = cudaGraphInstantiate(&exec[par], gr, 0);
                    cudaGraphDestroy(gr);
                    CK(e);
                } else {
                    // replaying advances the state exactly as the captured host code did
                    uint32_t *t = c.labels;
                    c.labels = c.labels_next;
                    c.labels_next = t;
                    c.cur ^= 1;
                }
                CK(cudaGraphLaunch(exec[par], s));
                c.launches += kernels[par];
            } else {
                iterate_async(c, threshold, trace_dev, max_trace);
            }
            CK(cudaMemcpyAsync(c.host_u32, b.n_active, 4, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (*c.host_u32 == 0) break;
        }
    } catch (...) {
        for (auto e : exec)
            if (e) cudaGraphExecDestroy(e);
        throw;
    }
    for (auto e : exec)
        if (e) cudaGraphExecDestroy(e);
    const double t2 = now_ms();
    out.best.resize(b.G);
    out.iters.resize(b.G);
    out.active.resize(b.G);
    CK(cudaMemcpyAsync(out.best.data(), b.best_wcc, 8 * b.G, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(out.iters.data(), b.iters, 4 * b.G, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(out.active.data(), b.active, b.G, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    out.distinct = distinct_per_graph(c, c.best);
    out.ms_partition = t1 - t0;
    out.ms_iterations = t2 - t1;
}



}  // namespace

extern "C" {

int scd_create(scd_ctx **out, int device_id, int work_group_size, unsigned flags) {
    if (!out) return SCD_ERR_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device_id < 0 || device_id >= count) return SCD_ERR_ARG;
    scd_ctx *ctx = new (std::nothrow) scd_ctx();
    if (!ctx) return SCD_ERR_OOM;
    Ctx &c = ctx->c;
    c.device = device_id;
    c.work_group_size = work_group_size > 0 ? work_group_size : 256;
    c.flags = flags;
    try {
        CK(cudaSetDevice(device_id));
        {   // keep freed pool memory cached for the next graph instead of returning it at every sync
            cudaMemPool_t pool;
            CK(cudaDeviceGetDefaultMemPool(&pool, device_id));
            uint64_t keep = ~0ull;
            CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
        }
        int prio = 0;   // the device's highest stream priority (numerically lowest) when asked for
        if (flags & SCD_FLAG_PRIORITY) {
            int lowest = 0;
            CK(cudaDeviceGetStreamPriorityRange(&lowest, &prio));
        }
        CK(cudaStreamCreateWithPriority(&c.stream, cudaStreamNonBlocking, prio));
        CK(cudaStreamCreateWithPriority(&c.side, cudaStreamNonBlocking, prio));
        CK(cudaStreamCreateWithPriority(&c.aux, cudaStreamNonBlocking, prio));
        CK(cudaEventCreateWithFlags(&c.aux_fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c.aux_join, cudaEventDisableTiming));
        CK(cudaMalloc((void **)&c.work_counter, 64));
        CK(cudaMallocHost((void **)&c.wcc_host, sizeof(double)));
        CK(cudaMallocHost((void **)&c.host_u32, 32 * sizeof(uint32_t)));
    } catch (const Error &e) {
        scd_destroy(ctx);
        return e.status;
    }
    *out = ctx;
    return SCD_OK;
}

void scd_destroy(scd_ctx *ctx) {
    if (!ctx) return;
    Ctx &c = ctx->c;
    cudaSetDevice(c.device);
    resident_destroy(c);
    c.free_all();
    if (c.stream) cudaStreamSynchronize(c.stream);
    {   // hand the cached pool memory back (arrays still in use elsewhere are not affected)
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, c.device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
    }
    if (c.work_counter) cudaFree(c.work_counter);
    if (c.wcc_host) cudaFreeHost(c.wcc_host);
    if (c.host_u32) cudaFreeHost(c.host_u32);
    for (int k = 0; k < 2; k++) {
        if (c.io_buf[k]) cudaFreeHost(c.io_buf[k]);
        if (c.io_done[k]) cudaEventDestroy(c.io_done[k]);
    }
    c.timers.destroy();
    if (c.pext_ready) cudaEventDestroy(c.pext_ready);
    if (c.stream) cudaStreamDestroy(c.stream);
    if (c.side) cudaStreamDestroy(c.side);
    if (c.aux) {
        cudaStreamSynchronize(c.aux);
        cudaStreamDestroy(c.aux);
    }
    if (c.aux_fork) cudaEventDestroy(c.aux_fork);
    if (c.aux_join) cudaEventDestroy(c.aux_join);
    delete ctx;
}

const char *scd_last_error(const scd_ctx *ctx) { return ctx ? ctx->c.err.c_str() : "null context"; }

int scd_convert_edges(scd_ctx *ctx, const uint32_t *pairs, uint64_t count, int pairs_on_device) {
    return guarded(ctx, [&](Ctx &c) {
        if (count && !pairs) throw Error(SCD_ERR_ARG, "pairs is NULL");
        if (pairs_on_device || count == 0) {
            convert_edges(c, pairs, count);
        } else {
            DevBuf<uint32_t> d(2 * count, c.stream);
            CK(cudaMemcpyAsync(d.get(), pairs, 2 * count * 4, cudaMemcpyHostToDevice, c.stream));
            convert_edges(c, d.get(), count);
        }
        CK(cudaStreamSynchronize(c.stream));
    });
}

int scd_transfer_graph(scd_ctx *ctx, uint32_t n, uint32_t m, const uint32_t *indices, const uint32_t *adj,
                       const int32_t *tri, const int32_t *tri_deg, double alpha) {
    return guarded(ctx, [&](Ctx &c) {
        if (!indices || (m && !adj) || (n && (!tri || !tri_deg))) throw Error(SCD_ERR_ARG, "NULL graph array");
        if (indices[0] != 0 || indices[n] != 2 * (uint64_t)m) throw Error(SCD_ERR_FORMAT, "indices do not match m");
        c.alpha = alpha;
        upload_graph(c, n, m, indices, adj, tri, tri_deg);
        CK(cudaStreamSynchronize(c.stream));
    });
}

namespace {

constexpr size_t IO_PIECE = 64u << 20;   // bytes per pinned piece of a graph file

// Piece [off, off + len) of a graph file's body (everything after the two header
// words) to the resident graph's arrays: the body is indices | adj | tri | tri_deg.
void body_to_device(Ctx &c, const char *src, uint64_t off, uint64_t len) {
    const Graph &g = c.g;
    const uint64_t seg_len[4] = {4 * ((uint64_t)g.n + 1), 8 * (uint64_t)g.m, 4 * (uint64_t)g.n, 4 * (uint64_t)g.n};
    char *seg_dst[4] = {(char *)g.indices, (char *)g.adj, (char *)g.tri, (char *)g.tri_deg};
    uint64_t seg_beg = 0;
    for (int k = 0; k < 4; k++) {
        const uint64_t a = off > seg_beg ? off : seg_beg, e = seg_beg + seg_len[k];
        const uint64_t b = off + len < e ? off + len : e;
        if (a < b) CK(cudaMemcpyAsync(seg_dst[k] + (a - seg_beg), src + (a - off), b - a, cudaMemcpyHostToDevice, c.stream));
        seg_beg = e;
    }
}

// the body is on the device: check its offsets, then the derived arrays
void finish_loaded_graph(Ctx &c, double alpha) {
    uint32_t ends[2] = {0, 0};
    CK(cudaMemcpyAsync(ends, c.g.indices, 4, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaMemcpyAsync(ends + 1, c.g.indices + c.g.n, 4, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (ends[0] != 0 || ends[1] != 2 * (uint64_t)c.g.m) {
        c.free_all();
        throw Error(SCD_ERR_FORMAT, "indices do not match m");
    }
    c.alpha = alpha;
    finish_graph(c);
    c.has_graph = true;
    CK(cudaStreamSynchronize(c.stream));
}

uint64_t graph_file_bytes(uint32_t n, uint32_t m) { return 4 * (2 + ((uint64_t)n + 1) + 2 * (uint64_t)m + 2 * (uint64_t)n); }

}  // namespace

int scd_transfer_graph_bytes(scd_ctx *ctx, const void *bytes, uint64_t size, double alpha) {
    return guarded(ctx, [&](Ctx &c) {
        if (!bytes || size < 8) throw Error(SCD_ERR_ARG, "no graph bytes");
        uint32_t hdr[2];
        memcpy(hdr, bytes, 8);
        if (graph_file_bytes(hdr[0], hdr[1]) != size) throw Error(SCD_ERR_FORMAT, "graph size does not match n and m");
        alloc_graph(c, hdr[0], hdr[1]);
        body_to_device(c, (const char *)bytes + 8, 0, size - 8);
        finish_loaded_graph(c, alpha);
    });
}

// Read in IO_PIECE pieces into two pinned buffers: the read of one piece overlaps
// the copy of the other; no pageable host copy of the graph is made.
int scd_load_graph_file(scd_ctx *ctx, const char *path, double alpha) {
    return guarded(ctx, [&](Ctx &c) {
        if (!path) throw Error(SCD_ERR_ARG, "NULL path");
        FILE *f = fopen(path, "rb");
        if (!f) throw Error(SCD_ERR_ARG, std::string("failed to open ") + path);
        struct Closer {
            FILE *f;
            ~Closer() { fclose(f); }
        } closer{f};
        const std::string bad = std::string("error while reading ") + path;
        uint32_t hdr[2];
        if (fread(hdr, 4, 2, f) != 2) throw Error(SCD_ERR_FORMAT, bad);
        if (fseek(f, 0, SEEK_END) != 0) throw Error(SCD_ERR_FORMAT, bad);
        const long long fsize = ftell(f);
        if (fsize < 0 || (uint64_t)fsize != graph_file_bytes(hdr[0], hdr[1]) || fseek(f, 8, SEEK_SET) != 0)
            throw Error(SCD_ERR_FORMAT, bad);
        for (int k = 0; k < 2; k++)
            if (!c.io_buf[k]) {
                CK(cudaMallocHost((void **)&c.io_buf[k], IO_PIECE));
                CK(cudaEventCreateWithFlags(&c.io_done[k], cudaEventDisableTiming));
            }
        alloc_graph(c, hdr[0], hdr[1]);
        const uint64_t body = (uint64_t)fsize - 8;
        bool used[2] = {false, false};
        int k = 0;
        for (uint64_t off = 0; off < body; off += IO_PIECE, k ^= 1) {
            const uint64_t len = body - off < IO_PIECE ? body - off : IO_PIECE;
            if (used[k]) CK(cudaEventSynchronize(c.io_done[k]));   // its previous piece has left
            if (fread(c.io_buf[k], 1, len, f) != len) {
                CK(cudaStreamSynchronize(c.stream));
                c.free_all();
                throw Error(SCD_ERR_FORMAT, bad);
            }
            body_to_device(c, c.io_buf[k], off, len);
            CK(cudaEventRecord(c.io_done[k], c.stream));
            used[k] = true;
        }
        finish_loaded_graph(c, alpha);
    });
}

int scd_graph_info(scd_ctx *ctx, uint32_t *n, uint32_t *m, double *cc) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        if (n) *n = c.g.n;
        if (m) *m = c.g.m;
        if (cc) {
            host_p_ext(c);
            *cc = c.g.p_ext;
        }
    });
}

int scd_graph_download(scd_ctx *ctx, uint32_t *indices, uint32_t *adj, int32_t *tri, int32_t *tri_deg) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        const Graph &g = c.g;
        cudaStream_t s = c.stream;
        if (indices) CK(cudaMemcpyAsync(indices, g.indices, ((size_t)g.n + 1) * 4, cudaMemcpyDeviceToHost, s));
        if (adj && g.m) CK(cudaMemcpyAsync(adj, g.adj, 2 * (size_t)g.m * 4, cudaMemcpyDeviceToHost, s));
        if (tri && g.n) CK(cudaMemcpyAsync(tri, g.tri, (size_t)g.n * 4, cudaMemcpyDeviceToHost, s));
        if (tri_deg && g.n) CK(cudaMemcpyAsync(tri_deg, g.tri_deg, (size_t)g.n * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int scd_initial_partition(scd_ctx *ctx, uint32_t *num_communities) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        initial_partition(c);
        CK(cudaStreamSynchronize(c.stream));
        if (num_communities) *num_communities = c.num_comms;
    });
}

int scd_labels_to_device(scd_ctx *ctx, const uint32_t *labels) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        if (c.g.n && !labels) throw Error(SCD_ERR_ARG, "labels is NULL");
        set_labels(c, labels);
        CK(cudaStreamSynchronize(c.stream));
    });
}

int scd_compute_wcc(scd_ctx *ctx, double *wcc) {
    return guarded(ctx, [&](Ctx &c) {
        require_labels(c);
        double w = compute_wcc(c, c.labels, c.st[c.cur]);
        if (wcc) *wcc = w;
    });
}

int scd_improve_labels(scd_ctx *ctx, double *wcc) {
    return guarded(ctx, [&](Ctx &c) {
        require_labels(c);
        double w = iterate(c);
        if (wcc) *wcc = w;
    });
}

int scd_store_labels(scd_ctx *ctx) {
    return guarded(ctx, [&](Ctx &c) {
        require_labels(c);
        if (c.g.n)
            CK(cudaMemcpyAsync(c.best, c.labels, (size_t)c.g.n * 4, cudaMemcpyDeviceToDevice, c.stream));
        CK(cudaStreamSynchronize(c.stream));
    });
}

int scd_labels_from_device(scd_ctx *ctx, uint32_t *labels) {
    return guarded(ctx, [&](Ctx &c) {
        require_labels(c);
        if (c.g.n) CK(cudaMemcpyAsync(labels, c.best, (size_t)c.g.n * 4, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
    });
}

int scd_current_labels(scd_ctx *ctx, uint32_t *labels) {
    return guarded(ctx, [&](Ctx &c) {
        require_labels(c);
        if (c.g.n) CK(cudaMemcpyAsync(labels, c.labels, (size_t)c.g.n * 4, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
    });
}

int scd_compressed_labels(scd_ctx *ctx, uint32_t *labels, uint32_t *num_communities) {
    return guarded(ctx, [&](Ctx &c) {
        require_labels(c);
        if (c.b.G != 1) throw Error(SCD_ERR_STATE, "the context holds a batch: compressed labels are per single graph");
        cudaStream_t s = c.stream;
        const uint32_t n = c.g.n;
        uint32_t total = 0;
        if (n) {
            const uint32_t nc = c.num_comms ? c.num_comms : 1;
            DevBuf<uint32_t> first(nc, s), rank((size_t)n + 1, s), out(n, s);
            CK(cudaMemsetAsync(first.get(), 0xff, (size_t)nc * 4, s));
            k_first_of_label<<<grid_for(n, TPB), TPB, 0, s>>>(n, c.best, first.get());
            CK_LAUNCH("k_first_of_label");
            scan_exclusive<uint32_t>(OpensCommunity{c.best, first.get()}, rank.get(), n, s);
            k_compressed<<<grid_for(n, TPB), TPB, 0, s>>>(n, c.best, first.get(), rank.get(), out.get());
            CK_LAUNCH("k_compressed");
            c.launches += 3;
            CK(cudaMemcpyAsync(&total, rank.get() + n, 4, cudaMemcpyDeviceToHost, s));
            if (labels) CK(cudaMemcpyAsync(labels, out.get(), (size_t)n * 4, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
        }
        if (num_communities) *num_communities = total;
    });
}

int scd_community_stats(scd_ctx *ctx, int32_t *sizes, int32_t *ext, int32_t *intl, uint32_t *nc) {
    return guarded(ctx, [&](Ctx &c) {
        require_labels(c);
        if (c.b.G != 1) throw Error(SCD_ERR_STATE, "the context holds a batch: statistics are per single graph");
        const Stats &st = c.st[c.cur];
        const size_t b = (size_t)c.num_comms * 4;
        if (sizes && b) CK(cudaMemcpyAsync(sizes, st.sizes, b, cudaMemcpyDeviceToHost, c.stream));
        if (ext && b) CK(cudaMemcpyAsync(ext, st.ext, b, cudaMemcpyDeviceToHost, c.stream));
        if (intl && b) CK(cudaMemcpyAsync(intl, st.intl, b, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
        if (nc) *nc = c.num_comms;
    });
}

int scd_run(scd_ctx *ctx, double threshold, int max_iters, double *wcc_trace, scd_result *res) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        if (c.b.G != 1) throw Error(SCD_ERR_STATE, "the context holds a batch: use scd_batch_run");
        if (max_iters < 0) throw Error(SCD_ERR_ARG, "max_iters < 0");
        DevBuf<double> trace(wcc_trace && max_iters ? max_iters : 0, c.stream);
        RunOut o;
        run_loop(c, threshold, max_iters, trace.get(), wcc_trace ? max_iters : 0, o);
        scd_result r;
        memset(&r, 0, sizeof r);
        r.iterations = o.iters[0];
        r.initial_wcc = o.wcc0[0];
        r.best_wcc = o.best[0];
        r.initial_communities = c.b.h_comm_off[1] - c.b.h_comm_off[0];
        r.distinct_communities = o.distinct[0];
        r.printed_communities = c.g.n - o.distinct[0];
        r.ms_partition = o.ms_partition;
        r.ms_iterations = o.ms_iterations;
        if (wcc_trace && r.iterations > 0) {
            CK(cudaMemcpyAsync(wcc_trace, trace.get(), 8 * std::min(r.iterations, max_iters), cudaMemcpyDeviceToHost,
                               c.stream));
            CK(cudaStreamSynchronize(c.stream));
        }
        if (res) *res = r;
        if (o.active[0] || (c.g.n == 0 && max_iters > 0))
            throw Error(SCD_ERR_LIMIT, "max_iters reached before convergence (or the WCC stays 0)");
    });
}

namespace {
// the text in device memory (copied in if it is on the host)
const char *device_text(Ctx &c, const char *text, uint64_t bytes, int on_device, DevBuf<char> &tmp) {
    if (bytes && !text) throw Error(SCD_ERR_ARG, "text is NULL");
    if (on_device || bytes == 0) return text;
    tmp.alloc(bytes, c.stream);
    CK(cudaMemcpyAsync(tmp.get(), text, bytes, cudaMemcpyHostToDevice, c.stream));
    return tmp.get();
}
}  // namespace

int scd_convert_text(scd_ctx *ctx, const char *text, uint64_t bytes, int text_on_device) {
    return guarded(ctx, [&](Ctx &c) {
        DevBuf<char> tmp;
        const char *d = device_text(c, text, bytes, text_on_device, tmp);
        DevBuf<uint32_t> pairs;
        uint64_t count;
        {
            PhaseScope ph(c, "parse");
            count = parse_edge_text(c, d, bytes, pairs);
        }
        tmp.release();
        convert_edges(c, pairs.get(), count);
        CK(cudaStreamSynchronize(c.stream));
    });
}

int scd_parse_text(scd_ctx *ctx, const char *text, uint64_t bytes, int text_on_device, uint32_t *pairs,
                   uint64_t *count) {
    return guarded(ctx, [&](Ctx &c) {
        if (!count) throw Error(SCD_ERR_ARG, "count is NULL");
        DevBuf<char> tmp;
        const char *d = device_text(c, text, bytes, text_on_device, tmp);
        DevBuf<uint32_t> out;
        *count = parse_edge_text(c, d, bytes, out);
        if (pairs && *count)
            CK(cudaMemcpyAsync(pairs, out.get(), 8 * *count, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
    });
}

int scd_batch_convert(scd_ctx *ctx, const uint32_t *pairs, const uint64_t *record_offsets, uint32_t num_graphs,
                      int pairs_on_device) {
    return guarded(ctx, [&](Ctx &c) {
        if (!record_offsets || num_graphs == 0) throw Error(SCD_ERR_ARG, "no graphs");
        std::vector<uint64_t> off(record_offsets, record_offsets + num_graphs + 1);
        for (uint32_t g = 0; g < num_graphs; g++)
            if (off[g + 1] < off[g]) throw Error(SCD_ERR_ARG, "record_offsets must be non-decreasing");
        if (off[0] != 0) throw Error(SCD_ERR_ARG, "record_offsets[0] must be 0");
        const uint64_t count = off[num_graphs];
        if (count && !pairs) throw Error(SCD_ERR_ARG, "pairs is NULL");
        if (pairs_on_device || count == 0) {
            convert_edges(c, pairs, count, &off);
        } else {
            DevBuf<uint32_t> d(2 * count, c.stream);
            CK(cudaMemcpyAsync(d.get(), pairs, 2 * count * 4, cudaMemcpyHostToDevice, c.stream));
            convert_edges(c, d.get(), count, &off);
        }
        CK(cudaStreamSynchronize(c.stream));
    });
}

int scd_batch_convert_lists(scd_ctx *ctx, const uint32_t *const *pairs, const uint64_t *counts,
                            uint32_t num_graphs) {
    return guarded(ctx, [&](Ctx &c) {
        if (!counts || num_graphs == 0) throw Error(SCD_ERR_ARG, "no graphs");
        std::vector<uint64_t> off(num_graphs + 1, 0);
        for (uint32_t g = 0; g < num_graphs; g++) {
            if (counts[g] && (!pairs || !pairs[g])) throw Error(SCD_ERR_ARG, "pairs[g] is NULL");
            off[g + 1] = off[g] + counts[g];
        }
        const uint64_t count = off[num_graphs];
        if (count >= (1ull << 31)) throw Error(SCD_ERR_LIMIT, "more than 2^31-1 edge records");
        DevBuf<uint32_t> d(2 * count, c.stream);
        for (uint32_t g = 0; g < num_graphs; g++)
            if (counts[g])
                CK(cudaMemcpyAsync(d.get() + 2 * off[g], pairs[g], 8 * counts[g], cudaMemcpyHostToDevice, c.stream));
        convert_edges(c, d.get(), count, &off);
        CK(cudaStreamSynchronize(c.stream));
    });
}

int scd_batch_size(scd_ctx *ctx, uint32_t *num_graphs) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        if (num_graphs) *num_graphs = c.b.G;
    });
}

int scd_batch_graph_info(scd_ctx *ctx, uint32_t g, uint32_t *n, uint32_t *m, double *cc) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        if (g >= c.b.G) throw Error(SCD_ERR_ARG, "graph index out of range");
        if (n) *n = c.b.h_fin_off[g + 1] - c.b.h_fin_off[g];
        if (m) *m = c.b.h_m[g];
        if (cc) {
            host_p_ext(c);
            *cc = c.b.h_p_ext[g];
        }
    });
}

int scd_batch_graph_download(scd_ctx *ctx, uint32_t g, uint32_t *indices, uint32_t *adj, int32_t *tri,
                             int32_t *tri_deg) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        if (g >= c.b.G) throw Error(SCD_ERR_ARG, "graph index out of range");
        cudaStream_t s = c.stream;
        const uint32_t v0 = c.b.h_fin_off[g], ng = c.b.h_fin_off[g + 1] - v0, m2 = 2 * c.b.h_m[g];
        DevBuf<uint32_t> ind((size_t)ng + 1, s), ad(m2 ? m2 : 1, s);
        k_local_graph<<<grid_for((uint64_t)ng + m2 + 1, 256), 256, 0, s>>>(ng, m2, v0, c.g.indices, c.g.adj, ind.get(),
                                                                       ad.get());
        CK_LAUNCH("k_local_graph");
        if (indices) CK(cudaMemcpyAsync(indices, ind.get(), 4 * ((size_t)ng + 1), cudaMemcpyDeviceToHost, s));
        if (adj && m2) CK(cudaMemcpyAsync(adj, ad.get(), 4 * (size_t)m2, cudaMemcpyDeviceToHost, s));
        if (tri && ng) CK(cudaMemcpyAsync(tri, c.g.tri + v0, 4 * (size_t)ng, cudaMemcpyDeviceToHost, s));
        if (tri_deg && ng) CK(cudaMemcpyAsync(tri_deg, c.g.tri_deg + v0, 4 * (size_t)ng, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int scd_batch_run(scd_ctx *ctx, double threshold, int max_iters, scd_result *results) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        if (max_iters < 0) throw Error(SCD_ERR_ARG, "max_iters < 0");
        RunOut o;
        run_loop(c, threshold, max_iters, nullptr, 0, o);
        bool all = true;
        for (uint32_t g = 0; g < c.b.G; g++) {
            const uint32_t ng = c.b.h_fin_off[g + 1] - c.b.h_fin_off[g];
            if (results) {
                scd_result &r = results[g];
                memset(&r, 0, sizeof r);
                r.iterations = o.iters[g];
                r.initial_wcc = o.wcc0[g];
                r.best_wcc = o.best[g];
                r.initial_communities = c.b.h_comm_off[g + 1] - c.b.h_comm_off[g];
                r.distinct_communities = o.distinct[g];
                r.printed_communities = ng - o.distinct[g];
                r.ms_partition = o.ms_partition;
                r.ms_iterations = o.ms_iterations;
            }
            if (o.active[g]) all = false;
        }
        if (!all) throw Error(SCD_ERR_LIMIT, "some graphs were still improving after max_iters");
    });
}

int scd_batch_labels(scd_ctx *ctx, uint32_t g, uint32_t *labels) {
    return guarded(ctx, [&](Ctx &c) {
        require_labels(c);
        if (g >= c.b.G) throw Error(SCD_ERR_ARG, "graph index out of range");
        cudaStream_t s = c.stream;
        const uint32_t v0 = c.b.h_fin_off[g], ng = c.b.h_fin_off[g + 1] - v0;
        if (!ng) return;
        DevBuf<uint32_t> tmp(ng, s);
        k_local_labels<<<grid_for(ng, 256), 256, 0, s>>>(ng, v0, c.b.h_comm_off[g], c.best, tmp.get());
        CK_LAUNCH("k_local_labels");
        CK(cudaMemcpyAsync(labels, tmp.get(), 4 * (size_t)ng, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int scd_batch_labels_all(scd_ctx *ctx, uint32_t *labels, uint64_t *vertex_offsets) {
    return guarded(ctx, [&](Ctx &c) {
        require_labels(c);
        if (!labels && !vertex_offsets) throw Error(SCD_ERR_ARG, "nothing to return");
        const Batch &b = c.b;
        if (vertex_offsets)
            for (uint32_t g = 0; g <= b.G; g++) vertex_offsets[g] = b.h_fin_off[g];
        const uint32_t n = c.g.n;
        if (!labels || n == 0) return;
        cudaStream_t s = c.stream;
        DevBuf<uint32_t> tmp(n, s);
        k_local_labels_all<<<grid_for(n, 256), 256, 0, s>>>(n, b.G > 1 ? b.gid : nullptr, b.comm_off, c.best, tmp.get());
        CK_LAUNCH("k_local_labels_all");
        c.launches++;
        CK(cudaMemcpyAsync(labels, tmp.get(), 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int scd_autotune(scd_ctx *ctx, uint32_t *small_max, uint32_t *warp_max, uint32_t *cta_max, double *best_ms,
                 char *report, uint64_t report_cap) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        if (c.res) throw Error(SCD_ERR_STATE, "a resident set keeps the split it was made with");
        std::vector<std::string> lines;
        const double ms = autotune_tc(c, &lines);
        if (c.g.n) {   // the WCC plan follows the chosen split
            c.wplan = TcPlan();
            tc_plan(c, Oriented{c.g.indices, c.g.nlow, c.g.adj, c.g.n}, c.wplan, c.stream, true, false);
        }
        if (small_max) *small_max = c.tc_small;
        if (warp_max) *warp_max = c.tc_b0;
        if (cta_max) *cta_max = c.tc_b1;
        if (best_ms) *best_ms = ms;
        if (report && report_cap) {
            std::string all;
            for (auto &l : lines) all += l + "\n";
            strncpy(report, all.c_str(), report_cap - 1);
            report[report_cap - 1] = 0;
        }
    });
}

int scd_set_memory_limit(scd_ctx *ctx, uint64_t bytes) {
    return guarded(ctx, [&](Ctx &c) { c.mem_limit = bytes; });
}

int scd_memory_usage(scd_ctx *ctx, uint64_t *bytes) {
    return guarded(ctx, [&](Ctx &c) {
        if (bytes) *bytes = c.bytes;
    });
}

int scd_kernel_launches(scd_ctx *ctx, uint64_t *count) {
    return guarded(ctx, [&](Ctx &c) {
        if (count) *count = c.launches;
    });
}

int scd_stream(scd_ctx *ctx, void **stream) {
    return guarded(ctx, [&](Ctx &c) {
        if (stream) *stream = (void *)c.stream;
    });
}

int scd_profile_get(scd_ctx *ctx, const char *phase, double *total_ms, uint64_t *count) {
    return guarded(ctx, [&](Ctx &c) {
        if (!phase) throw Error(SCD_ERR_ARG, "phase is NULL");
        c.timers.flush();
        const int i = c.timers.index(phase);
        if (total_ms) *total_ms = c.timers.phases[i].ms;
        if (count) *count = c.timers.phases[i].count;
    });
}

int scd_profile_reset(scd_ctx *ctx) {
    return guarded(ctx, [&](Ctx &c) { c.timers.reset(); });
}

}  // extern "C"
