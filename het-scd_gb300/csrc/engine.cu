// Context management, per-graph setup and the C ABI (include/scd_gb300.h).
#include <chrono>
#include <cstring>
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

struct InClass {
    const uint32_t *indices;
    uint32_t lo, hi;   // lo < deg <= hi
    __device__ uint32_t operator[](size_t v) const {
        const uint32_t d = indices[v + 1] - indices[v];
        return d > lo && d <= hi;
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

__global__ void k_mark_labels(uint32_t n, const uint32_t *__restrict__ labels, uint32_t *seen, uint32_t nc) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t l = labels[v];
        if (l != INVALID && l < nc) seen[l] = 1;
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

uint32_t class_list(Ctx &c, uint32_t lo, uint32_t hi, uint32_t **out) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    DevBuf<uint32_t> pos((size_t)g.n + 1, s);
    InClass f{g.indices, lo, hi};
    scan_exclusive<uint32_t>(f, pos.get(), g.n, s);
    uint32_t cnt = 0;
    CK(cudaMemcpyAsync(&cnt, pos.get() + g.n, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *out = c.alloc<uint32_t>(cnt);
    if (cnt) {
        k_class_scatter<<<grid_for(g.n, TPB), TPB, 0, s>>>(g.n, f, pos.get(), *out);
        CK_LAUNCH("k_class_scatter");
    }
    return cnt;
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
    if (!(ctx.flags & SCD_FLAG_PROFILE)) return;
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
    for (void *p : owned) cudaFree(p);
    owned.clear();
    bytes = 0;
    g = Graph();
    has_graph = has_labels = false;
    labels = labels_next = best = nullptr;
    st[0] = st[1] = Stats();
    slot_flag = nullptr;
    itcount = nullptr;
    itdeg = nullptr;
    wplan = TcPlan();
    wcc_part = wcc_sum = nullptr;
    big_tables = nullptr;
    pin64 = nullptr;
    pin32 = nullptr;
    num_comms = 0;
}

void finish_graph(Ctx &c) {
    Graph &g = c.g;
    cudaStream_t s = c.stream;
    const uint32_t n = g.n;
    g.nlow = c.alloc<uint32_t>(n);
    g.p_ext_dev = c.alloc<double>(1);
    if (n) {
        k_nlow<<<grid_for(n, TPB), TPB, 0, s>>>(n, g.indices, g.adj, g.nlow);
        CK_LAUNCH("k_nlow");
    }
    uint32_t lo = 0;
    for (int k = 0; k < DegreeClasses::K; k++) {
        g.cls.count[k] = class_list(c, lo, DegreeClasses::upper[k], &g.cls.list[k]);
        lo = DegreeClasses::upper[k];
    }
    const uint32_t n_big = g.cls.count[DegreeClasses::K - 1];
    g.big_table_off = c.alloc<uint64_t>((size_t)n_big + 1);
    if (n_big) {
        scan_exclusive<uint64_t>(TableWords{g.cls.list[DegreeClasses::K - 1], g.indices}, g.big_table_off, n_big, s);
        CK(cudaMemcpyAsync(&g.big_table_words, g.big_table_off + n_big, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        c.big_tables = c.alloc<uint32_t>(g.big_table_words);
    }
    c.labels = c.alloc<uint32_t>(n);
    c.labels_next = c.alloc<uint32_t>(n);
    c.best = c.alloc<uint32_t>(n);
    for (int k = 0; k < 2; k++) {
        c.st[k].sizes = c.alloc<int32_t>(n);
        c.st[k].ext = c.alloc<int32_t>(n);
        c.st[k].intl = c.alloc<int32_t>(n);
    }
    c.pin64 = c.alloc<double>(n);
    c.pin32 = c.alloc<float2>(n);
    c.slot_flag = c.alloc<uint8_t>(2 * (size_t)g.m);
    c.itcount = c.alloc<uint32_t>(n);
    c.itdeg = c.alloc<int32_t>(n);
    if (n) tc_plan(c, Oriented{g.indices, g.nlow, g.adj, n}, c.wplan, s, true);
    c.wcc_part = c.alloc<double>((n + 2047) / 2048 + 1);
    c.wcc_sum = c.alloc<double>(1);
    compute_p_ext(c);
    c.launches += 4;
}

}  // namespace scd

using namespace scd;

struct scd_ctx {
    Ctx c;
};

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
    c.cur = 0;
    collect_stats(c, c.labels, c.st[0]);
    if (g.n) CK(cudaMemcpyAsync(c.best, c.labels, (size_t)g.n * 4, cudaMemcpyDeviceToDevice, s));
    c.has_labels = true;
}

double iterate(Ctx &c) {
    // improve (old labels -> labels_next), statistics and WCC of the new labels
    improve(c, c.labels, c.st[c.cur], c.labels_next);
    uint32_t *t = c.labels;
    c.labels = c.labels_next;
    c.labels_next = t;
    c.cur ^= 1;
    collect_stats(c, c.labels, c.st[c.cur]);
    return compute_wcc(c, c.labels, c.st[c.cur]);
}

uint32_t distinct_labels(Ctx &c, const uint32_t *labels) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    if (g.n == 0 || c.num_comms == 0) return 0;
    DevBuf<uint32_t> seen(c.num_comms, s), pre((size_t)c.num_comms + 1, s);
    CK(cudaMemsetAsync(seen.get(), 0, (size_t)c.num_comms * 4, s));
    k_mark_labels<<<grid_for(g.n, TPB), TPB, 0, s>>>(g.n, labels, seen.get(), c.num_comms);
    CK_LAUNCH("k_mark_labels");
    scan_exclusive<uint32_t>((const uint32_t *)seen.get(), pre.get(), c.num_comms, s);
    uint32_t cnt = 0;
    CK(cudaMemcpyAsync(&cnt, pre.get() + c.num_comms, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return cnt;
}

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
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
        CK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking));
        CK(cudaMalloc((void **)&c.work_counter, 64));
        CK(cudaMallocHost((void **)&c.wcc_host, sizeof(double)));
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
    c.free_all();
    if (c.work_counter) cudaFree(c.work_counter);
    if (c.wcc_host) cudaFreeHost(c.wcc_host);
    c.timers.destroy();
    if (c.stream) cudaStreamDestroy(c.stream);
    if (c.side) cudaStreamDestroy(c.side);
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

int scd_graph_info(scd_ctx *ctx, uint32_t *n, uint32_t *m, double *cc) {
    return guarded(ctx, [&](Ctx &c) {
        require_graph(c);
        if (n) *n = c.g.n;
        if (m) *m = c.g.m;
        if (cc) *cc = c.g.p_ext;
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

int scd_community_stats(scd_ctx *ctx, int32_t *sizes, int32_t *ext, int32_t *intl, uint32_t *nc) {
    return guarded(ctx, [&](Ctx &c) {
        require_labels(c);
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
        scd_result r;
        memset(&r, 0, sizeof r);
        double t0 = now_ms();
        if (!c.has_labels) initial_partition(c);
        r.initial_communities = c.num_comms;
        double best_wcc = compute_wcc(c, c.labels, c.st[c.cur]);
        r.initial_wcc = best_wcc;
        double t1 = now_ms();
        bool converged = false;
        int iters = 0;
        while (iters < max_iters) {
            iters++;
            double w = iterate(c);
            if (w > best_wcc && c.g.n)
                CK(cudaMemcpyAsync(c.best, c.labels, (size_t)c.g.n * 4, cudaMemcpyDeviceToDevice, c.stream));
            if (wcc_trace) wcc_trace[iters - 1] = w;
            if (w < best_wcc * (1 + threshold)) {
                converged = true;
                break;
            }
            best_wcc = w;
        }
        CK(cudaStreamSynchronize(c.stream));
        double t2 = now_ms();
        r.iterations = iters;
        r.best_wcc = best_wcc;
        r.distinct_communities = distinct_labels(c, c.best);
        r.printed_communities = c.g.n - r.distinct_communities;
        r.ms_partition = t1 - t0;
        r.ms_iterations = t2 - t1;
        if (res) *res = r;
        if (!converged) throw Error(SCD_ERR_LIMIT, "max_iters reached before convergence");
    });
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
