// Community statistics (collect_stats, src/scd.cpp:57-111), the WCC metric
// (compute_wcc, src/wcc.cpp:31-141) and the clustering coefficient p_ext
// (src/graph.cpp:57-68); the label improvement itself is in improve.cu.
//
// wcc: the internal out-lists (out-neighbours with the vertex's own label), the
// oriented triangle count on them (internal triangles per vertex and the flags
// of internal edges on one), per-vertex sums, per-vertex WCC terms and a
// fixed-order (deterministic) tree reduction.
#include "engine.cuh"
#include "rows.cuh"
#include "gain.cuh"

namespace scd {

namespace {

constexpr unsigned TPB = 256;

// ---- collect_stats ---------------------------------------------------------

// A row segment for one warp: a whole short row or one piece of a long row.
struct RowSeg {
    uint32_t v, row0, beg, end;   // vertex, start of its row, [beg, end) of the segment in adj
    bool first, live;             // first segment of the row
};

__device__ __forceinline__ RowSeg chunk_seg(const RowWork &rw, uint32_t c, const uint32_t *indices) {
    uint32_t lo = 0, hi = rw.nlong;   // last row whose first chunk is <= c
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (rw.chunk_off[mid] <= c) lo = mid;
        else hi = mid;
    }
    const uint32_t k = c - rw.chunk_off[lo];
    RowSeg r;
    r.v = rw.llong[lo];
    const uint32_t b0 = indices[r.v], e0 = indices[r.v + 1];
    r.row0 = b0;
    r.beg = b0 + k * RowWork::CHUNK;
    r.end = min(e0, r.beg + RowWork::CHUNK);
    r.first = k == 0;
    r.live = true;
    return r;
}

// collect_stats for one row segment: sizes once per vertex, ext/int from the segment
template <int G>
__device__ __forceinline__ void stats_seg(RowSeg r, const uint32_t *adj, const uint32_t *labels, Stats st,
                                          LabelFilter skip) {
    const int gl = (threadIdx.x & 31) % G;
    const uint32_t l = r.live ? labels[r.v] : INVALID;
    const bool live = l != INVALID && !skip.frozen(r.v);
    uint32_t same = 0;
    if (live)
        for (uint32_t i = r.beg + gl; i < r.end; i += G) same += labels[adj[i]] == l;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) same += __shfl_xor_sync(FULL, same, o);
    if (live && gl == 0) {
        const uint32_t len = r.end - r.beg;
        if (r.first) atomicAdd(st.sizes + l, 1);
        if (len - same) atomicAdd(st.ext + l, (int)(len - same));
        if (same) atomicAdd(st.intl + l, (int)same);
    }
}

// collect_stats (src/scd.cpp:57-111): rows of degree <= 256 as 32-row streams in id
// order, the rows longer than 256 as RowWork chunks after them
__global__ void __launch_bounds__(TPB)
k_stats(uint32_t n, RowWork rw, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ adj,
        const uint32_t *__restrict__ labels, Stats st, LabelFilter skip) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t groups = (n + 31) / 32, nchunks = rw.nchunks;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < groups + nchunks; w += warps) {
        if (w >= groups) {   // a piece of a long row
            stats_seg<32>(chunk_seg(rw, w - groups, indices), adj, labels, st, skip);
            continue;
        }
        const uint32_t r = w * 32 + lane;
        uint32_t b = 0, deg = 0, l = INVALID;
        if (r < n) {
            b = indices[r];
            deg = indices[r + 1] - b;
            l = labels[r];
            if (skip.frozen(r)) l = INVALID;
        }
        const bool mine = l != INVALID && deg <= RowWork::CHUNK;   // long rows: chunk units
        const RowStream rs(mine ? deg : 0u);
        uint32_t same = 0;
        for (uint32_t t0 = 0; t0 < rs.total; t0 += 32) {
            const uint32_t t = t0 + lane;
            const int j = rs.owner(t < rs.total ? t : rs.total - 1);
            const uint32_t pos = __shfl_sync(FULL, b, j) + (t - __shfl_sync(FULL, rs.pre, j));
            const uint32_t lj = __shfl_sync(FULL, l, j);
            const bool hit = t < rs.total && labels[adj[pos]] == lj;
            same += __popc(__ballot_sync(FULL, hit) & rs.my_lanes(t0));
        }
        if (mine) {
            atomicAdd(st.sizes + l, 1);
            if (deg - same) atomicAdd(st.ext + l, (int)(deg - same));
            if (same) atomicAdd(st.intl + l, (int)same);
        }
    }
}

// ---- WCC ---------------------------------------------------------------------

// int_tri_deg for one row segment: its out-slots (the first nlow entries of the row)
template <int G>
__device__ __forceinline__ void intdeg_seg(RowSeg r, const uint32_t *nlow, const uint32_t *adj, const uint8_t *flag,
                                           int32_t *itdeg, LabelFilter skip) {
    const int gl = (threadIdx.x & 31) % G;
    const bool live = r.live && !skip.frozen(r.v);
    uint32_t edges = 0;
    if (live) {
        const uint32_t stop = min(r.end, r.row0 + nlow[r.v]);
        for (uint32_t i = r.beg + gl; i < stop; i += G) {
            if (flag[i]) {
                atomicAdd(itdeg + adj[i], 1);
                edges++;
            }
        }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) edges += __shfl_xor_sync(FULL, edges, o);
    if (live && gl == 0 && edges) atomicAdd(itdeg + r.v, (int)edges);
}

// int_tri_deg (src/wcc.cpp:124-126): per vertex, the internal edges that lie on an
// internal triangle, counted from the out-slot flags of both endpoints; the out-slots
// of rows of degree <= 256 as 32-row streams in id order, longer rows as RowWork chunks
__global__ void __launch_bounds__(TPB)
k_internal_degrees(uint32_t n, RowWork rw, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ nlow,
                   const uint32_t *__restrict__ adj, const uint8_t *__restrict__ flag, int32_t *itdeg,
                   LabelFilter skip) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t groups = (n + 31) / 32, nchunks = rw.nchunks;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < groups + nchunks; w += warps) {
        if (w >= groups) {   // a piece of a long row
            intdeg_seg<32>(chunk_seg(rw, w - groups, indices), nlow, adj, flag, itdeg, skip);
            continue;
        }
        const uint32_t u = w * 32 + lane;
        uint32_t b = 0, len = 0;
        if (u < n && !skip.frozen(u)) {
            b = indices[u];
            if (indices[u + 1] - b <= RowWork::CHUNK) len = nlow[u];
        }
        const RowStream rs(len);
        uint32_t edges = 0;
        for (uint32_t t0 = 0; t0 < rs.total; t0 += 32) {
            const uint32_t t = t0 + lane;
            const int j = rs.owner(t < rs.total ? t : rs.total - 1);
            const uint32_t pos = __shfl_sync(FULL, b, j) + (t - __shfl_sync(FULL, rs.pre, j));
            const bool f = t < rs.total && flag[pos];
            if (f) atomicAdd(itdeg + adj[pos], 1);
            edges += __popc(__ballot_sync(FULL, f) & rs.my_lanes(t0));
        }
        if (edges) atomicAdd(itdeg + u, (int)edges);
    }
}

constexpr int WCC_ITEMS = 8;
constexpr int WCC_CHUNK = TPB * WCC_ITEMS;

// WCC_p of src/wcc.cpp:129-134
__device__ __forceinline__ double wcc_term(uint32_t p, const uint32_t *labels, const Stats &st,
                                           const int32_t *tri, const int32_t *tri_deg, const uint32_t *itcount,
                                           const int32_t *itdeg, double alpha) {
    const uint32_t l = labels[p];
    if (l == INVALID) return 0.0;
    const int size = st.sizes[l], td = tri_deg[p];
    if (size <= 2 || td == 0) return 0.0;
    const int it = (int)(2u * itcount[p]), itd = itdeg[p];   // int_tri = 2 x internal triangles
    const double nom = (double)imul_wrap(it, td);
    const double den = dmul((double)tri[p], dadd((double)td, dmul(alpha, (double)(size - 1 - itd))));
    return den != 0.0 ? ddiv(nom, den) : 0.0;
}

__device__ __forceinline__ double block_sum_fixed(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = dadd(v, __shfl_xor_sync(FULL, v, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) r = dadd(r, sh[w]);
    __syncthreads();
    return r;
}

// Graph-aligned blocks: block b sums WCC_CHUNK consecutive vertices of graph
// blk_gid[b], counted from that graph's first vertex, so every graph's sum has
// the same shape as when the graph is processed alone.
__global__ void __launch_bounds__(TPB)
k_wcc_partial(const uint32_t *__restrict__ fin_off, const uint32_t *__restrict__ blk_off,
              const uint32_t *__restrict__ blk_gid, const uint32_t *__restrict__ labels, Stats st,
              const int32_t *__restrict__ tri, const int32_t *__restrict__ tri_deg,
              const uint32_t *__restrict__ itcount, const int32_t *__restrict__ itdeg, double alpha,
              double *partial, const uint8_t *__restrict__ active) {
    __shared__ double sh[TPB / 32];
    const uint32_t g = blk_gid[blockIdx.x];
    if (active && !active[g]) return;   // a graph of the batch that stopped iterating
    const uint32_t end = fin_off[g + 1];
    const uint32_t base = fin_off[g] + (blockIdx.x - blk_off[g]) * WCC_CHUNK + threadIdx.x * WCC_ITEMS;
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < WCC_ITEMS; i++)
        if (base + i < end) s = dadd(s, wcc_term(base + i, labels, st, tri, tri_deg, itcount, itdeg, alpha));
    double r = block_sum_fixed(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

// one block per graph: fixed-order sum of the graph's partials, divided by its n
__global__ void __launch_bounds__(TPB) k_wcc_final(const double *__restrict__ partial,
                                                   const uint32_t *__restrict__ blk_off,
                                                   const uint32_t *__restrict__ fin_off, double *out,
                                                   const uint8_t *__restrict__ active = nullptr) {
    __shared__ double sh[TPB / 32];
    const uint32_t g = blockIdx.x;
    if (active && !active[g]) return;
    const uint32_t p0 = blk_off[g], parts = blk_off[g + 1] - p0, n = fin_off[g + 1] - fin_off[g];
    double s = 0.0;
    for (uint32_t i = threadIdx.x; i < parts; i += TPB) s = dadd(s, partial[p0 + i]);
    double r = block_sum_fixed(s, sh);
    if (threadIdx.x == 0) out[g] = n > 0 ? ddiv(r, (double)n) : 0.0;
}

// ---- p_ext ---------------------------------------------------------------------

__global__ void k_pext_terms(uint32_t n, const uint32_t *__restrict__ indices, const int32_t *__restrict__ tri,
                             double *term) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const uint32_t d = indices[p + 1] - indices[p];
        term[p] = d > 1 ? ddiv((double)tri[p], dmul((double)d, dsub((double)d, 1.0))) : 0.0;
    }
}

// The reference's single-thread order (src/graph.cpp:59-68 at one thread),
// s = ((t0 + t1) + t2) + ..., reproduced bit for bit without a 1.2M-long chain
// of dependent FP64 adds (67 cycles each on GB300).  All terms are >= 0 (zero
// for degree <= 1, which leaves s unchanged).  While s stays in one binade
// [2^e, 2^(e+1)) it is an integer S times u = 2^(e-52), and fl(s + t) is
// (S + round(t/u)) * u with round-to-nearest of the exact t/u — unless t/u has
// a fractional part of exactly 1/2 (then ties-to-even depends on S) or the sum
// leaves the binade.  So one CTA walks the terms in tiles of 8192: integer
// roundings + a block prefix sum give every in-binade partial sum exactly, and
// only the first tie or binade crossing in a tile is done with a real DADD,
// after which the tile restarts from the next term.
constexpr int SEQ_THREADS = 1024;
constexpr int SEQ_ITEMS = 8;
constexpr int SEQ_TILE = SEQ_THREADS * SEQ_ITEMS;

__global__ void __launch_bounds__(SEQ_THREADS)
k_sequential_sum_exact(const double *__restrict__ terms, const uint32_t *__restrict__ seg_off, double *out) {
    // one block per segment (graph): sum of terms[seg_off[g] .. seg_off[g+1]) / length
    const double *term = terms + seg_off[blockIdx.x];
    const uint32_t n = seg_off[blockIdx.x + 1] - seg_off[blockIdx.x];
    const double divisor = (double)n;
    __shared__ long long warp_tot[SEQ_THREADS / 32];
    __shared__ double s_val;
    __shared__ uint32_t s_pos, s_event;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long TWO53 = 1ll << 53;
    if (threadIdx.x == 0) {
        double s = 0.0;
        uint32_t p = 0;
        while (p < n && s == 0.0) s = dadd(s, term[p++]);   // leading zero terms
        s_val = s;
        s_pos = p;
    }
    __syncthreads();
    while (true) {
        const uint32_t pos = s_pos;
        if (pos >= n) break;
        const double s = s_val;
        if (!(s >= 2.2250738585072014e-308) || s > 1e300) {
            // not a positive normal number (e.g. after a negative term): one plain step
            __syncthreads();
            if (threadIdx.x == 0) {
                s_val = dadd(s, term[pos]);
                s_pos = pos + 1;
            }
            __syncthreads();
            continue;
        }
        const int e = (int)((__double_as_longlong(s) >> 52) & 0x7ff) - 1023;   // s in [2^e, 2^(e+1))
        const double scale = __longlong_as_double((long long)(1023 + 52 - e) << 52);   // 2^(52-e)
        const double u = __longlong_as_double((long long)(1023 - 52 + e) << 52);       // 2^(e-52)
        const long long S = __double2ll_rz(dmul(s, scale));
        const uint32_t base = pos + threadIdx.x * SEQ_ITEMS;
        long long r[SEQ_ITEMS];
        bool ev[SEQ_ITEMS];
        long long local = 0;
#pragma unroll
        for (int i = 0; i < SEQ_ITEMS; i++) {
            r[i] = 0;
            ev[i] = false;
            if (base + i < n) {
                const double x = dmul(term[base + i], scale);   // exact: power-of-two scaling
                if (!(x >= 0.0) || x >= 9007199254740992.0) {
                    ev[i] = true;
                } else {
                    const double q = floor(x), f = dsub(x, q);
                    ev[i] = f == 0.5;
                    r[i] = (long long)q + (f > 0.5 ? 1 : 0);
                }
            }
            local += r[i];
        }
        // block exclusive scan of the per-thread totals
        long long inc = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long v = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) warp_tot[warp] = inc;
        if (threadIdx.x == 0) s_event = INVALID;
        __syncthreads();
        if (warp == 0) {
            long long w = warp_tot[lane];
            long long wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                long long v = __shfl_up_sync(FULL, wi, o);
                if (lane >= o) wi += v;
            }
            warp_tot[lane] = wi - w;   // exclusive offset of each warp
        }
        __syncthreads();
        long long run = S + warp_tot[warp] + (inc - local);   // value before this thread's first item
        uint32_t first_event = INVALID;
        long long before_event = 0;
#pragma unroll
        for (int i = 0; i < SEQ_ITEMS; i++) {
            if (base + i < n && first_event == INVALID) {
                if (ev[i] || run + r[i] >= TWO53) {
                    first_event = base + i;
                    before_event = run;
                } else {
                    run += r[i];
                }
            }
        }
        if (first_event != INVALID) atomicMin(&s_event, first_event);
        __syncthreads();
        const uint32_t evi = s_event;
        if (evi == INVALID) {
            const uint32_t last = min(n, pos + (uint32_t)SEQ_TILE) - 1;
            if (last >= base && last < base + SEQ_ITEMS) {   // owner of the tile's last term
                s_val = dmul((double)run, u);
                s_pos = last + 1;
            }
        } else if (first_event == evi) {
            s_val = dadd(dmul((double)before_event, u), term[evi]);
            s_pos = evi + 1;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = ddiv(s_val, divisor);
}

__global__ void k_pext_tree(const uint32_t *__restrict__ fin_off, const uint32_t *__restrict__ blk_off,
                            const uint32_t *__restrict__ blk_gid, const double *__restrict__ term, double *partial) {
    __shared__ double sh[TPB / 32];
    const uint32_t g = blk_gid[blockIdx.x];
    const uint32_t end = fin_off[g + 1];
    const uint32_t base = fin_off[g] + (blockIdx.x - blk_off[g]) * WCC_CHUNK + threadIdx.x * WCC_ITEMS;
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < WCC_ITEMS; i++)
        if (base + i < end) s = dadd(s, term[base + i]);
    double r = block_sum_fixed(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

// ---- per-graph loop control ---------------------------------------------------

// src/main.cpp:68-81 for every graph still iterating: count the iteration,
// remember whether it beat the best WCC, stop when it is below best*(1+threshold)
__global__ void k_batch_step(uint32_t G, const double *__restrict__ wcc, double *best, uint8_t *active,
                             uint8_t *improved, int32_t *iters, double threshold, uint32_t *n_active, double *trace,
                             int max_trace) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < G; g += gridDim.x * blockDim.x) {
        improved[g] = 0;
        if (!active[g]) continue;
        const double w = wcc[g], b = best[g];
        const int it = ++iters[g];
        if (trace && it <= max_trace) trace[(size_t)g * max_trace + it - 1] = w;
        if (w > b) improved[g] = 1;
        if (w < dmul(b, dadd(1.0, threshold))) {
            active[g] = 0;
        } else {
            best[g] = w;
            atomicAdd(n_active, 1u);
        }
    }
}

__global__ void k_copy_improved(uint32_t n, const uint32_t *__restrict__ gid, const uint8_t *__restrict__ improved,
                                const uint32_t *__restrict__ labels, uint32_t *best) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (improved[gid ? gid[v] : 0]) best[v] = labels[v];
}

__global__ void k_batch_reset(uint32_t G, const uint32_t *__restrict__ fin_off, const double *__restrict__ wcc,
                              double *best, uint8_t *active, int32_t *iters) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < G; g += gridDim.x * blockDim.x) {
        best[g] = wcc[g];
        active[g] = fin_off[g + 1] > fin_off[g];
        iters[g] = 0;
    }
}

}  // namespace

void batch_step(Ctx &c, double threshold, double *trace, int max_trace) {
    Batch &b = c.b;
    cudaStream_t s = c.stream;
    CK(cudaMemsetAsync(b.n_active, 0, 4, s));
    k_batch_step<<<grid_for(b.G, TPB), TPB, 0, s>>>(b.G, b.wcc, b.best_wcc, b.active, b.improved, b.iters, threshold,
                                                     b.n_active, trace, max_trace);
    CK_LAUNCH("k_batch_step");
    if (c.g.n) {
        k_copy_improved<<<grid_for(c.g.n, TPB), TPB, 0, s>>>(c.g.n, b.gid, b.improved, c.labels, c.best);
        CK_LAUNCH("k_copy_improved");
    }
    c.launches += 2;
}

void batch_reset(Ctx &c) {
    Batch &b = c.b;
    k_batch_reset<<<grid_for(b.G, TPB), TPB, 0, c.stream>>>(b.G, b.fin_off, b.wcc, b.best_wcc, b.active, b.iters);
    CK_LAUNCH("k_batch_reset");
    c.launches++;
}

void collect_stats(Ctx &c, const uint32_t *labels, Stats &st, bool frozen_graphs) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    const size_t bytes = (size_t)(c.num_comms ? c.num_comms : 1) * 4;
    CK(cudaMemsetAsync(st.sizes, 0, bytes, s));
    CK(cudaMemsetAsync(st.ext, 0, bytes, s));
    CK(cudaMemsetAsync(st.intl, 0, bytes, s));
    if (g.n == 0) return;
    PhaseScope ph(c, "stats");
    const LabelFilter skip{nullptr, c.b.gid, frozen_graphs ? c.b.active : nullptr};
    k_stats<<<grid_for(((uint64_t)(g.n + 31) / 32 + g.rows.nchunks) * 32, TPB), TPB, 0, s>>>(
        g.n, g.rows, g.indices, g.adj, labels, st, skip);
    CK_LAUNCH("k_stats");
    c.launches++;
}

// Internal out-lists for the label-mode triangle count: the out-neighbours of v
// that carry v's (valid) label, in order, at v's CSR offset; length 0 for
// unlabelled vertices and those of converged graphs.  The internal triangles of
// compute_wcc (src/wcc.cpp:84-127) are exactly the triangles of this subgraph, so
// the count walks internal lists only instead of filtering whole out-lists.
template <int G>
__global__ void __launch_bounds__(TPB)
k_internal_outlists(uint32_t n, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ nlow,
                    const uint32_t *__restrict__ adj, LabelFilter lf, uint32_t *ilen, uint32_t *iadj) {
    // a group of G lanes per vertex (out-lists of most vertices are short; ids are
    // degree ranks, so the vertices of a warp have out-lists of similar length)
    const int lane = threadIdx.x & 31, gl = lane % G, g0 = lane - gl;
    const unsigned gmask = (G == 32) ? FULL : (((1u << G) - 1u) << g0);
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t groups = (gridDim.x * blockDim.x) / G;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) / G - (lane / G); base < n;
         base += groups) {
        const uint32_t v = base + lane / G;   // (base: the warp's first vertex)
        const bool live = v < n;
        const uint32_t l = live ? lf.labels[v] : INVALID;
        const bool on = live && l != INVALID && !lf.frozen(v);
        const uint32_t beg = on ? indices[v] : 0u, len = on ? nlow[v] : 0u;
        uint32_t steps = (len + G - 1) / G;
#pragma unroll
        for (int d = G; d < 32; d <<= 1) steps = max(steps, __shfl_xor_sync(FULL, steps, d));
        uint32_t cnt = 0;
        for (uint32_t s = 0; s < steps; s++) {
            const uint32_t i = s * G + gl;
            const uint32_t w = i < len ? adj[beg + i] : 0u;
            const bool keep = i < len && lf.labels[w] == l;
            const unsigned kb = __ballot_sync(FULL, keep) & gmask;
            if (keep) iadj[beg + cnt + __popc(kb & lt)] = w;
            cnt += __popc(kb);
        }
        if (live && gl == 0) ilen[v] = cnt;
    }
}

void launch_wcc(Ctx &c, const uint32_t *labels, const Stats &st, bool frozen_graphs) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    if (g.n == 0) {
        CK(cudaMemsetAsync(c.b.wcc, 0, sizeof(double) * c.b.G, s));
        return;
    }
    PhaseScope ph(c, "wcc");
    CK(cudaMemsetAsync(c.slot_flag, 0, 2 * (size_t)g.m, s));
    CK(cudaMemsetAsync(c.itcount, 0, (size_t)g.n * 4, s));
    CK(cudaMemsetAsync(c.itdeg, 0, (size_t)g.n * 4, s));
    const Batch &b = c.b;
    const uint8_t *active = frozen_graphs ? b.active : nullptr;
    const LabelFilter lf{labels, b.gid, active};
    k_internal_outlists<8><<<grid_for((uint64_t)g.n * 8, TPB), TPB, 0, s>>>(g.n, g.indices, g.nlow, g.adj, lf, c.int_len,
                                                                        c.int_adj);
    CK_LAUNCH("k_internal_outlists");
    // the plan's buckets (by full out-degree) stay valid: internal lists are never longer
    const Oriented o{g.indices, c.int_len, c.int_adj, g.n};
    count_triangles(c, o, c.wplan, LabelFilter{}, c.itcount, c.slot_flag, s, "wcc_tc");
    k_internal_degrees<<<grid_for(((uint64_t)(g.n + 31) / 32 + g.rows.nchunks) * 32, TPB), TPB, 0, s>>>(
        g.n, g.rows, g.indices, c.int_len, c.int_adj, c.slot_flag, c.itdeg, lf);
    CK_LAUNCH("k_internal_degrees");
    c.launches++;
    if (b.blocks) {
        k_wcc_partial<<<b.blocks, TPB, 0, s>>>(b.fin_off, b.blk_off, b.blk_gid, labels, st, g.tri, g.tri_deg,
                                               c.itcount, c.itdeg, c.alpha, c.wcc_part, active);
        CK_LAUNCH("k_wcc_partial");
    }
    k_wcc_final<<<b.G, TPB, 0, s>>>(c.wcc_part, b.blk_off, b.fin_off, b.wcc, active);
    CK_LAUNCH("k_wcc_final");
    c.launches += 3;
}

double compute_wcc(Ctx &c, const uint32_t *labels, const Stats &st) {
    launch_wcc(c, labels, st);
    CK(cudaMemcpyAsync(c.wcc_host, c.b.wcc, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return *c.wcc_host;
}

// FP32 enclosure of every p_ext (directed conversions), for the interval gains
__global__ void k_pe32(uint32_t G, const double *__restrict__ p_ext, float2 *pe32) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < G; g += gridDim.x * blockDim.x)
        pe32[g] = make_float2(__double2float_rd(p_ext[g]), __double2float_ru(p_ext[g]));
}

// p_ext of every graph on the side stream: the index-ordered sum is one CTA per
// graph and runs alongside the initial partition and WCC on the main stream;
// join_p_ext (before the first improvement) and host_p_ext (host reads) wait for it.
void compute_p_ext(Ctx &c) {
    Graph &g = c.g;
    Batch &b = c.b;
    cudaStream_t s = c.side;
    if (!c.pext_ready) CK(cudaEventCreateWithFlags(&c.pext_ready, cudaEventDisableTiming));
    CK(cudaEventRecord(c.pext_ready, c.stream));   // the graph arrays are ready
    CK(cudaStreamWaitEvent(s, c.pext_ready, 0));
    DevBuf<double> term(g.n ? g.n : 1, s);
    if (g.n) {
        k_pext_terms<<<grid_for(g.n, TPB), TPB, 0, s>>>(g.n, g.indices, g.tri, term.get());
        CK_LAUNCH("k_pext_terms");
        c.launches++;
    }
    if ((c.flags & SCD_FLAG_PEXT_TREE) && g.n) {
        DevBuf<double> part(b.blocks ? b.blocks : 1, s);
        if (b.blocks) {
            k_pext_tree<<<b.blocks, TPB, 0, s>>>(b.fin_off, b.blk_off, b.blk_gid, term.get(), part.get());
            CK_LAUNCH("k_pext_tree");
        }
        k_wcc_final<<<b.G, TPB, 0, s>>>(part.get(), b.blk_off, b.fin_off, b.p_ext);
        CK_LAUNCH("k_wcc_final");
        c.launches += 2;
        // (an empty graph's p_ext is 0 here, NaN in the index-ordered mode like the reference's 0/0)
    } else {
        k_sequential_sum_exact<<<b.G, SEQ_THREADS, 0, s>>>(term.get(), b.fin_off, b.p_ext);
        CK_LAUNCH("k_sequential_sum_exact");
        c.launches++;
    }
    k_pe32<<<grid_for(b.G, TPB), TPB, 0, s>>>(b.G, b.p_ext, b.pe32);
    CK_LAUNCH("k_pe32");
    c.launches++;
    term.release();
    CK(cudaEventRecord(c.pext_ready, s));
    c.pext_join_pending = true;
    c.pext_host_valid = false;
}

void join_p_ext(Ctx &c) {
    if (!c.pext_join_pending) return;
    CK(cudaStreamWaitEvent(c.stream, c.pext_ready, 0));
    c.pext_join_pending = false;
}

void host_p_ext(Ctx &c) {
    if (c.pext_host_valid) return;
    Batch &b = c.b;
    b.h_p_ext.assign(b.G, 0.0);
    if (c.pext_ready) CK(cudaEventSynchronize(c.pext_ready));
    if (b.G && b.p_ext) CK(cudaMemcpy(b.h_p_ext.data(), b.p_ext, sizeof(double) * b.G, cudaMemcpyDeviceToHost));
    c.g.p_ext = b.G ? b.h_p_ext[0] : 0.0;
    c.pext_host_valid = true;
}

}  // namespace scd
