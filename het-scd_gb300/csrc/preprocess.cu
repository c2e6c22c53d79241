// Preprocessing on the device: the work of the reference's `convert` tool
// (src/convert.cpp:141-463), which the reference runs on the CPU only.
//
//  1. first-appearance renumbering (src/convert.cpp:141-170): first position of
//     every raw id (atomicMin over the 2E endpoint slots), a bitmap of those
//     positions and a popcount prefix give each id its rank of first appearance;
//  2. both directions of every renamed non-loop pair placed by a counting sort
//     on the row, every row sorted and its repeated values marked (csr.cu): the
//     de-duplicated symmetric rows (src/convert.cpp:252-268 + 417-463);
//  3. degree orientation (u -> v iff (deg v, v) > (deg u, u)) read straight off
//     those rows into out-lists and in-lists, triangles per vertex and "edge lies
//     on a triangle" flags (triangles.cu); tri = 2 x the vertex's triangles,
//     tri_deg = number of flagged edges (src/convert.cpp:271-340);
//  4. triangle-free edges dropped and the kept vertices ranked by (tri_deg, id)
//     descending, degree-0 vertices trimmed (src/convert.cpp:342-414);
//  5. the final symmetric CSR: rows of the kept edges in rank ids, placed by
//     the known row lengths (tri_deg) and sorted row by row (src/convert.cpp:417-455).
#include "engine.cuh"

namespace scd {

namespace {

constexpr unsigned TPB = 256;

__global__ void k_first_pos(const uint32_t *__restrict__ pairs, uint64_t count, uint32_t *first) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t a = pairs[2 * i], b = pairs[2 * i + 1];
        uint32_t pa = (uint32_t)(2 * i), pb = pa + 1;
        if (first[a] > pa) atomicMin(first + a, pa);
        if (first[b] > pb) atomicMin(first + b, pb);
    }
}

__global__ void k_mark_first(const uint32_t *__restrict__ first, uint32_t n_raw, uint32_t *bits) {
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n_raw; x += gridDim.x * blockDim.x) {
        uint32_t p = first[x];
        if (p != INVALID) atomicOr(bits + (p >> 5), 1u << (p & 31));
    }
}

struct PopcountOf {
    const uint32_t *bits;
    __device__ uint32_t operator[](size_t i) const { return __popc(bits[i]); }
};

// first[x] (position of first appearance) -> new id (rank of that position)
__global__ void k_rename(uint32_t *first, uint32_t n_raw, const uint32_t *__restrict__ bits,
                         const uint32_t *__restrict__ word_prefix) {
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n_raw; x += gridDim.x * blockDim.x) {
        uint32_t p = first[x];
        if (p != INVALID) {
            uint32_t w = p >> 5, b = p & 31;
            first[x] = word_prefix[w] + __popc(bits[w] & ((1u << b) - 1u));
        }
    }
}

// row lengths of the renamed, loop-free pairs in both directions
__global__ void k_pair_degrees(const uint32_t *__restrict__ pairs, uint64_t count, const uint32_t *__restrict__ rename,
                               uint32_t *cnt) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = rename[pairs[2 * i]], b = rename[pairs[2 * i + 1]];
        if (a != b) {   // (input lists are often sorted by the first id: aggregate its increments)
            warp_atomic_inc(cnt + a, __activemask());
            atomicAdd(cnt + b, 1u);
        }
    }
}

// both directions of every pair into their rows (order inside a row is fixed by the row sort)
__global__ void k_pair_fill(const uint32_t *__restrict__ pairs, uint64_t count, const uint32_t *__restrict__ rename,
                            const uint32_t *__restrict__ off, uint32_t *fill, uint32_t *vals) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = rename[pairs[2 * i]], b = rename[pairs[2 * i + 1]];
        if (a != b) {
            vals[off[a] + warp_atomic_inc(fill + a, __activemask())] = b;
            vals[off[b] + atomicAdd(fill + b, 1u)] = a;
        }
    }
}

// u -> v iff (deg v, v) > (deg u, u): the degree orientation
__device__ __forceinline__ bool is_out(uint32_t u, uint32_t du, uint32_t v, uint32_t dv) {
    return dv > du || (dv == du && v > u);
}

// rows of more than LONG_ROW entries (repeats included) go to a CTA each
constexpr uint32_t LONG_ROW = 4096;
constexpr int LONG_THREADS = 512;

struct LongRow {
    const uint32_t *off;
    __device__ uint32_t operator[](size_t u) const { return off[u + 1] - off[u] > LONG_ROW; }
};

__global__ void k_long_list(const uint32_t *__restrict__ off, uint32_t n, const uint32_t *__restrict__ lpos,
                            uint32_t *longs) {
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x)
        if (off[u + 1] - off[u] > LONG_ROW) longs[lpos[u]] = u;
}

// out-slots of every short de-duplicated row (one warp per row; INVALID holes skipped)
__global__ void k_row_out_count(const uint32_t *__restrict__ off, uint32_t n, const uint32_t *__restrict__ vals,
                                const uint32_t *__restrict__ deg, uint32_t *olen) {
    const uint32_t lane = threadIdx.x & 31, warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += warps) {
        const uint32_t b = off[u], e = off[u + 1];
        if (e - b > LONG_ROW) continue;
        const uint32_t du = deg[u];
        uint32_t c = 0;
        for (uint32_t i = b + lane; i < e; i += 32) {
            const uint32_t v = vals[i];
            if (v != INVALID && is_out(u, du, v, deg[v])) c++;
        }
        c = warp_sum(c);
        if (lane == 0) olen[u] = c;
    }
}

// the same for the long rows, one CTA per row
__global__ void __launch_bounds__(LONG_THREADS)
k_long_out_count(const uint32_t *__restrict__ off, const uint32_t *__restrict__ longs, const uint32_t *__restrict__ nlong,
                 const uint32_t *__restrict__ vals, const uint32_t *__restrict__ deg, uint32_t *olen) {
    __shared__ uint32_t wsum[LONG_THREADS / 32];
    const uint32_t nl = *nlong, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t k = blockIdx.x; k < nl; k += gridDim.x) {
        const uint32_t u = longs[k], du = deg[u], e = off[u + 1];
        uint32_t c = 0;
        for (uint32_t i = off[u] + threadIdx.x; i < e; i += LONG_THREADS) {
            const uint32_t v = vals[i];
            if (v != INVALID && is_out(u, du, v, deg[v])) c++;
        }
        c = warp_sum(c);
        if (lane == 0) wsum[w] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int j = 0; j < LONG_THREADS / 32; j++) t += wsum[j];
            olen[u] = t;
        }
        __syncthreads();
    }
}

struct InCount {   // in-slots of row u: its distinct values that are not out-slots
    const uint32_t *deg, *olen;
    __device__ uint32_t operator[](size_t u) const { return deg[u] - olen[u]; }
};

// out-slots (u, v) of the short rows to orow/ocol from obeg[u] on, in-slots (v -> u)
// to icol from ibeg[u] on, both in row order (so out- and in-lists stay sorted)
__global__ void k_row_orient(const uint32_t *__restrict__ off, uint32_t n, const uint32_t *__restrict__ vals,
                             const uint32_t *__restrict__ deg, const uint32_t *__restrict__ obeg,
                             const uint32_t *__restrict__ ibeg, uint32_t *orow, uint32_t *ocol, uint32_t *icol) {
    const uint32_t lane = threadIdx.x & 31, warps = (gridDim.x * blockDim.x) >> 5;
    const unsigned lt = lanemask_lt();
    for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += warps) {
        const uint32_t b = off[u], e = off[u + 1];
        if (e - b > LONG_ROW) continue;
        const uint32_t du = deg[u];
        uint32_t ob = obeg[u], ib = ibeg[u];
        for (uint32_t i0 = b; i0 < e; i0 += 32) {
            const uint32_t i = i0 + lane;
            const uint32_t v = i < e ? vals[i] : INVALID;
            const bool valid = v != INVALID, out = valid && is_out(u, du, v, deg[v]);
            const unsigned mo = __ballot_sync(FULL, out), mi = __ballot_sync(FULL, valid && !out);
            if (out) {
                const uint32_t p = ob + __popc(mo & lt);
                orow[p] = u;
                ocol[p] = v;
            } else if (valid) {
                icol[ib + __popc(mi & lt)] = v;
            }
            ob += __popc(mo);
            ib += __popc(mi);
        }
    }
}

// the same for the long rows: one CTA per row, LONG_THREADS entries at a time,
// positions from a block scan of the out / in flags
__global__ void __launch_bounds__(LONG_THREADS)
k_long_orient(const uint32_t *__restrict__ off, const uint32_t *__restrict__ longs, const uint32_t *__restrict__ nlong,
              const uint32_t *__restrict__ vals, const uint32_t *__restrict__ deg, const uint32_t *__restrict__ obeg,
              const uint32_t *__restrict__ ibeg, uint32_t *orow, uint32_t *ocol, uint32_t *icol) {
    constexpr int NW = LONG_THREADS / 32;
    __shared__ uint32_t so[NW], si[NW];
    const uint32_t nl = *nlong, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt = lanemask_lt();
    for (uint32_t k = blockIdx.x; k < nl; k += gridDim.x) {
        const uint32_t u = longs[k], du = deg[u], e = off[u + 1];
        uint32_t ob = obeg[u], ib = ibeg[u];
        for (uint32_t i0 = off[u]; i0 < e; i0 += LONG_THREADS) {
            const uint32_t i = i0 + threadIdx.x;
            const uint32_t v = i < e ? vals[i] : INVALID;
            const bool valid = v != INVALID, out = valid && is_out(u, du, v, deg[v]);
            const unsigned mo = __ballot_sync(FULL, out), mi = __ballot_sync(FULL, valid && !out);
            if (lane == 0) {
                so[w] = __popc(mo);
                si[w] = __popc(mi);
            }
            __syncthreads();
            uint32_t po = 0, pi = 0, to = 0, ti = 0;   // warps before this one, and the whole chunk
            for (int j = 0; j < NW; j++) {
                const uint32_t a = so[j], c = si[j];
                if (j < (int)w) {
                    po += a;
                    pi += c;
                }
                to += a;
                ti += c;
            }
            if (out) {
                const uint32_t p = ob + po + __popc(mo & lt);
                orow[p] = u;
                ocol[p] = v;
            } else if (valid) {
                icol[ib + pi + __popc(mi & lt)] = v;
            }
            ob += to;
            ib += ti;
            __syncthreads();   // so / si are rewritten by the next chunk
        }
    }
}

__global__ void k_in_len(const uint32_t *__restrict__ deg, const uint32_t *__restrict__ olen, uint32_t n,
                         uint32_t *ilen) {
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x)
        ilen[u] = deg[u] - olen[u];
}

// tri_deg[v] = number of v's edges that lie on a triangle (src/convert.cpp:327-340)
__global__ void k_flag_degrees(const uint32_t *__restrict__ orow, const uint32_t *__restrict__ ocol,
                               const uint8_t *__restrict__ flag, uint32_t count, int32_t *tri_deg) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        if (flag[i]) {   // out-slots are grouped by row: one atomic per row and warp for that side
            warp_atomic_inc((uint32_t *)(tri_deg + orow[i]), __activemask());
            atomicAdd(tri_deg + ocol[i], 1);
        }
    }
}

// tri[v] = sum of the per-edge counts at v = 2 x triangles at v, in int32
// two's-complement arithmetic like the reference's int accumulator
__global__ void k_tri_from_count(const uint32_t *__restrict__ tcount, uint32_t n, int32_t *tri) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        tri[v] = (int32_t)(2u * tcount[v]);
}

// the kept vertices (tri_deg > 0) at their id-order positions kscan[v], with the
// key ((maxd - tri_deg) << k) | (2^k-1 - v): ascending = (tri_deg, v) descending
__global__ void k_kept_keys(const int32_t *__restrict__ tri_deg, uint32_t n, const uint32_t *__restrict__ kscan,
                            uint32_t maxd, int k, uint64_t *keys, uint32_t *vals) {
    const uint64_t vmax = (1ull << k) - 1;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int32_t d = tri_deg[v];
        if (d > 0) {
            const uint32_t i = kscan[v];
            keys[i] = ((uint64_t)(maxd - (uint32_t)d) << k) | (vmax - v);
            vals[i] = v;
        }
    }
}

// final id = position in the sorted order of the kept vertices
__global__ void k_rank_of(const uint32_t *__restrict__ order, uint32_t n2, const int32_t *__restrict__ tri,
                          const int32_t *__restrict__ tri_deg, uint32_t *rank, int32_t *tri_out,
                          int32_t *tri_deg_out) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n2; r += gridDim.x * blockDim.x) {
        const uint32_t v = order[r];
        rank[v] = r;
        tri_out[r] = tri[v];
        tri_deg_out[r] = tri_deg[v];
    }
}

// the kept (flagged) edges in rank ids into the rows of the final CSR, both directions
__global__ void k_final_fill(const uint32_t *__restrict__ orow, const uint32_t *__restrict__ ocol,
                             const uint8_t *__restrict__ flag, uint32_t count, const uint32_t *__restrict__ rank,
                             const uint32_t *__restrict__ ind, uint32_t *fill, uint32_t *adj) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        if (flag[i]) {
            const uint32_t a = rank[orow[i]], b = rank[ocol[i]];
            adj[ind[a] + warp_atomic_inc(fill + a, __activemask())] = b;
            adj[ind[b] + atomicAdd(fill + b, 1u)] = a;
        }
    }
}

struct DegreeOf {   // final row length of a ranked vertex: its kept (triangle) edges
    const int32_t *tri_deg;
    __device__ uint32_t operator[](size_t i) const { return (uint32_t)tri_deg[i]; }
};

// ---- batches: graph g's records are [rec_off[g], rec_off[g+1]) --------------

__device__ __forceinline__ uint32_t segment_of(const uint64_t *off, uint32_t G, uint64_t i) {
    uint32_t lo = 0, hi = G + 1;   // last g with off[g] <= i
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= i) lo = mid + 1;
        else hi = mid;
    }
    return lo - 1;
}

__device__ __forceinline__ uint32_t segment_of32(const uint32_t *off, uint32_t G, uint32_t i) {
    uint32_t lo = 0, hi = G + 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= i) lo = mid + 1;
        else hi = mid;
    }
    return lo - 1;
}

// Each CTA takes one contiguous range of items (loads stay coalesced: its
// threads stride by blockDim inside the range) and a thread looks its graph up
// only when it crosses into the next one, so per-graph totals need one atomic
// per thread and graph met, not one per item.
struct BlockRange {
    uint64_t lo, hi;
    __device__ BlockRange(uint64_t count) {
        const uint64_t span = (count + gridDim.x - 1) / gridDim.x;
        lo = min(count, (uint64_t)blockIdx.x * span);
        hi = min(count, lo + span);
    }
};

// ids of graph g span [0, gmax[g]): one past its largest id
__global__ void k_graph_id_span(const uint32_t *__restrict__ pairs, uint64_t count, const uint64_t *__restrict__ rec_off,
                                uint32_t G, uint32_t *gmax) {
    const BlockRange r(count);
    uint32_t g = INVALID, cur = 0;
    uint64_t end = 0;
    for (uint64_t i = r.lo + threadIdx.x; i < r.hi; i += blockDim.x) {
        if (g == INVALID || i >= end) {
            if (g != INVALID) atomicMax(gmax + g, cur);
            g = segment_of(rec_off, G, i);
            end = rec_off[g + 1];
            cur = 0;
        }
        const uint32_t a = pairs[2 * i], b = pairs[2 * i + 1];
        cur = max(cur, (a > b ? a : b) + 1);
    }
    if (g != INVALID) atomicMax(gmax + g, cur);
}

// disjoint id ranges: graph g's ids shifted by raw_off[g]
__global__ void k_offset_pairs(const uint32_t *__restrict__ pairs, uint64_t count, const uint64_t *__restrict__ rec_off,
                               uint32_t G, const uint64_t *__restrict__ raw_off, uint32_t *out) {
    const BlockRange r(count);
    uint32_t d = 0;
    uint64_t end = 0;
    bool have = false;
    for (uint64_t i = r.lo + threadIdx.x; i < r.hi; i += blockDim.x) {
        if (!have || i >= end) {
            const uint32_t g = segment_of(rec_off, G, i);
            end = rec_off[g + 1];
            d = (uint32_t)raw_off[g];
            have = true;
        }
        out[2 * i] = pairs[2 * i] + d;
        out[2 * i + 1] = pairs[2 * i + 1] + d;
    }
}

// renamed vertices per graph (raw ids of graph g lie in [raw_off[g], raw_off[g+1]))
__global__ void k_count_renamed(const uint32_t *__restrict__ rename, uint32_t n_raw, const uint64_t *__restrict__ raw_off,
                                uint32_t G, uint32_t *ndist) {
    const BlockRange r(n_raw);
    uint32_t g = INVALID, cur = 0;
    uint64_t end = 0;
    for (uint64_t x = r.lo + threadIdx.x; x < r.hi; x += blockDim.x) {
        if (g == INVALID || x >= end) {
            if (g != INVALID && cur) atomicAdd(ndist + g, cur);
            g = segment_of(raw_off, G, x);
            end = raw_off[g + 1];
            cur = 0;
        }
        cur += rename[x] != INVALID;
    }
    if (g != INVALID && cur) atomicAdd(ndist + g, cur);
}

__global__ void k_graph_of_order(const uint32_t *__restrict__ order, uint32_t n, const uint32_t *__restrict__ ren_off,
                                 uint32_t G, uint64_t *keys) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        keys[i] = segment_of32(ren_off, G, order[i]);
}

struct Kept {
    const int32_t *tri_deg;
    __device__ uint32_t operator[](size_t v) const { return tri_deg[v] > 0; }
};

// first final id of every graph: kept vertices before the graph's first renamed id
// (renamed ids, and so the kept vertices in id order, are graph-contiguous)
__global__ void k_final_offsets(uint32_t G, const uint32_t *__restrict__ ren_off, const uint32_t *__restrict__ kscan,
                                uint32_t *fin_off) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += gridDim.x * blockDim.x)
        fin_off[g] = kscan[ren_off[g]];
}

template <typename T>
T read_scalar(const T *dev, cudaStream_t s) {
    T h;
    CK(cudaMemcpyAsync(&h, dev, sizeof(T), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return h;
}

}  // namespace

void convert_edges(Ctx &c, const uint32_t *pairs_in, uint64_t count, const std::vector<uint64_t> *rec_off_h) {
    cudaStream_t s = c.stream;
    if (count >= (1ull << 31)) throw Error(SCD_ERR_LIMIT, "more than 2^31-1 edge records");
    const uint32_t NG = rec_off_h ? (uint32_t)rec_off_h->size() - 1 : 1;
    c.free_all();
    if (count == 0 && NG == 1) {
        upload_graph(c, 0, 0, nullptr, nullptr, nullptr, nullptr);
        return;
    }
    PhaseScope ph(c, "convert");
    const unsigned G = grid_for(count ? count : 1, TPB, 152 * 32);
    prepare_tc_kernels();

    // 0. a batch: disjoint raw id ranges per graph
    const uint32_t *pairs = pairs_in;
    DevBuf<uint64_t> rec_off, raw_off;
    DevBuf<uint32_t> shifted;
    if (NG > 1) {
        rec_off.alloc(NG + 1, s);
        CK(cudaMemcpyAsync(rec_off.get(), rec_off_h->data(), 8 * (NG + 1), cudaMemcpyHostToDevice, s));
        DevBuf<uint32_t> gmax(NG, s);
        CK(cudaMemsetAsync(gmax.get(), 0, 4 * NG, s));
        if (count) {
            k_graph_id_span<<<G, TPB, 0, s>>>(pairs_in, count, rec_off.get(), NG, gmax.get());
            CK_LAUNCH("k_graph_id_span");
        }
        raw_off.alloc(NG + 1, s);
        scan_exclusive<uint64_t>(gmax.get(), raw_off.get(), NG, s);
        if (read_scalar(raw_off.get() + NG, s) >= 0xffffffffull)
            throw Error(SCD_ERR_LIMIT, "the graphs of a batch need more than 2^32-1 vertex ids together");
        shifted.alloc(2 * count + 1, s);
        if (count) {
            k_offset_pairs<<<G, TPB, 0, s>>>(pairs_in, count, rec_off.get(), NG, raw_off.get(), shifted.get());
            CK_LAUNCH("k_offset_pairs");
        }
        pairs = shifted.get();
        c.launches += 3;
    }
    if (count == 0) {   // a batch of empty graphs
        c.b.G = NG;
        c.b.h_fin_off.assign(NG + 1, 0);
        upload_graph(c, 0, 0, nullptr, nullptr, nullptr, nullptr);
        return;
    }

    // 1. first-appearance renumbering
    DevBuf<uint32_t> mx(1, s);
    CK(cudaMemsetAsync(mx.get(), 0, 4, s));
    k_reduce_max<uint32_t><<<grid_for(2 * count, TPB, 152 * 16), TPB, 0, s>>>(pairs, 2 * count, mx.get());
    CK_LAUNCH("k_reduce_max");
    const uint32_t n_raw = read_scalar(mx.get(), s) + 1;
    if (n_raw == 0) throw Error(SCD_ERR_LIMIT, "vertex id 2^32-1 is not supported");
    DevBuf<uint32_t> rename(n_raw, s);
    CK(cudaMemsetAsync(rename.get(), 0xff, (size_t)n_raw * 4, s));
    k_first_pos<<<G, TPB, 0, s>>>(pairs, count, rename.get());
    CK_LAUNCH("k_first_pos");
    const size_t words = (2 * count + 31) / 32;
    DevBuf<uint32_t> bits(words, s), wpre(words + 1, s);
    CK(cudaMemsetAsync(bits.get(), 0, words * 4, s));
    k_mark_first<<<grid_for(n_raw, TPB), TPB, 0, s>>>(rename.get(), n_raw, bits.get());
    CK_LAUNCH("k_mark_first");
    scan_exclusive<uint32_t>(PopcountOf{bits.get()}, wpre.get(), words, s);
    k_rename<<<grid_for(n_raw, TPB), TPB, 0, s>>>(rename.get(), n_raw, bits.get(), wpre.get());
    CK_LAUNCH("k_rename");
    const uint32_t n1 = read_scalar(wpre.get() + words, s);
    bits.release();
    wpre.release();
    DevBuf<uint32_t> ren_off(NG + 1, s);   // renamed ids of graph g: [ren_off[g], ren_off[g+1])
    if (NG > 1) {
        DevBuf<uint32_t> ndist(NG, s);
        CK(cudaMemsetAsync(ndist.get(), 0, 4 * NG, s));
        k_count_renamed<<<grid_for(n_raw, TPB, 152 * 8), TPB, 0, s>>>(rename.get(), n_raw, raw_off.get(), NG, ndist.get());
        CK_LAUNCH("k_count_renamed");
        scan_exclusive<uint32_t>((const uint32_t *)ndist.get(), ren_off.get(), NG, s);
        c.launches += 2;
    } else {
        const uint32_t h[2] = {0, n1};
        CK(cudaMemcpyAsync(ren_off.get(), h, 8, cudaMemcpyHostToDevice, s));
    }

    // 2. de-duplicated symmetric CSR over the renamed ids: rows by a counting sort, then sorted row by row
    const int k1 = ceil_log2(n1 < 2 ? 2 : n1);
    DevBuf<uint32_t> cnt(n1, s), off1((size_t)n1 + 1, s);
    CK(cudaMemsetAsync(cnt.get(), 0, (size_t)n1 * 4, s));
    k_pair_degrees<<<G, TPB, 0, s>>>(pairs, count, rename.get(), cnt.get());
    CK_LAUNCH("k_pair_degrees");
    scan_exclusive<uint32_t>((const uint32_t *)cnt.get(), off1.get(), n1, s);
    const uint32_t entries = read_scalar(off1.get() + n1, s);
    DevBuf<uint32_t> vals(entries ? entries : 1, s);
    CK(cudaMemsetAsync(cnt.get(), 0, (size_t)n1 * 4, s));
    k_pair_fill<<<G, TPB, 0, s>>>(pairs, count, rename.get(), off1.get(), cnt.get(), vals.get());
    CK_LAUNCH("k_pair_fill");
    rename.release();
    sort_rows(c, off1.get(), n1, vals.get(), true, cnt.get(), s);   // cnt := distinct values of each row
    // 3. degree orientation straight from the sorted rows (repeated values are
    //    INVALID holes): out-slots per row, their offsets, then out-lists (orow,
    //    ocol) and in-lists (icol) in row order; a warp per row, a CTA per row of
    //    more than LONG_ROW entries (a hub's row would be one warp's serial loop)
    DevBuf<uint32_t> olen(n1, s), obeg((size_t)n1 + 1, s), ibeg((size_t)n1 + 1, s);
    DevBuf<uint32_t> lpos((size_t)n1 + 1, s), longs(n1, s);
    scan_exclusive<uint32_t>(LongRow{off1.get()}, lpos.get(), n1, s);
    k_long_list<<<grid_for(n1, TPB), TPB, 0, s>>>(off1.get(), n1, lpos.get(), longs.get());
    CK_LAUNCH("k_long_list");
    k_row_out_count<<<grid_for((uint64_t)n1 * 32, TPB), TPB, 0, s>>>(off1.get(), n1, vals.get(), cnt.get(), olen.get());
    CK_LAUNCH("k_row_out_count");
    k_long_out_count<<<152 * 2, LONG_THREADS, 0, s>>>(off1.get(), longs.get(), lpos.get() + n1, vals.get(), cnt.get(),
                                                      olen.get());
    CK_LAUNCH("k_long_out_count");
    scan_exclusive<uint32_t>((const uint32_t *)olen.get(), obeg.get(), n1, s);
    scan_exclusive<uint32_t>(InCount{cnt.get(), olen.get()}, ibeg.get(), n1, s);
    const uint32_t m1 = read_scalar(obeg.get() + n1, s);
    DevBuf<uint32_t> orow(m1 ? m1 : 1, s), ocol(m1 ? m1 : 1, s), icol(m1 ? m1 : 1, s);
    k_row_orient<<<grid_for((uint64_t)n1 * 32, TPB), TPB, 0, s>>>(off1.get(), n1, vals.get(), cnt.get(), obeg.get(),
                                                                  ibeg.get(), orow.get(), ocol.get(), icol.get());
    CK_LAUNCH("k_row_orient");
    k_long_orient<<<152 * 2, LONG_THREADS, 0, s>>>(off1.get(), longs.get(), lpos.get() + n1, vals.get(), cnt.get(),
                                                   obeg.get(), ibeg.get(), orow.get(), ocol.get(), icol.get());
    CK_LAUNCH("k_long_orient");
    c.launches += 8;
    vals.release();
    off1.release();
    lpos.release();
    longs.release();
    DevBuf<uint32_t> ilen(n1, s);
    k_in_len<<<grid_for(n1, TPB), TPB, 0, s>>>(cnt.get(), olen.get(), n1, ilen.get());
    CK_LAUNCH("k_in_len");
    cnt.release();
    DevBuf<uint32_t> tcount(n1, s);
    DevBuf<uint8_t> oflag(m1, s);
    CK(cudaMemsetAsync(tcount.get(), 0, (size_t)n1 * 4, s));
    CK(cudaMemsetAsync(oflag.get(), 0, m1, s));
    Oriented o{obeg.get(), olen.get(), ocol.get(), n1, ibeg.get(), ilen.get(), icol.get()};
    {
        TcPlan plan;
        tc_plan_counting(c, o, m1, plan, s);
        count_triangles(c, o, plan, LabelFilter{}, tcount.get(), oflag.get(), s);
    }
    icol.release();
    ibeg.release();
    ilen.release();
    DevBuf<int32_t> tri1(n1, s), tdeg1(n1, s);
    CK(cudaMemsetAsync(tdeg1.get(), 0, (size_t)n1 * 4, s));
    k_tri_from_count<<<grid_for(n1, TPB), TPB, 0, s>>>(tcount.get(), n1, tri1.get());
    CK_LAUNCH("k_tri_from_count");
    k_flag_degrees<<<grid_for(m1, TPB), TPB, 0, s>>>(orow.get(), ocol.get(), oflag.get(), m1, tdeg1.get());
    CK_LAUNCH("k_flag_degrees");
    tcount.release();
    obeg.release();
    olen.release();

    // 4. rank by (tri_deg, id) descending within each graph; vertices without
    //    triangle edges are trimmed, so only the kept ones are sorted (those with
    //    tri_deg 0 would sort after all of them), on keys as wide as the largest
    //    tri_deg needs
    DevBuf<uint32_t> kscan(n1 + 1, s), dmax(1, s);
    scan_exclusive<uint32_t>(Kept{tdeg1.get()}, kscan.get(), n1, s);
    CK(cudaMemsetAsync(dmax.get(), 0, 4, s));
    k_reduce_max<uint32_t><<<grid_for(n1, TPB, 152 * 8), TPB, 0, s>>>((const uint32_t *)tdeg1.get(), n1, dmax.get());
    CK_LAUNCH("k_reduce_max");
    uint32_t *hk = c.host_u32 + 2;   // pinned words: kept vertices, largest tri_deg
    CK(cudaMemcpyAsync(hk, kscan.get() + n1, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hk + 1, dmax.get(), 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const uint32_t n2 = hk[0], maxd = hk[1];
    DevBuf<uint64_t> dkeys(n2 ? n2 : 1, s);
    DevBuf<uint32_t> order(n2 ? n2 : 1, s), rank(n1, s);
    k_kept_keys<<<grid_for(n1, TPB), TPB, 0, s>>>(tdeg1.get(), n1, kscan.get(), maxd, k1, dkeys.get(), order.get());
    CK_LAUNCH("k_kept_keys");
    radix_sort<uint64_t>(dkeys.get(), order.get(), n2, 0, k1 + ceil_log2((uint64_t)maxd + 1), s);
    if (NG > 1) {   // graph-major (stable): each graph's vertices stay contiguous
        k_graph_of_order<<<grid_for(n2 ? n2 : 1, TPB), TPB, 0, s>>>(order.get(), n2, ren_off.get(), NG, dkeys.get());
        CK_LAUNCH("k_graph_of_order");
        radix_sort<uint64_t>(dkeys.get(), order.get(), n2, 0, ceil_log2(NG), s);
    }
    dkeys.release();

    // 5. final symmetric CSR in rank ids: row lengths are the kept edges (tri_deg), rows filled then sorted
    Graph &g = c.g;
    g.n = n2;
    g.indices = c.alloc<uint32_t>((size_t)n2 + 1);
    g.tri = c.alloc<int32_t>(n2);
    g.tri_deg = c.alloc<int32_t>(n2);
    k_rank_of<<<grid_for(n2 ? n2 : 1, TPB), TPB, 0, s>>>(order.get(), n2, tri1.get(), tdeg1.get(), rank.get(), g.tri,
                                                       g.tri_deg);
    CK_LAUNCH("k_rank_of");
    scan_exclusive<uint32_t>(DegreeOf{g.tri_deg}, g.indices, n2, s);
    const uint32_t m2 = read_scalar(g.indices + n2, s) / 2;
    g.m = m2;
    g.adj = c.alloc<uint32_t>(2 * (size_t)m2);
    c.b.G = NG;
    c.b.fin_off = c.alloc<uint32_t>(NG + 1);
    k_final_offsets<<<grid_for(NG + 1, TPB), TPB, 0, s>>>(NG, ren_off.get(), kscan.get(), c.b.fin_off);
    CK_LAUNCH("k_final_offsets");
    c.b.h_fin_off.resize(NG + 1);
    CK(cudaMemcpyAsync(c.b.h_fin_off.data(), c.b.fin_off, 4 * (NG + 1), cudaMemcpyDeviceToHost, s));
    if (m2 > 0) {
        DevBuf<uint32_t> fill(n2, s);
        CK(cudaMemsetAsync(fill.get(), 0, (size_t)n2 * 4, s));
        k_final_fill<<<grid_for(m1, TPB), TPB, 0, s>>>(orow.get(), ocol.get(), oflag.get(), m1, rank.get(), g.indices,
                                                      fill.get(), g.adj);
        CK_LAUNCH("k_final_fill");
        sort_rows(c, g.indices, n2, g.adj, false, nullptr, s);
        c.launches++;
    }
    finish_graph(c);
    c.has_graph = true;   // only once every array exists: a failure above leaves no graph
}

void alloc_graph(Ctx &c, uint32_t n, uint32_t m) {
    const uint32_t NG = c.b.G;   // > 1 only for a batch of empty graphs
    c.free_all();
    c.b.G = NG;
    c.b.h_fin_off.assign(NG + 1, 0);
    c.b.h_fin_off[NG] = n;
    Graph &g = c.g;
    g.n = n;
    g.m = m;
    g.indices = c.alloc<uint32_t>((size_t)n + 1);
    g.adj = c.alloc<uint32_t>(2 * (size_t)m);
    g.tri = c.alloc<int32_t>(n);
    g.tri_deg = c.alloc<int32_t>(n);
}

void upload_graph(Ctx &c, uint32_t n, uint32_t m, const uint32_t *indices, const uint32_t *adj,
                  const int32_t *tri, const int32_t *tri_deg) {
    cudaStream_t s = c.stream;
    alloc_graph(c, n, m);
    Graph &g = c.g;
    if (indices) {
        CK(cudaMemcpyAsync(g.indices, indices, ((size_t)n + 1) * 4, cudaMemcpyHostToDevice, s));
        if (m) CK(cudaMemcpyAsync(g.adj, adj, 2 * (size_t)m * 4, cudaMemcpyHostToDevice, s));
        if (n) {
            CK(cudaMemcpyAsync(g.tri, tri, (size_t)n * 4, cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(g.tri_deg, tri_deg, (size_t)n * 4, cudaMemcpyHostToDevice, s));
        }
    } else {
        CK(cudaMemsetAsync(g.indices, 0, ((size_t)n + 1) * 4, s));
    }
    finish_graph(c);
    c.has_graph = true;
}

}  // namespace scd
