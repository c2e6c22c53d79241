// Triangle counting on a degree-oriented graph: per-vertex triangle counts and
// per-edge "lies on a triangle" flags.
//
// Every undirected edge has one out-slot in the out-list of its lower-ranked
// endpoint.  A triangle {a, b, c} with a -> b, a -> c, b -> c is found once:
// c in out(b) ∩ out(a).  That is all the reference's outputs need
// (src/convert.cpp:290-340): tri[v] = sum of the per-edge counts at v =
// 2 x (triangles at v), and tri_deg[v] and the filter need only whether an
// edge's count is > 0.  So the kernels produce
//   tcount[v]  triangles at v (tri = 2 tcount),
//   flag[slot] 1 if the edge of that out-slot lies on a triangle,
// and never a per-edge counter: the centre's, the partners' and the table
// entries' counts and flags are aggregated in shared memory per work unit; the
// only per-triangle global write is the byte store of the walked slot's flag
// (idempotent, no atomic).  The reference's id-oriented merge is quadratic in
// hub degree; this does sum over a->b of min(d+(a), d+(b)) hash probes.
//
// Which vertex's table counts a triangle: an edge a -> b whose b has the longer
// out-list (d+(a) < d+(b), b in the CTA buckets) is b-centric: instead of
// walking out(b) against a's table, the unit of b walks out(a) against b's
// table (b's in-lists give the a).  Every triangle a -> b -> c is still found
// exactly once, at a's table or at b's.
//
// With labels, only internal triangles count (all three vertices carry the
// same valid label): only partners and table entries with the centre's label
// take part.  (compute_wcc gives the kernels internal out-lists instead, which
// is faster; the label filter stays for callers with whole out-lists.)
//
// Work unit = (vertex a, its out-list whole) for a register group, (a, up to
// 32 consecutive b of out(a)) for one warp, or (centre, up to 512 partners) for
// one CTA when the centre's out-list is long.  The centre's out-list is staged
// in a shared-memory open-addressing table with a one-hash bitmap (>= 16 bits
// per entry) in front, which answers most lookups (misses) with one shared load;
// the unit's items (partner, c in the partner's walk) are flattened with a
// prefix sum; a warp takes 256 consecutive items, lane L every 32nd from L
// (coalesced loads), walking the partner boundaries forward.  Centres are
// grouped by out-degree into buckets so that each kernel's shared memory
// matches its lists.
//
// The preprocessing count takes its upper CTA bucket (out-degree > T, where
// nearly all the work of skewed graphs lies) with an exact bitmap instead of a
// hash table: those centres' out-lists all lie among the vertices of degree >
// T, numbered densely, so a small shared bitmap holds each one (k_tc_core).
// T is the lowest of 64, 128, 256, 512, 1024 whose core has at most 128K
// vertices (R-MAT scale 22: 128; Chung-Lu 8M: 256).
#include "engine.cuh"

namespace scd {

namespace {

constexpr uint32_t EMPTY = 0xffffffffu;
constexpr int ITEMS = 8;   // consecutive items per thread

constexpr uint32_t HASH_MUL = 0x9E3779B1u;   // multiplicative hash: table index = top bits

// a -> b (d+(a), d+(b)) is counted at b's table iff d+(a) < d+(b), lo < d+(b) <= hi
// and d+(a) > amin (amin > 0 keeps short out-lists with the register-group kernel,
// whose binary searches make a long out(b) cheap; which is faster depends on the
// graph, so amin is one of the autotuned splits)
struct Dir {
    uint32_t lo, hi, amin;
    __device__ __forceinline__ bool bcentric(uint32_t da, uint32_t db) const {
        return da < db && da > amin && db > lo && db <= hi;
    }
};

// units of the centres verts[i]: out-list centres (i < nfwd) have d+ partners, in-list centres their in-degree
struct UnitsOf {
    Oriented o;
    const uint32_t *verts;
    uint32_t per_unit, nfwd;
    __device__ uint32_t operator[](size_t i) const {
        const uint32_t v = verts[i], p = i < nfwd ? o.len[v] : o.in_len(v);
        return (p + per_unit - 1) / per_unit;
    }
};

struct InBucket {
    Oriented o;
    uint32_t lo, hi;
    bool in_list;   // in-list centres: also a non-empty in-list
    __device__ uint32_t operator[](size_t v) const {
        return o.len[v] > lo && o.len[v] <= hi && (!in_list || o.in_len((uint32_t)v) > 0);
    }
};

__global__ void k_bucket_scatter(uint32_t n, InBucket f, const uint32_t *__restrict__ pos, uint32_t *out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (f[v]) out[pos[v]] = v;
}

// Short out-lists (d+(a) <= G, G = 16 or 32): one group of G lanes per vertex
// a, no table.  Lane i holds out(a)[i] in a register (out-lists are sorted
// ascending); the (b, c in out(b)) items of a are flattened by a group scan
// and taken G at a time, the owner b of an item and the position of c in
// out(a) are both found by binary search over registers (shuffles).  Per-slot
// hit counts go to a 32-entry shared array per warp: a hit adds one for b and
// one for c, both entries of out(a), and flags the (b, c) slot.  An out(b) at
// least 4x longer than out(a) (a hub's) is not walked: every lane searches its
// out(a) entry in out(b) instead (alen searches of log2 d+(b) steps).
template <int G>
__global__ void __launch_bounds__(256)
k_tc_small(Oriented o, const uint32_t *__restrict__ verts, uint32_t nverts, Dir dir, LabelFilter lf,
           uint32_t *tcount, uint8_t *flag) {
    constexpr int PER_WARP = 32 / G;
    __shared__ uint32_t acc[8][32];
    const uint32_t *labels = lf.labels;
    const int lane = threadIdx.x & 31, gl = lane % G, g0 = lane - gl, w = threadIdx.x >> 5;
    const unsigned gmask = (G == 32) ? FULL : (((1u << G) - 1u) << g0);
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * PER_WARP; base < nverts;
         base += warps * PER_WARP) {
        const uint32_t vi = base + lane / G;
        bool live = vi < nverts;
        const uint32_t a = live ? verts[vi] : 0u;
        uint32_t la = 0;
        if (live && labels) {
            la = labels[a];
            live = la != INVALID && !lf.frozen(a);
        }
        const uint32_t abeg = live ? o.beg[a] : 0u, alen = live ? o.len[a] : 0u;   // alen <= G
        const bool in_a = (uint32_t)gl < alen;
        const uint32_t x = in_a ? o.adj[abeg + gl] : 0xffffffffu;
        const bool ok = in_a && (!labels || labels[x] == la);   // usable as b and as c
        const uint32_t dx = ok ? o.len[x] : 0u;
        const bool walk = ok && !dir.bcentric(alen, dx);        // a -> x is counted here
        const uint32_t wfull = walk ? dx : 0u, bb = walk ? o.beg[x] : 0u;
        // a long out(b) is searched for the entries of out(a) (below) instead of walked
        const bool far = wfull >= 32 && wfull >= 4 * alen;
        const uint32_t wb = far ? 0u : wfull;
        uint32_t incl = wb;
#pragma unroll
        for (int d = 1; d < G; d <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, d, G);
            if (gl >= d) incl += y;
        }
        const uint32_t total = __shfl_sync(FULL, incl, G - 1, G), pre = incl - wb;
        uint32_t tmax = total;
#pragma unroll
        for (int d = G; d < 32; d <<= 1) tmax = max(tmax, __shfl_xor_sync(FULL, tmax, d));
        acc[w][lane] = 0;
        __syncwarp();
        uint32_t hits = 0;
        for (uint32_t t0 = 0; t0 < tmax; t0 += G) {
            const uint32_t t = t0 + gl;
            uint32_t j = 0;   // owner: last lane with pre <= t
#pragma unroll
            for (int st = G / 2; st > 0; st >>= 1)
                if (__shfl_sync(FULL, pre, j + st, G) <= t) j += st;
            const uint32_t bj = __shfl_sync(FULL, bb, j, G), pj = __shfl_sync(FULL, pre, j, G);
            const bool valid = t < total;
            const uint32_t cpos = bj + (t - pj);
            const uint32_t cv = valid ? o.adj[cpos] : 0xffffffffu;
            uint32_t k = 0;   // last entry of out(a) <= c
#pragma unroll
            for (int st = G / 2; st > 0; st >>= 1)
                if (__shfl_sync(FULL, x, k + st, G) <= cv) k += st;
            const uint32_t xk = __shfl_sync(FULL, x, k, G);        // every lane shuffles
            const int okk = __shfl_sync(FULL, (int)ok, k, G);
            const bool hit = valid && xk == cv && okk;
            if (hit) {
                atomicAdd(&acc[w][g0 + j], 1u);
                atomicAdd(&acc[w][g0 + k], 1u);
                flag[cpos] = 1;
                hits++;
            }
        }
        // long out-lists: lane k binary-searches its out(a) entry in out(b), one b at a time
        __syncwarp();
        uint32_t selfc = 0;
        // positions j that hold a far b in some group of the warp (groups search side by side)
        const unsigned fm = __ballot_sync(FULL, far);
        unsigned fpos = 0;
#pragma unroll
        for (int g = 0; g < PER_WARP; g++) fpos |= (G == 32) ? fm : (fm >> (g * G)) & ((1u << G) - 1u);
        for (; fpos; fpos &= fpos - 1) {
            const int j = __ffs(fpos) - 1;
            const bool fj = __shfl_sync(FULL, far, j, G);
            const uint32_t bj = __shfl_sync(FULL, bb, j, G), wj = __shfl_sync(FULL, wfull, j, G);
            bool hit = false;
            uint32_t lo = 0;
            if (fj && ok) {
                uint32_t hi = wj;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (o.adj[bj + mid] < x) lo = mid + 1;
                    else hi = mid;
                }
                hit = lo < wj && o.adj[bj + lo] == x;
            }
            if (hit) {
                flag[bj + lo] = 1;
                selfc++;
                hits++;
            }
            const uint32_t nb = __popc(__ballot_sync(FULL, hit) & gmask);
            if (gl == j && nb) acc[w][lane] += nb;
        }
        __syncwarp();
        const uint32_t hc = acc[w][lane] + selfc;
        if (hc && in_a) {
            atomicAdd(tcount + x, hc);
            flag[abeg + gl] = 1;
        }
#pragma unroll
        for (int d = G / 2; d > 0; d >>= 1) hits += __shfl_xor_sync(FULL, hits, d);
        if (gl == 0 && hits) atomicAdd(tcount + a, hits);
        __syncwarp();
    }
}

// Warp units.  Per warp: table of TCAP (key, index) entries, LCAP counters.
template <int WARPS, int TCAP, int LCAP, int FBITS>
__global__ void __launch_bounds__(WARPS * 32)
k_tc_warp(Oriented o, const uint32_t *__restrict__ verts, const uint32_t *__restrict__ unit_off, uint32_t nverts,
          Dir dir, LabelFilter lf, uint32_t *tcount, uint8_t *flag, uint32_t *next_unit) {
    const uint32_t *labels = lf.labels;
    __shared__ uint32_t filt[WARPS][(1 << FBITS) / 32];
    __shared__ uint32_t keys[WARPS][TCAP];
    __shared__ uint16_t idxs[WARPS][TCAP];
    __shared__ uint32_t cnt[WARPS][LCAP];
    __shared__ uint32_t pre[WARPS][32], bbase[WARPS][32], bhits[WARPS][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t n_units = unit_off[nverts];
    while (true) {
        uint32_t unit = 0;
        if (lane == 0) unit = atomicAdd(next_unit, 1u);
        unit = __shfl_sync(FULL, unit, 0);
        if (unit >= n_units) break;
        uint32_t lo = 0, hi = nverts + 1;   // vertex index: unit_off[i] <= unit < unit_off[i+1]
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (unit_off[mid] <= unit) lo = mid + 1;
            else hi = mid;
        }
        const uint32_t vi = lo - 1;
        const uint32_t a = verts[vi], ch = unit - unit_off[vi];
        const uint32_t la = labels ? labels[a] : 0u;
        if (labels && (la == INVALID || lf.frozen(a))) continue;
        const uint32_t abeg = o.beg[a], alen = o.len[a];
        int bits = 1;
        while ((1u << bits) < 4 * alen) bits++;
        if ((1 << bits) > TCAP) bits = 31 - __clz(TCAP);
        const uint32_t tmask = (1u << bits) - 1;
        for (uint32_t i = lane; i < (1u << bits); i += 32) keys[w][i] = EMPTY;
        for (uint32_t i = lane; i < (1u << FBITS) / 32; i += 32) filt[w][i] = 0;
        for (uint32_t i = lane; i < alen; i += 32) cnt[w][i] = 0;
        __syncwarp();
        for (uint32_t i = lane; i < alen; i += 32) {
            const uint32_t id = o.adj[abeg + i];
            if (labels && labels[id] != la) continue;   // only internal c can close an internal triangle
            const uint32_t hv = id * HASH_MUL, fi = hv >> (32 - FBITS);
            atomicOr(&filt[w][fi >> 5], 1u << (fi & 31));
            uint32_t h = hv >> (32 - bits);
            while (atomicCAS(&keys[w][h], EMPTY, id) != EMPTY) h = (h + 1) & tmask;
            idxs[w][h] = (uint16_t)i;
        }
        __syncwarp();
        const uint32_t j = ch * 32 + lane;
        uint32_t wb = 0, bb = 0, b = 0;
        if (j < alen) {
            b = o.adj[abeg + j];
            const uint32_t db = o.len[b];
            if ((!labels || labels[b] == la) && !dir.bcentric(alen, db)) {
                wb = db;
                bb = o.beg[b];
            }
        }
        const uint32_t incl = warp_inclusive_scan(wb);
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        pre[w][lane] = incl - wb;
        bbase[w][lane] = bb;
        bhits[w][lane] = 0;
        __syncwarp();
        for (uint32_t t0 = 0; t0 < total; t0 += 32 * ITEMS) {
            const uint32_t tl = t0 + lane;   // lane L takes items t0 + L + 32k (coalesced)
            uint32_t l0 = 0, l1 = 32;        // owner lane of tl: last lane with pre <= tl
            while (l0 < l1) {
                const uint32_t mid = (l0 + l1) >> 1;
                if (pre[w][mid] <= tl) l0 = mid + 1;
                else l1 = mid;
            }
            uint32_t jb = l0 - 1;
            uint32_t nxt = jb + 1 < 32 ? pre[w][jb + 1] : total;
            uint32_t cbase = bbase[w][jb] - pre[w][jb];
            uint32_t cpos[ITEMS], cv[ITEMS], own[ITEMS];
#pragma unroll
            for (int k = 0; k < ITEMS; k++) {
                const uint32_t t = tl + 32 * k;
                own[k] = INVALID;
                if (t < total) {
                    while (t >= nxt) {
                        jb++;
                        nxt = jb + 1 < 32 ? pre[w][jb + 1] : total;
                        cbase = bbase[w][jb] - pre[w][jb];
                    }
                    own[k] = jb;
                    cpos[k] = cbase + t;
                    cv[k] = o.adj[cpos[k]];
                }
            }
#pragma unroll
            for (int k = 0; k < ITEMS; k++) {
                if (own[k] == INVALID) continue;
                const uint32_t c = cv[k];
                const uint32_t hv = c * HASH_MUL, fi = hv >> (32 - FBITS);
                if (!((filt[w][fi >> 5] >> (fi & 31)) & 1u)) continue;   // certainly not in out(a)
                uint32_t h = hv >> (32 - bits), key;
                while ((key = keys[w][h]) != c && key != EMPTY) h = (h + 1) & tmask;
                if (key == c) {
                    atomicAdd(&cnt[w][idxs[w][h]], 1u);
                    atomicAdd(&bhits[w][own[k]], 1u);
                    flag[cpos[k]] = 1;
                }
            }
        }
        __syncwarp();
        const uint32_t hb = j < alen ? bhits[w][lane] : 0;
        if (hb) {
            atomicAdd(tcount + b, hb);
            flag[abeg + j] = 1;
        }
        const uint32_t sa = warp_sum(hb);
        if (lane == 0 && sa) atomicAdd(tcount + a, sa);
        for (uint32_t i = lane; i < alen; i += 32) {
            const uint32_t cc = cnt[w][i];
            if (cc) {
                atomicAdd(tcount + o.adj[abeg + i], cc);
                flag[abeg + i] = 1;
            }
        }
        __syncwarp();
    }
}

// CTA units for longer out-lists: (centre x, up to THREADS x ROUNDS partners),
// one shared table of out(x) per CTA, partners THREADS at a time.  Out-list
// centres (vi < nfwd) take the partners b = out(x)[j] of edges x -> b counted at
// x and walk out(b); in-list centres take the a = in(x)[j] of b-centric edges
// a -> x and walk out(a).  A hit c closes the triangle (x, partner, c): the
// walked slot is flagged at once, the partner's and the table entry's counts
// and flags are aggregated in shared memory.  The out-slot of a -> x (in-list
// centre) is found by a binary search of x in out(a), for partners with hits.
//
// The table entries' hit counts are 16-bit halves of shared words (a count is at
// most the unit's THREADS x ROUNDS partners), which with the register bound lets
// MIN_CTAS CTAs share an SM.
template <int THREADS, int ROUNDS, int TCAP, int LCAP, int FBITS, int MIN_CTAS>
__global__ void __launch_bounds__(THREADS, MIN_CTAS)
k_tc_cta(Oriented o, const uint32_t *__restrict__ verts, const uint32_t *__restrict__ unit_off, uint32_t nverts,
         uint32_t nfwd, Dir dir, LabelFilter lf, uint32_t *tcount, uint8_t *flag, uint32_t *next_unit) {
    constexpr uint32_t PER_UNIT = (uint32_t)THREADS * ROUNDS;
    static_assert(PER_UNIT < 65536, "16-bit hit counts");
    const uint32_t *labels = lf.labels;
    extern __shared__ uint32_t sm[];
    uint32_t *keys = sm;                                  // TCAP
    uint32_t *cnt = sm + TCAP;                            // LCAP 16-bit counts
    uint32_t *filt = sm + TCAP + LCAP / 2;                // 2^FBITS bits
    uint16_t *idxs = (uint16_t *)(filt + (1 << FBITS) / 32);   // TCAP
    __shared__ uint32_t pre[THREADS], bbase[THREADS], bhits[THREADS], wsum[THREADS / 32];
    __shared__ uint32_t s_unit, s_total;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t n_units = unit_off[nverts];
    while (true) {
        if (threadIdx.x == 0) s_unit = atomicAdd(next_unit, 1u);
        __syncthreads();
        const uint32_t unit = s_unit;
        if (unit >= n_units) break;
        uint32_t lo = 0, hi = nverts + 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (unit_off[mid] <= unit) lo = mid + 1;
            else hi = mid;
        }
        const uint32_t vi = lo - 1;
        const uint32_t x = verts[vi], ch = unit - unit_off[vi];
        const bool fwd = vi < nfwd;
        const uint32_t la = labels ? labels[x] : 0u;
        if (labels && (la == INVALID || lf.frozen(x))) {
            __syncthreads();
            continue;
        }
        const uint32_t xbeg = o.beg[x], xlen = o.len[x];
        int bits = 1;
        while ((1u << bits) < 2 * xlen) bits++;
        const uint32_t tmask = (1u << bits) - 1;
        for (uint32_t i = threadIdx.x; i < (1u << bits); i += THREADS) keys[i] = EMPTY;
        for (uint32_t i = threadIdx.x; i < (1u << FBITS) / 32; i += THREADS) filt[i] = 0;
        for (uint32_t i = threadIdx.x; i < (xlen + 1) / 2; i += THREADS) cnt[i] = 0;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < xlen; i += THREADS) {
            const uint32_t id = o.adj[xbeg + i];
            if (labels && labels[id] != la) continue;   // only internal c can close an internal triangle
            const uint32_t hv = id * HASH_MUL, fi = hv >> (32 - FBITS);
            atomicOr(&filt[fi >> 5], 1u << (fi & 31));
            uint32_t h = hv >> (32 - bits);
            while (atomicCAS(&keys[h], EMPTY, id) != EMPTY) h = (h + 1) & tmask;
            idxs[h] = (uint16_t)i;
        }
        const uint32_t *padj = fwd ? o.adj : o.in_adj();
        const uint32_t pbeg = fwd ? xbeg : o.in_beg(x), plen = fwd ? xlen : o.in_len(x);
        const uint32_t pend = min(plen, (ch + 1) * PER_UNIT);
        uint32_t xhits = 0;
        for (uint32_t r0 = ch * PER_UNIT; r0 < pend; r0 += THREADS) {
            const uint32_t j = r0 + threadIdx.x;
            uint32_t wb = 0, bb = 0, y = 0;
            if (j < pend) {
                y = padj[pbeg + j];
                const uint32_t dy = o.len[y];
                const bool here = fwd ? !dir.bcentric(xlen, dy) : dir.bcentric(dy, xlen);
                if (here && (!labels || labels[y] == la)) {
                    wb = dy;
                    bb = o.beg[y];
                }
            }
            uint32_t incl = warp_inclusive_scan(wb);   // block inclusive scan of wb
            if (lane == 31) wsum[w] = incl;
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t run = 0;
                for (int k = 0; k < THREADS / 32; k++) {
                    const uint32_t v = wsum[k];
                    wsum[k] = run;
                    run += v;
                }
                s_total = run;
            }
            __syncthreads();
            incl += wsum[w];
            pre[threadIdx.x] = incl - wb;
            bbase[threadIdx.x] = bb;
            bhits[threadIdx.x] = 0;
            const uint32_t total = s_total;
            __syncthreads();
            // warp chunks of 32*ITEMS consecutive items; lane L takes items chunk + L + 32k
            // (coalesced loads) and walks the owner boundaries forward
            for (uint32_t t0 = (uint32_t)w * 32 * ITEMS; t0 < total; t0 += THREADS * ITEMS) {
                const uint32_t tl = t0 + lane;
                uint32_t l0 = 0, l1 = THREADS;   // owner of tl: last thread with pre <= tl
                while (l0 < l1) {
                    const uint32_t mid = (l0 + l1) >> 1;
                    if (pre[mid] <= tl) l0 = mid + 1;
                    else l1 = mid;
                }
                uint32_t jb = l0 - 1;
                uint32_t nxt = jb + 1 < THREADS ? pre[jb + 1] : total;
                uint32_t cbase = bbase[jb] - pre[jb];
                uint32_t cpos[ITEMS], cv[ITEMS], own[ITEMS];
#pragma unroll
                for (int k = 0; k < ITEMS; k++) {
                    const uint32_t t = tl + 32 * k;
                    own[k] = INVALID;
                    if (t < total) {
                        while (t >= nxt) {
                            jb++;
                            nxt = jb + 1 < THREADS ? pre[jb + 1] : total;
                            cbase = bbase[jb] - pre[jb];
                        }
                        own[k] = jb;
                        cpos[k] = cbase + t;
                        cv[k] = o.adj[cpos[k]];
                    }
                }
#pragma unroll
                for (int k = 0; k < ITEMS; k++) {
                    if (own[k] == INVALID) continue;
                    const uint32_t c = cv[k];
                    const uint32_t hv = c * HASH_MUL, fi = hv >> (32 - FBITS);
                    if (!((filt[fi >> 5] >> (fi & 31)) & 1u)) continue;   // certainly not in out(x)
                    uint32_t h = hv >> (32 - bits), key;
                    while ((key = keys[h]) != c && key != EMPTY) h = (h + 1) & tmask;
                    if (key == c) {
                        const uint32_t ic = idxs[h];
                        atomicAdd(&cnt[ic >> 1], 1u << ((ic & 1) << 4));
                        atomicAdd(&bhits[own[k]], 1u);
                        flag[cpos[k]] = 1;
                    }
                }
            }
            __syncthreads();
            const uint32_t hb = j < pend ? bhits[threadIdx.x] : 0;
            if (hb) {
                atomicAdd(tcount + y, hb);
                const uint32_t yb = o.beg[y];
                flag[fwd ? xbeg + j : yb + lower_bound(o.adj + yb, o.len[y], x)] = 1;
            }
            xhits += hb;
        }
        const uint32_t sa = warp_sum(xhits);
        if (lane == 0 && sa) atomicAdd(tcount + x, sa);
        for (uint32_t i = threadIdx.x; i < xlen; i += THREADS) {
            const uint32_t cc = (cnt[i >> 1] >> ((i & 1) << 4)) & 0xffffu;
            if (cc) {
                atomicAdd(tcount + o.adj[xbeg + i], cc);
                flag[xbeg + i] = 1;
            }
        }
        __syncthreads();
    }
}

template <int TCAP, int LCAP, int FBITS>
constexpr size_t tc_cta_smem() {
    return (size_t)TCAP * 4 + (size_t)LCAP * 2 + ((size_t)1 << FBITS) / 8 + (size_t)TCAP * 2;
}

template <int THREADS, int ROUNDS, int TCAP, int LCAP, int FBITS, int MIN_CTAS>
void set_tc_attr() {
    if (tc_cta_smem<TCAP, LCAP, FBITS>() > 48 * 1024)
        CK(cudaFuncSetAttribute((const void *)k_tc_cta<THREADS, ROUNDS, TCAP, LCAP, FBITS, MIN_CTAS>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_cta_smem<TCAP, LCAP, FBITS>()));
}

template <int THREADS, int ROUNDS, int TCAP, int LCAP, int FBITS, int MIN_CTAS>
void launch_tc_cta(const Oriented &o, const TcPlan &plan, int k, LabelFilter labels, uint32_t *tcount,
                   uint8_t *flag, uint32_t *ctr, unsigned grid, cudaStream_t s) {
    const size_t smem = tc_cta_smem<TCAP, LCAP, FBITS>();
    k_tc_cta<THREADS, ROUNDS, TCAP, LCAP, FBITS, MIN_CTAS><<<grid, THREADS, smem, s>>>(
        o, plan.verts[k], plan.unit_off[k], plan.nverts[k], plan.nfwd[k], Dir{plan.dir_lo, plan.dir_hi, plan.dir_amin},
        labels, tcount, flag, ctr);
    CK_LAUNCH("k_tc_cta");
}

// partners per CTA unit of the two CTA buckets
constexpr int CTA1_THREADS = 128, CTA1_ROUNDS = 4, CTA2_THREADS = 256, CTA2_ROUNDS = 2;

// CTA units of the upper CTA bucket (out-degree in (cta_hi, 8192]) over a core
// bitmap, when the plan has a core map and no labels filter.  Every out-list
// of such a centre lies in the core, the vertices of degree > cta_hi (their
// degrees are at least the centre's), so the centre's out-list in core numbers
// is held exactly by a shared bitmap of core_n bits (plus the outside marker
// core_n, never set).  pre[w] is the out-list position of the first member in
// bitmap word w; core numbers ascend with ids, so the position of a member c
// is pre[c/32] + the popcount of the word's bits below c.  A lookup is one
// shared load and a bit test: no hash, no probe sequence, no false positives.
// The core of the upper bucket is small (R-MAT scale 22: 110,575 vertices of
// degree > 128, a 13.5 KB bitmap), so many CTAs share an SM.
//
// The walk: THREADS partners per round; every list in the core-number array
// starts on a 16-byte boundary and is padded with core_n to whole quads, the
// quads of the round are flattened by a block scan, and a warp takes 32 x K
// consecutive quads of its own contiguous range, lane L every 32nd (one 16-byte
// load each: 4K items of a lane in flight).  A hit flags the walked slot at
// once and counts in the member's shared count and, per quad, in the partner's.
template <int THREADS, int K>
__global__ void __launch_bounds__(THREADS, 6)
k_tc_core(Oriented o, const uint32_t *__restrict__ cpad, const uint32_t *__restrict__ cbeg, uint32_t core_n,
          uint32_t kwords, uint32_t lcap, const uint32_t *__restrict__ verts, const uint32_t *__restrict__ unit_off,
          uint32_t nverts, uint32_t nfwd, uint32_t per_unit, Dir dir, uint32_t *tcount, uint8_t *flag,
          uint32_t *next_unit) {
    extern __shared__ __align__(16) uint32_t sm[];
    uint32_t *bm = sm;                           // kwords
    uint32_t *cnt = bm + kwords;                 // lcap hit counts of the centre's members
    uint16_t *pre = (uint16_t *)(cnt + lcap);    // kwords
    __shared__ uint32_t qpre[THREADS], sq0[THREADS], sdl[THREADS], sh[THREADS], wsum[THREADS / 32];
    __shared__ uint32_t s_unit, s_total, s_xhits;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint4 *cq = reinterpret_cast<const uint4 *>(cpad);
    for (uint32_t i = threadIdx.x; i < kwords; i += THREADS) bm[i] = 0;
    const uint32_t n_units = unit_off[nverts];
    while (true) {
        if (threadIdx.x == 0) {
            s_unit = atomicAdd(next_unit, 1u);
            s_xhits = 0;
        }
        __syncthreads();
        const uint32_t unit = s_unit;
        if (unit >= n_units) break;
        uint32_t lo = 0, hi = nverts + 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (unit_off[mid] <= unit) lo = mid + 1;
            else hi = mid;
        }
        const uint32_t vi = lo - 1;
        const uint32_t x = verts[vi], ch = unit - unit_off[vi];
        const bool fwd = vi < nfwd;
        const uint32_t xbeg = o.beg[x], xlen = o.len[x];
        const uint32_t *xc = cpad + cbeg[x];
        for (uint32_t i = threadIdx.x; i < xlen; i += THREADS) {
            const uint32_t c = xc[i];
            if (c < core_n) {
                atomicOr(&bm[c >> 5], 1u << (c & 31));
                if (i == 0 || (xc[i - 1] >> 5) != (c >> 5)) pre[c >> 5] = (uint16_t)i;
            }
        }
        for (uint32_t i = threadIdx.x; i < xlen; i += THREADS) cnt[i] = 0;
        const uint32_t *padj = fwd ? o.adj : o.in_adj();
        const uint32_t pbeg = fwd ? xbeg : o.in_beg(x), plen = fwd ? xlen : o.in_len(x);
        const uint32_t pend = min(plen, (ch + 1) * per_unit);
        uint32_t xh = 0;
        for (uint32_t r0 = ch * per_unit; r0 < pend; r0 += THREADS) {
            const uint32_t j = r0 + threadIdx.x;
            uint32_t y = 0, wb = 0, cb = 0, ob = 0;
            if (j < pend) {
                y = padj[pbeg + j];
                const uint32_t dy = o.len[y];
                if (fwd ? !dir.bcentric(xlen, dy) : dir.bcentric(dy, xlen)) {
                    wb = dy;
                    cb = cbeg[y];
                    ob = o.beg[y];
                }
            }
            const uint32_t nq = (wb + 3) >> 2;
            uint32_t incl = warp_inclusive_scan(nq);   // block scan of the quad counts
            if (lane == 31) wsum[w] = incl;
            __syncthreads();   // also orders the bitmap build before the walk
            if (threadIdx.x == 0) {
                uint32_t run = 0;
                for (int k = 0; k < THREADS / 32; k++) {
                    const uint32_t v = wsum[k];
                    wsum[k] = run;
                    run += v;
                }
                s_total = run;
            }
            __syncthreads();
            qpre[threadIdx.x] = incl + wsum[w] - nq;
            sq0[threadIdx.x] = cb >> 2;
            sdl[threadIdx.x] = ob - cb;   // core-array position -> out-slot (mod 2^32)
            sh[threadIdx.x] = 0;
            const uint32_t total = s_total;
            __syncthreads();
            // warp w walks its own contiguous range of the round's quads, 32 x K at a
            // time (lane L every 32nd: coalesced); each lane finds the owner of its first
            // quad once and then only walks the partner boundaries forward
            const uint32_t wbeg = (uint32_t)(((uint64_t)total * w) / (THREADS / 32));
            const uint32_t wend = (uint32_t)(((uint64_t)total * (w + 1)) / (THREADS / 32));
            uint32_t jb = 0, nxt = 0;
            if (wbeg + lane < wend) {
                uint32_t l0 = 0, l1 = THREADS;   // owner: last partner with qpre <= the quad
                while (l0 < l1) {
                    const uint32_t mid = (l0 + l1) >> 1;
                    if (qpre[mid] <= wbeg + lane) l0 = mid + 1;
                    else l1 = mid;
                }
                jb = l0 - 1;
                nxt = jb + 1 < THREADS ? qpre[jb + 1] : total;
            }
            for (uint32_t t0 = wbeg; t0 < wend; t0 += 32 * K) {
                uint4 v[K];
                uint32_t qa[K], own[K];
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const uint32_t t = t0 + lane + 32 * k;
                    own[k] = INVALID;
                    if (t < wend) {
                        while (t >= nxt) {
                            jb++;
                            nxt = jb + 1 < THREADS ? qpre[jb + 1] : total;
                        }
                        own[k] = jb;
                        qa[k] = sq0[jb] + (t - qpre[jb]);
                        v[k] = __ldg(cq + qa[k]);
                    }
                }
#pragma unroll
                for (int k = 0; k < K; k++) {
                    if (own[k] == INVALID) continue;
                    const uint32_t fo = qa[k] * 4 + sdl[own[k]];
                    const uint32_t vals[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
                    uint32_t h = 0;
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const uint32_t c = vals[e], wd = bm[c >> 5], bit = c & 31;
                        if ((wd >> bit) & 1u) {
                            const uint32_t r = pre[c >> 5] + __popc(wd & ((1u << bit) - 1u));
                            if (r < xlen) atomicAdd(&cnt[r], 1u);
                            flag[fo + e] = 1;
                            h++;
                        }
                    }
                    if (h) atomicAdd(&sh[own[k]], h);
                }
            }
            __syncthreads();
            const uint32_t hb = j < pend ? sh[threadIdx.x] : 0u;
            if (hb) {
                atomicAdd(tcount + y, hb);
                flag[fwd ? xbeg + j : ob + lower_bound(o.adj + ob, wb, x)] = 1;
                xh += hb;
            }
        }
        xh = warp_sum(xh);
        if (lane == 0 && xh) atomicAdd(&s_xhits, xh);
        __syncthreads();
        if (threadIdx.x == 0 && s_xhits) atomicAdd(tcount + x, s_xhits);
        const uint32_t *xa = o.adj + xbeg;
        for (uint32_t i = threadIdx.x; i < xlen; i += THREADS) {
            const uint32_t cc = cnt[i];
            if (cc) {
                atomicAdd(tcount + xa[i], cc);
                flag[xbeg + i] = 1;
            }
            const uint32_t c = xc[i];
            if (c < core_n) bm[c >> 5] = 0;
        }
        __syncthreads();
    }
}

constexpr int CORE_THREADS = 256, CORE_K = 2;
constexpr size_t CORE_SMEM_MAX = 200 * 1024;   // below the 227 KB opt-in limit with the static part
// core size (vertices) whose bitmap and position table (24 KB) leave room for six CTAs per SM
constexpr uint32_t CORE_BUDGET = 128 * 1024;

inline size_t tc_core_smem(uint32_t kwords, uint32_t lcap) {
    return (size_t)kwords * 4 + (size_t)lcap * 4 + ((size_t)kwords * 2 + 3) / 4 * 4;
}

void launch_tc_core(const Oriented &o, const TcPlan &plan, int k, uint32_t lcap, uint32_t *tcount, uint8_t *flag,
                    uint32_t *ctr, cudaStream_t s) {
    const uint32_t kwords = plan.core_n / 32 + 1;
    const size_t smem = tc_core_smem(kwords, lcap);
    const void *fn = (const void *)k_tc_core<CORE_THREADS, CORE_K>;
    int dev = 0, per_sm = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, CORE_THREADS, smem));
    if (per_sm < 1) throw Error(SCD_ERR_CUDA, "core triangle-count kernel does not fit an SM");
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    k_tc_core<CORE_THREADS, CORE_K><<<sms * per_sm, CORE_THREADS, smem, s>>>(
        o, plan.core_adj, plan.core_beg, plan.core_n, kwords, lcap, plan.verts[k], plan.unit_off[k], plan.nverts[k],
        plan.nfwd[k], CTA2_THREADS * CTA2_ROUNDS, Dir{plan.dir_lo, plan.dir_hi, plan.dir_amin}, tcount, flag, ctr);
    CK_LAUNCH("k_tc_core");
}

// Lists longer than 8192 (none in the benchmark graphs): items looked up
// by binary search in the sorted out-list in global memory, per-triangle
// atomics.  Kept for generality.
__global__ void __launch_bounds__(256)
k_tc_huge(Oriented o, const uint32_t *__restrict__ verts, uint32_t nverts, LabelFilter lf, uint32_t *tcount,
          uint8_t *flag) {
    const uint32_t *labels = lf.labels;
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t vi = 0; vi < nverts; vi++) {
        const uint32_t a = verts[vi];
        const uint32_t la = labels ? labels[a] : 0u;
        if (labels && (la == INVALID || lf.frozen(a))) continue;
        const uint32_t abeg = o.beg[a], alen = o.len[a];
        const uint32_t *A = o.adj + abeg;
        for (uint32_t j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < alen; j += warps) {
            const uint32_t b = A[j];
            if (labels && labels[b] != la) continue;
            const uint32_t bbeg = o.beg[b], blen = o.len[b];
            uint32_t hits = 0;
            for (uint32_t i = lane; i < blen; i += 32) {
                const uint32_t c = o.adj[bbeg + i];
                const uint32_t ic = lower_bound(A, alen, c);
                if (ic < alen && A[ic] == c && (!labels || labels[c] == la)) {
                    hits++;
                    atomicAdd(tcount + c, 1u);
                    flag[abeg + ic] = 1;
                    flag[bbeg + i] = 1;
                }
            }
            hits = warp_sum(hits);
            if (lane == 0 && hits) {
                atomicAdd(tcount + a, hits);
                atomicAdd(tcount + b, hits);
                flag[abeg + j] = 1;
            }
        }
    }
}

// out-degree buckets: (0,16] and (16,S] register groups (S = 0, 16 or 32), (S,B0] warp
// units, (B0,B1] and (B1,8192] CTA units, > 8192 fallback; B0 <= 64 and B1 <= 1024
// (the kernels' shared-memory capacities); S, B0, B1 tuned per context
constexpr uint32_t B2 = 8192;


// v lies in the core: symmetric degree above the CTA buckets' lower bound
struct CoreFlag {
    Oriented o;
    uint32_t bound;
    __device__ uint32_t operator[](size_t v) const { return o.len[v] + o.in_len((uint32_t)v) > bound; }
};

// for the candidate core bounds t[j]: cnt[j] = vertices of symmetric degree
// > t[j] (the core), cnt[K + j] = the largest out-degree in (t[j], 8192] (the
// upper CTA bucket's longest out-list, which sizes the per-member counts)
struct CoreBounds {
    static constexpr int K = 5;
    uint32_t t[K];
};
__global__ void k_core_counts(Oriented o, CoreBounds cb, uint32_t *cnt) {
    uint32_t m[CoreBounds::K] = {}, mx[CoreBounds::K] = {};
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < o.n; v += gridDim.x * blockDim.x) {
        const uint32_t len = o.len[v], d = len + o.in_len(v);
#pragma unroll
        for (int j = 0; j < CoreBounds::K; j++) {
            m[j] += d > cb.t[j];
            if (len > cb.t[j] && len <= 8192u) mx[j] = max(mx[j], len);
        }
    }
#pragma unroll
    for (int j = 0; j < CoreBounds::K; j++) {
        uint32_t t = warp_sum(m[j]), x = mx[j];
        for (int d = 16; d > 0; d >>= 1) x = max(x, __shfl_xor_sync(FULL, x, d));
        if ((threadIdx.x & 31) == 0) {
            if (t) atomicAdd(cnt + j, t);
            if (x) atomicMax(cnt + CoreBounds::K + j, x);
        }
    }
}

// padded list length: every list starts on a 16-byte boundary
struct PadLen {
    const uint32_t *len;
    __device__ uint32_t operator[](size_t v) const { return (len[v] + 3u) & ~3u; }
};

// v's out-list in core numbers (core_n: outside the core) at cpad[cbeg[v]..],
// padded with core_n to a multiple of 4; one warp per vertex
__global__ void k_core_pad(Oriented o, const uint32_t *__restrict__ cpos, uint32_t core_n,
                           const uint32_t *__restrict__ cbeg, uint32_t *cpad) {
    const uint32_t lane = threadIdx.x & 31, warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < o.n; v += warps) {
        const uint32_t len = o.len[v], b = o.beg[v], d = cbeg[v], plen = (len + 3u) & ~3u;
        for (uint32_t i = lane; i < plen; i += 32) {
            uint32_t c = core_n;
            if (i < len) {
                const uint32_t u = o.adj[b + i], a = cpos[u];
                if (cpos[u + 1] > a) c = a;
            }
            cpad[d + i] = c;
        }
    }
}

}  // namespace

void tc_plan(Ctx &c, const Oriented &o, TcPlan &plan, cudaStream_t s, bool owned, bool in_lists, uint32_t core_from) {
    const uint32_t sm = c.tc_small, s16 = sm < 16 ? sm : 16, s8 = sm < 8 ? sm : 8, b0 = c.tc_b0 > sm ? c.tc_b0 : sm;
    // the core-bitmap kernel takes the upper CTA bucket from core_from on; the hash
    // kernels' upper bucket (one CTA per SM, 16K-entry tables) from tc_b1 on
    const uint32_t b1 = core_from ? (core_from > b0 ? core_from : b0) : c.tc_b1;
    const uint32_t bounds[TcPlan::K + 1] = {0, s8, s16, sm, b0, b1, B2, 0xffffffffu};
    const uint32_t per_unit[TcPlan::K] = {1, 1, 1, 32, CTA1_THREADS * CTA1_ROUNDS, CTA2_THREADS * CTA2_ROUNDS, 1};
    const bool split = in_lists && !(c.flags & SCD_FLAG_TC_OUT_ONLY);
    plan.dir_lo = split ? b0 : 0;
    plan.dir_hi = split ? B2 : 0;
    plan.dir_amin = c.tc_amin < sm ? c.tc_amin : sm;
    plan.cta_lo = b0;
    plan.cta_hi = b1;
    // every bucket's scans first, then one host read of all the counts
    DevBuf<uint32_t> pos[TcPlan::K], ipos[TcPlan::K], counts(2 * TcPlan::K, s);
    for (int k = 0; k < TcPlan::K; k++) {
        const bool cta = k == 4 || k == 5;
        pos[k].alloc((size_t)o.n + 1, s);
        scan_exclusive<uint32_t>(InBucket{o, bounds[k], bounds[k + 1], false}, pos[k].get(), o.n, s);
        CK(cudaMemcpyAsync(counts.get() + 2 * k, pos[k].get() + o.n, 4, cudaMemcpyDeviceToDevice, s));
        if (split && cta) {
            ipos[k].alloc((size_t)o.n + 1, s);
            scan_exclusive<uint32_t>(InBucket{o, bounds[k], bounds[k + 1], true}, ipos[k].get(), o.n, s);
            CK(cudaMemcpyAsync(counts.get() + 2 * k + 1, ipos[k].get() + o.n, 4, cudaMemcpyDeviceToDevice, s));
        } else {
            CK(cudaMemsetAsync(counts.get() + 2 * k + 1, 0, 4, s));
        }
    }
    uint32_t cnts[2 * TcPlan::K];
    CK(cudaMemcpyAsync(cnts, counts.get(), sizeof cnts, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int k = 0; k < TcPlan::K; k++) {
        const InBucket fa{o, bounds[k], bounds[k + 1], false}, fb{o, bounds[k], bounds[k + 1], true};
        const uint32_t na = cnts[2 * k], nb = cnts[2 * k + 1], cnt = na + nb;
        plan.nverts[k] = cnt;
        plan.nfwd[k] = na;
        if (owned) {
            plan.verts[k] = c.alloc<uint32_t>(cnt);
            plan.unit_off[k] = c.alloc<uint32_t>((size_t)cnt + 1);
        } else {
            plan.tmp[2 * k].alloc(cnt ? cnt : 1, s);
            plan.tmp[2 * k + 1].alloc((size_t)cnt + 1, s);
            plan.verts[k] = plan.tmp[2 * k].get();
            plan.unit_off[k] = plan.tmp[2 * k + 1].get();
        }
        if (na) {
            k_bucket_scatter<<<grid_for(o.n, 256), 256, 0, s>>>(o.n, fa, pos[k].get(), plan.verts[k]);
            CK_LAUNCH("k_bucket_scatter");
        }
        if (nb) {
            k_bucket_scatter<<<grid_for(o.n, 256), 256, 0, s>>>(o.n, fb, ipos[k].get(), plan.verts[k] + na);
            CK_LAUNCH("k_bucket_scatter");
        }
        scan_exclusive<uint32_t>(UnitsOf{o, plan.verts[k], per_unit[k], na}, plan.unit_off[k], cnt, s);
    }
}

void tc_core_map(Ctx &c, const Oriented &o, uint64_t slots, TcPlan &plan, uint32_t core_n, uint32_t lcap,
                 cudaStream_t s) {
    plan.core_adj = plan.core_beg = nullptr;
    plan.core_n = plan.core_lcap = 0;
    if (o.n == 0 || plan.nverts[5] == 0) return;
    const uint64_t padded = slots + 3ull * o.n;   // at most: every list padded by three
    if (padded >= 0xffffffffull) return;          // the padded layout is indexed in 32 bits
    DevBuf<uint32_t> cpos((size_t)o.n + 1, s);
    plan.core_beg_buf.alloc((size_t)o.n + 1, s);
    plan.core_buf.alloc((size_t)padded + 4, s);
    scan_exclusive<uint32_t>(CoreFlag{o, plan.cta_hi}, cpos.get(), o.n, s);
    scan_exclusive<uint32_t>(PadLen{o.len}, plan.core_beg_buf.get(), o.n, s);
    k_core_pad<<<grid_for((uint64_t)o.n * 32, 256, 152 * 16), 256, 0, s>>>(o, cpos.get(), core_n,
                                                                           plan.core_beg_buf.get(), plan.core_buf.get());
    CK_LAUNCH("k_core_pad");
    c.launches++;
    plan.core_adj = plan.core_buf.get();
    plan.core_beg = plan.core_beg_buf.get();
    plan.core_n = core_n;
    plan.core_lcap = (lcap + 1) & ~1u;
}

void tc_plan_counting(Ctx &c, const Oriented &o, uint64_t slots, TcPlan &plan, cudaStream_t s) {
    if (c.flags & SCD_FLAG_TC_HASH || o.n == 0) {
        tc_plan(c, o, plan, s, false, true);
        return;
    }
    // the core kernel starts at the lowest candidate bound whose core fits the
    // bitmap budget (many CTAs per SM), else at the lowest one that fits at all
    const uint32_t b0 = c.tc_b0 > c.tc_small ? c.tc_b0 : c.tc_small;
    constexpr int K = CoreBounds::K;
    if (o.n <= CORE_BUDGET) {   // every core fits the budget: the lowest split, no host read
        tc_plan(c, o, plan, s, false, true, b0);
        tc_core_map(c, o, slots, plan, o.n, B2, s);   // core_n <= n; counts sized for the cap
        if (plan.core_n || !plan.nverts[5]) return;
        plan = TcPlan();
        tc_plan(c, o, plan, s, false, true);
        return;
    }
    CoreBounds cb{};
    const uint32_t cand[K] = {b0, 128, 256, 512, 1024};
    for (int j = 0; j < K; j++) cb.t[j] = cand[j] > b0 ? cand[j] : b0;
    DevBuf<uint32_t> cnt(2 * K, s);
    CK(cudaMemsetAsync(cnt.get(), 0, 8 * K, s));
    k_core_counts<<<grid_for(o.n, 256, 152 * 8), 256, 0, s>>>(o, cb, cnt.get());
    CK_LAUNCH("k_core_counts");
    c.launches++;
    uint32_t *h = c.host_u32 + 2;   // pinned planning words
    CK(cudaMemcpyAsync(h, cnt.get(), 8 * K, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    int pick = -1;
    for (int j = 0; j < K && pick < 0; j++)
        if (h[j] <= CORE_BUDGET) pick = j;
    for (int j = 0; j < K && pick < 0; j++)
        if (tc_core_smem(h[j] / 32 + 1, h[K + j]) <= CORE_SMEM_MAX) pick = j;
    if (pick >= 0) {
        const uint32_t core_n = h[pick], lcap = h[K + pick];
        tc_plan(c, o, plan, s, false, true, cb.t[pick]);
        tc_core_map(c, o, slots, plan, core_n, lcap, s);
        if (plan.core_n || !plan.nverts[5]) return;
        plan = TcPlan();
    }
    tc_plan(c, o, plan, s, false, true);   // no map: the hash kernels' split
}

void prepare_tc_kernels() {
    static thread_local int done_device = -1;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (done_device == dev) return;
    set_tc_attr<CTA1_THREADS, CTA1_ROUNDS, 2048, 1024, 14, 12>();
    set_tc_attr<CTA2_THREADS, CTA2_ROUNDS, 16384, 8192, 17, 1>();
    // no carveout preference: the driver's split keeps L1 for the list loads (a
    // maximal shared-memory carveout made the kernel 17 % slower on R-MAT-22)
    CK(cudaFuncSetAttribute((const void *)k_tc_core<CORE_THREADS, CORE_K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)CORE_SMEM_MAX));
    done_device = dev;
}

double autotune_tc(Ctx &c, std::vector<std::string> *report) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    if (!c.has_graph || g.n == 0) return 0.0;
    const Oriented o{g.indices, g.nlow, g.adj, g.n};
    DevBuf<uint32_t> tcount(g.n, s);
    DevBuf<uint8_t> flag(2 * (size_t)g.m + 1, s);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const uint32_t sms[] = {0, 16, 32}, b0s[] = {16, 32, 64}, b1s[] = {256, 512, 1024}, amins[] = {0, 16, 32};
    const uint32_t cur_s = c.tc_small, cur0 = c.tc_b0, cur1 = c.tc_b1, cur_a = c.tc_amin;
    double best = 1e300, cur_ms = 1e300;
    uint32_t best_s = cur_s, best0 = cur0, best1 = cur1, best_a = cur_a;
    for (uint32_t sm : sms)
        for (uint32_t b0 : b0s)
            for (uint32_t b1 : b1s)
                for (uint32_t am : amins) {
                    if (b0 < sm) continue;   // (S, B0] would be empty: same plan as B0 = S
                    if (am > sm) continue;   // same plan as am = S
                    c.tc_small = sm;
                    c.tc_b0 = b0;
                    c.tc_b1 = b1;
                    c.tc_amin = am;
                    TcPlan plan;
                    tc_plan(c, o, plan, s, false, true);
                    double ms_min = 1e300;
                    for (int rep = 0; rep < 2; rep++) {
                        CK(cudaMemsetAsync(tcount.get(), 0, (size_t)g.n * 4, s));
                        CK(cudaMemsetAsync(flag.get(), 0, 2 * (size_t)g.m, s));
                        CK(cudaEventRecord(e0, s));
                        count_triangles(c, o, plan, LabelFilter{}, tcount.get(), flag.get(), s);
                        CK(cudaEventRecord(e1, s));
                        CK(cudaEventSynchronize(e1));
                        float ms = 0;
                        CK(cudaEventElapsedTime(&ms, e0, e1));
                        ms_min = ms < ms_min ? ms : ms_min;
                    }
                    if (report) {
                        char buf[112];
                        snprintf(buf, sizeof buf, "small<=%u warp<=%u cta<=%u in-list>%u: %.3f ms", sm, b0, b1, am,
                                 ms_min);
                        report->push_back(buf);
                    }
                    if (sm == cur_s && b0 == cur0 && b1 == cur1 && am == cur_a) cur_ms = ms_min;
                    if (ms_min < best) {
                        best = ms_min;
                        best_s = sm;
                        best0 = b0;
                        best1 = b1;
                        best_a = am;
                    }
                }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // keep the current split unless another is clearly faster: single timings of a
    // few milliseconds are noisy, and a noise-driven pick can cost more than it gains
    if (best > 0.95 * cur_ms) {
        best = cur_ms;
        best_s = cur_s;
        best0 = cur0;
        best1 = cur1;
        best_a = cur_a;
    }
    c.tc_small = best_s;
    c.tc_b0 = best0;
    c.tc_b1 = best1;
    c.tc_amin = best_a;
    return best;
}

void count_triangles(Ctx &c, const Oriented &o, const TcPlan &plan, LabelFilter labels, uint32_t *tcount,
                     uint8_t *flag, cudaStream_t s, const char *phase) {
    if (o.n == 0) return;
    PhaseScope ph(c, phase ? phase : labels.labels ? "wcc_tc" : "tc");
    prepare_tc_kernels();
    uint32_t *ctr = c.work_counter;
    CK(cudaMemsetAsync(ctr, 0, 16, s));
    const Dir dir{plan.dir_lo, plan.dir_hi, plan.dir_amin};
    const bool core = plan.nverts[5] && plan.core_n && !labels.labels;
    if (plan.nverts[0]) {
        k_tc_small<8><<<grid_for((uint64_t)plan.nverts[0] * 8, 256, 152 * 8), 256, 0, s>>>(
            o, plan.verts[0], plan.nverts[0], dir, labels, tcount, flag);
        CK_LAUNCH("k_tc_small8");
        c.launches++;
    }
    if (plan.nverts[1]) {
        k_tc_small<16><<<grid_for((uint64_t)plan.nverts[1] * 16, 256, 152 * 8), 256, 0, s>>>(
            o, plan.verts[1], plan.nverts[1], dir, labels, tcount, flag);
        CK_LAUNCH("k_tc_small16");
        c.launches++;
    }
    if (plan.nverts[2]) {
        k_tc_small<32><<<grid_for((uint64_t)plan.nverts[2] * 32, 256, 152 * 8), 256, 0, s>>>(
            o, plan.verts[2], plan.nverts[2], dir, labels, tcount, flag);
        CK_LAUNCH("k_tc_small32");
        c.launches++;
    }
    if (plan.nverts[3]) {
        k_tc_warp<16, 256, 64, 10><<<152 * 4, 16 * 32, 0, s>>>(o, plan.verts[3], plan.unit_off[3], plan.nverts[3],
                                                           dir, labels, tcount, flag, ctr);
        CK_LAUNCH("k_tc_warp64");
        c.launches++;
    }
    if (plan.nverts[4]) {
        launch_tc_cta<CTA1_THREADS, CTA1_ROUNDS, 2048, 1024, 14, 12>(o, plan, 4, labels, tcount, flag, ctr + 1, 152 * 12,
                                                                     s);
        c.launches++;
    }
    if (core) {
        launch_tc_core(o, plan, 5, plan.core_lcap, tcount, flag, ctr + 2, s);
        c.launches++;
    } else if (plan.nverts[5]) {
        launch_tc_cta<CTA2_THREADS, CTA2_ROUNDS, 16384, 8192, 17, 1>(o, plan, 5, labels, tcount, flag, ctr + 2, 152, s);
        c.launches++;
    }
    if (plan.nverts[6]) {
        k_tc_huge<<<152 * 4, 256, 0, s>>>(o, plan.verts[6], plan.nverts[6], labels, tcount, flag);
        CK_LAUNCH("k_tc_huge");
        c.launches++;
    }
}

}  // namespace scd
