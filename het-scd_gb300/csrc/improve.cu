// improve_partition (src/scd.cpp:221-341) on the device.
//
// For every vertex p the multiset of its neighbours' labels (old labels) is
// reduced to (label, frequency) pairs without sorting:
//   degree <= 32     a group of 8, 16 or 32 lanes of a warp, one lane per
//                    neighbour; __match_any_sync finds equal labels (groups
//                    are separated by a lane mask), the lowest lane of each
//                    equal-label set owns the label;
//   33 .. 256        one warp per vertex, open-addressing (label, count) table
//                    in shared memory;
//   257 .. 4096      one CTA per vertex, the table in shared memory (three
//                    sizes, so that short tables leave room for more CTAs);
//   > 4096           one CTA per vertex, per-vertex table in global memory.
// Every distinct label first gets an FP32 interval enclosure of its FP64 gain
// (gain_interval.cuh); for short label lists the intervals of many vertices are
// evaluated together, 32 per warp pass.  The intervals settle most vertices:
// no foreign label can have a positive gain and the own label's sign is known,
// or exactly one foreign label can hold the maximum and it clearly beats (or
// loses to) the own label.  Only the rest get exact FP64 gains: the foreign
// labels whose interval could still hold the maximum and, if needed, the own
// label (the remove gain).  The winner is the largest exact positive gain, ties
// to the smaller label — the candidate the reference's ascending scan with a
// strict '>' keeps (src/scd.cpp:313-316) — and the decision of
// src/scd.cpp:321-330 follows.  Labels update Jacobi-style.
#include "engine.cuh"
#include "gain_interval.cuh"

namespace scd {

namespace {

constexpr unsigned TPB = 256;

struct ImproveArgs {
    const uint32_t *indices, *adj, *labels;
    Stats st;
    const double *pin64;   // p_in of every community (src/scd.cpp:296-298)
    const int4 *civ;       // per label: size, external edges, FP32 enclosure of p_in (bits)
    const double *p_ext;      // per graph
    const float2 *pe32;       // per graph: FP32 enclosure of p_ext
    const uint32_t *gid;      // graph of each vertex (nullptr: one graph)
    const uint8_t *active;    // per graph: still iterating (nullptr: all)
    double alpha;
    uint32_t *next;
};

__device__ __forceinline__ uint32_t graph_of(const ImproveArgs &a, uint32_t p) { return a.gid ? a.gid[p] : 0u; }

__device__ __forceinline__ Iv pe_of(const ImproveArgs &a, uint32_t gp) {
    const float2 v = a.pe32[gp];
    return Iv{v.x, v.y};
}

__device__ __forceinline__ bool better(double g1, uint32_t l1, double g2, uint32_t l2) {
    return g1 > g2 || (g1 == g2 && l1 < l2);
}

// exact FP64 gain of moving p (degree deg, label mine) to label l seen freq times
__device__ __forceinline__ double exact_gain(const ImproveArgs &a, uint32_t l, uint32_t freq, uint32_t deg,
                                             uint32_t mine, double p_ext) {
    int size = a.st.sizes[l], ext = a.st.ext[l];
    double p_in;
    if (l == mine) {
        int in = a.st.intl[l] / 2;
        size--;
        ext += (int)(freq - (deg - freq));
        in -= (int)freq;
        p_in = community_p_in(size, in);
    } else {
        p_in = a.pin64[l];
    }
    return wcc_gain(size, (int)freq, (int)deg - (int)freq, ext, p_in, p_ext, a.alpha);
}

// Interval of the gain of label l, own label included (the negated remove gain:
// the community without p, as exact_gain's l == mine branch, with
// community_p_in enclosed).  One wcc_gain_iv call for both kinds, so lanes of a
// warp holding own and foreign labels do not diverge through it.
__device__ __forceinline__ Iv interval_any_gain(const ImproveArgs &a, uint32_t l, bool own, uint32_t freq,
                                                uint32_t deg, Iv p_ext, Iv alpha, bool *exact_needed) {
    const int4 cv = a.civ[l];   // one 16-byte read: size, external edges, p_in enclosure
    int size = cv.x, ext = cv.y;
    Iv pin;
    bool pin_bad = false;
    if (own) {
        size--;
        ext += (int)(freq - (deg - freq));
        const int in = a.st.intl[l] / 2 - (int)freq;
        pin = size > 1 ? iv_div(iv_int(2 * in), iv_mul(iv_int(size), iv_int(size - 1)), &pin_bad) : Iv{0.f, 0.f};
    } else {
        pin = Iv{__int_as_float(cv.z), __int_as_float(cv.w)};
    }
    const Iv g = wcc_gain_iv(size, (int)freq, (int)deg - (int)freq, ext, pin, p_ext, alpha, exact_needed);
    *exact_needed = *exact_needed || pin_bad;
    return g;
}

// The own label's exact gain is needed unless no foreign label survives the
// interval test and the interval alone fixes the sign of the remove gain
// (remove gain > 0 exactly when the own gain is < 0).
__device__ __forceinline__ bool own_sign_known(Iv iv, bool need) { return !need && (iv.hi < 0.f || iv.lo >= 0.f); }

// The decision from intervals alone where they settle it.  b (label bl) is the
// only foreign label that can hold the maximum gain and its lower bound is > 0
// (so bl is the exact arg-max and the best gain bg > 0); own encloses the own
// label's gain G (remove gain rg = -G; no own label among the neighbours: rg = 0).
// Move if bg > G (then bg + rg > 0, and bg is far above half an ulp of rg, so
// fl(bg + rg) > rg); stay if bg <= G (then bg + rg <= 0 and rg < 0).  Otherwise
// the exact gains decide.
constexpr uint32_t UNDECIDED = 0xfffffffeu;

__device__ __forceinline__ uint32_t decide_iv(Iv b, uint32_t bl, bool has_own, Iv own, uint32_t mine) {
    if (!has_own) return bl;
    const float r = fmaxf(fabsf(own.lo), fabsf(own.hi));
    if (b.lo > own.hi && b.lo > r * 0x1p-40f) return bl;
    if (b.hi <= own.lo) return mine;
    return UNDECIDED;
}

__device__ __forceinline__ uint32_t decide(double best_gain, uint32_t best_label, double remove_gain,
                                           uint32_t mine) {
    const double insert = dadd(best_gain, remove_gain);
    if (insert > remove_gain && insert > 0.0) return best_label;
    if (remove_gain > 0) return INVALID;
    return mine;
}

__global__ void k_comm_prep(uint32_t nc, Stats st, double *pin64, int4 *civ) {
    for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < nc; l += gridDim.x * blockDim.x) {
        const double p = community_p_in(st.sizes[l], st.intl[l] / 2);
        pin64[l] = p;
        civ[l] = make_int4(st.sizes[l], st.ext[l], __float_as_int(__double2float_rd(p)),
                           __float_as_int(__double2float_ru(p)));
    }
}

// ---- degree <= G: groups of G lanes ---------------------------------------
//
// A group of G lanes finds the (label, frequency) pairs of its vertex with
// __match_any_sync; the pairs go to the warp's candidate queue (below).

constexpr unsigned GROUP_GRID = 152 * 4;   // resident CTAs (64 registers x 256 threads): warps loop over many rounds

// Candidate queue of a warp for the group kernels: the (label, frequency) pairs
// of the pending vertices.  The interval of every candidate is evaluated 32 at
// a time with all lanes busy (a vertex of degree <= 32 has only a few distinct
// labels, so evaluating them where they arise would leave most lanes idle);
// then one lane per vertex decides from the intervals, and the rare vertices
// that need exact gains are evaluated one at a time, lane-parallel over their
// candidates.
constexpr int CQ = 64;

struct CandQueue {
    uint32_t label[CQ], freq[CQ];
    float lo[CQ], hi[CQ];
    uint8_t vert[CQ], need[CQ];
    uint32_t p[CQ], deg[CQ], mine[CQ], gp[CQ];   // pending vertices (each has >= 1 candidate)
    uint8_t first[CQ], cnt[CQ], exact[CQ];
};

__device__ __forceinline__ void process_candidates(const ImproveArgs &a, CandQueue &q, uint32_t cn, uint32_t vn,
                                                int lane, Iv al) {
    __syncwarp();
    for (uint32_t i = lane; i < cn; i += 32) {
        const uint32_t v = q.vert[i], l = q.label[i];
        bool need = false;
        const Iv iv = interval_any_gain(a, l, l == q.mine[v], q.freq[i], q.deg[v], pe_of(a, q.gp[v]), al, &need);
        q.lo[i] = iv.lo;
        q.hi[i] = iv.hi;
        q.need[i] = need;
    }
    __syncwarp();
    for (uint32_t v = lane; v < vn; v += 32) {
        const uint32_t mine = q.mine[v], f = q.first[v], e = f + q.cnt[v];
        float m = -INFINITY, m_hi = -INFINITY;
        uint32_t m_label = INVALID;
        bool need_any = false, has_own = false, own_need = false;
        Iv own = {0.f, 0.f};
        for (uint32_t k = f; k < e; k++) {
            const uint32_t l = q.label[k];
            if (l == mine) {
                has_own = true;
                own_need = q.need[k];
                own = Iv{q.lo[k], q.hi[k]};
            } else if (q.need[k]) {
                need_any = true;
            } else if (q.lo[k] > m) {
                m = q.lo[k];
                m_hi = q.hi[k];
                m_label = l;
            }
        }
        uint32_t survivors = 0;
        for (uint32_t k = f; k < e; k++)
            survivors += q.label[k] != mine && (q.need[k] || (q.hi[k] > 0.f && q.hi[k] >= m));
        uint32_t dec = UNDECIDED;
        if (survivors == 1 && !need_any && m > 0.f && !(has_own && own_need))
            dec = decide_iv(Iv{m, m_hi}, m_label, has_own, own, mine);
        else if (survivors == 0 && !(has_own && !own_sign_known(own, own_need)))
            dec = (has_own && own.hi < 0.f) ? INVALID : mine;   // no foreign label can have a positive gain
        q.exact[v] = dec == UNDECIDED;
        if (dec != UNDECIDED) a.next[q.p[v]] = dec;
    }
    __syncwarp();
    // exact gains: one vertex at a time, a lane per candidate (<= 32 of them)
    for (uint32_t v0 = 0; v0 < vn; v0 += 32) {
        unsigned xb = __ballot_sync(FULL, v0 + lane < vn && q.exact[v0 + lane]);
        while (xb) {
            const uint32_t v = v0 + __ffs(xb) - 1;
            xb &= xb - 1;
            const uint32_t mine = q.mine[v], c = q.cnt[v], k = q.first[v] + lane;
            const bool in = (uint32_t)lane < c;
            const uint32_t l = in ? q.label[k] : INVALID;
            const bool is_own = in && l == mine, need = in && q.need[k];
            const float lo = in ? q.lo[k] : -INFINITY, hi = in ? q.hi[k] : -INFINITY;
            float m = (in && !is_own && !need) ? lo : -INFINITY;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL, m, o));
            const bool survive = in && !is_own && (need || (hi > 0.f && hi >= m));
            const bool any_survivor = __any_sync(FULL, survive);
            const bool own_item = is_own && (any_survivor || !own_sign_known(Iv{lo, hi}, need));
            const double p_ext = a.p_ext[q.gp[v]];
            double g = 0.0;
            if (survive || own_item) g = exact_gain(a, l, q.freq[k], q.deg[v], mine, p_ext);
            const unsigned own_lanes = __ballot_sync(FULL, is_own);
            const double own_g = __shfl_sync(FULL, g, own_lanes ? __ffs(own_lanes) - 1 : 0);
            // remove gain: exact if evaluated; else only its sign matters (nothing survives)
            const bool own_eval = __shfl_sync(FULL, own_item, own_lanes ? __ffs(own_lanes) - 1 : 0);
            const float own_hi = __shfl_sync(FULL, hi, own_lanes ? __ffs(own_lanes) - 1 : 0);
            const double rg = !own_lanes ? 0.0 : own_eval ? -own_g : (own_hi < 0.f ? 1.0 : 0.0);
            double bg = 0.0;
            uint32_t bl = INVALID;
            if (survive && g > 0.0) {
                bg = g;
                bl = l;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double og = __shfl_xor_sync(FULL, bg, o);
                const uint32_t olb = __shfl_xor_sync(FULL, bl, o);
                if (olb != INVALID && (bl == INVALID || better(og, olb, bg, bl))) {
                    bg = og;
                    bl = olb;
                }
            }
            if (lane == 0) a.next[q.p[v]] = decide(bl == INVALID ? 0.0 : bg, bl == INVALID ? 0u : bl, rg, mine);
        }
    }
    __syncwarp();
}

template <int G>
__global__ void __launch_bounds__(TPB)
k_improve_group(const uint32_t *__restrict__ verts, uint32_t count, ImproveArgs a) {
    constexpr int PER_WARP = 32 / G;
    __shared__ CandQueue queues[TPB / 32];
    const int lane = threadIdx.x & 31, gl = lane % G, g0 = lane - gl;
    const unsigned gmask = (G == 32) ? FULL : (((1u << G) - 1u) << g0);
    const unsigned below = (1u << lane) - 1u;
    CandQueue &q = queues[threadIdx.x >> 5];
    const Iv al = iv_of(a.alpha);
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t cn = 0, vn = 0;   // warp-uniform
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;; w += warps) {
        const bool done = w * PER_WARP >= count;
        if (cn > CQ - 32 || (done && cn)) {   // one call site: the evaluation is inlined once
            process_candidates(a, q, cn, vn, lane, al);
            cn = vn = 0;
        }
        if (done) break;
        const uint32_t slot = w * PER_WARP + lane / G;
        const bool active = slot < count;
        const uint32_t p = active ? verts[slot] : 0;
        const uint32_t beg = active ? a.indices[p] : 0;
        const uint32_t deg = active ? a.indices[p + 1] - beg : 0;
        const uint32_t mine = active ? a.labels[p] : INVALID;
        const uint32_t gp = active ? graph_of(a, p) : 0u;
        const bool frozen = active && a.active && !a.active[gp];   // graph already converged
        const uint32_t l = (uint32_t)gl < deg && !frozen ? a.labels[a.adj[beg + gl]] : INVALID;
        const unsigned peers = __match_any_sync(FULL, l) & gmask;
        const bool owner = l != INVALID && lane == __ffs(peers) - 1;
        const uint32_t freq = __popc(peers);
        const unsigned ob = __ballot_sync(FULL, owner);
        const uint32_t gcnt = __popc(ob & gmask);
        // no labelled neighbour (or the graph converged): the label stays
        if (active && gl == 0 && gcnt == 0) a.next[p] = mine;
        const unsigned vb = __ballot_sync(FULL, active && gl == 0 && gcnt != 0);
        const uint32_t vidx = vn + __popc(vb & below);
        if (active && gl == 0 && gcnt != 0) {
            q.p[vidx] = p;
            q.deg[vidx] = deg;
            q.mine[vidx] = mine;
            q.gp[vidx] = gp;
            q.first[vidx] = (uint8_t)(cn + __popc(ob & ((1u << g0) - 1u)));
            q.cnt[vidx] = (uint8_t)gcnt;
        }
        const uint32_t my_v = __shfl_sync(FULL, vidx, g0);
        if (owner) {
            const uint32_t pos = cn + __popc(ob & below);
            q.label[pos] = l;
            q.freq[pos] = freq;
            q.vert[pos] = (uint8_t)my_v;
        }
        cn += __popc(ob);
        vn += __popc(vb);
    }
}

// ---- degree 33 .. 256: one warp per vertex, (label, count) hash table -------
// ---- degree > 256: one CTA per vertex ---------------------------------------

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// One warp per vertex (degree <= WLIST): the warp's own open-addressing table
// in shared memory and the list of its occupied entries.  A vertex with at most
// 32 distinct labels goes to the warp's candidate queue like the group kernels'
// vertices; one with more has its intervals evaluated lane-parallel over the
// list and, where they do not settle it, its exact gains too.
constexpr int WCAP = 512, WLIST = 256, WWARPS = 4;

struct WarpTable {
    uint32_t keys[WCAP], vals[WCAP];
    float hi[WLIST];   // upper bound of each listed foreign label (+inf: interval unusable)
    uint16_t list[WLIST];
    uint32_t n;
};

__device__ __forceinline__ bool survives(float hi, float m) { return hi > 0.f && hi >= m; }

// a vertex with more than 32 distinct labels, on its own
__device__ __forceinline__ void improve_many_labels(const ImproveArgs &a, WarpTable &T, uint32_t nl, uint32_t p,
                                                    uint32_t gp, uint32_t mine, uint32_t deg, Iv al, int lane) {
    const double p_ext = a.p_ext[gp];
    const Iv pe = pe_of(a, gp);
    float m = -INFINITY, mh = -INFINITY, m_hi = -INFINITY;   // m_hi: upper bound of the label holding m
    uint32_t m_label = INVALID;
    bool need_any = false, has_own = false, own_need = false;
    Iv own_iv = {0.f, 0.f};
    for (uint32_t k = lane; k < nl; k += 32) {
        const uint32_t h = T.list[k], l = T.keys[h], f = T.vals[h];
        bool need = false;
        const Iv iv = interval_any_gain(a, l, l == mine, f, deg, pe, al, &need);
        if (l == mine) {
            has_own = true;
            own_need = need;
            own_iv = iv;
            T.hi[k] = -INFINITY;
        } else if (need) {
            need_any = true;
            T.hi[k] = INFINITY;
        } else {
            if (iv.lo > m) {
                m = iv.lo;
                m_hi = iv.hi;
                m_label = l;
            }
            mh = fmaxf(mh, iv.hi);
            T.hi[k] = iv.hi;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float om = __shfl_xor_sync(FULL, m, o), omh = __shfl_xor_sync(FULL, m_hi, o);
        const uint32_t oml = __shfl_xor_sync(FULL, m_label, o);
        if (om > m || (om == m && oml < m_label)) {
            m = om;
            m_hi = omh;
            m_label = oml;
        }
        mh = fmaxf(mh, __shfl_xor_sync(FULL, mh, o));
    }
    need_any = __any_sync(FULL, need_any);
    const unsigned own_lanes = __ballot_sync(FULL, has_own);
    const int ol = own_lanes ? __ffs(own_lanes) - 1 : 0;
    own_need = __shfl_sync(FULL, own_need, ol);
    own_iv.lo = __shfl_sync(FULL, own_iv.lo, ol);
    own_iv.hi = __shfl_sync(FULL, own_iv.hi, ol);
    __syncwarp();
    const bool any_survivor = need_any || (mh > 0.f && mh >= m);
    uint32_t survivors = 0;
    for (uint32_t kb = 0; kb < nl; kb += 32) {
        const uint32_t k = kb + lane;
        survivors += __popc(__ballot_sync(FULL, k < nl && survives(T.hi[k], m)));
    }
    uint32_t dec = UNDECIDED;
    if (survivors == 1 && !need_any && m > 0.f && !(own_lanes && own_need))
        dec = decide_iv(Iv{m, m_hi}, m_label, own_lanes != 0, own_iv, mine);
    else if (survivors == 0 && !(own_lanes && !own_sign_known(own_iv, own_need)))
        dec = (own_lanes && own_iv.hi < 0.f) ? INVALID : mine;
    if (dec != UNDECIDED) {
        if (lane == 0) a.next[p] = dec;
        return;
    }
    // exact gains of the survivors and of the own label, lane-parallel over the list
    const bool own_item = own_lanes && (own_need || !own_sign_known(own_iv, own_need) || any_survivor);
    double bg = 0.0, rg = 0.0;
    uint32_t bl = INVALID;
    for (uint32_t k = lane; k < nl; k += 32) {
        const uint32_t h = T.list[k], l = T.keys[h];
        if (l == mine) {
            if (own_item) rg = -exact_gain(a, l, T.vals[h], deg, mine, p_ext);
        } else if (survives(T.hi[k], m)) {
            const double g = exact_gain(a, l, T.vals[h], deg, mine, p_ext);
            if (g > 0.0 && (bl == INVALID || better(g, l, bg, bl))) {
                bg = g;
                bl = l;
            }
        }
    }
    rg = __shfl_sync(FULL, rg, ol);
    if (own_lanes && !own_item) rg = own_iv.hi < 0.f ? 1.0 : 0.0;   // only its sign matters then
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double og = __shfl_xor_sync(FULL, bg, o);
        const uint32_t olb = __shfl_xor_sync(FULL, bl, o);
        if (olb != INVALID && (bl == INVALID || better(og, olb, bg, bl))) {
            bg = og;
            bl = olb;
        }
    }
    if (lane == 0) a.next[p] = decide(bl == INVALID ? 0.0 : bg, bl == INVALID ? 0u : bl, rg, mine);
}

__global__ void __launch_bounds__(WWARPS * 32)
k_improve_warp(const uint32_t *__restrict__ verts, uint32_t count, ImproveArgs a) {
    __shared__ WarpTable tabs[WWARPS];
    __shared__ CandQueue queues[WWARPS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    WarpTable &T = tabs[wid];
    CandQueue &q = queues[wid];
    const Iv al = iv_of(a.alpha);
    for (uint32_t i = lane; i < WCAP; i += 32) {
        T.keys[i] = INVALID;
        T.vals[i] = 0;
    }
    if (lane == 0) T.n = 0;
    __syncwarp();
    uint32_t cn = 0, vn = 0;   // warp-uniform
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t vi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;; vi += warps) {
        const bool done = vi >= count;
        // the label table of this vertex, before a flush needs the queue
        uint32_t p = 0, gp = 0, mine = INVALID, deg = 0, nl = 0;
        bool frozen = false;
        if (!done) {
            p = verts[vi];
            gp = graph_of(a, p);
            mine = a.labels[p];
            frozen = a.active && !a.active[gp];
        }
        if (!done && !frozen) {
            const uint32_t beg = a.indices[p];
            deg = a.indices[p + 1] - beg;
            uint32_t cap = 64;
            while (cap < 2 * deg) cap <<= 1;
            const uint32_t mask = cap - 1;
            for (uint32_t k = lane; k < deg; k += 32) {
                const uint32_t l = a.labels[a.adj[beg + k]];
                if (l == INVALID) continue;
                uint32_t h = hash32(l) & mask;
                while (true) {
                    uint32_t key = T.keys[h];
                    if (key == INVALID) {
                        key = atomicCAS(T.keys + h, INVALID, l);
                        if (key == INVALID) {
                            T.list[atomicAdd(&T.n, 1u)] = (uint16_t)h;
                            key = l;
                        }
                    }
                    if (key == l) {
                        atomicAdd(T.vals + h, 1u);
                        break;
                    }
                    h = (h + 1) & mask;
                }
            }
            __syncwarp();
            nl = T.n;
        }
        const bool queued = !done && !frozen && nl > 0 && nl <= 32;
        if ((queued && cn + nl > (uint32_t)CQ) || (done && cn)) {   // one call site
            process_candidates(a, q, cn, vn, lane, al);
            cn = vn = 0;
        }
        if (done) break;
        if (frozen || nl == 0) {   // converged graph, or no labelled neighbour: the label stays
            if (lane == 0) a.next[p] = mine;
        } else if (queued) {
            if ((uint32_t)lane < nl) {
                const uint32_t h = T.list[lane];
                q.label[cn + lane] = T.keys[h];
                q.freq[cn + lane] = T.vals[h];
                q.vert[cn + lane] = (uint8_t)vn;
            }
            if (lane == 0) {
                q.p[vn] = p;
                q.deg[vn] = deg;
                q.mine[vn] = mine;
                q.gp[vn] = gp;
                q.first[vn] = (uint8_t)cn;
                q.cnt[vn] = (uint8_t)nl;
            }
            cn += nl;
            vn++;
        } else {
            improve_many_labels(a, T, nl, p, gp, mine, deg, al, lane);
        }
        // empty the table through its list
        __syncwarp();
        for (uint32_t k = lane; k < nl; k += 32) {
            const uint32_t h = T.list[k];
            T.keys[h] = INVALID;
            T.vals[h] = 0;
        }
        __syncwarp();
        if (lane == 0) T.n = 0;
        __syncwarp();
    }
}

// One vertex per CTA.  keys/vals is an open-addressing table of cap (label,
// count) entries; list receives the index of every occupied entry, so both
// passes touch only the distinct labels.
template <int THREADS>
__device__ void improve_cta(const ImproveArgs &a, uint32_t p, uint32_t *keys, uint32_t *vals, uint32_t *list,
                            float *hi_of, uint32_t cap, double p_ext, Iv pe, Iv al) {
    __shared__ double s_gain[THREADS / 32];
    __shared__ uint32_t s_label[THREADS / 32];
    __shared__ float s_lo[THREADS / 32], s_hi[THREADS / 32];
    __shared__ double s_remove;
    __shared__ uint32_t s_n;
    __shared__ int s_need;        // some foreign interval was not usable
    __shared__ int s_own;         // 0 no own label among the neighbours, 1 sign known, 2 exact needed
    __shared__ float s_own_lo, s_own_hi;
    __shared__ uint32_t s_own_i;  // the own label's position in the entry list
    __shared__ float s_mhi[THREADS / 32];
    __shared__ uint32_t s_mlab[THREADS / 32], s_surv[THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t beg = a.indices[p], deg = a.indices[p + 1] - beg, mine = a.labels[p];
    const uint32_t mask = cap - 1;
    for (uint32_t i = threadIdx.x; i < cap; i += THREADS) {
        keys[i] = INVALID;
        vals[i] = 0;
    }
    if (threadIdx.x == 0) {
        s_remove = 0.0;
        s_n = 0;
        s_need = 0;
        s_own = 0;
    }
    __syncthreads();
    // LB neighbour labels per thread are gathered before any is inserted, so their
    // loads overlap instead of one load chain per neighbour
    constexpr int LB = 4;
    for (uint32_t i0 = threadIdx.x; i0 < deg; i0 += THREADS * LB) {
        uint32_t lb[LB];
#pragma unroll
        for (int k = 0; k < LB; k++) {
            const uint32_t i = i0 + k * THREADS;
            lb[k] = i < deg ? a.adj[beg + i] : INVALID;
        }
#pragma unroll
        for (int k = 0; k < LB; k++) lb[k] = lb[k] != INVALID ? a.labels[lb[k]] : INVALID;
#pragma unroll
        for (int k = 0; k < LB; k++) {
            const uint32_t l = lb[k];
            if (l == INVALID) continue;
            uint32_t h = hash32(l) & mask;
            while (true) {
                uint32_t key = keys[h];
                if (key == INVALID) {
                    key = atomicCAS(keys + h, INVALID, l);
                    if (key == INVALID) {
                        list[atomicAdd(&s_n, 1u)] = h;   // first occurrence of l
                        key = l;
                    }
                }
                if (key == l) {
                    atomicAdd(vals + h, 1u);
                    break;
                }
                h = (h + 1) & mask;
            }
        }
    }
    __syncthreads();
    const uint32_t nl = s_n;
    // pass 1: best lower and upper bounds among foreign labels, the own label's
    // interval; hi_of[i] keeps label i's upper bound for pass 2 (+inf: unusable)
    float m = -INFINITY, mh = -INFINITY, m_hi = -INFINITY;   // m_hi: upper bound of the label holding m
    uint32_t m_label = INVALID;
    for (uint32_t i = threadIdx.x; i < nl; i += THREADS) {
        const uint32_t h = list[i], l = keys[h];
        bool need = false;
        const Iv iv = interval_any_gain(a, l, l == mine, vals[h], deg, pe, al, &need);
        if (l == mine) {
            s_own = own_sign_known(iv, need) ? 1 : 2;
            s_own_lo = iv.lo;
            s_own_hi = iv.hi;
            s_own_i = i;
            hi_of[i] = -INFINITY;
            continue;
        }
        if (need) {
            s_need = 1;
            hi_of[i] = INFINITY;
        } else {
            if (iv.lo > m || (iv.lo == m && l < m_label)) {
                m = iv.lo;
                m_hi = iv.hi;
                m_label = l;
            }
            mh = fmaxf(mh, iv.hi);
            hi_of[i] = iv.hi;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float om = __shfl_xor_sync(FULL, m, o), omh = __shfl_xor_sync(FULL, m_hi, o);
        const uint32_t oml = __shfl_xor_sync(FULL, m_label, o);
        if (om > m || (om == m && oml < m_label)) {
            m = om;
            m_hi = omh;
            m_label = oml;
        }
        mh = fmaxf(mh, __shfl_xor_sync(FULL, mh, o));
    }
    if (lane == 0) {
        s_lo[warp] = m;
        s_hi[warp] = mh;
        s_mhi[warp] = m_hi;
        s_mlab[warp] = m_label;
    }
    __syncthreads();
    m = s_lo[0];
    mh = s_hi[0];
    m_hi = s_mhi[0];
    m_label = s_mlab[0];
#pragma unroll
    for (int w = 1; w < THREADS / 32; w++) {
        if (s_lo[w] > m || (s_lo[w] == m && s_mlab[w] < m_label)) {
            m = s_lo[w];
            m_hi = s_mhi[w];
            m_label = s_mlab[w];
        }
        mh = fmaxf(mh, s_hi[w]);
    }
    // a foreign label survives iff its interval is unusable or hi > 0 and hi >= m;
    // the one with the largest hi decides whether any does
    const bool any_survivor = s_need || (mh > 0.f && mh >= m);
    // the intervals alone decide when the label holding m > 0 is the only survivor
    // and the own label's interval is usable (decide_iv); no exact gain is then needed
    if (!s_need && m > 0.f && s_own != 2) {
        uint32_t surv = 0;
        for (uint32_t i0 = 0; i0 < nl; i0 += THREADS) {
            const uint32_t i = i0 + threadIdx.x;
            const float hi = i < nl ? hi_of[i] : -INFINITY;
            surv += __popc(__ballot_sync(FULL, hi > 0.f && hi >= m));
        }
        if (lane == 0) s_surv[warp] = surv;
        __syncthreads();
        surv = 0;
#pragma unroll
        for (int w = 0; w < THREADS / 32; w++) surv += s_surv[w];
        if (surv == 1) {
            const uint32_t dec = decide_iv(Iv{m, m_hi}, m_label, s_own != 0, Iv{s_own_lo, s_own_hi}, mine);
            if (dec != UNDECIDED) {
                if (threadIdx.x == 0) a.next[p] = dec;
                __syncthreads();
                return;
            }
        }
    }
    // pass 2: exact gains of the survivors and, if needed, of the own label (remove gain)
    double bg = 0.0;
    uint32_t bl = INVALID;
    if (s_own && threadIdx.x == (s_own_i & (THREADS - 1))) {   // the own label (remove gain)
        const uint32_t h = list[s_own_i];
        if (any_survivor || s_own == 2) s_remove = -exact_gain(a, mine, vals[h], deg, mine, p_ext);
        else if (s_own_hi < 0.f) s_remove = 1.0;   // only its sign matters when nothing survives
    }
    for (uint32_t i = threadIdx.x; i < nl; i += THREADS) {
        const float hi = hi_of[i];   // -inf for the own label
        if (hi > 0.f && hi >= m) {
            const uint32_t h = list[i], l = keys[h];
            const double g = exact_gain(a, l, vals[h], deg, mine, p_ext);
            if (g > 0.0 && (bl == INVALID || better(g, l, bg, bl))) {
                bg = g;
                bl = l;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double og = __shfl_xor_sync(FULL, bg, o);
        const uint32_t ol = __shfl_xor_sync(FULL, bl, o);
        if (ol != INVALID && (bl == INVALID || better(og, ol, bg, bl))) {
            bg = og;
            bl = ol;
        }
    }
    if (lane == 0) {
        s_gain[warp] = bg;
        s_label[warp] = bl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < THREADS / 32; w++)
            if (s_label[w] != INVALID && (bl == INVALID || better(s_gain[w], s_label[w], bg, bl))) {
                bg = s_gain[w];
                bl = s_label[w];
            }
        a.next[p] = decide(bl == INVALID ? 0.0 : bg, bl == INVALID ? 0u : bl, s_remove, mine);
    }
    __syncthreads();
}

template <int THREADS, uint32_t CAP>
__global__ void __launch_bounds__(THREADS)
k_improve_cta(const uint32_t *__restrict__ verts, uint32_t count, ImproveArgs a) {
    extern __shared__ uint32_t smem[];
    uint32_t *keys = smem, *vals = smem + CAP, *list = smem + 2 * CAP;
    float *hi_of = (float *)(list + CAP / 2);
    const Iv al = iv_of(a.alpha);
    for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
        const uint32_t p = verts[i];
        const uint32_t gp = graph_of(a, p);
        if (a.active && !a.active[gp]) {   // graph already converged: labels stay
            if (threadIdx.x == 0) a.next[p] = a.labels[p];
            continue;
        }
        const uint32_t deg = a.indices[p + 1] - a.indices[p];
        uint32_t cap = 64;
        while (cap < 2 * deg) cap <<= 1;
        improve_cta<THREADS>(a, p, keys, vals, list, hi_of, cap, a.p_ext[gp], pe_of(a, gp), al);
    }
}

constexpr int GLOBAL_THREADS = 512;

// tables: per vertex 3*cap words (keys, counts; then the occupied-entry list and
// the labels' upper bounds, cap / 2 each)
__global__ void __launch_bounds__(GLOBAL_THREADS, 2)
k_improve_global(const uint32_t *__restrict__ verts, uint32_t count, ImproveArgs a, uint32_t *tables,
                 const uint64_t *__restrict__ table_off) {
    const Iv al = iv_of(a.alpha);
    for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
        const uint32_t p = verts[i];
        const uint32_t gp = graph_of(a, p);
        if (a.active && !a.active[gp]) {
            if (threadIdx.x == 0) a.next[p] = a.labels[p];
            continue;
        }
        const uint64_t off = table_off[i];
        const uint32_t cap = (uint32_t)((table_off[i + 1] - off) / 3);
        uint32_t *t = tables + off;
        improve_cta<GLOBAL_THREADS>(a, p, t, t + cap, t + 2 * cap, (float *)(t + 2 * cap + cap / 2), cap, a.p_ext[gp],
                                    pe_of(a, gp), al);
    }
}

template <int THREADS, uint32_t CAP>
constexpr size_t cta_smem() {   // keys, counts (CAP each), entry list and upper bounds (CAP / 2 each)
    return 3 * CAP * sizeof(uint32_t);
}

template <int THREADS, uint32_t CAP>
void set_cta_attr() {   // always: dynamic plus static shared memory may pass 48 KB
    CK(cudaFuncSetAttribute((const void *)k_improve_cta<THREADS, CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)cta_smem<THREADS, CAP>()));
}

}  // namespace

void prepare_improve_kernels() {
    static thread_local int done_device = -1;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (done_device == dev) return;
    set_cta_attr<128, 2048>();
    set_cta_attr<256, 4096>();
    set_cta_attr<512, 8192>();
    done_device = dev;
}

namespace {

template <int THREADS, uint32_t CAP>
void launch_cta(const uint32_t *verts, uint32_t count, const ImproveArgs &a, cudaStream_t s, unsigned max_grid) {
    k_improve_cta<THREADS, CAP><<<grid_for(count, 1, max_grid), THREADS, cta_smem<THREADS, CAP>(), s>>>(verts, count, a);
    CK_LAUNCH("k_improve_cta");
}

}  // namespace

void improve(Ctx &c, const uint32_t *labels, const Stats &st, uint32_t *next, bool frozen_graphs) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    if (g.n == 0) return;
    PhaseScope ph(c, "improve");
    prepare_improve_kernels();
    if (c.num_comms) {
        k_comm_prep<<<grid_for(c.num_comms, TPB), TPB, 0, s>>>(c.num_comms, st, c.pin64, c.civ);
        CK_LAUNCH("k_comm_prep");
        c.launches++;
    }
    ImproveArgs a{g.indices, g.adj, labels, st, c.pin64, c.civ, c.b.p_ext, c.b.pe32, c.b.gid,
                  frozen_graphs ? c.b.active : nullptr, c.alpha, next};
    const DegreeClasses &k = g.cls;
    // the hub class (one CTA per vertex of degree > 4096, bound by the latency of its
    // global-memory tables) runs on the auxiliary stream beside the other classes;
    // the classes decide disjoint vertices from the same labels and statistics
    const bool fork = k.count[7] && c.aux;
    if (fork) {
        CK(cudaEventRecord(c.aux_fork, s));
        CK(cudaStreamWaitEvent(c.aux, c.aux_fork, 0));
        k_improve_global<<<grid_for(k.count[7], 1, 152 * 2), GLOBAL_THREADS, 0, c.aux>>>(k.list[7], k.count[7], a,
                                                                                        c.big_tables, g.big_table_off);
        CK_LAUNCH("k_improve_global");
        CK(cudaEventRecord(c.aux_join, c.aux));
        c.launches++;
    }
    if (k.count[0]) {
        k_improve_group<8><<<grid_for((uint64_t)k.count[0] * 8, TPB, GROUP_GRID), TPB, 0, s>>>(k.list[0], k.count[0], a);
        CK_LAUNCH("k_improve_group8");
        c.launches++;
    }
    if (k.count[1]) {
        k_improve_group<16><<<grid_for((uint64_t)k.count[1] * 16, TPB, GROUP_GRID), TPB, 0, s>>>(k.list[1], k.count[1], a);
        CK_LAUNCH("k_improve_group16");
        c.launches++;
    }
    if (k.count[2]) {
        k_improve_group<32><<<grid_for((uint64_t)k.count[2] * 32, TPB, GROUP_GRID), TPB, 0, s>>>(k.list[2], k.count[2], a);
        CK_LAUNCH("k_improve_group32");
        c.launches++;
    }
    if (k.count[3]) {
        k_improve_warp<<<grid_for((uint64_t)k.count[3] * 32, WWARPS * 32, 152 * 7), WWARPS * 32, 0, s>>>(
            k.list[3], k.count[3], a);
        CK_LAUNCH("k_improve_warp");
        c.launches++;
    }
    if (k.count[4]) {
        launch_cta<128, 2048>(k.list[4], k.count[4], a, s, 152 * 16);
        c.launches++;
    }
    if (k.count[5]) {
        launch_cta<256, 4096>(k.list[5], k.count[5], a, s, 152 * 7);
        c.launches++;
    }
    if (k.count[6]) {
        launch_cta<512, 8192>(k.list[6], k.count[6], a, s, 152 * 2);
        c.launches++;
    }
    if (fork) {
        CK(cudaStreamWaitEvent(s, c.aux_join, 0));
    } else if (k.count[7]) {
        k_improve_global<<<grid_for(k.count[7], 1, 152 * 2), GLOBAL_THREADS, 0, s>>>(k.list[7], k.count[7], a,
                                                                                    c.big_tables, g.big_table_off);
        CK_LAUNCH("k_improve_global");
        c.launches++;
    }
}

}  // namespace scd
