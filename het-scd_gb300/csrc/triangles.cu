// Triangle counting on a degree-oriented graph, with per-edge counters.
//
// Every undirected edge has one out-slot (in the out-list of its lower-ranked
// endpoint).  A triangle {a, b, c} with a -> b, a -> c, b -> c is found once,
// from a: for b in out(a), every c in out(b) ∩ out(a) adds 1 to the counters of
// the three slots (a,b), (a,c), (b,c).  The per-edge totals are exactly the
// per-edge triangle counts t[e] of the reference's merge over the id-oriented
// list (src/convert.cpp:290-319), computed with O(sum d+(a) d+(b)) work instead
// of the reference's id orientation, whose hubs make it quadratic.
//
// With labels, only internal triangles count (all three vertices share a valid
// label): the per-edge internal counts that compute_wcc derives by merging each
// vertex's same-label neighbours (src/wcc.cpp:84-127), and that the reference
// GPU path gets from a compacted internal CSR (src/cuda.cu:285-330,
// src/kernels.cuh:299-356).
//
// Work decomposition: a unit is (vertex a, 32 consecutive entries b of out(a)).
// Units are handed to warps dynamically (heavy out-lists are split across
// warps).  out(a) is staged in the warp's shared memory; the warp flattens the
// items (b, c in out(b)) of its 32 b's with a prefix sum, each lane takes items
// and looks c up in out(a) by binary search.
#include "engine.cuh"

namespace scd {

namespace {

constexpr int TC_WARPS = 8;
constexpr int TC_THREADS = TC_WARPS * 32;
constexpr int TC_STAGE = 1024;   // out-list entries staged per warp

struct UnitsOf {
    const uint32_t *len;
    const uint32_t *labels;
    __device__ uint32_t operator[](size_t a) const {
        if (labels && labels[a] == INVALID) return 0;
        return (len[a] + 31) >> 5;
    }
};

__global__ void __launch_bounds__(TC_THREADS)
k_tc_units(Oriented o, const uint32_t *__restrict__ labels, const uint32_t *__restrict__ unit_off,
           uint32_t *slot_cnt, uint32_t *next_unit) {
    __shared__ uint32_t stage[TC_WARPS][TC_STAGE];
    __shared__ uint32_t pre[TC_WARPS][32];
    __shared__ uint32_t bbase[TC_WARPS][32];
    __shared__ uint32_t bhits[TC_WARPS][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t n_units = unit_off[o.n];
    while (true) {
        uint32_t unit = 0;
        if (lane == 0) unit = atomicAdd(next_unit, 1u);
        unit = __shfl_sync(FULL, unit, 0);
        if (unit >= n_units) break;
        // vertex a: unit_off[a] <= unit < unit_off[a+1]
        uint32_t lo = 0, hi = o.n + 1;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (unit_off[mid] <= unit) lo = mid + 1;
            else hi = mid;
        }
        const uint32_t a = lo - 1;
        const uint32_t ch = unit - unit_off[a];
        const uint32_t la = labels ? labels[a] : 0u;
        const uint32_t abeg = o.beg[a], alen = o.len[a];
        const bool staged = alen <= TC_STAGE;
        if (staged)
            for (uint32_t i = lane; i < alen; i += 32) stage[w][i] = o.adj[abeg + i];
        __syncwarp();
        const uint32_t *A = staged ? stage[w] : o.adj + abeg;

        const uint32_t j = ch * 32 + lane;
        uint32_t wb = 0, bb = 0;
        if (j < alen) {
            uint32_t b = A[j];
            if (!labels || labels[b] == la) {
                wb = o.len[b];
                bb = o.beg[b];
            }
        }
        const uint32_t incl = warp_inclusive_scan(wb);
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        pre[w][lane] = incl - wb;
        bbase[w][lane] = bb;
        bhits[w][lane] = 0;
        __syncwarp();
        for (uint32_t t = lane; t < total; t += 32) {
            // owner lane of item t: last lane with pre <= t
            uint32_t l0 = 0, l1 = 32;
            while (l0 < l1) {
                uint32_t mid = (l0 + l1) >> 1;
                if (pre[w][mid] <= t) l0 = mid + 1;
                else l1 = mid;
            }
            const uint32_t jb = l0 - 1;
            const uint32_t cpos = bbase[w][jb] + (t - pre[w][jb]);
            const uint32_t c = o.adj[cpos];
            const uint32_t ic = lower_bound(A, alen, c);
            bool hit = ic < alen && A[ic] == c;
            if (hit && labels) hit = labels[c] == la;
            if (hit) {
                atomicAdd(&bhits[w][jb], 1u);
                atomicAdd(slot_cnt + abeg + ic, 1u);
                atomicAdd(slot_cnt + cpos, 1u);
            }
        }
        __syncwarp();
        if (j < alen && bhits[w][lane]) atomicAdd(slot_cnt + abeg + j, bhits[w][lane]);
        __syncwarp();
    }
}

}  // namespace

void count_oriented_triangles(Ctx &c, const Oriented &o, const uint32_t *labels, uint32_t *slot_cnt,
                              cudaStream_t s) {
    if (o.n == 0) return;
    DevBuf<uint32_t> unit_off((size_t)o.n + 1, s);
    scan_exclusive<uint32_t>(UnitsOf{o.len, labels}, unit_off.get(), o.n, s);
    CK(cudaMemsetAsync(c.work_counter, 0, 4, s));
    PhaseScope ph(c, labels ? "wcc_tc" : "tc");
    k_tc_units<<<152 * 4, TC_THREADS, 0, s>>>(o, labels, unit_off.get(), slot_cnt, c.work_counter);
    CK_LAUNCH("k_tc_units");
    c.launches += 3;
}

}  // namespace scd
