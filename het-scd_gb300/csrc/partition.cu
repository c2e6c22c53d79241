// Initial partition on the device (create_initial_partition,
// src/scd.cpp:113-171).
//
// The reference sorts vertices by ((cc, deg), id) descending and walks them
// sequentially: a still-unlabelled vertex opens the next label and claims its
// unlabelled neighbours.  Exact parallel form used here: a vertex is a seed iff
// no neighbour earlier in the order is a seed (the lexicographically-first
// maximal independent set of that order); a seed's label is its rank among the
// seeds; a non-seed takes the label of its earliest seed neighbour (that seed
// reached it first).  The order comes from two stable LSD radix sorts:
// (deg, id) then the cc bits (positive doubles order like their bit patterns).
// The independent set is found in rounds: an undecided vertex becomes a
// non-seed as soon as an earlier neighbour is a seed, and a seed once every
// earlier neighbour is a decided non-seed.
#include "engine.cuh"

namespace scd {

namespace {

constexpr unsigned TPB = 256;
constexpr uint8_t UNDECIDED = 0, SEED = 1, NONSEED = 2;

__global__ void k_order_keys(uint32_t n, const uint32_t *__restrict__ indices, uint64_t *keys, uint32_t *vals) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t d = indices[v + 1] - indices[v];
        keys[v] = ((uint64_t)(0xffffffffu - d) << 32) | (0xffffffffu - v);
        vals[v] = v;
    }
}

// cc = tri / (deg * (deg - 1.0)) (src/scd.cpp:129-131); key = ~bits so that
// ascending order is cc descending
__global__ void k_cc_keys(uint32_t n, const uint32_t *__restrict__ order, const uint32_t *__restrict__ indices,
                          const int32_t *__restrict__ tri, uint64_t *keys) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t v = order[i];
        const uint32_t d = indices[v + 1] - indices[v];
        const double cc = __ddiv_rn((double)tri[v], __dmul_rn((double)d, __dsub_rn((double)d, 1.0)));
        keys[i] = ~(uint64_t)__double_as_longlong(cc);
    }
}

__global__ void k_graph_keys(uint32_t n, const uint32_t *__restrict__ order, const uint32_t *__restrict__ gid,
                             uint64_t *keys) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) keys[i] = gid[order[i]];
}

// label offset of every graph: the seed rank at the graph's first position
__global__ void k_comm_off(uint32_t G, const uint32_t *__restrict__ fin_off, const uint32_t *__restrict__ rank,
                           uint32_t *comm_off) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += gridDim.x * blockDim.x)
        comm_off[g] = rank[fin_off[g]];
}

__global__ void k_positions(uint32_t n, const uint32_t *__restrict__ order, uint32_t *pos) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) pos[order[i]] = i;
}

// vertices of degree > HUB_DEG are scanned by a whole CTA (k_mis_round_hub, k_claim_hub):
// a hub has thousands of earlier neighbours, one warp would walk them one load chain at a time
constexpr uint32_t HUB_DEG = 4096, HUB_TPB = 1024;

__global__ void __launch_bounds__(TPB)
k_mis_round(uint32_t n, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ adj,
            const uint32_t *__restrict__ pos, uint8_t *state, uint32_t *undecided) {
    const int lane = threadIdx.x & 31;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += (gridDim.x * blockDim.x) >> 5) {
        if (((volatile uint8_t *)state)[v] != UNDECIDED) continue;
        const uint32_t pv = pos[v], beg = indices[v], deg = indices[v + 1] - beg;
        if (deg > HUB_DEG) continue;
        bool seed_seen = false, open = false;
        for (uint32_t i0 = 0; i0 < deg && !seed_seen; i0 += 32) {
            bool s = false, u = false;
            if (i0 + lane < deg) {
                const uint32_t w = adj[beg + i0 + lane];
                if (pos[w] < pv) {
                    const uint8_t st = ((volatile uint8_t *)state)[w];
                    s = st == SEED;
                    u = st == UNDECIDED;
                }
            }
            seed_seen = __any_sync(FULL, s);
            open = open || __any_sync(FULL, u);
        }
        if (lane == 0) {
            if (seed_seen) state[v] = NONSEED;
            else if (!open) state[v] = SEED;
            else atomicAdd(undecided, 1u);
        }
    }
}

// the same round for the hubs (list hubs[count], all of degree > HUB_DEG), one CTA each
__global__ void __launch_bounds__(HUB_TPB)
k_mis_round_hub(const uint32_t *__restrict__ hubs, uint32_t count, const uint32_t *__restrict__ indices,
                const uint32_t *__restrict__ adj, const uint32_t *__restrict__ pos, uint8_t *state,
                uint32_t *undecided) {
    for (uint32_t h = blockIdx.x; h < count; h += gridDim.x) {
        const uint32_t v = hubs[h];
        if (((volatile uint8_t *)state)[v] != UNDECIDED) continue;   // CTA-uniform
        const uint32_t pv = pos[v], beg = indices[v], deg = indices[v + 1] - beg;
        int seed_seen = 0, open = 0;
        for (uint32_t i0 = 0; i0 < deg && !seed_seen; i0 += HUB_TPB) {
            bool s = false, u = false;
            const uint32_t i = i0 + threadIdx.x;
            if (i < deg) {
                const uint32_t w = adj[beg + i];
                if (pos[w] < pv) {
                    const uint8_t st = ((volatile uint8_t *)state)[w];
                    s = st == SEED;
                    u = st == UNDECIDED;
                }
            }
            seed_seen = __syncthreads_or(s);
            open = __syncthreads_or(u) || open;
        }
        if (threadIdx.x == 0) {
            if (seed_seen) state[v] = NONSEED;
            else if (!open) state[v] = SEED;
            else atomicAdd(undecided, 1u);
        }
        __syncthreads();
    }
}

struct SeedAt {
    const uint32_t *order;
    const uint8_t *state;
    __device__ uint32_t operator[](size_t i) const { return state[order[i]] == SEED; }
};

__global__ void k_seed_labels(uint32_t n, const uint32_t *__restrict__ pos, const uint8_t *__restrict__ state,
                              const uint32_t *__restrict__ seed_rank, uint32_t *labels) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (state[v] == SEED) labels[v] = seed_rank[pos[v]];
}

__global__ void __launch_bounds__(TPB)
k_claim_labels(uint32_t n, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ adj,
               const uint32_t *__restrict__ pos, const uint8_t *__restrict__ state, uint32_t *labels) {
    const int lane = threadIdx.x & 31;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += (gridDim.x * blockDim.x) >> 5) {
        if (state[v] != NONSEED) continue;
        const uint32_t beg = indices[v], deg = indices[v + 1] - beg;
        if (deg > HUB_DEG) continue;
        uint32_t best_pos = INVALID, best = INVALID;
        for (uint32_t i = lane; i < deg; i += 32) {
            const uint32_t w = adj[beg + i];
            if (state[w] == SEED && pos[w] < best_pos) {
                best_pos = pos[w];
                best = w;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            uint32_t op = __shfl_xor_sync(FULL, best_pos, o), ob = __shfl_xor_sync(FULL, best, o);
            if (op < best_pos) {
                best_pos = op;
                best = ob;
            }
        }
        if (lane == 0) labels[v] = labels[best];
    }
}

// the earliest seed neighbour of a non-seed hub, one CTA per hub
__global__ void __launch_bounds__(HUB_TPB)
k_claim_hub(const uint32_t *__restrict__ hubs, uint32_t count, const uint32_t *__restrict__ indices,
            const uint32_t *__restrict__ adj, const uint32_t *__restrict__ pos, const uint8_t *__restrict__ state,
            uint32_t *labels) {
    __shared__ unsigned long long s_best;
    for (uint32_t h = blockIdx.x; h < count; h += gridDim.x) {
        const uint32_t v = hubs[h];
        if (state[v] != NONSEED) continue;   // CTA-uniform
        if (threadIdx.x == 0) s_best = ~0ull;
        __syncthreads();
        const uint32_t beg = indices[v], deg = indices[v + 1] - beg;
        unsigned long long best = ~0ull;   // (position, vertex) of the earliest seed neighbour
        for (uint32_t i = threadIdx.x; i < deg; i += HUB_TPB) {
            const uint32_t w = adj[beg + i];
            if (state[w] == SEED) {
                const unsigned long long key = ((unsigned long long)pos[w] << 32) | w;
                best = key < best ? key : best;
            }
        }
        if (best != ~0ull) atomicMin(&s_best, best);
        __syncthreads();
        if (threadIdx.x == 0) labels[v] = labels[(uint32_t)s_best];
        __syncthreads();
    }
}

}  // namespace

void initial_partition(Ctx &c) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    const uint32_t n = g.n;
    c.num_comms = 0;
    if (n == 0) {
        c.b.h_comm_off.assign(c.b.G + 1, 0);
        CK(cudaMemsetAsync(c.b.comm_off, 0, 4 * (c.b.G + 1), s));
        c.has_labels = true;
        return;
    }
    PhaseScope ph(c, "partition");
    DevBuf<uint64_t> keys(n, s);
    DevBuf<uint32_t> order(n, s), pos(n, s), undecided(1, s);
    k_order_keys<<<grid_for(n, TPB), TPB, 0, s>>>(n, g.indices, keys.get(), order.get());
    CK_LAUNCH("k_order_keys");
    radix_sort<uint64_t>(keys.get(), order.get(), n, 0, 64, s);
    k_cc_keys<<<grid_for(n, TPB), TPB, 0, s>>>(n, order.get(), g.indices, g.tri, keys.get());
    CK_LAUNCH("k_cc_keys");
    radix_sort<uint64_t>(keys.get(), order.get(), n, 0, 64, s);
    if (c.b.G > 1) {   // graph-major: each graph's order stays contiguous
        k_graph_keys<<<grid_for(n, TPB), TPB, 0, s>>>(n, order.get(), c.b.gid, keys.get());
        CK_LAUNCH("k_graph_keys");
        radix_sort<uint64_t>(keys.get(), order.get(), n, 0, ceil_log2(c.b.G), s);
        c.launches++;
    }
    keys.release();
    k_positions<<<grid_for(n, TPB), TPB, 0, s>>>(n, order.get(), pos.get());
    CK_LAUNCH("k_positions");
    c.launches += 3;

    DevBuf<uint8_t> state(n, s);
    CK(cudaMemsetAsync(state.get(), UNDECIDED, n, s));
    const unsigned G = grid_for((uint64_t)n * 32, TPB);
    const uint32_t *hubs = g.cls.list[DegreeClasses::K - 1];   // degree > 4096 = HUB_DEG
    const uint32_t nhubs = g.cls.count[DegreeClasses::K - 1];
    static_assert(DegreeClasses::upper[DegreeClasses::K - 2] == HUB_DEG, "hub class");
    for (int round = 0;; round++) {
        CK(cudaMemsetAsync(undecided.get(), 0, 4, s));
        if (nhubs) {
            k_mis_round_hub<<<grid_for(nhubs, 1, 152 * 2), HUB_TPB, 0, s>>>(hubs, nhubs, g.indices, g.adj, pos.get(),
                                                                         state.get(), undecided.get());
            CK_LAUNCH("k_mis_round_hub");
            c.launches++;
        }
        k_mis_round<<<G, TPB, 0, s>>>(n, g.indices, g.adj, pos.get(), state.get(), undecided.get());
        CK_LAUNCH("k_mis_round");
        c.launches++;
        uint32_t left = 0;
        CK(cudaMemcpyAsync(&left, undecided.get(), 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (left == 0) break;
        if (round > 4 * (int)n + 8) throw Error(SCD_ERR_TIMEOUT, "initial partition did not converge");
    }

    DevBuf<uint32_t> rank((size_t)n + 1, s);
    scan_exclusive<uint32_t>(SeedAt{order.get(), state.get()}, rank.get(), n, s);
    k_seed_labels<<<grid_for(n, TPB), TPB, 0, s>>>(n, pos.get(), state.get(), rank.get(), c.labels);
    CK_LAUNCH("k_seed_labels");
    k_claim_labels<<<G, TPB, 0, s>>>(n, g.indices, g.adj, pos.get(), state.get(), c.labels);
    CK_LAUNCH("k_claim_labels");
    if (nhubs) {
        k_claim_hub<<<grid_for(nhubs, 1, 152 * 2), HUB_TPB, 0, s>>>(hubs, nhubs, g.indices, g.adj, pos.get(),
                                                                 state.get(), c.labels);
        CK_LAUNCH("k_claim_hub");
        c.launches++;
    }
    c.launches += 4;
    k_comm_off<<<grid_for(c.b.G + 1, TPB), TPB, 0, s>>>(c.b.G, c.b.fin_off, rank.get(), c.b.comm_off);
    CK_LAUNCH("k_comm_off");
    c.b.h_comm_off.resize(c.b.G + 1);
    CK(cudaMemcpyAsync(c.b.h_comm_off.data(), c.b.comm_off, 4 * (c.b.G + 1), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    c.num_comms = c.b.h_comm_off[c.b.G];
    c.cur = 0;
    collect_stats(c, c.labels, c.st[0]);
    CK(cudaMemcpyAsync(c.best, c.labels, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    c.has_labels = true;
}

}  // namespace scd
