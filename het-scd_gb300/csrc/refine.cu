// One refinement iteration on the device: improve_partition
// (src/scd.cpp:221-341), collect_stats (src/scd.cpp:57-111) and compute_wcc
// (src/wcc.cpp:31-141), plus the clustering coefficient p_ext
// (src/graph.cpp:57-68).
//
// improve: for every vertex, the multiset of its neighbours' labels is reduced
// to (label, frequency) runs without sorting: degree <= 32 by one warp with
// __match_any_sync (one lane per neighbour); larger degrees by one CTA with an
// open-addressing hash table in shared memory (global memory for the few
// vertices whose table does not fit).  Each distinct label's FP64 gain is
// evaluated once; the winner is the maximal positive gain, ties to the
// smallest label, which is what the reference's ascending scan with a strict
// '>' picks (src/scd.cpp:313-316).  Labels are updated Jacobi-style
// (old labels in, new labels out).
//
// wcc: internal triangles per edge by the oriented counting kernel restricted
// to same-label triangles, per-vertex sums, per-vertex WCC terms and a
// fixed-order (deterministic) tree reduction.
#include "engine.cuh"
#include "gain.cuh"

namespace scd {

namespace {

constexpr unsigned TPB = 256;

struct Best {
    double gain;
    uint32_t label;
};

// (g1,l1) better than (g2,l2): larger gain, ties to the smaller label
__device__ __forceinline__ bool better(double g1, uint32_t l1, double g2, uint32_t l2) {
    return g1 > g2 || (g1 == g2 && l1 < l2);
}

__device__ __forceinline__ double gain_of(uint32_t l, uint32_t freq, uint32_t deg, uint32_t mine,
                                          const Stats &st, double p_ext, double alpha) {
    int size = st.sizes[l], ext = st.ext[l], in = st.intl[l] / 2;
    if (l == mine) {
        size--;
        ext += (int)(freq - (deg - freq));
        in -= (int)freq;
    }
    const double p_in = community_p_in(size, in);
    return wcc_gain(size, (int)freq, (int)deg - (int)freq, ext, p_in, p_ext, alpha);
}

// decision of src/scd.cpp:321-330
__device__ __forceinline__ uint32_t decide(double best_gain, uint32_t best_label, double remove_gain,
                                           uint32_t mine) {
    const double insert = dadd(best_gain, remove_gain);
    if (insert > remove_gain && insert > 0.0) return best_label;
    if (remove_gain > 0) return INVALID;
    return mine;
}

// ---- degree <= 32: one warp per vertex -----------------------------------

__global__ void __launch_bounds__(TPB)
k_improve_warp(const uint32_t *__restrict__ verts, uint32_t count, const uint32_t *__restrict__ indices,
               const uint32_t *__restrict__ adj, const uint32_t *__restrict__ labels, Stats st,
               const double *__restrict__ p_ext_ptr, double alpha, uint32_t *next) {
    const int lane = threadIdx.x & 31;
    const double p_ext = *p_ext_ptr;
    for (uint32_t wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < count;
         wi += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t p = verts[wi];
        const uint32_t beg = indices[p], deg = indices[p + 1] - beg;
        const uint32_t mine = labels[p];
        const uint32_t l = lane < (int)deg ? labels[adj[beg + lane]] : INVALID;
        const unsigned peers = __match_any_sync(FULL, l);
        const bool leader = l != INVALID && lane == __ffs(peers) - 1;
        double g = 0.0;
        if (leader) g = gain_of(l, __popc(peers), deg, mine, st, p_ext, alpha);
        // own community's gain -> remove gain
        const unsigned own = __ballot_sync(FULL, leader && l == mine);
        double remove_gain = 0.0;
        {
            double gm = __shfl_sync(FULL, g, own ? __ffs(own) - 1 : 0);
            if (own) remove_gain = -gm;
        }
        // arg-max over positive gains
        double bg = (leader && g > 0.0) ? g : 0.0;
        uint32_t bl = (leader && g > 0.0) ? l : INVALID;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double og = __shfl_xor_sync(FULL, bg, o);
            uint32_t ol = __shfl_xor_sync(FULL, bl, o);
            if (ol != INVALID && (bl == INVALID || better(og, ol, bg, bl))) {
                bg = og;
                bl = ol;
            }
        }
        if (lane == 0) next[p] = decide(bl == INVALID ? 0.0 : bg, bl == INVALID ? 0u : bl, remove_gain, mine);
    }
}

// ---- degree > 32: one CTA per vertex, hash table of (label, count) --------

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

template <int THREADS>
__device__ void improve_cta(uint32_t p, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ adj,
                            const uint32_t *__restrict__ labels, const Stats &st, double p_ext, double alpha,
                            uint32_t *next, uint32_t *keys, uint32_t *vals, uint32_t cap) {
    __shared__ double s_gain[THREADS / 32];
    __shared__ uint32_t s_label[THREADS / 32];
    __shared__ double s_remove;
    __shared__ int s_has_remove;
    const uint32_t beg = indices[p], deg = indices[p + 1] - beg, mine = labels[p];
    const uint32_t mask = cap - 1;
    for (uint32_t i = threadIdx.x; i < cap; i += THREADS) {
        keys[i] = INVALID;
        vals[i] = 0;
    }
    if (threadIdx.x == 0) {
        s_remove = 0.0;
        s_has_remove = 0;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < deg; i += THREADS) {
        const uint32_t l = labels[adj[beg + i]];
        if (l == INVALID) continue;
        uint32_t h = hash32(l) & mask;
        while (true) {
            uint32_t k = keys[h];
            if (k == INVALID) {
                k = atomicCAS(keys + h, INVALID, l);
                if (k == INVALID) k = l;
            }
            if (k == l) {
                atomicAdd(vals + h, 1u);
                break;
            }
            h = (h + 1) & mask;
        }
    }
    __syncthreads();
    double bg = 0.0;
    uint32_t bl = INVALID;
    for (uint32_t i = threadIdx.x; i < cap; i += THREADS) {
        const uint32_t l = keys[i];
        if (l == INVALID) continue;
        const double g = gain_of(l, vals[i], deg, mine, st, p_ext, alpha);
        if (l == mine) {
            s_remove = -g;
            s_has_remove = 1;
        }
        if (g > 0.0 && (bl == INVALID || better(g, l, bg, bl))) {
            bg = g;
            bl = l;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double og = __shfl_xor_sync(FULL, bg, o);
        uint32_t ol = __shfl_xor_sync(FULL, bl, o);
        if (ol != INVALID && (bl == INVALID || better(og, ol, bg, bl))) {
            bg = og;
            bl = ol;
        }
    }
    if ((threadIdx.x & 31) == 0) {
        s_gain[threadIdx.x >> 5] = bg;
        s_label[threadIdx.x >> 5] = bl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < THREADS / 32; w++)
            if (s_label[w] != INVALID && (bl == INVALID || better(s_gain[w], s_label[w], bg, bl))) {
                bg = s_gain[w];
                bl = s_label[w];
            }
        next[p] = decide(bl == INVALID ? 0.0 : bg, bl == INVALID ? 0u : bl, s_has_remove ? s_remove : 0.0, mine);
    }
    __syncthreads();
}

constexpr int MID_THREADS = 256;
constexpr uint32_t MID_CAP = 8192;   // shared-memory table entries (64 KB)

__global__ void __launch_bounds__(MID_THREADS)
k_improve_mid(const uint32_t *__restrict__ verts, uint32_t count, const uint32_t *__restrict__ indices,
              const uint32_t *__restrict__ adj, const uint32_t *__restrict__ labels, Stats st,
              const double *__restrict__ p_ext_ptr, double alpha, uint32_t *next) {
    extern __shared__ uint32_t smem[];
    uint32_t *keys = smem, *vals = smem + MID_CAP;
    const double p_ext = *p_ext_ptr;
    for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
        const uint32_t p = verts[i];
        const uint32_t deg = indices[p + 1] - indices[p];
        uint32_t cap = 64;
        while (cap < 2 * deg) cap <<= 1;
        improve_cta<MID_THREADS>(p, indices, adj, labels, st, p_ext, alpha, next, keys, vals, cap);
    }
}

__global__ void __launch_bounds__(MID_THREADS)
k_improve_big(const uint32_t *__restrict__ verts, uint32_t count, const uint32_t *__restrict__ indices,
              const uint32_t *__restrict__ adj, const uint32_t *__restrict__ labels, Stats st,
              const double *__restrict__ p_ext_ptr, double alpha, uint32_t *next, uint32_t *tables,
              const uint64_t *__restrict__ table_off) {
    const double p_ext = *p_ext_ptr;
    for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
        const uint32_t p = verts[i];
        const uint64_t off = table_off[i];
        const uint32_t cap = (uint32_t)((table_off[i + 1] - off) / 2);
        improve_cta<MID_THREADS>(p, indices, adj, labels, st, p_ext, alpha, next, tables + off, tables + off + cap,
                                 cap);
    }
}

// ---- collect_stats ---------------------------------------------------------

__global__ void __launch_bounds__(TPB)
k_stats(uint32_t n, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ adj,
        const uint32_t *__restrict__ labels, Stats st) {
    const int lane = threadIdx.x & 31;
    for (uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < n; p += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t l = labels[p];
        if (l == INVALID) continue;
        const uint32_t beg = indices[p], deg = indices[p + 1] - beg;
        uint32_t same = 0;
        for (uint32_t i = lane; i < deg; i += 32) same += labels[adj[beg + i]] == l;
        same = warp_sum(same);
        if (lane == 0) {
            atomicAdd(st.sizes + l, 1);
            if (deg - same) atomicAdd(st.ext + l, (int)(deg - same));
            if (same) atomicAdd(st.intl + l, (int)same);
        }
    }
}

// ---- WCC ---------------------------------------------------------------------

// per-vertex sums of the internal per-edge triangle counts
__global__ void __launch_bounds__(TPB)
k_internal_sums(uint32_t n, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ nlow,
                const uint32_t *__restrict__ adj, const uint32_t *__restrict__ cnt, int32_t *itri,
                int32_t *itdeg) {
    const int lane = threadIdx.x & 31;
    for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t beg = indices[u], len = nlow[u];
        uint32_t sum = 0, edges = 0;
        for (uint32_t i = lane; i < len; i += 32) {
            const uint32_t c = cnt[beg + i];
            if (c) {
                const uint32_t v = adj[beg + i];
                atomicAdd((uint32_t *)itri + v, c);
                atomicAdd(itdeg + v, 1);
                sum += c;
                edges++;
            }
        }
        sum = warp_sum(sum);
        edges = warp_sum(edges);
        if (lane == 0 && edges) {
            atomicAdd((uint32_t *)itri + u, sum);
            atomicAdd(itdeg + u, (int)edges);
        }
    }
}

constexpr int WCC_ITEMS = 8;
constexpr int WCC_CHUNK = TPB * WCC_ITEMS;

// WCC_p of src/wcc.cpp:129-134
__device__ __forceinline__ double wcc_term(uint32_t p, const uint32_t *labels, const Stats &st,
                                           const int32_t *tri, const int32_t *tri_deg, const int32_t *itri,
                                           const int32_t *itdeg, double alpha) {
    const uint32_t l = labels[p];
    if (l == INVALID) return 0.0;
    const int size = st.sizes[l], td = tri_deg[p];
    if (size <= 2 || td == 0) return 0.0;
    const int it = itri[p], itd = itdeg[p];
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

__global__ void __launch_bounds__(TPB)
k_wcc_partial(uint32_t n, const uint32_t *__restrict__ labels, Stats st, const int32_t *__restrict__ tri,
              const int32_t *__restrict__ tri_deg, const int32_t *__restrict__ itri,
              const int32_t *__restrict__ itdeg, double alpha, double *partial) {
    __shared__ double sh[TPB / 32];
    const uint32_t base = blockIdx.x * WCC_CHUNK + threadIdx.x * WCC_ITEMS;
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < WCC_ITEMS; i++)
        if (base + i < n) s = dadd(s, wcc_term(base + i, labels, st, tri, tri_deg, itri, itdeg, alpha));
    double r = block_sum_fixed(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

__global__ void __launch_bounds__(TPB) k_wcc_final(const double *__restrict__ partial, uint32_t parts, uint32_t n,
                                                   double *out) {
    __shared__ double sh[TPB / 32];
    double s = 0.0;
    for (uint32_t i = threadIdx.x; i < parts; i += TPB) s = dadd(s, partial[i]);
    double r = block_sum_fixed(s, sh);
    if (threadIdx.x == 0) *out = n > 0 ? ddiv(r, (double)n) : 0.0;
}

// ---- p_ext ---------------------------------------------------------------------

__global__ void k_pext_terms(uint32_t n, const uint32_t *__restrict__ indices, const int32_t *__restrict__ tri,
                             double *term) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const uint32_t d = indices[p + 1] - indices[p];
        term[p] = d > 1 ? ddiv((double)tri[p], dmul((double)d, dsub((double)d, 1.0))) : 0.0;
    }
}

// the reference's single-thread order (src/graph.cpp:59-68 at one thread):
// ((t0 + t1) + t2) + ... over vertices with degree > 1, then / n
__global__ void k_pext_sequential(uint32_t n, const uint32_t *__restrict__ indices, const double *__restrict__ term,
                                  double *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    uint32_t p = 0;
    for (; p + 8 <= n; p += 8) {
        double t[8];
        uint32_t d[9];
#pragma unroll
        for (int k = 0; k < 9; k++) d[k] = indices[p + k];
#pragma unroll
        for (int k = 0; k < 8; k++) t[k] = term[p + k];
#pragma unroll
        for (int k = 0; k < 8; k++)
            if (d[k + 1] - d[k] > 1) s = dadd(s, t[k]);
    }
    for (; p < n; p++)
        if (indices[p + 1] - indices[p] > 1) s = dadd(s, term[p]);
    *out = ddiv(s, (double)n);
}

__global__ void k_pext_tree(uint32_t n, const double *__restrict__ term, double *partial) {
    __shared__ double sh[TPB / 32];
    const uint32_t base = blockIdx.x * WCC_CHUNK + threadIdx.x * WCC_ITEMS;
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < WCC_ITEMS; i++)
        if (base + i < n) s = dadd(s, term[base + i]);
    double r = block_sum_fixed(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

}  // namespace

void collect_stats(Ctx &c, const uint32_t *labels, Stats &st) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    const size_t bytes = (size_t)(c.num_comms ? c.num_comms : 1) * 4;
    CK(cudaMemsetAsync(st.sizes, 0, bytes, s));
    CK(cudaMemsetAsync(st.ext, 0, bytes, s));
    CK(cudaMemsetAsync(st.intl, 0, bytes, s));
    if (g.n == 0) return;
    PhaseScope ph(c, "stats");
    k_stats<<<grid_for((uint64_t)g.n * 32, TPB), TPB, 0, s>>>(g.n, g.indices, g.adj, labels, st);
    CK_LAUNCH("k_stats");
    c.launches += 1;
}

void improve(Ctx &c, const uint32_t *labels, const Stats &st, uint32_t *next) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    if (g.n == 0) return;
    PhaseScope ph(c, "improve");
    if (g.n_small) {
        k_improve_warp<<<grid_for((uint64_t)g.n_small * 32, TPB), TPB, 0, s>>>(
            g.cls_small, g.n_small, g.indices, g.adj, labels, st, g.p_ext_dev, c.alpha, next);
        CK_LAUNCH("k_improve_warp");
        c.launches++;
    }
    if (g.n_mid) {
        const size_t smem = 2 * MID_CAP * sizeof(uint32_t);
        CK(cudaFuncSetAttribute((const void *)k_improve_mid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_improve_mid<<<grid_for(g.n_mid, 1, 152 * 3), MID_THREADS, smem, s>>>(
            g.cls_mid, g.n_mid, g.indices, g.adj, labels, st, g.p_ext_dev, c.alpha, next);
        CK_LAUNCH("k_improve_mid");
        c.launches++;
    }
    if (g.n_big) {
        k_improve_big<<<grid_for(g.n_big, 1, 152 * 2), MID_THREADS, 0, s>>>(
            g.cls_big, g.n_big, g.indices, g.adj, labels, st, g.p_ext_dev, c.alpha, next, c.big_tables,
            g.big_table_off);
        CK_LAUNCH("k_improve_big");
        c.launches++;
    }
}

void launch_wcc(Ctx &c, const uint32_t *labels, const Stats &st) {
    const Graph &g = c.g;
    cudaStream_t s = c.stream;
    if (g.n == 0) {
        CK(cudaMemsetAsync(c.wcc_sum, 0, sizeof(double), s));
        return;
    }
    PhaseScope ph(c, "wcc");
    CK(cudaMemsetAsync(c.slot_cnt, 0, 2 * (size_t)g.m * 4, s));
    CK(cudaMemsetAsync(c.itri, 0, (size_t)g.n * 4, s));
    CK(cudaMemsetAsync(c.itdeg, 0, (size_t)g.n * 4, s));
    Oriented o{g.indices, g.nlow, g.adj, g.n};
    count_oriented_triangles(c, o, labels, c.slot_cnt, s);
    k_internal_sums<<<grid_for((uint64_t)g.n * 32, TPB), TPB, 0, s>>>(g.n, g.indices, g.nlow, g.adj, c.slot_cnt,
                                                                     c.itri, c.itdeg);
    CK_LAUNCH("k_internal_sums");
    const uint32_t parts = (g.n + WCC_CHUNK - 1) / WCC_CHUNK;
    k_wcc_partial<<<parts, TPB, 0, s>>>(g.n, labels, st, g.tri, g.tri_deg, c.itri, c.itdeg, c.alpha, c.wcc_part);
    CK_LAUNCH("k_wcc_partial");
    k_wcc_final<<<1, TPB, 0, s>>>(c.wcc_part, parts, g.n, c.wcc_sum);
    CK_LAUNCH("k_wcc_final");
    c.launches += 3;
}

double compute_wcc(Ctx &c, const uint32_t *labels, const Stats &st) {
    launch_wcc(c, labels, st);
    CK(cudaMemcpyAsync(c.wcc_host, c.wcc_sum, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return *c.wcc_host;
}

void compute_p_ext(Ctx &c) {
    Graph &g = c.g;
    cudaStream_t s = c.stream;
    if (g.n == 0) {
        const double nan = 0.0 / 0.0;
        CK(cudaMemcpyAsync(g.p_ext_dev, &nan, sizeof(double), cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
        g.p_ext = nan;
        return;
    }
    DevBuf<double> term(g.n, s);
    k_pext_terms<<<grid_for(g.n, TPB), TPB, 0, s>>>(g.n, g.indices, g.tri, term.get());
    CK_LAUNCH("k_pext_terms");
    if (c.flags & SCD_FLAG_PEXT_TREE) {
        const uint32_t parts = (g.n + WCC_CHUNK - 1) / WCC_CHUNK;
        DevBuf<double> part(parts, s);
        k_pext_tree<<<parts, TPB, 0, s>>>(g.n, term.get(), part.get());
        CK_LAUNCH("k_pext_tree");
        k_wcc_final<<<1, TPB, 0, s>>>(part.get(), parts, g.n, g.p_ext_dev);
        CK_LAUNCH("k_wcc_final");
        c.launches += 2;
    } else {
        k_pext_sequential<<<1, 32, 0, s>>>(g.n, g.indices, term.get(), g.p_ext_dev);
        CK_LAUNCH("k_pext_sequential");
        c.launches += 1;
    }
    c.launches += 1;
    CK(cudaMemcpyAsync(&g.p_ext, g.p_ext_dev, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
}

}  // namespace scd
