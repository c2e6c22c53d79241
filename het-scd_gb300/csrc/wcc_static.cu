// scd_wcc_static: the WCC of a labelling (src/wcc.cpp:31-141) for callers that
// must not allocate device memory.
//
// Who needs it: code that runs inside a host that owns all device memory —
// a serving process whose pool has already reserved the free HBM, a plugin
// host whose allocator accounting must not be bypassed, or a latency-critical
// loop that cannot afford the device-wide synchronisation cudaFree implies.
// Such callers hold the graph, the labels and the community sizes in their
// own buffers and cannot let the library call cudaMalloc.
//
// The only scratch is two file-scope __device__ arrays, held by every GPU that
// loads the library until the process exits: the per-block partial sums of the
// fixed-order reduction, sized for SCD_WCC_STATIC_MAX_VERTICES vertices (64 KB),
// and the internal-triangle counts of hub rows (131072 x 8 B = 1 MB).  All calls
// share them: calls that overlap on the GPU race on them, so a caller must order
// them (same stream, or events).  Every call overwrites the partials it reads and
// clears the hub counts before it adds to them.
//
// The per-vertex terms and the summation order are those of the engine's
// scd_compute_wcc (blocks of 2048 vertices, 8 consecutive vertices per
// thread, warp then block tree), so both entry points give the same value.
#include <mutex>

#include "engine.cuh"
#include "gain.cuh"

namespace scd {

namespace {

constexpr int TPB = 256;
constexpr int ITEMS = 8;
constexpr int CHUNK = TPB * ITEMS;   // vertices per block
constexpr uint32_t MAX_PARTS = SCD_WCC_STATIC_MAX_VERTICES / CHUNK;

static __device__ __align__(256) double g_wcc_partials[MAX_PARTS];

// Hub rows: a vertex p < HUB_MAX of degree > HUB_DEG has its neighbour pairs spread
// over HUB_CHUNKS CTAs (one warp per vertex would serialise a whole block on it; in
// `convert`'s graphs ids are degree ranks, so the hubs are the first vertices); its
// internal-triangle count and triangle degree are summed into g_hub_acc[p] as
// (count << 32) | degree with 64-bit atomics (integers: the order of the additions
// does not matter), and the partial kernel reads them back.  Hubs with ids beyond
// HUB_MAX take the warp path (same value, slower).
constexpr uint32_t HUB_DEG = 128, HUB_MAX = 131072, HUB_CHUNKS = 16;
static __device__ __align__(256) unsigned long long g_hub_acc[HUB_MAX];

// |{r in adj(p) ∩ adj(q) : label(r) == l}|, searching the shorter row in the longer
__device__ uint32_t common_same_label(const uint32_t *__restrict__ adj, uint32_t bp, uint32_t ep, uint32_t bq,
                                      uint32_t eq, const uint32_t *__restrict__ labels, uint32_t l) {
    if (ep - bp > eq - bq) {
        uint32_t t = bp; bp = bq; bq = t;
        t = ep; ep = eq; eq = t;
    }
    uint32_t c = 0;
    for (uint32_t i = bp; i < ep; i++) {
        const uint32_t r = adj[i];
        if (labels[r] != l) continue;
        const uint32_t k = lower_bound(adj + bq, eq - bq, r);
        c += (k < eq - bq && adj[bq + k] == r);
    }
    return c;
}

// one CTA per (hub p, piece); a warp per internal neighbour q of p, its lanes
// taking the entries of the shorter of the two rows (a pair of hubs is too long
// for one thread), pieces taking every HUB_CHUNKS-th run of warps' neighbours
__global__ void __launch_bounds__(TPB)
k_wcc_static_hubs(uint32_t n, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ adj,
                  const int32_t *__restrict__ tri_deg, const uint32_t *__restrict__ labels,
                  const int32_t *__restrict__ sizes, unsigned long long *acc) {
    constexpr uint32_t WARPS = TPB / 32;
    __shared__ uint32_t s_it[WARPS], s_itd[WARPS];
    const uint32_t p = blockIdx.x;   // (grid x: up to 2^31-1 blocks; y and z stop at 65535)
    if (p >= n) return;
    const uint32_t bp = indices[p], ep = indices[p + 1];
    if (ep - bp <= HUB_DEG) return;
    const uint32_t l = labels[p];
    if (l == INVALID || sizes[l] <= 2 || tri_deg[p] == 0) return;   // its term is 0 without the counts
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t it = 0, itd = 0;
    for (uint32_t i = bp + blockIdx.y * WARPS + warp; i < ep; i += HUB_CHUNKS * WARPS) {
        const uint32_t q = adj[i];
        if (labels[q] != l) continue;   // the same q for the whole warp
        uint32_t sb = bp, se = ep, gb = indices[q], ge = indices[q + 1];
        if (se - sb > ge - gb) {
            uint32_t t = sb; sb = gb; gb = t;
            t = se; se = ge; ge = t;
        }
        uint32_t c = 0;
        for (uint32_t j = sb + lane; j < se; j += 32) {
            const uint32_t r = adj[j];
            if (labels[r] != l) continue;
            const uint32_t k = lower_bound(adj + gb, ge - gb, r);
            c += (k < ge - gb && adj[gb + k] == r);
        }
        c = warp_sum(c);
        it += c;
        itd += c > 0;
    }
    if (lane == 0) {
        s_it[warp] = it;
        s_itd[warp] = itd;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t a = 0, b = 0;
        for (uint32_t w = 0; w < WARPS; w++) {
            a += s_it[w];
            b += s_itd[w];
        }
        if (a || b) atomicAdd(acc + p, ((unsigned long long)a << 32) | b);
    }
}

__global__ void __launch_bounds__(TPB)
k_wcc_static_partial(uint32_t n, const uint32_t *__restrict__ indices, const uint32_t *__restrict__ adj,
                     const int32_t *__restrict__ tri, const int32_t *__restrict__ tri_deg,
                     const uint32_t *__restrict__ labels, const int32_t *__restrict__ sizes, double alpha,
                     double *partials, const unsigned long long *__restrict__ hub_acc) {
    __shared__ double terms[CHUNK];
    __shared__ double sh[TPB / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t base = blockIdx.x * CHUNK;
    // terms of this block's vertices, one warp per vertex
    for (int k = warp; k < CHUNK; k += TPB / 32) {
        const uint32_t p = base + k;
        double term = 0.0;
        if (p < n) {
            const uint32_t l = labels[p];
            const int size = l != INVALID ? sizes[l] : 0;
            const int td = tri_deg[p];
            if (l != INVALID && size > 2 && td != 0) {
                const uint32_t bp = indices[p], ep = indices[p + 1];
                uint32_t it = 0, itd = 0;
                if (p < HUB_MAX && ep - bp > HUB_DEG) {   // counted by k_wcc_static_hubs
                    const unsigned long long h = hub_acc[p];
                    it = (uint32_t)(h >> 32);
                    itd = (uint32_t)h;
                } else {
                    for (uint32_t i = bp + lane; i < ep; i += 32) {
                        const uint32_t q = adj[i];
                        if (labels[q] != l) continue;
                        const uint32_t c = common_same_label(adj, bp, ep, indices[q], indices[q + 1], labels, l);
                        it += c;
                        itd += c > 0;
                    }
                    it = warp_sum(it);
                    itd = warp_sum(itd);
                }
                const double nom = (double)imul_wrap((int)it, td);
                const double den = dmul((double)tri[p], dadd((double)td, dmul(alpha, (double)(size - 1 - (int)itd))));
                term = den != 0.0 ? ddiv(nom, den) : 0.0;
            }
        }
        if (lane == 0) terms[k] = term;
    }
    __syncthreads();
    // the engine's order: 8 consecutive terms per thread, then the block tree
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
        if (base + threadIdx.x * ITEMS + i < n) s = dadd(s, terms[threadIdx.x * ITEMS + i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = dadd(s, __shfl_xor_sync(FULL, s, o));
    if (lane == 0) sh[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < TPB / 32; w++) r = dadd(r, sh[w]);
        partials[blockIdx.x] = r;
    }
}

__global__ void __launch_bounds__(TPB)
k_wcc_static_final(const double *__restrict__ partials, uint32_t parts, uint32_t n, double *out) {
    __shared__ double sh[TPB / 32];
    double s = 0.0;
    for (uint32_t i = threadIdx.x; i < parts; i += TPB) s = dadd(s, partials[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = dadd(s, __shfl_xor_sync(FULL, s, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < TPB / 32; w++) r = dadd(r, sh[w]);
        *out = n > 0 ? ddiv(r, (double)n) : 0.0;
    }
}

// device address of g_wcc_partials per device: set up by the first call on a
// device, refreshed by every call made outside a stream capture (a device reset
// or a new primary context reloads the module and moves the array), reused as is
// by calls made while the stream is being captured
constexpr int MAX_DEVICES = 64;
std::mutex g_setup_lock;
double *g_partials_addr[MAX_DEVICES] = {};
unsigned long long *g_hub_addr[MAX_DEVICES] = {};

}  // namespace
}  // namespace scd

using namespace scd;

extern "C" int scd_wcc_static(const uint32_t *indices, const uint32_t *adj, const int32_t *tri,
                              const int32_t *tri_deg, const uint32_t *labels, const int32_t *sizes, uint32_t n,
                              double alpha, double *wcc, void *stream) {
    if (n > SCD_WCC_STATIC_MAX_VERTICES) return SCD_ERR_LIMIT;
    if (!indices || !wcc || (n && (!adj || !tri || !tri_deg || !labels || !sizes))) return SCD_ERR_ARG;
    // an error already pending on this thread belongs to the caller: report it
    // without clearing it, and without launching anything
    if (cudaPeekAtLastError() != cudaSuccess) return SCD_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return SCD_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return SCD_ERR_CUDA;
    double *partials = nullptr;
    unsigned long long *hub_acc = nullptr;
    {
        std::lock_guard<std::mutex> hold(g_setup_lock);
        if (cap == cudaStreamCaptureStatusNone || !g_partials_addr[dev]) {
            // a host-side lookup of the array's device address; the first call on
            // a device must not be made while its stream is being captured
            if (cap != cudaStreamCaptureStatusNone) return SCD_ERR_STATE;
            void *p = nullptr, *h = nullptr;
            if (cudaGetSymbolAddress(&p, g_wcc_partials) != cudaSuccess || !p) return SCD_ERR_CUDA;
            if (cudaGetSymbolAddress(&h, g_hub_acc) != cudaSuccess || !h) return SCD_ERR_CUDA;
            g_partials_addr[dev] = (double *)p;
            g_hub_addr[dev] = (unsigned long long *)h;
        }
        partials = g_partials_addr[dev];
        hub_acc = g_hub_addr[dev];
    }
    const uint32_t parts = n ? (n + CHUNK - 1) / CHUNK : 0;
    if (parts) {
        // the hub counts start from zero on every call (the array keeps the last call's)
        const uint32_t hubs = n < HUB_MAX ? n : HUB_MAX;
        if (cudaMemsetAsync(hub_acc, 0, sizeof(unsigned long long) * hubs, s) != cudaSuccess) return SCD_ERR_CUDA;
        k_wcc_static_hubs<<<dim3(hubs, HUB_CHUNKS), TPB, 0, s>>>(n, indices, adj, tri_deg, labels, sizes, hub_acc);
        if (cudaGetLastError() != cudaSuccess) return SCD_ERR_CUDA;
        k_wcc_static_partial<<<parts, TPB, 0, s>>>(n, indices, adj, tri, tri_deg, labels, sizes, alpha, partials,
                                                   hub_acc);
        if (cudaGetLastError() != cudaSuccess) return SCD_ERR_CUDA;
    }
    k_wcc_static_final<<<1, TPB, 0, s>>>(partials, parts, n, wcc);
    return cudaGetLastError() == cudaSuccess ? SCD_OK : SCD_ERR_CUDA;
}
