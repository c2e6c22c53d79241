// Row-wise CSR construction for the preprocessing (src/convert.cpp:252-268 and
// 417-455: sort, de-duplicate, write both directions with sorted rows).
//
// Instead of one global sort of 64-bit (row, value) keys, whose every radix
// pass moves every entry, the entries are placed by a counting sort on the row
// (row lengths, offsets, one scatter) and then every row is sorted on its own:
//   rows of length <= 512     a warp, bitonic network in registers and
//                             shuffles (1, 2, 4, 8 or 16 values per lane);
//   513 .. 4096, .. 16384     a CTA, 8 or 16 values per thread: the stages
//                             whose partner is in the same warp in registers
//                             and shuffles, the cross-warp ones in shared memory;
//   longer rows               one radix sort of (row rank, value) keys.
// With de-duplication a repeated value of a row becomes INVALID and the number
// of distinct values of the row is written out; the caller compacts.
#include "engine.cuh"

namespace scd {

namespace {

constexpr unsigned TPB = 256;
constexpr uint32_t WARP_ROW = 32, MID_ROW = 512, BIG_ROW = 4096, HUGE_ROW = 16384;

__device__ __forceinline__ uint32_t bitonic32(uint32_t v, int lane) {
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const uint32_t o = __shfl_xor_sync(FULL, v, j);
            const bool asc = (lane & k) == 0, low = (lane & j) == 0;
            v = (low == asc) ? min(v, o) : max(v, o);
        }
    }
    return v;
}

// every row of length <= 32: one warp per row
__global__ void __launch_bounds__(TPB)
k_sort_rows_warp(const uint32_t *__restrict__ off, uint32_t nrows, uint32_t *vals, bool dedup, uint32_t *udeg) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nrows; r += warps) {
        const uint32_t beg = off[r], len = off[r + 1] - beg;
        if (len > WARP_ROW) continue;
        uint32_t v = (uint32_t)lane < len ? vals[beg + lane] : INVALID;
        v = bitonic32(v, lane);
        const uint32_t prev = __shfl_up_sync(FULL, v, 1);
        const bool in = (uint32_t)lane < len;
        const bool keep = in && (!dedup || lane == 0 || v != prev);
        if (in) vals[beg + lane] = keep ? v : INVALID;
        const unsigned kb = __ballot_sync(FULL, keep);
        if (udeg && lane == 0) udeg[r] = __popc(kb);
    }
}

// rows of one list with 32 < len <= 32 * E: one warp per row, E values per lane
// (value index = lane * E + i), bitonic network in registers
template <int E>
__global__ void __launch_bounds__(TPB)
k_sort_rows_warp_e(const uint32_t *__restrict__ list, uint32_t count, const uint32_t *__restrict__ off, uint32_t *vals,
                   bool dedup, uint32_t *udeg) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < count; w += warps) {
        const uint32_t r = list[w], beg = off[r], len = off[r + 1] - beg;
        uint32_t v[E];
#pragma unroll
        for (int i = 0; i < E; i++) {
            const uint32_t idx = lane * E + i;
            v[i] = idx < len ? vals[beg + idx] : INVALID;
        }
#pragma unroll
        for (int k = 2; k <= 32 * E; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                if (j >= E) {   // partner in lane ^ (j / E)
#pragma unroll
                    for (int i = 0; i < E; i++) {
                        const int idx = lane * E + i;
                        const uint32_t o = __shfl_xor_sync(FULL, v[i], j / E);
                        const bool asc = (idx & k) == 0, low = (idx & j) == 0;
                        v[i] = (low == asc) ? min(v[i], o) : max(v[i], o);
                    }
                } else {        // partner in this lane: i ^ j
#pragma unroll
                    for (int i = 0; i < E; i++) {
                        const int q = i ^ j;
                        if (q > i) {
                            const bool asc = ((lane * E + i) & k) == 0;
                            const uint32_t x = v[i], y = v[q];
                            if ((x > y) == asc) {
                                v[i] = y;
                                v[q] = x;
                            }
                        }
                    }
                }
            }
        }
        const uint32_t last_prev = __shfl_up_sync(FULL, v[E - 1], 1);
        uint32_t kept = 0;
#pragma unroll
        for (int i = 0; i < E; i++) {
            const uint32_t idx = lane * E + i;
            const uint32_t prev = i ? v[i - 1] : last_prev;
            const bool keep = idx < len && (!dedup || idx == 0 || v[i] != prev);
            if (idx < len) vals[beg + idx] = keep ? v[i] : INVALID;
            kept += keep;
        }
        kept = warp_sum(kept);
        if (udeg && lane == 0) udeg[r] = kept;
    }
}

// rows of one list, one CTA of W warps per row, E values per thread in index
// order (value index = threadIdx.x * E + i); bitonic network over the next power
// of two P >= len: stages with partner distance j < E in registers, E <= j < 32E
// by shuffles, j >= 32E through shared memory (pairs enumerated directly)
template <int W, int E>
__global__ void __launch_bounds__(W * 32)
k_sort_rows_cta(const uint32_t *__restrict__ list, uint32_t count, const uint32_t *__restrict__ off, uint32_t *vals,
                bool dedup, uint32_t *udeg) {
    constexpr int THREADS = W * 32;
    constexpr uint32_t WSPAN = 32u * E;
    extern __shared__ uint32_t sh[];   // THREADS * E values
    __shared__ uint32_t wsum[W];
    const uint32_t base = threadIdx.x * E;
    for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
        const uint32_t r = list[i], beg = off[r], len = off[r + 1] - beg;
        uint32_t P = WSPAN;
        while (P < len) P <<= 1;
        for (uint32_t t = threadIdx.x; t < P; t += THREADS) sh[t] = t < len ? vals[beg + t] : INVALID;
        __syncthreads();
        uint32_t v[E];
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = base + e < P ? sh[base + e] : INVALID;
        const bool live = base < P;   // warp-uniform: P is a multiple of the warp span
        for (uint32_t k = 2; k <= P; k <<= 1) {
            if (k > WSPAN) {   // distances j >= 32E: shared memory
                __syncthreads();
#pragma unroll
                for (int e = 0; e < E; e++)
                    if (live) sh[base + e] = v[e];
                __syncthreads();
                for (uint32_t j = k >> 1; j >= WSPAN; j >>= 1) {
                    for (uint32_t q = threadIdx.x; q < P / 2; q += THREADS) {
                        const uint32_t t = ((q & ~(j - 1)) << 1) | (q & (j - 1)), x = t | j;
                        const uint32_t a = sh[t], b = sh[x];
                        if ((a > b) == ((t & k) == 0)) {
                            sh[t] = b;
                            sh[x] = a;
                        }
                    }
                    __syncthreads();
                }
#pragma unroll
                for (int e = 0; e < E; e++)
                    if (live) v[e] = sh[base + e];
            }
            if (!live) continue;
#pragma unroll
            for (int j = 16 * E; j >= E; j >>= 1) {   // partner in lane ^ (j / E)
                if ((uint32_t)j >= k) continue;
#pragma unroll
                for (int e = 0; e < E; e++) {
                    const uint32_t idx = base + e;
                    const uint32_t o = __shfl_xor_sync(FULL, v[e], j / E);
                    const bool asc = (idx & k) == 0, low = (idx & j) == 0;
                    v[e] = (low == asc) ? min(v[e], o) : max(v[e], o);
                }
            }
#pragma unroll
            for (int j = E / 2; j > 0; j >>= 1) {    // partner in this thread: e ^ j
                if ((uint32_t)j >= k) continue;
#pragma unroll
                for (int e = 0; e < E; e++) {
                    const int q = e ^ j;
                    if (q > e) {
                        const bool asc = ((base + e) & k) == 0;
                        const uint32_t x = v[e], y = v[q];
                        if ((x > y) == asc) {
                            v[e] = y;
                            v[q] = x;
                        }
                    }
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < E; e++)
            if (live) sh[base + e] = v[e];
        __syncthreads();
        uint32_t kept = 0;
        for (uint32_t t = threadIdx.x; t < len; t += THREADS) {
            const uint32_t v = sh[t];
            const bool keep = !dedup || t == 0 || v != sh[t - 1];
            vals[beg + t] = keep ? v : INVALID;
            kept += keep;
        }
        kept = warp_sum(kept);
        if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = kept;
        __syncthreads();
        if (threadIdx.x == 0 && udeg) {
            uint32_t tot = 0;
            for (int w = 0; w < THREADS / 32; w++) tot += wsum[w];
            udeg[r] = tot;
        }
        __syncthreads();
    }
}

struct RowLenIn {
    const uint32_t *off;
    uint32_t lo, hi;   // lo < len <= hi
    __device__ uint32_t operator[](size_t r) const {
        const uint32_t len = off[r + 1] - off[r];
        return len > lo && len <= hi;
    }
};

__global__ void k_row_scatter(uint32_t nrows, RowLenIn f, const uint32_t *__restrict__ pos, uint32_t *list) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x)
        if (f[r]) list[pos[r]] = r;
}

struct RowLenOf {
    const uint32_t *list, *off;
    __device__ uint32_t operator[](size_t i) const { return off[list[i] + 1] - off[list[i]]; }
};

// long rows: key = (rank of the row in the list) << 32 | value
__global__ void k_big_keys(const uint32_t *__restrict__ list, uint32_t count, const uint32_t *__restrict__ off,
                           const uint32_t *__restrict__ koff, const uint32_t *__restrict__ vals, uint64_t *keys) {
    for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
        const uint32_t r = list[i], beg = off[r], len = off[r + 1] - beg, k0 = koff[i];
        for (uint32_t t = threadIdx.x; t < len; t += blockDim.x) keys[k0 + t] = ((uint64_t)i << 32) | vals[beg + t];
    }
}

__global__ void k_big_back(const uint64_t *__restrict__ keys, uint32_t total, const uint32_t *__restrict__ list,
                           const uint32_t *__restrict__ off, const uint32_t *__restrict__ koff, uint32_t *vals,
                           bool dedup, uint32_t *udeg) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
        const uint64_t key = keys[p];
        const uint32_t i = (uint32_t)(key >> 32), v = (uint32_t)key;
        const uint32_t t = p - koff[i], r = list[i];
        const bool keep = !dedup || t == 0 || (uint32_t)keys[p - 1] != v;
        vals[off[r] + t] = keep ? v : INVALID;
        if (udeg) {
            const unsigned peers = __match_any_sync(__activemask(), i);
            const unsigned kb = __ballot_sync(__activemask(), keep) & peers;
            if ((threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1) && kb) atomicAdd(udeg + r, (uint32_t)__popc(kb));
        }
    }
}

__global__ void k_zero_rows(const uint32_t *__restrict__ list, uint32_t count, uint32_t *udeg) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) udeg[list[i]] = 0;
}

void prepare_sort_kernels() {
    static thread_local int done_device = -1;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (done_device == dev) return;
    CK(cudaFuncSetAttribute((const void *)k_sort_rows_cta<32, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)(HUGE_ROW * 4)));
    done_device = dev;
}

}  // namespace

void sort_rows(Ctx &c, const uint32_t *off, uint32_t nrows, uint32_t *vals, bool dedup, uint32_t *udeg,
               cudaStream_t s) {
    if (nrows == 0) return;
    k_sort_rows_warp<<<grid_for((uint64_t)nrows * 32, TPB), TPB, 0, s>>>(off, nrows, vals, dedup, udeg);
    CK_LAUNCH("k_sort_rows_warp");
    c.launches++;
    // the longer rows, listed by length class (one host read for all the counts)
    constexpr int NC = 8;
    const uint32_t bounds[NC + 1] = {WARP_ROW, 64, 128, 256, MID_ROW, BIG_ROW, HUGE_ROW, 0xffffffffu};
    prepare_sort_kernels();
    DevBuf<uint32_t> pos[NC];
    for (int k = 0; k < NC; k++) {
        pos[k].alloc((size_t)nrows + 1, s);
        scan_exclusive<uint32_t>(RowLenIn{off, bounds[k], bounds[k + 1]}, pos[k].get(), nrows, s);
    }
    uint32_t cnt[NC];
    for (int k = 0; k < NC; k++) CK(cudaMemcpyAsync(cnt + k, pos[k].get() + nrows, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    DevBuf<uint32_t> list[NC];
    for (int k = 0; k < NC; k++) {
        if (!cnt[k]) continue;
        list[k].alloc(cnt[k], s);
        k_row_scatter<<<grid_for(nrows, TPB), TPB, 0, s>>>(nrows, RowLenIn{off, bounds[k], bounds[k + 1]},
                                                          pos[k].get(), list[k].get());
        CK_LAUNCH("k_row_scatter");
        c.launches++;
    }
    if (cnt[0]) {
        k_sort_rows_warp_e<2><<<grid_for((uint64_t)cnt[0] * 32, TPB), TPB, 0, s>>>(list[0].get(), cnt[0], off, vals,
                                                                                dedup, udeg);
        CK_LAUNCH("k_sort_rows_warp64");
        c.launches++;
    }
    if (cnt[1]) {
        k_sort_rows_warp_e<4><<<grid_for((uint64_t)cnt[1] * 32, TPB), TPB, 0, s>>>(list[1].get(), cnt[1], off, vals,
                                                                                dedup, udeg);
        CK_LAUNCH("k_sort_rows_warp128");
        c.launches++;
    }
    if (cnt[2]) {
        k_sort_rows_warp_e<8><<<grid_for((uint64_t)cnt[2] * 32, TPB), TPB, 0, s>>>(list[2].get(), cnt[2], off, vals,
                                                                                dedup, udeg);
        CK_LAUNCH("k_sort_rows_warp256");
        c.launches++;
    }
    if (cnt[3]) {
        k_sort_rows_warp_e<16><<<grid_for((uint64_t)cnt[3] * 32, TPB), TPB, 0, s>>>(list[3].get(), cnt[3], off, vals,
                                                                                 dedup, udeg);
        CK_LAUNCH("k_sort_rows_warp512");
        c.launches++;
    }
    if (cnt[4]) {
        k_sort_rows_cta<16, 8><<<grid_for(cnt[4], 1, 152 * 4), 512, BIG_ROW * 4, s>>>(list[4].get(), cnt[4], off, vals,
                                                                                    dedup, udeg);
        CK_LAUNCH("k_sort_rows_cta4096");
        c.launches++;
    }
    if (cnt[5]) {
        k_sort_rows_cta<32, 16><<<grid_for(cnt[5], 1, 152 * 2), 1024, HUGE_ROW * 4, s>>>(list[5].get(), cnt[5], off,
                                                                                      vals, dedup, udeg);
        CK_LAUNCH("k_sort_rows_cta16384");
        c.launches++;
    }
    if (cnt[6]) {
        DevBuf<uint32_t> koff((size_t)cnt[6] + 1, s);
        scan_exclusive<uint32_t>(RowLenOf{list[6].get(), off}, koff.get(), cnt[6], s);
        uint32_t total = 0;
        CK(cudaMemcpyAsync(&total, koff.get() + cnt[6], 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        DevBuf<uint64_t> keys(total, s);
        k_big_keys<<<grid_for(cnt[6], 1, 152 * 8), TPB, 0, s>>>(list[6].get(), cnt[6], off, koff.get(), vals,
                                                               keys.get());
        CK_LAUNCH("k_big_keys");
        radix_sort<uint64_t>(keys.get(), nullptr, total, 0, 32 + ceil_log2(cnt[6] < 2 ? 2 : cnt[6]), s);
        if (udeg) {
            k_zero_rows<<<grid_for(cnt[6], TPB), TPB, 0, s>>>(list[6].get(), cnt[6], udeg);
            CK_LAUNCH("k_zero_rows");
        }
        k_big_back<<<grid_for(total, TPB), TPB, 0, s>>>(keys.get(), total, list[6].get(), off, koff.get(), vals,
                                                        dedup, udeg);
        CK_LAUNCH("k_big_back");
        c.launches += 3;
    }
}

}  // namespace scd
