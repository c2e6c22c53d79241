// Device-wide building blocks written for this engine (no CUB/moderngpu):
// exclusive scan, stable LSD radix sort of 32/64-bit keys with optional
// 32-bit payloads, max-reduce, and stream-ordered temporary buffers.
//
// These replace the moderngpu primitives the reference GPU path calls
// (Scan, SegSortKeysFromIndices, ReduceByKey, Reduce; src/cuda.cu:205-345).
#pragma once

#include "common.cuh"

namespace scd {

// ---------------------------------------------------------------------------
// stream-ordered temporary device buffer

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    DevBuf() = default;
    DevBuf(size_t count, cudaStream_t stream) { alloc(count, stream); }
    void alloc(size_t count, cudaStream_t stream) {
        release();
        s = stream;
        n = count;
        if (count) CK(cudaMallocAsync((void **)&p, count * sizeof(T), stream));
    }
    void release() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { release(); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        release();
        p = o.p; n = o.n; s = o.s;
        o.p = nullptr; o.n = 0;
        return *this;
    }
    T *get() const { return p; }
};

// ---------------------------------------------------------------------------
// exclusive scan: out[0..n] with out[n] = total (n+1 outputs)

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *total, T *smem_warp /*[8]*/) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T inc = warp_inclusive_scan(v);
    if (lane == 31) smem_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < (SCAN_THREADS / 32) ? smem_warp[lane] : T(0);
        T wi = warp_inclusive_scan(w);
        if (lane < (SCAN_THREADS / 32)) smem_warp[lane] = wi - w;
        if (lane == (SCAN_THREADS / 32) - 1) smem_warp[SCAN_THREADS / 32] = wi;
    }
    __syncthreads();
    T res = smem_warp[warp] + inc - v;
    *total = smem_warp[SCAN_THREADS / 32];
    __syncthreads();
    return res;
}

template <typename T, typename In>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(In in, size_t n, T *out, T *tile_sums) {
    __shared__ T sw[SCAN_THREADS / 32 + 1];
    const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
    T v[SCAN_ITEMS];
    T sum = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        size_t idx = base + i;
        v[i] = idx < n ? T(in[idx]) : T(0);
        sum += v[i];
    }
    T total;
    T run = block_exclusive_scan(sum, &total, sw);
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        size_t idx = base + i;
        if (idx <= n) out[idx] = run;
        run += v[i];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

template <typename T>
__global__ void k_scan_add(T *out, size_t n, const T *tile_offsets) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i <= n; i += stride) out[i] += tile_offsets[i / SCAN_TILE];
}

// in may be a pointer or any functor-like indexable; out must hold n+1 entries.
template <typename T, typename In>
void scan_exclusive(In in, T *out, size_t n, cudaStream_t s) {
    size_t tiles = (n + 1 + SCAN_TILE - 1) / SCAN_TILE;
    DevBuf<T> sums(tiles + 1, s);
    k_scan_tiles<T, In><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n, out, sums.get());
    CK_LAUNCH("k_scan_tiles");
    if (tiles > 1) {
        DevBuf<T> offs(tiles + 1, s);
        scan_exclusive<T, const T *>(sums.get(), offs.get(), tiles, s);
        k_scan_add<T><<<grid_for(n + 1, 256), 256, 0, s>>>(out, n, offs.get());
        CK_LAUNCH("k_scan_add");
    }
}

// ---------------------------------------------------------------------------
// reductions

template <typename T>
__global__ void k_reduce_max(const T *in, size_t n, T *out) {
    T m = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        m = in[i] > m ? in[i] : m;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T u = __shfl_xor_sync(FULL, m, o);
        m = u > m ? u : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// ---------------------------------------------------------------------------
// stable LSD radix sort, 8-bit digits, reduce-then-scan per pass.
//
// A tile is RS_WARPS*32*RS_ITEMS keys; warp w of a tile owns the contiguous
// run [w*32*RS_ITEMS, (w+1)*32*RS_ITEMS) and walks it 32 keys at a time, so
// (step, lane) order equals input order and __match_any_sync ranking keeps the
// sort stable.

constexpr int RS_WARPS = 8;
constexpr int RS_THREADS = RS_WARPS * 32;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;

template <typename K>
__global__ void __launch_bounds__(RS_THREADS) k_rs_upsweep(const K *keys, size_t n, int shift,
                                                           unsigned mask, uint32_t *hist,
                                                           size_t tiles) {
    __shared__ uint32_t cnt[RS_WARPS][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_THREADS) (&cnt[0][0])[i] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * RS_TILE + (size_t)warp * 32 * RS_ITEMS;
#pragma unroll 4
    for (int k = 0; k < RS_ITEMS; k++) {
        size_t idx = base + (size_t)k * 32 + lane;
        bool valid = idx < n;
        unsigned d = valid ? (unsigned)(keys[idx] >> shift) & mask : 0xffffffffu;
        unsigned peers = __match_any_sync(FULL, d);
        if (valid && lane == __ffs(peers) - 1) cnt[warp][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += RS_THREADS) {
        uint32_t s = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) s += cnt[w][d];
        hist[(size_t)d * tiles + blockIdx.x] = s;
    }
}

// Ranks every key of the tile stably by digit, reorders the tile in shared
// memory, then writes it out in tile order so that keys of one digit leave as
// one contiguous run (coalesced) at the digit's global offset.
template <typename K, bool HAS_VALS>
__global__ void __launch_bounds__(RS_THREADS, 4) k_rs_downsweep(const K *keys_in, const uint32_t *vals_in,
                                                                K *keys_out, uint32_t *vals_out,
                                                                size_t n, int shift, unsigned mask,
                                                                const uint32_t *offsets, size_t tiles) {
    __shared__ uint32_t cnt[RS_WARPS][256];
    __shared__ uint32_t tile_start[256];   // first tile position of each digit
    __shared__ uint32_t glob[256];         // global position of that first key
    __shared__ K skeys[RS_TILE];
    __shared__ uint32_t svals[HAS_VALS ? RS_TILE : 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_THREADS) (&cnt[0][0])[i] = 0;
    __syncthreads();
    const size_t tile_base = (size_t)blockIdx.x * RS_TILE;
    const size_t base = tile_base + (size_t)warp * 32 * RS_ITEMS;
    K key[RS_ITEMS];
    uint32_t val[RS_ITEMS];
    uint32_t rank[RS_ITEMS];
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++) {
        size_t idx = base + (size_t)k * 32 + lane;
        bool valid = idx < n;
        key[k] = valid ? keys_in[idx] : K(0);
        if (HAS_VALS) val[k] = valid ? vals_in[idx] : 0u;
        unsigned d = valid ? (unsigned)(key[k] >> shift) & mask : 0xffffffffu;
        unsigned peers = __match_any_sync(FULL, d);
        int leader = __ffs(peers) - 1;
        uint32_t before = 0;
        if (valid && lane == leader) {
            before = cnt[warp][d];
            cnt[warp][d] = before + __popc(peers);
        }
        before = __shfl_sync(FULL, before, leader);
        rank[k] = before + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();
    // per digit: exclusive prefix over warps (in place) and the digit's tile total
    uint32_t total = 0;
    if (threadIdx.x < 256) {
        const int d = threadIdx.x;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) {
            uint32_t c = cnt[w][d];
            cnt[w][d] = total;
            total += c;
        }
        glob[d] = offsets[(size_t)d * tiles + blockIdx.x];
    }
    // exclusive scan of the 256 digit totals (RS_THREADS == 256: one per thread)
    {
        __shared__ uint32_t wsum[RS_WARPS];
        uint32_t inc = warp_inclusive_scan(total);
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        uint32_t off = 0;
        for (int w = 0; w < warp; w++) off += wsum[w];
        tile_start[threadIdx.x] = off + inc - total;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++) {
        size_t idx = base + (size_t)k * 32 + lane;
        if (idx < n) {
            unsigned d = (unsigned)(key[k] >> shift) & mask;
            uint32_t p = tile_start[d] + cnt[warp][d] + rank[k];
            skeys[p] = key[k];
            if (HAS_VALS) svals[p] = val[k];
        }
    }
    __syncthreads();
    const uint32_t count = (uint32_t)min((size_t)RS_TILE, n - tile_base);
    for (uint32_t i = threadIdx.x; i < count; i += RS_THREADS) {
        const K kk = skeys[i];
        const unsigned d = (unsigned)(kk >> shift) & mask;
        const uint32_t dst = glob[d] + (i - tile_start[d]);
        keys_out[dst] = kk;
        if (HAS_VALS) vals_out[dst] = svals[i];
    }
}

// Sorts keys[0..n) (and vals, if non-null) by bits [begin_bit, end_bit).
// n must be < 2^32.  Uses one temporary copy of the arrays.
template <typename K>
void radix_sort(K *keys, uint32_t *vals, size_t n, int begin_bit, int end_bit, cudaStream_t s) {
    if (n < 2 || end_bit <= begin_bit) return;
    if (n >= (size_t(1) << 32)) throw Error(SCD_ERR_LIMIT, "radix_sort: more than 2^32 keys");
    const size_t tiles = (n + RS_TILE - 1) / RS_TILE;
    DevBuf<K> kt(n, s);
    DevBuf<uint32_t> vt(vals ? n : 0, s);
    DevBuf<uint32_t> hist(256 * tiles + 1, s);
    K *kin = keys, *kout = kt.get();
    uint32_t *vin = vals, *vout = vt.get();
    int passes = 0;
    for (int b = begin_bit; b < end_bit; b += 8) {
        int bits = end_bit - b < 8 ? end_bit - b : 8;
        unsigned mask = (1u << bits) - 1u;
        k_rs_upsweep<K><<<(unsigned)tiles, RS_THREADS, 0, s>>>(kin, n, b, mask, hist.get(), tiles);
        CK_LAUNCH("k_rs_upsweep");
        scan_exclusive<uint32_t, const uint32_t *>(hist.get(), hist.get(), 256 * tiles, s);
        if (vals)
            k_rs_downsweep<K, true><<<(unsigned)tiles, RS_THREADS, 0, s>>>(kin, vin, kout, vout, n, b, mask,
                                                                           hist.get(), tiles);
        else
            k_rs_downsweep<K, false><<<(unsigned)tiles, RS_THREADS, 0, s>>>(kin, nullptr, kout, nullptr, n, b,
                                                                            mask, hist.get(), tiles);
        CK_LAUNCH("k_rs_downsweep");
        K *tk = kin; kin = kout; kout = tk;
        uint32_t *tv = vin; vin = vout; vout = tv;
        passes++;
    }
    if (passes & 1) {
        CK(cudaMemcpyAsync(keys, kin, n * sizeof(K), cudaMemcpyDeviceToDevice, s));
        if (vals) CK(cudaMemcpyAsync(vals, vin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    }
}

}  // namespace scd
