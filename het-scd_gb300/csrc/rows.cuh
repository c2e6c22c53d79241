// Row streams: a warp walks the entries of 32 consecutive CSR rows as one
// stream (see RowStream).
#pragma once

#include "common.cuh"

namespace scd {

// A warp takes 32 consecutive rows (lane k: row r0 + k, its entries [b_k, b_k + len_k))
// and walks their concatenated entries 32 at a time: coalesced loads and many
// independent gathers in flight instead of one short row per warp.  For the entry
// of lane L the owning row is found by a binary search over the lanes' prefix
// sums (shuffles); each lane then counts, with one ballot, the hits of its own
// row in the chunk (the chunk lanes owned by row k form one contiguous range).
struct RowStream {
    uint32_t pre, len, total;
    __device__ __forceinline__ RowStream(uint32_t l) : len(l) {
        const int lane = threadIdx.x & 31;
        uint32_t incl = l;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, d);
            if (lane >= d) incl += y;
        }
        total = __shfl_sync(FULL, incl, 31);
        pre = incl - l;
    }
    // owner lane of stream position t (t < total)
    __device__ __forceinline__ int owner(uint32_t t) const {
        int j = 0;
#pragma unroll
        for (int st = 16; st > 0; st >>= 1)
            if (__shfl_sync(FULL, pre, j + st) <= t) j += st;
        return j;
    }
    // lanes of the chunk [t0, t0 + 32) that hold this lane's row
    __device__ __forceinline__ unsigned my_lanes(uint32_t t0) const {
        const long long lo = (long long)pre - t0, hi = (long long)pre + len - t0;
        const int a = lo <= 0 ? 0 : lo >= 32 ? 32 : (int)lo, b = hi <= 0 ? 0 : hi >= 32 ? 32 : (int)hi;
        const unsigned upto_b = b >= 32 ? FULL : ((1u << b) - 1u);
        const unsigned upto_a = a >= 32 ? FULL : ((1u << a) - 1u);
        return upto_b & ~upto_a;
    }
};

}  // namespace scd
