// Shared device/host helpers of the SCD engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>

#include "scd_gb300.h"

namespace scd {

constexpr uint32_t INVALID = 0xffffffffu;   // src/scd.hpp:23 INVALID_LABEL
constexpr unsigned FULL = 0xffffffffu;
constexpr int NUM_SMS_HINT = 152;

// Errors inside the engine are C++ exceptions carrying an SCD_ERR_* status;
// every C-ABI entry point catches them and returns the status (the reference
// calls exit() instead, src/cuda-common.cuh:67-77).
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void cuda_check(cudaError_t e, const char *what, const char *file, int line) {
    if (e != cudaSuccess) {
        char buf[512];
        snprintf(buf, sizeof buf, "%s: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
        throw Error(e == cudaErrorMemoryAllocation ? SCD_ERR_OOM : SCD_ERR_CUDA, buf);
    }
}
#define CK(call) ::scd::cuda_check((call), #call, __FILE__, __LINE__)
#define CK_LAUNCH(name) ::scd::cuda_check(cudaGetLastError(), name, __FILE__, __LINE__)

inline unsigned grid_for(uint64_t items, unsigned per_block, unsigned cap = 152u * 64u) {
    uint64_t g = (items + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

inline int ceil_log2(uint64_t x) {
    int b = 0;
    while ((uint64_t(1) << b) < x) b++;
    return b;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp-aggregated atomicAdd of 1 (the common case: counting / slot claims).
__device__ __forceinline__ uint32_t warp_atomic_inc(uint32_t *addr, unsigned active = FULL) {
    unsigned peers = __match_any_sync(active, (unsigned long long)addr);
    int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(addr, (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & lanemask_lt());
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T u = __shfl_up_sync(FULL, v, o);
        if ((int)lane_id() >= o) v += u;
    }
    return v;
}

// first index in sorted a[0..len) with a[i] >= key
template <typename T>
__device__ __forceinline__ uint32_t lower_bound(const T *a, uint32_t len, T key) {
    uint32_t lo = 0, hi = len;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

}  // namespace scd
