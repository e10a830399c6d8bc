// Device-side helpers shared by the libmbe kernels (sm_103a only).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <type_traits>

#include "mbe.h"
#include "mbe_internal.h"

#define MBE_CUDA_TRY(expr)                                                              \
    do {                                                                                \
        cudaError_t err__ = (expr);                                                     \
        if (err__ != cudaSuccess)                                                       \
            return ::mbe::fail(err__ == cudaErrorMemoryAllocation ? MBE_ERR_OUT_OF_MEMORY \
                                                                   : MBE_ERR_CUDA,      \
                               std::string(#expr) + ": " + cudaGetErrorString(err__));  \
    } while (0)

namespace mbe {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

// Sum over the warp of an integer, wrapping like the type: one redux.sync
// for 32-bit values; for 64-bit values three independent ones (the high
// words mod 2^32 and the two 16-bit halves of the low words, whose totals
// stay below 2^21), recombined mod 2^64.
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
    static_assert(std::is_integral<T>::value && (sizeof(T) == 4 || sizeof(T) == 8), "32/64-bit integers");
    if constexpr (sizeof(T) == 4) {
        return (T)__reduce_add_sync(kFull, (uint32_t)v);
    } else {
        const uint64_t u = (uint64_t)v;
        const uint32_t lo = (uint32_t)u;
        const uint32_t shi = __reduce_add_sync(kFull, (uint32_t)(u >> 32));
        const uint32_t s0 = __reduce_add_sync(kFull, lo & 0xFFFFu);
        const uint32_t s1 = __reduce_add_sync(kFull, lo >> 16);
        return (T)(((uint64_t)shi << 32) + ((uint64_t)s1 << 16) + s0);
    }
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Exclusive prefix sum over a device array (n <= 2^31), in place into out.
// Three launches: per-block sums, scan of block sums, add-back.
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* tmp_blocks,
                               uint32_t* total, cudaStream_t s);
size_t exclusive_scan_tmp_words(uint32_t n);

}  // namespace mbe
