// Device-side helpers shared by the libmbe kernels (sm_103a only).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

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

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
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
