/* Force-included when compiling the reference's sources with CUDA 13:
 * the reference calls the pre-CUDA-13 four-argument cudaMemPrefetchAsync
 * (src/main.cu:149-181), which CUDA 13 replaced by a cudaMemLocation form.
 * This overload forwards the old call shape to the new one. */
#pragma once
#include <cuda_runtime.h>
static inline cudaError_t cudaMemPrefetchAsync(const void* ptr, size_t count, int device, cudaStream_t stream) {
    cudaMemLocation loc;
    loc.type = cudaMemLocationTypeDevice;
    loc.id = device;
    return cudaMemPrefetchAsync(ptr, count, loc, 0u, stream);
}
