// Host interface of the enumeration engine (used by capi.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "engine.cuh"
#include "graph_dev.cuh"

namespace mbe {

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    mbe_status ensure(size_t need);
    void free();
};

// Device memory reused across calls on one context.
struct EngineBuffers {
    DevBuf graphs, roots, ctrl, tasks, ready, cmap, a_cl, a_cnt, a_keys, pool, arena, frames, scratch, results,
        retry_in, retry_list;
    DevBuf e_ids, e_start, e_nrows, e_ncols, e_ctl;  // output stream
    // sizes chosen at first use from the device's free memory
    uint32_t arena_words = 0;
    uint64_t pool_words = 0;
    void release();
};

// Device buffers of the output stream (MBE_OPT_EMIT), owned by the caller
// of engine_run; emission is off when EngineConfig::emit is null.
struct EmitTarget {
    uint32_t* ids = nullptr;
    unsigned long long cap_ids = 0;
    unsigned long long* start = nullptr;
    uint32_t* nrows = nullptr;
    uint32_t* ncols = nullptr;
    unsigned long long cap_b = 0;
    unsigned long long* ctl = nullptr;  // 3 words, reset by engine_run at every attempt
};

struct EngineConfig {
    uint32_t variant = 0;
    uint32_t minL = 0, minR = 0;        // thresholds in L/R orientation
    uint32_t donate_min = 2;
    uint32_t blocks_per_sm = 0;         // 0 = occupancy limit
    uint32_t max_frames = 512;
    uint32_t arena_words = 0;           // per warp; 0 = engine default
    uint64_t pool_words = 0;            // node pool cap; 0 = engine default (grows on demand)
    uint64_t chunk_words = 0;           // root records per chunk; 0 = half the pool
    uint64_t extra_tasks = 1ull << 16;  // ring slots beyond the roots and the margin
    unsigned long long timeout_ns = 60ull * 1000000000ull;
    const EmitTarget* emit = nullptr;
};

struct EngineStats {
    float ms_expand = 0, ms_dfs = 0;
    uint32_t chunks = 0, grid_a = 0, grid_b = 0;
};

// Runs root expansion + DFS for the given (graph, rank) roots.  results[g]
// receives the accumulated count / hash / nodes / words of graph g.
mbe_status engine_run(EngineBuffers& eb, cudaStream_t s, const EngineConfig& cfg,
                      const std::vector<const DeviceGraph*>& graphs, const std::vector<uint2>& roots,
                      std::vector<ResultAcc>& results, EngineStats* stats, IoCounters* io);

// Enumeration of resident graphs with opts applied (capi.cu).
mbe_status run_devs(EngineBuffers& eb, cudaStream_t s, IoCounters* io, const std::vector<const DeviceGraph*>& devs,
                    mbe_variant variant, const mbe_opts* opts, std::vector<ResultAcc>& acc, EngineStats& stats,
                    const EmitTarget* emit = nullptr);

// Raw launchers of the two enumeration kernels (root expansion: 256 threads
// per block; DFS: kDfsWarps warps per block).
cudaError_t launch_expand_roots(const EngineArgs& a, unsigned grid, cudaStream_t s);
cudaError_t launch_dfs(const EngineArgs& a, unsigned grid, cudaStream_t s);

}  // namespace mbe
