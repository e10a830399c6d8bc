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

// Pinned host memory reused across calls: every per-launch transfer goes
// through it, so a copy never takes the driver's pageable path (which
// returns only when the copy is done and can hold up other streams' small
// copies while a long kernel runs ahead of it).
struct HostBuf {
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
    HostBuf pin_in, pin_out, pin_retry;               // staging of the launch inputs, the readbacks, retry lists
    // sizes chosen at first use from the device's free memory
    uint32_t arena_words = 0;
    uint64_t pool_words = 0;
    // State the kernels leave behind: after a run that ended without an
    // error every candidate-map entry is -1 again (each root restores what
    // it touched) and every task-ring flag is 0 (every pushed task was
    // taken).  Bytes known to be in that state, so they need no clearing.
    size_t cmap_clean = 0;
    size_t ready_clean = 0;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // timing events, created once
    void release();
    size_t bytes() const;  // device memory held
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
    uint32_t min_rows = 0, min_cols = 0;  // thresholds in file orientation, for every entry ...
    const std::vector<uint2>* entry_thr = nullptr;  // ... or per entry: (min_rows, min_cols)
    uint32_t donate_min = 2;
    uint32_t blocks_per_sm = 0;         // 0 = occupancy limit
    uint32_t max_frames = 512;
    uint32_t arena_words = 0;           // per warp; 0 = engine default
    uint64_t pool_words = 0;            // node pool cap; 0 = engine default (grows on demand)
    uint64_t chunk_words = 0;           // root records per chunk; 0 = half the pool
    uint32_t solve_rows = 32;           // packed records with at most this many rows (<= 32) use the register search
    bool l2_pin = false;                // single-graph, uncapped runs: keep the L-side adjacency persisting in L2
    uint64_t extra_tasks = 1ull << 16;  // ring slots beyond the roots and the margin
    // Multi-graph runs: chunks captured per CUDA graph launch, the chunk loop
    // then running on the device (0 = host-driven chunk loop)
    uint32_t graph_chunks = 8;
    unsigned long long timeout_ns = 60ull * 1000000000ull;
    const EmitTarget* emit = nullptr;
    // Bytes of device memory the run's buffers may hold in total (0 = no
    // cap): arenas shrink to at most a quarter of it, the node pool gets
    // what the other buffers leave and never grows past it.
    uint64_t mem_cap = 0;
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
// Engine knobs an autotuner sets for a group of graphs (0 = default).
struct BatchKnobs {
    uint32_t blocks_per_sm = 0;
    uint32_t donate_min = 0;
    uint32_t solve_rows = 32;
    uint64_t chunk_words = 0;
};

mbe_status run_devs(EngineBuffers& eb, cudaStream_t s, IoCounters* io, const std::vector<const DeviceGraph*>& devs,
                    mbe_variant variant, const mbe_opts* opts, std::vector<ResultAcc>& acc, EngineStats& stats,
                    const EmitTarget* emit = nullptr, uint64_t mem_cap = 0, const BatchKnobs* knobs = nullptr,
                    const std::vector<uint2>* entry_thr = nullptr);

// Resident DFS blocks per SM on device dev (the launch's upper bound).
cudaError_t dfs_blocks_per_sm(int dev, int* occ);

// Raw launchers of the two enumeration kernels (root expansion: 256 threads
// per block; DFS: kDfsWarps warps per block).
cudaError_t launch_expand_roots(const EngineArgs& a, unsigned grid, cudaStream_t s);
cudaError_t launch_dfs(const EngineArgs& a, unsigned grid, cudaStream_t s);

}  // namespace mbe
