// Device-resident graph in R/L orientation.
//
// R = the smaller side (the branching side of the search), L = the larger
// side, as the reference orients its input (src/main.cu:65-70).  R
// vertices are relabelled by processing rank: rank r is the r-th vertex in
// (degree ascending, original id ascending) order.  Both CSRs are sorted.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "mbe_internal.h"

namespace mbe {

struct DeviceGraph {
    uint32_t nR = 0, nL = 0;
    uint64_t nE = 0;
    uint32_t swapped = 0;       // 1: R = file cols, L = file rows
    uint32_t max_rdeg = 0, max_ldeg = 0;
    uint64_t uid = 0;
    uint32_t* r_ptr = nullptr;  // [nR+1] rank -> offsets into r_adj
    uint32_t* r_adj = nullptr;  // L ids, ascending within a row
    uint32_t* l_ptr = nullptr;  // [nL+1]
    uint32_t* l_adj = nullptr;  // ranks, ascending within a row
    uint32_t* r_orig = nullptr; // [nR] original (file) id of each rank
    uint64_t* eR = nullptr;     // [nR] canonical-hash element of each rank
    uint64_t* eL = nullptr;     // [nL] canonical-hash element of each L id
    uint32_t n_isolated = 0;    // ranks [0, n_isolated) have degree 0
    std::vector<uint32_t> deg_by_rank;  // host copy of the R degrees
    void release();
};

// Words allocated past the end of a device adjacency array, so that a copy
// rounded out to 16-byte boundaries stays inside the allocation.
constexpr uint32_t kAdjSlack = 4;

// Flat view passed to kernels (by value).
struct GraphView {
    uint32_t nR, nL, swapped;
    uint32_t r_adj_slack;       // readable words allocated past r_adj[r_ptr[nR]] (for 16-byte bulk copies)
    const uint32_t* r_ptr;
    const uint32_t* r_adj;
    const uint32_t* l_ptr;
    const uint32_t* l_adj;
    const uint32_t* r_orig;
    const uint64_t* eR;
    const uint64_t* eL;
    uint32_t minL, minR;        // thresholds of this entry, L/R orientation (|L| >= minL, |R| >= minR)
};

inline GraphView view_of(const DeviceGraph& d) {
    return GraphView{d.nR, d.nL, d.swapped, kAdjSlack, d.r_ptr, d.r_adj, d.l_ptr, d.l_adj, d.r_orig, d.eR, d.eL, 0u, 0u};
}

mbe_status build_device_graph(const mbe_graph* g, cudaStream_t s, int n_sm, DeviceGraph* out, IoCounters* io);

}  // namespace mbe
