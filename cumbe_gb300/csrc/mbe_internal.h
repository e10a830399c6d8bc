// Internal declarations shared by the host translation units of libmbe.
#pragma once
#include <stdint.h>
#include <string>
#include <vector>

#include "mbe.h"

struct mbe_graph {
    uint32_t n_rows = 0;
    uint32_t n_cols = 0;
    std::vector<uint64_t> row_ptr;   // n_rows + 1
    std::vector<uint32_t> col_idx;   // sorted, unique per row
    uint32_t max_row_deg = 0;
    uint32_t max_col_deg = 0;
    uint32_t n_dup = 0;
    uint64_t uid = 0;                // identity for device residency
};

namespace mbe {

// Per-context accounting of what crossed the host/device boundary.
struct IoCounters {
    uint64_t launches = 0;   // kernels of this library launched
    uint64_t h2d = 0;        // bytes copied host -> device
    uint64_t d2h = 0;        // bytes copied device -> host
};

// Thread-local error message plumbing.
mbe_status fail(mbe_status st, const std::string& msg);
void clear_error();

// Sort + dedupe each row, fill degree maxima.  Returns MBE_ERR_FORMAT when
// an id is out of range.
mbe_status normalise(mbe_graph* g);

uint64_t next_graph_uid();

}  // namespace mbe
