// Device-resident graph construction: orientation, root order, and the two
// sorted CSRs the enumeration kernels read.
//
// Replaces, on the reference side:
//   - the orientation swap (src/main.cu:65-70): R = smaller side;
//   - CUDA_TRANSPOSE (src/transpose.cuh:1-52), which scatters one input
//     row per grid-wide barrier: here the transpose is count -> scan ->
//     atomic scatter -> segmented sort, with no grid barrier;
//   - my_memset_sort (src/header.cuh:55-63): R vertices are relabelled by
//     their processing rank (degree ascending, id ascending), so rank order
//     is id order on the device and the root queue needs no indirection.
#include <algorithm>
#include <cstring>
#include <vector>

#include "dev_common.cuh"
#include "graph_dev.cuh"
#include "mbe_hash.h"

namespace mbe {

// ---------------------------------------------------------------------------
// exclusive scan (tile = 4096 elements per 1024-thread block)

namespace {
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanTile = kScanThreads * kScanPer;

__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
    unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(kFull, s, o);
            if (lane >= (unsigned)o) s += y;
        }
        warp_sums[lane] = s;  // inclusive
    }
    __syncthreads();
    uint32_t base = warp ? warp_sums[warp - 1] : 0;
    if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
    return base + x - v;
}

__global__ void scan_tile_sums(const uint32_t* in, uint32_t n, uint32_t* tile_sums) {
    __shared__ uint32_t ws[32];
    uint64_t base = (uint64_t)blockIdx.x * kScanTile + threadIdx.x * kScanPer;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanPer; i++)
        if (base + i < n) s += in[base + i];
    uint32_t tot;
    block_exclusive_scan(s, ws, &tot);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void scan_tile_offsets(uint32_t* tile_sums, uint32_t n_tiles, uint32_t* total) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t b = 0; b < n_tiles; b += blockDim.x) {
        uint32_t i = b + threadIdx.x;
        uint32_t v = i < n_tiles ? tile_sums[i] : 0;
        uint32_t tot;
        uint32_t ex = block_exclusive_scan(v, ws, &tot);
        if (i < n_tiles) tile_sums[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void scan_tile_apply(const uint32_t* in, uint32_t* out, uint32_t n, const uint32_t* tile_offsets) {
    __shared__ uint32_t ws[32];
    uint64_t base = (uint64_t)blockIdx.x * kScanTile + threadIdx.x * kScanPer;
    uint32_t v[kScanPer];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanPer; i++) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    uint32_t ex = block_exclusive_scan(s, ws, nullptr) + tile_offsets[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanPer; i++) {
        if (base + i < n) out[base + i] = ex;
        ex += v[i];
    }
}
}  // namespace

size_t exclusive_scan_tmp_words(uint32_t n) { return (size_t)(n + kScanTile - 1) / kScanTile + 1; }

cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* tmp, uint32_t* total,
                               cudaStream_t s) {
    uint32_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
        return cudaSuccess;
    }
    scan_tile_sums<<<tiles, kScanThreads, 0, s>>>(in, n, tmp);
    scan_tile_offsets<<<1, kScanThreads, 0, s>>>(tmp, tiles, total);
    scan_tile_apply<<<tiles, kScanThreads, 0, s>>>(in, out, n, tmp);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// edge expansion and CSR construction

namespace {

// One thread per edge: find its row by binary search in the file CSR and
// emit (rank, L id) in R/L orientation.
__global__ void expand_edges(const uint64_t* row_ptr, const uint32_t* col_idx, uint32_t n_rows, uint64_t n_edges,
                             const uint32_t* rank_of, int swapped, uint32_t* e_rank, uint32_t* e_l) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_edges;
         e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n_rows;  // find r with row_ptr[r] <= e < row_ptr[r+1]
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (row_ptr[mid] <= e)
                lo = mid;
            else
                hi = mid;
        }
        uint32_t r = lo, c = col_idx[e];
        if (!swapped) {
            e_rank[e] = rank_of[r];
            e_l[e] = c;
        } else {
            e_rank[e] = rank_of[c];
            e_l[e] = r;
        }
    }
}

__global__ void count_keys(const uint32_t* keys, uint64_t n, uint32_t* deg) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&deg[keys[e]], 1u);
}

__global__ void scatter_keys(const uint32_t* keys, const uint32_t* vals, uint64_t n, uint32_t* cursor, uint32_t* adj) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t pos = atomicAdd(&cursor[keys[e]], 1u);
        adj[pos] = vals[e];
    }
}

// Segments of length 2..32: one warp, register bitonic network.
__global__ void sort_segments_warp(const uint32_t* ptr, uint32_t n_seg, uint32_t* adj) {
    unsigned lane = threadIdx.x & 31u;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t s = gw; s < n_seg; s += nw) {
        uint32_t b = ptr[s], len = ptr[s + 1] - b;
        if (len < 2 || len > 32) continue;
        uint32_t v = lane < len ? adj[b + lane] : 0xFFFFFFFFu;
        for (int k = 2; k <= 32; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                uint32_t o = __shfl_xor_sync(kFull, v, j);
                bool up = (lane & k) == 0, lower = (lane & j) == 0;
                v = (lower == up) ? min(v, o) : max(v, o);
            }
        if (lane < len) adj[b + lane] = v;
    }
}

// Segments of length 33..4096: one block, shared-memory bitonic sort.
constexpr uint32_t kMedMax = 4096;
__global__ void sort_segments_block(const uint32_t* ptr, uint32_t n_seg, uint32_t* adj) {
    __shared__ uint32_t sm[kMedMax];
    for (uint32_t s = blockIdx.x; s < n_seg; s += gridDim.x) {
        uint32_t b = ptr[s], len = ptr[s + 1] - b;
        if (len <= 32 || len > kMedMax) continue;
        uint32_t n = 64;
        while (n < len) n <<= 1;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) sm[i] = i < len ? adj[b + i] : 0xFFFFFFFFu;
        __syncthreads();
        for (uint32_t k = 2; k <= n; k <<= 1)
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                    uint32_t ixj = i ^ j;
                    if (ixj > i) {
                        uint32_t a = sm[i], c = sm[ixj];
                        bool asc = (i & k) == 0;
                        if ((a > c) == asc) {
                            sm[i] = c;
                            sm[ixj] = a;
                        }
                    }
                }
                __syncthreads();
            }
        for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) adj[b + i] = sm[i];
        __syncthreads();
    }
}

// Segments longer than 4096: values in a segment are distinct and below
// max_val, so a bitmap of max_val bits sorts them: set, then compact in
// word order with a block prefix sum.
__global__ void sort_segments_bitmap(const uint32_t* ptr, uint32_t n_seg, uint32_t* adj, uint32_t max_val,
                                     uint32_t* bitmaps) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t carry;
    uint32_t nwords = (max_val + 31) / 32;
    uint32_t* bm = bitmaps + (size_t)blockIdx.x * nwords;
    for (uint32_t s = blockIdx.x; s < n_seg; s += gridDim.x) {
        uint32_t b = ptr[s], len = ptr[s + 1] - b;
        if (len <= kMedMax) continue;
        for (uint32_t i = threadIdx.x; i < nwords; i += blockDim.x) bm[i] = 0;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) {
            uint32_t v = adj[b + i];
            atomicOr(&bm[v >> 5], 1u << (v & 31));
        }
        __syncthreads();
        if (threadIdx.x == 0) carry = 0;
        __syncthreads();
        for (uint32_t w0 = 0; w0 < nwords; w0 += blockDim.x) {
            uint32_t w = w0 + threadIdx.x;
            uint32_t bits = w < nwords ? bm[w] : 0;
            uint32_t tot;
            uint32_t ex = block_exclusive_scan(__popc(bits), ws, &tot) + carry;
            while (bits) {
                uint32_t t = __ffs(bits) - 1;
                bits &= bits - 1;
                adj[b + ex++] = w * 32 + t;
            }
            __syncthreads();
            if (threadIdx.x == 0) carry += tot;
            __syncthreads();
        }
    }
}

__global__ void elem_hashes(uint32_t nR, uint32_t nL, const uint32_t* r_orig, int swapped, uint64_t* eR,
                            uint64_t* eL) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // R side = file rows unless swapped; L side = file cols unless swapped.
    if (i < nR) eR[i] = swapped ? mbe_elem_col(r_orig[i]) : mbe_elem_row(r_orig[i]);
    if (i < nL) eL[i] = swapped ? mbe_elem_row(i) : mbe_elem_col(i);
}

cudaError_t build_csr(uint32_t n_keys, uint64_t n_edges, const uint32_t* keys, const uint32_t* vals, uint32_t* ptr,
                      uint32_t* adj, uint32_t* cursor, uint32_t* scan_tmp, uint32_t max_val, uint32_t* bitmaps,
                      uint32_t n_bitmaps, int n_sm, cudaStream_t s, IoCounters* io) {
    cudaError_t err;
    if ((err = cudaMemsetAsync(cursor, 0, sizeof(uint32_t) * ((size_t)n_keys + 1), s))) return err;
    int grid = n_sm * 8;
    if (n_edges) {
        count_keys<<<grid, 256, 0, s>>>(keys, n_edges, cursor);
        io->launches++;
    }
    if ((err = exclusive_scan_u32(cursor, ptr, n_keys + 1, scan_tmp, nullptr, s))) return err;
    io->launches += 3;
    if ((err = cudaMemcpyAsync(cursor, ptr, sizeof(uint32_t) * n_keys, cudaMemcpyDeviceToDevice, s))) return err;
    if (n_edges) {
        scatter_keys<<<grid, 256, 0, s>>>(keys, vals, n_edges, cursor, adj);
        io->launches++;
    }
    if (n_keys) {
        sort_segments_warp<<<n_sm * 8, 256, 0, s>>>(ptr, n_keys, adj);
        sort_segments_block<<<n_sm * 4, 256, 0, s>>>(ptr, n_keys, adj);
        io->launches += 2;
        if (n_bitmaps) {
            sort_segments_bitmap<<<n_bitmaps, 512, 0, s>>>(ptr, n_keys, adj, max_val, bitmaps);
            io->launches++;
        }
    }
    return cudaGetLastError();
}

}  // namespace

void DeviceGraph::release() {
    for (void* p : {(void*)r_ptr, (void*)r_adj, (void*)l_ptr, (void*)l_adj, (void*)r_orig, (void*)eR, (void*)eL})
        if (p) cudaFree(p);
    r_ptr = r_adj = l_ptr = l_adj = r_orig = nullptr;
    eR = eL = nullptr;
}

// Root order on the host, as the reference does (src/header.cuh:55-63),
// but by a counting sort: rank = position in (degree asc, id asc) order.
// The reference grabs roots from the tail of a degree-DESCENDING list
// (src/mbe_cuMBE.cuh:125-133), i.e. it also processes low degree first.
static void compute_ranks(const mbe_graph* g, bool swapped, std::vector<uint32_t>& rank_of,
                          std::vector<uint32_t>& by_rank, uint32_t* max_rdeg, std::vector<uint32_t>& deg_by_rank,
                          uint32_t* n_isolated) {
    uint32_t nR = swapped ? g->n_cols : g->n_rows;
    std::vector<uint32_t> deg(nR, 0);
    if (!swapped)
        for (uint32_t r = 0; r < nR; r++) deg[r] = (uint32_t)(g->row_ptr[r + 1] - g->row_ptr[r]);
    else
        for (uint32_t c : g->col_idx) deg[c]++;
    uint32_t md = 0;
    for (uint32_t d : deg) md = std::max(md, d);
    std::vector<uint32_t> start((size_t)md + 2, 0);
    for (uint32_t d : deg) start[d + 1]++;
    for (uint32_t d = 0; d <= md; d++) start[d + 1] += start[d];
    rank_of.resize(nR);
    by_rank.resize(nR);
    for (uint32_t v = 0; v < nR; v++) {
        uint32_t r = start[deg[v]]++;
        rank_of[v] = r;
        by_rank[r] = v;
    }
    *max_rdeg = md;
    deg_by_rank.resize(nR);
    for (uint32_t r = 0; r < nR; r++) deg_by_rank[r] = deg[by_rank[r]];
    *n_isolated = 0;
    while (*n_isolated < nR && deg_by_rank[*n_isolated] == 0) (*n_isolated)++;
}

mbe_status build_device_graph(const mbe_graph* g, cudaStream_t s, int n_sm, DeviceGraph* out, IoCounters* io) {
    DeviceGraph d;
    d.swapped = g->n_rows > g->n_cols ? 1u : 0u;
    d.nR = d.swapped ? g->n_cols : g->n_rows;
    d.nL = d.swapped ? g->n_rows : g->n_cols;
    d.nE = g->col_idx.size();
    d.uid = g->uid;
    if (d.nE >= 0xFFFFFFFFull) return fail(MBE_ERR_CAPACITY, "graphs with 2^32 or more edges are not supported");
    std::vector<uint32_t> rank_of, by_rank;
    compute_ranks(g, d.swapped, rank_of, by_rank, &d.max_rdeg, d.deg_by_rank, &d.n_isolated);
    d.max_ldeg = d.swapped ? g->max_row_deg : g->max_col_deg;

    // pinned staging of the inputs: row_ptr (u64), col_idx, rank_of, by_rank
    size_t n_rp = (size_t)g->n_rows + 1, n_e = d.nE;
    size_t stage_bytes = n_rp * 8 + n_e * 4 + (size_t)d.nR * 8 + 64;
    void* stage = nullptr;
    MBE_CUDA_TRY(cudaMallocHost(&stage, stage_bytes));
    uint8_t* sp = (uint8_t*)stage;
    std::memcpy(sp, g->row_ptr.data(), n_rp * 8);
    std::memcpy(sp + n_rp * 8, g->col_idx.data(), n_e * 4);
    std::memcpy(sp + n_rp * 8 + n_e * 4, rank_of.data(), (size_t)d.nR * 4);
    std::memcpy(sp + n_rp * 8 + n_e * 4 + (size_t)d.nR * 4, by_rank.data(), (size_t)d.nR * 4);

    uint64_t* d_row_ptr = nullptr;
    uint32_t *d_col = nullptr, *d_rank_of = nullptr, *e_rank = nullptr, *e_l = nullptr, *cursor = nullptr,
             *scan_tmp = nullptr, *bitmaps = nullptr;
    mbe_status st = MBE_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(s);
        for (void* p : {(void*)d_row_ptr, (void*)d_col, (void*)d_rank_of, (void*)e_rank, (void*)e_l, (void*)cursor,
                        (void*)scan_tmp, (void*)bitmaps})
            if (p) cudaFree(p);
        cudaFreeHost(stage);
    };
#define GD_TRY(expr)                                                                           \
    do {                                                                                       \
        cudaError_t e__ = (expr);                                                              \
        if (e__ != cudaSuccess) {                                                              \
            st = fail(e__ == cudaErrorMemoryAllocation ? MBE_ERR_OUT_OF_MEMORY : MBE_ERR_CUDA, \
                      std::string(#expr) + ": " + cudaGetErrorString(e__));                    \
            cleanup();                                                                         \
            d.release();                                                                       \
            return st;                                                                         \
        }                                                                                      \
    } while (0)
    size_t ne1 = n_e ? n_e : 1;
    uint32_t nmax = std::max(d.nR, d.nL) + 1;
    GD_TRY(cudaMalloc(&d_row_ptr, n_rp * 8));
    GD_TRY(cudaMalloc(&d_col, ne1 * 4));
    GD_TRY(cudaMalloc(&d_rank_of, ((size_t)d.nR + 1) * 4));
    GD_TRY(cudaMalloc(&e_rank, ne1 * 4));
    GD_TRY(cudaMalloc(&e_l, ne1 * 4));
    GD_TRY(cudaMalloc(&cursor, (size_t)nmax * 4 + 4));
    GD_TRY(cudaMalloc(&scan_tmp, exclusive_scan_tmp_words(nmax) * 4));
    GD_TRY(cudaMalloc(&d.r_ptr, ((size_t)d.nR + 1) * 4));
    GD_TRY(cudaMalloc(&d.r_adj, (ne1 + kAdjSlack) * 4));
    GD_TRY(cudaMalloc(&d.l_ptr, ((size_t)d.nL + 1) * 4));
    GD_TRY(cudaMalloc(&d.l_adj, ne1 * 4));
    GD_TRY(cudaMalloc(&d.r_orig, ((size_t)d.nR + 1) * 4));
    GD_TRY(cudaMalloc(&d.eR, ((size_t)d.nR + 1) * 8));
    GD_TRY(cudaMalloc(&d.eL, ((size_t)d.nL + 1) * 8));
    uint32_t n_big = 0;
    if (std::max(d.max_rdeg, d.max_ldeg) > kMedMax) {
        n_big = (uint32_t)n_sm * 2;
        GD_TRY(cudaMalloc(&bitmaps, (size_t)n_big * ((nmax + 31) / 32) * 4));
    }
    io->h2d += n_rp * 8 + n_e * 4 + (size_t)d.nR * 8;
    GD_TRY(cudaMemcpyAsync(d_row_ptr, sp, n_rp * 8, cudaMemcpyHostToDevice, s));
    if (n_e) GD_TRY(cudaMemcpyAsync(d_col, sp + n_rp * 8, n_e * 4, cudaMemcpyHostToDevice, s));
    if (d.nR) {
        GD_TRY(cudaMemcpyAsync(d_rank_of, sp + n_rp * 8 + n_e * 4, (size_t)d.nR * 4, cudaMemcpyHostToDevice, s));
        GD_TRY(cudaMemcpyAsync(d.r_orig, sp + n_rp * 8 + n_e * 4 + (size_t)d.nR * 4, (size_t)d.nR * 4,
                               cudaMemcpyHostToDevice, s));
    }
    if (n_e) {
        expand_edges<<<n_sm * 8, 256, 0, s>>>(d_row_ptr, d_col, g->n_rows, n_e, d_rank_of, (int)d.swapped, e_rank,
                                              e_l);
        io->launches++;
        GD_TRY(cudaGetLastError());
    }
    GD_TRY(build_csr(d.nR, n_e, e_rank, e_l, d.r_ptr, d.r_adj, cursor, scan_tmp, d.nL, bitmaps, n_big, n_sm, s, io));
    GD_TRY(build_csr(d.nL, n_e, e_l, e_rank, d.l_ptr, d.l_adj, cursor, scan_tmp, d.nR, bitmaps, n_big, n_sm, s, io));
    uint32_t nh = std::max(d.nR, d.nL);
    if (nh) {
        elem_hashes<<<(nh + 255) / 256, 256, 0, s>>>(d.nR, d.nL, d.r_orig, (int)d.swapped, d.eR, d.eL);
        io->launches++;
        GD_TRY(cudaGetLastError());
    }
    GD_TRY(cudaStreamSynchronize(s));
#undef GD_TRY
    cleanup();
    *out = d;
    return MBE_OK;
}

}  // namespace mbe
