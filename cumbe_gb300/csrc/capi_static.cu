// mbe_enumerate_static: maximal biclique enumeration that allocates no
// device memory.
//
// Some callers cannot allocate device memory while they run: applications
// that reserve the whole device up front through their own pool allocator
// and forbid third-party cudaMalloc, serving loops that must not pay the
// device-wide synchronisation cudaMalloc/cudaFree can cause, and plugin
// hosts that hand a plugin its device buffers but no allocation budget.
// This entry point serves them: the caller passes the graph and the result
// buffer in device memory, and every byte of working memory comes from one
// fixed array compiled into the library (kStaticScratchBytes, 64 MiB),
// which every GPU that loads the library holds until the process exits.
//
// Set-up: the first call on a device, with that device current, looks the
// array's device address up with cudaGetSymbolAddress (in host code the
// array's name is only a host-side stand-in, never a device address) and
// caches it.  Make that first call before any stream capture.
//
// Sharing: all calls use the same array and it keeps the last call's
// contents.  Each call clears what must start cleared (control block, task
// ring flags, result accumulator, candidate map) before its kernels run.
// Calls whose work overlaps on the GPU (other streams, other host threads)
// race on the array and corrupt each other: serialise them.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "dev_common.cuh"
#include "engine_host.h"
#include "mbe_hash.h"
#include "mbe_internal.h"

namespace mbe {
namespace {

constexpr size_t kStaticScratchBytes = (size_t)MBE_STATIC_SCRATCH_BYTES;
constexpr uint32_t kStaticMaxVertices = MBE_STATIC_MAX_VERTICES;
constexpr uint32_t kGridA = 32;          // root-expansion blocks
constexpr uint32_t kWarps = 128;                   // DFS warps
constexpr uint32_t kGridB = kWarps / kDfsWarps;    // DFS blocks
constexpr uint32_t kArenaWords = 16384;  // 64 KiB DFS arena per warp
constexpr uint32_t kMaxFrames = 256;
constexpr uint32_t kRetryCap = 1024;
constexpr int kMaxDevices = 128;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Control block of one call (same fields the enumeration kernels use).
struct StaticCtrl {
    unsigned long long pool_top;
    unsigned long long progress;
    unsigned long long error_info;
    uint32_t root_next;
    uint32_t n_retry;
    uint32_t q_tail;
    uint32_t q_head;
    int pending;
    uint32_t q_done;
    int error;
    uint32_t max_n;
    uint32_t pad[2];
};

// Element hashes of the identity labelling (R = rows, L = cols) and the
// root list (every row; rows without edges are skipped by the expansion).
__global__ void static_prep(uint32_t nR, uint32_t nL, uint64_t* eR, uint64_t* eL, uint2* roots) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (nR > nL ? nR : nL); i += gridDim.x * blockDim.x) {
        if (i < nR) {
            eR[i] = mbe_elem_row(i);
            roots[i] = make_uint2(0u, nR - 1u - i);
        }
        if (i < nL) eL[i] = mbe_elem_col(i);
    }
}

struct Carver {
    unsigned char* base;
    size_t used = 0, cap;
    void* take(size_t bytes) {
        size_t off = (used + 255) & ~(size_t)255;
        if (off + bytes > cap) return nullptr;
        used = off + bytes;
        return base + off;
    }
};

mbe_status scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(MBE_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(MBE_ERR_NO_DEVICE, "device index out of range");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            return fail(MBE_ERR_CUDA, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return MBE_OK;
}

}  // namespace
}  // namespace mbe

using namespace mbe;

extern "C" mbe_status mbe_enumerate_static(uint32_t n_rows, uint32_t n_cols, const uint32_t* d_row_ptr,
                                           const uint32_t* d_row_idx, const uint32_t* d_col_ptr,
                                           const uint32_t* d_col_idx, mbe_variant variant, uint64_t* d_result,
                                           void* stream) {
    clear_error();
    if (!d_result) return fail(MBE_ERR_INVALID_ARG, "null result buffer");
    if (n_rows > kStaticMaxVertices || n_cols > kStaticMaxVertices)
        return fail(MBE_ERR_CAPACITY, "mbe_enumerate_static handles at most " + std::to_string(kStaticMaxVertices) +
                                          " rows and " + std::to_string(kStaticMaxVertices) + " cols; got " +
                                          std::to_string(n_rows) + " x " + std::to_string(n_cols));
    if ((n_rows && (!d_row_ptr || !d_row_idx)) || (n_cols && (!d_col_ptr || !d_col_idx)))
        return fail(MBE_ERR_INVALID_ARG, "null CSR array");
    cudaStream_t s = (cudaStream_t)stream;
    void* base = nullptr;
    mbe_status st = scratch_address(&base);
    if (st != MBE_OK) return st;
    if (n_rows == 0 || n_cols == 0) {
        MBE_CUDA_TRY(cudaMemsetAsync(d_result, 0, 2 * sizeof(uint64_t), s));
        return MBE_OK;
    }

    // R = rows (the branching side), L = cols, identity labelling: any total
    // order of the roots gives the same set of maximal bicliques.
    const uint32_t nR = n_rows, nL = n_cols;
    const uint32_t maxW = (nL + 31) / 32;
    // Per-block root scratch (u64 words): the root expansion keeps its
    // count histogram (2 x degree u32) and its Q keep flags (one u32 per
    // candidate) there once they outgrow shared memory.  A row's degree is
    // at most n_cols, so n_cols + 1 bounds the first; pow2(n_rows) the second.
    uint32_t keys_cap = 2048;
    while (keys_cap < nR) keys_cap <<= 1;
    if (keys_cap < nL + 1) keys_cap = nL + 1;
    const uint32_t scr_n = nR < 32 ? 32 : nR;
    uint32_t kc = 32;
    while (kc < scr_n) kc <<= 1;
    const size_t sw = scratch_words(maxW, scr_n, kc, false);
    const uint32_t q_margin = 32 * kWarps + 1024;  // a donor pushes up to 31 tasks after its check
    const uint32_t task_cap = nR + q_margin + 4096;

    Carver cv{(unsigned char*)base, 0, kStaticScratchBytes};
    auto* ctrl = (StaticCtrl*)cv.take(sizeof(StaticCtrl));
    auto* gview = (GraphView*)cv.take(sizeof(GraphView));
    auto* roots = (uint2*)cv.take(sizeof(uint2) * nR);
    auto* tasks = (Task*)cv.take(sizeof(Task) * task_cap);
    auto* ready = (uint32_t*)cv.take(sizeof(uint32_t) * task_cap);
    const size_t cmap_bytes = sizeof(int) * (size_t)kGridA * nR;
    auto* cmap = (int*)cv.take(cmap_bytes);
    auto* a_cl = (uint32_t*)cv.take(sizeof(uint32_t) * (size_t)kGridA * nR);
    auto* a_cnt = (uint32_t*)cv.take(sizeof(uint32_t) * (size_t)kGridA * nR);
    auto* a_keys = (unsigned long long*)cv.take(sizeof(unsigned long long) * (size_t)kGridA * keys_cap);
    auto* eR = (uint64_t*)cv.take(sizeof(uint64_t) * nR);
    auto* eL = (uint64_t*)cv.take(sizeof(uint64_t) * nL);
    auto* results = (ResultAcc*)cv.take(sizeof(ResultAcc));
    auto* retry = (uint32_t*)cv.take(sizeof(uint32_t) * kRetryCap);
    auto* frames = (Frame*)cv.take(sizeof(Frame) * (size_t)kWarps * kMaxFrames);
    auto* scratch = (uint32_t*)cv.take(sizeof(uint32_t) * (size_t)kWarps * sw);
    auto* arena = (uint32_t*)cv.take(sizeof(uint32_t) * (size_t)kWarps * kArenaWords);
    const size_t pool_min = (size_t)1 << 20;
    size_t pool_bytes = (cv.cap - ((cv.used + 255) & ~(size_t)255)) & ~(size_t)127;
    auto* pool = pool_bytes >= pool_min ? (uint32_t*)cv.take(pool_bytes) : nullptr;
    if (!ctrl || !gview || !roots || !tasks || !ready || !cmap || !a_cl || !a_cnt || !a_keys || !eR || !eL ||
        !results || !retry || !frames || !scratch || !arena || !pool)
        return fail(MBE_ERR_CAPACITY, "graph too large for the static scratch of mbe_enumerate_static");

    // clear what must start cleared; the rest is written before it is read
    MBE_CUDA_TRY(cudaMemsetAsync(ctrl, 0, sizeof(StaticCtrl), s));
    MBE_CUDA_TRY(cudaMemsetAsync(ready, 0, sizeof(uint32_t) * task_cap, s));
    MBE_CUDA_TRY(cudaMemsetAsync(results, 0, sizeof(ResultAcc), s));
    MBE_CUDA_TRY(cudaMemsetAsync(cmap, 0xFF, cmap_bytes, s));
    GraphView gv{nR, nL, 0u, 0u, d_row_ptr, d_row_idx, d_col_ptr, d_col_idx, nullptr, eR, eL};
    MBE_CUDA_TRY(cudaMemcpyAsync(gview, &gv, sizeof gv, cudaMemcpyHostToDevice, s));
    static_prep<<<64, 256, 0, s>>>(nR, nL, eR, eL, roots);
    MBE_CUDA_TRY(cudaGetLastError());

    EngineArgs a;
    std::memset(&a, 0, sizeof a);
    a.graphs = gview;
    a.n_graphs = 1;
    a.variant = (uint32_t)variant;
    a.donate_min = 2;
    a.donate_copy = 1;
    a.solve_rows = 32;
    a.roots = roots;
    a.n_roots = nR;
    a.root_next = &ctrl->root_next;
    a.retry = retry;
    a.n_retry = &ctrl->n_retry;
    a.retry_cap = kRetryCap;
    a.pool = pool;
    a.pool_words = pool_bytes / 4;
    a.pool_top = &ctrl->pool_top;
    a.pool_watermark = a.pool_words;  // one pass: a root that does not fit fails the call
    a.tasks = tasks;
    a.ready = ready;
    a.task_cap = task_cap;
    a.q_tail = &ctrl->q_tail;
    a.q_head = &ctrl->q_head;
    a.q_done = &ctrl->q_done;
    a.q_margin = q_margin;
    a.pending = &ctrl->pending;
    a.progress = &ctrl->progress;
    a.cmap = cmap;
    a.a_cl = a_cl;
    a.a_cnt = a_cnt;
    a.a_keys = a_keys;
    a.maxNR = nR;
    a.keys_cap = keys_cap;
    a.stage_words = 4096;  // the root expansion's L0 staging buffer (dynamic shared memory)
    a.max_n = &ctrl->max_n;
    a.arena = arena;
    a.arena_stride = kArenaWords;
    a.arena_words = arena_usable_words(kArenaWords);
    a.frames = frames;
    a.max_frames = kMaxFrames;
    a.frame_stride = kMaxFrames;
    a.frame_skew = 0;
    a.scratch = scratch;
    a.scratch_words = (uint32_t)sw;
    a.scr_n = scr_n;
    a.scr_kc = kc;
    a.max_W = maxW;
    a.results = results;
    a.error = &ctrl->error;
    a.error_info = &ctrl->error_info;
    a.timeout_ns = 60ull * 1000000000ull;
    MBE_CUDA_TRY(launch_expand_roots(a, kGridA, s));
    MBE_CUDA_TRY(launch_dfs(a, kGridB, s));
    StaticCtrl hc;
    MBE_CUDA_TRY(cudaMemcpyAsync(&hc, ctrl, sizeof hc, cudaMemcpyDeviceToHost, s));
    MBE_CUDA_TRY(cudaStreamSynchronize(s));
    if (hc.error == kErrTimeout) return fail(MBE_ERR_DEVICE_TIMEOUT, "mbe_enumerate_static: a device wait timed out");
    if (hc.error || hc.n_retry)
        return fail(MBE_ERR_OUT_OF_MEMORY, "mbe_enumerate_static: the search outgrew the static scratch (error " +
                                               std::to_string(hc.error) + ")");
    // ResultAcc starts with count, hash
    MBE_CUDA_TRY(cudaMemcpyAsync(d_result, results, 2 * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
    return MBE_OK;
}
