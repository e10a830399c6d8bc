// Enumeration kernels (sm_103a) and their host driver.
//
// Reference path replaced: CUDA_MBE_cuMBE / noES / noRS / noWS
// (src/mbe_cuMBE.cuh, src/mbe_noES.cuh, src/mbe_noRS.cuh, src/mbe_noWS.cuh)
// and the per-block state plan around them (src/main.cu:72-119,
// src/global_extension.cuh).  The reference runs one tree node per
// 512-thread block with __syncthreads between every step, serial
// thread-0 partition loops, an O(|R|) P reset per root and grid-wide
// barriers for stealing.  Here:
//   - expand_roots_kernel (one block per root, persistent): builds the
//     root's bit-row universe by reverse scanning N(N(x)) (the reference's
//     RS, src/mbe_cuMBE.cuh:215-263), tests root maximality, counts the
//     root biclique and publishes the root's record as a task;
//   - dfs_kernel (one warp per task, persistent): depth-first search over
//     node records with popcount intersections, no block barriers, and
//     work donation to hungry warps through a device task queue (the
//     reference's level-1 stealing, src/mbe_cuMBE.cuh:570-621,1208-1256,
//     generalised to any depth).  Termination is an outstanding-task
//     counter, not a grid barrier; every wait is bounded by %globaltimer.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "dev_common.cuh"
#include "engine.cuh"
#include "engine_host.h"
#include "mbe_hash.h"

namespace mbe {

namespace {

constexpr int kThreadsA = 256;
constexpr int kWarpsB = kDfsWarps;
constexpr int kThreadsB = kWarpsB * 32;
// Shared-memory sizes per DFS warp, chosen so that MBE_DFS_MIN_BLOCKS
// blocks fit the 64 KB carveout (the rest of the SM's memory stays L1).
// At seven blocks: 16 L_i words and 24 packed-build rows (26/16 measured
// the same, 30/8 and 16/16 slower).
#ifndef MBE_SMEM_W
#define MBE_SMEM_W 16
#endif
#ifndef MBE_SH_ROWS
#define MBE_SH_ROWS 24
#endif
constexpr uint32_t kSmemW = MBE_SMEM_W;  // Li words cached in shared memory per warp
constexpr unsigned long long kInvalidKey = ~0ull;
#ifndef MBE_KEEP_WINDOW
#define MBE_KEEP_WINDOW 32
#endif
#ifndef MBE_POP_SLEEP_MAX
#define MBE_POP_SLEEP_MAX 1024
#endif
constexpr uint32_t kKeepWindow = MBE_KEEP_WINDOW;  // Q rows a dropped Q row is tested against (<= 32)
constexpr unsigned kPopSleepMax = MBE_POP_SLEEP_MAX;  // ns, back-off ceiling of a warp waiting for a task
constexpr uint32_t kShRows = MBE_SH_ROWS;  // Q' rows / P' keys of a packed build kept in shared memory
// The set-word counter (mbe_result.words: 32-bit words of set data the DFS
// kernel's evaluations stream) is a diagnostic, compiled in by
// MBE_COUNT_WORDS=1 and by profile builds.  Left out, the DFS kernel runs
// 0.55% faster on the 94k x 30k graph and 0.6% on a 600-graph batch (its
// 64-bit adds sit in every scan chunk and its lane counts in the batch
// prefilter's inner loop), and words reads 0.
#ifndef MBE_COUNT_WORDS
#ifdef MBE_PROFILE
#define MBE_COUNT_WORDS 1
#else
#define MBE_COUNT_WORDS 0
#endif
#endif
constexpr bool kCountWords = MBE_COUNT_WORDS != 0;
#ifndef MBE_UNROLL_E
#define MBE_UNROLL_E 1
#endif
#ifndef MBE_UNROLL_G
#define MBE_UNROLL_G 1
#endif
// Prefilter rows in flight per lane: 5 measured fastest on the bench graph
// at 7 blocks per SM (2 to 6 within 1% of each other, 8 2.4% slower; 8 was
// 1.2% faster on the mixed batch).
#ifndef MBE_UNROLL_P
#define MBE_UNROLL_P 5
#endif
constexpr int kUnrollE = MBE_UNROLL_E;   // 32-row chunks in flight per step of the expansion scan
constexpr int kUnrollG = MBE_UNROLL_G;   // ... of the Q' gather of a packed build
constexpr int kUnrollP = MBE_UNROLL_P;   // rows in flight per lane in the batch prefilter
constexpr uint32_t kSolveRows = 32;      // packed records with at most this many rows are solved in registers
#ifndef MBE_POLL_CYCLES
#define MBE_POLL_CYCLES 0
#endif
constexpr uint32_t kPollCycles = MBE_POLL_CYCLES;  // least SM cycles between two reads of the queue counters

// One saved level of the register-resident small-record search (row masks
// over the record's rows, one row per lane).
struct SolveLevel {
    uint32_t L, Q, P, pend, nR, Rm;  // Rm: rows added to R below the record (output stream)
    unsigned long long sR;
};
constexpr uint32_t kDonateSlabMax = 8192;      // arena records up to this size are copied into a slab
constexpr uint32_t kDonateCopyMax = 1u << 20;  // larger ones up to this size by a direct pool allocation
constexpr uint32_t kSlabWords = 1u << 16;      // pool slab a warp takes for donation copies

__device__ __forceinline__ void set_error(const EngineArgs& a, int code, unsigned long long info) {
    if (atomicCAS(a.error, 0, code) == 0) *a.error_info = info;
}

// ---------------------------------------------------------------------------
// Asynchronous bulk copy (global -> this CTA's shared memory) completing on an
// mbarrier: the TMA unit moves the bytes while the threads go on; they wait
// on the barrier's phase before reading.  Both addresses 16-byte aligned,
// size a multiple of 16 (the caller rounds).
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the init is seen by the async proxy
}

// One thread: expect `bytes` on the barrier and start the copy.  The fence
// orders the block's earlier (generic) reads of dst before the async writes.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Waits until the barrier completes phase `parity`; false if that takes
// longer than limit_ns (checked every 64 polls).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity, unsigned long long limit_ns) {
    const uint32_t b = smem_addr(bar);
    unsigned long long t0 = 0;
    for (uint32_t it = 1;; it++) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(b), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 63u) == 0) {
            const unsigned long long now = globaltimer_ns();
            if (t0 == 0)
                t0 = now;
            else if (now - t0 > limit_ns)
                return false;
        }
    }
}

__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }
__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) { return *(const volatile uint32_t*)p; }
__device__ __forceinline__ unsigned long long ld_volatile(const unsigned long long* p) {
    return *(const volatile unsigned long long*)p;
}

// Publishes a task in the ring.  pending is raised before the slot becomes
// visible so that pending == 0 implies no queued and no running task.
// Callers leave q_margin slots free (donors check before calling; the root
// expansion pushes at most n_roots <= capacity - margin), so the slot of
// ticket t was released by the consumer of ticket t - capacity long ago;
// the wait below is a bounded guard, never expected to spin.
__device__ bool push_task(const EngineArgs& a, Task t) {
    atomicAdd(a.pending, 1);
    uint32_t tk = atomicAdd(a.q_tail, 1u);
    uint32_t slot = tk % a.task_cap;
    unsigned long long t0 = 0;
    while (ld_volatile(&a.ready[slot]) != 0) {
        if (t0 == 0) t0 = globaltimer_ns();
        if (globaltimer_ns() - t0 > 1000000000ull) {
            set_error(a, kErrQueue, tk);
            atomicSub(a.pending, 1);
            return false;
        }
        __nanosleep(64);
    }
    volatile Task* dst = (volatile Task*)&a.tasks[slot];
    dst->node = t.node;
    dst->begin = t.begin;
    dst->end = t.end;
    dst->plen = t.plen;
    for (uint32_t j = 0; j < t.plen && j < kMaxPath; j++) dst->path[j] = t.path[j];
    __threadfence();
    atomicExch(&a.ready[slot], tk + 1u);
    return true;
}

#ifdef MBE_PROFILE
#define PROF_TAB(cls, c0, v)                                                                              \
    do {                                                                                                  \
        if (lane == 0) {                                                                                  \
            unsigned tb__ = (unsigned)min((globaltimer_ns() - wc.t_start) / kProfTabNs, (unsigned long long)kProfTB - 1); \
            atomicAdd(&sTab[(tb__ * kProfTC + (cls)) * 2], (unsigned long long)(v));                      \
            atomicAdd(&sTab[(tb__ * kProfTC + (cls)) * 2 + 1], 1ull);                                     \
        }                                                                                                 \
    } while (0)
#define PROF_T0() long long prof_t0__ = clock64()
// root-expansion sections (thread 0 after a block barrier): cycles, events
#define PA_MARK(sec)                                                                    \
    do {                                                                                \
        if (threadIdx.x == 0 && a.prof_a) {                                             \
            long long t__ = clock64();                                                  \
            atomicAdd(&a.prof_a[2 * (sec)], (unsigned long long)(t__ - pa_t));         \
            atomicAdd(&a.prof_a[2 * (sec) + 1], 1ull);                                  \
            pa_t = t__;                                                                 \
        }                                                                               \
    } while (0)
#define PROF_VAL(acc_arr, sec, v) do { if (lane_id() == 0) { (acc_arr)[2 * (sec)] += (v); (acc_arr)[2 * (sec) + 1]++; } } while (0)
#define PROF_ADD(acc_arr, sec) do { const long long t__ = clock64(); if (lane_id() == 0) { (acc_arr)[2 * (sec)] += t__ - prof_t0__; (acc_arr)[2 * (sec) + 1]++; } prof_t0__ = clock64(); } while (0)
#else
#define PROF_T0() do {} while (0)
#define PROF_ADD(acc_arr, sec) do {} while (0)
#define PA_MARK(sec) do {} while (0)
#define PROF_VAL(acc_arr, sec, v) do {} while (0)
#define PROF_TAB(cls, c0, v) do {} while (0)
#endif

// Bump allocation from the node pool; ~0 when it does not fit.  Sizes are
// rounded to 128-byte lines so that records written by one SM and read by
// another never share a cache line with a record read earlier (L1 is not
// coherent across SMs).
__device__ unsigned long long pool_alloc(const EngineArgs& a, unsigned long long words) {
    words = (words + 31) & ~31ull;
    unsigned long long old = ld_volatile(a.pool_top);
    for (;;) {
        if (old + words > a.pool_words) return ~0ull;
        unsigned long long prev = atomicCAS(a.pool_top, old, old + words);
        if (prev == old) return old;
        old = prev;
    }
}

__device__ __forceinline__ uint64_t side_hash(const GraphView& G, uint64_t sL, uint32_t nl, uint64_t sR,
                                              uint32_t nr) {
    // A = rows, B = cols of the file; R is the file's rows unless swapped.
    return G.swapped ? mbe_pair_hash(sL, nl, sR, nr) : mbe_pair_hash(sR, nr, sL, nl);
}


// register bitonic sort across the 32 lanes (ascending by lane)
__device__ __forceinline__ unsigned long long warp_sort_reg(unsigned long long v) {
    unsigned lane = lane_id();
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1)
#pragma unroll
        for (int j = size >> 1; j > 0; j >>= 1) {
            unsigned long long o = __shfl_xor_sync(kFull, v, j);
            bool up = (lane & size) == 0, lower = (lane & j) == 0;
            v = (lower == up) ? (v < o ? v : o) : (v > o ? v : o);
        }
    return v;
}

// A row of a root record (word-major rows, n2 of them) by its first four
// non-zero words; most candidate rows meet only a few words of N(x).
struct SparseRow {
    uint32_t w0, w1, w2, w3, v0, v1, v2, v3, nz;
};

__device__ __forceinline__ SparseRow sparse_row(const uint32_t* M, uint32_t n2, uint32_t W, uint32_t p) {
    SparseRow r{0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t w = 0; w < W; w++) {
        const uint32_t v = M[(size_t)w * n2 + p];
        if (v) {
            if (r.nz == 0) { r.w0 = w; r.v0 = v; }
            else if (r.nz == 1) { r.w1 = w; r.v1 = v; }
            else if (r.nz == 2) { r.w2 = w; r.v2 = v; }
            else if (r.nz == 3) { r.w3 = w; r.v3 = v; }
            r.nz++;
        }
    }
    return r;
}

// Row p (described by r) is a subset of row q.
__device__ __forceinline__ bool row_subset(const SparseRow& r, const uint32_t* M, uint32_t n2, uint32_t W,
                                           uint32_t p, uint32_t q) {
    if (r.nz > 4) {
        for (uint32_t w = 0; w < W; w++)
            if (M[(size_t)w * n2 + p] & ~M[(size_t)w * n2 + q]) return false;
        return true;
    }
    if (r.nz > 0 && (r.v0 & ~M[(size_t)r.w0 * n2 + q])) return false;
    if (r.nz > 1 && (r.v1 & ~M[(size_t)r.w1 * n2 + q])) return false;
    if (r.nz > 2 && (r.v2 & ~M[(size_t)r.w2 * n2 + q])) return false;
    if (r.nz > 3 && (r.v3 & ~M[(size_t)r.w3 * n2 + q])) return false;
    return true;
}

// In-place exclusive prefix sum of a[0..m) by the whole block (each thread
// a contiguous chunk); s_part holds one word per warp.  Ends with a barrier.
__device__ void block_exclusive_scan(uint32_t* a, uint32_t m, uint32_t* s_part) {
    const uint32_t t = threadIdx.x, nt = blockDim.x, lane = t & 31u, warp = t >> 5;
    const uint32_t ch = (m + nt - 1) / nt, b = min(m, t * ch), e = min(m, b + ch);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; i++) sum += a[i];
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, inc, o);
        if (lane >= (uint32_t)o) inc += y;
    }
    if (lane == 31) s_part[warp] = inc;
    __syncthreads();
    uint32_t run = inc - sum;
    for (uint32_t w = 0; w < warp; w++) run += s_part[w];
    for (uint32_t i = b; i < e; i++) {
        const uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
    __syncthreads();
}


// ---------------------------------------------------------------------------
// Output stream (MBE_OPT_EMIT).  A counted biclique reserves room for its
// file rows then its file cols (ids in no particular order within a side);
// a biclique that does not fit is dropped and the overflow flag set, while
// the count and hash still cover it.  R members are ranks on the device and
// leave as file ids through r_orig; L members are file ids already.

// Reserves room for a biclique with nr R members and nl L members; returns
// the id offset, or ~0 when the buffers are full.  Warp-collective.
__device__ __noinline__ unsigned long long emit_reserve(const EngineArgs& a, uint32_t nr, uint32_t nl,
                                                        uint32_t swapped) {
    unsigned long long o = ~0ull;
    if (lane_id() == 0) {
        const uint32_t na = swapped ? nl : nr, nb = swapped ? nr : nl;
        const unsigned long long sz = (unsigned long long)na + nb;
        const unsigned long long oo = atomicAdd(&a.emit_ctl[0], sz);
        unsigned long long k = ~0ull;
        if (oo + sz <= a.emit_cap_ids) k = atomicAdd(&a.emit_ctl[1], 1ull);
        if (k < a.emit_cap_b) {
            a.emit_start[k] = oo;
            a.emit_nrows[k] = na;
            a.emit_ncols[k] = nb;
            o = oo;
        } else {
            atomicExch(&a.emit_ctl[2], 1ull);
        }
    }
    return __shfl_sync(kFull, o, 0);
}

// Copies the R list of record nd (ranks) to dst, as file ids when r_orig is
// given.  Warp-collective.
__device__ __forceinline__ void copy_rlist(const uint32_t* nd, uint32_t* dst, const uint32_t* r_orig) {
    const NodeHdr* h = (const NodeHdr*)nd;
    const uint32_t* rl = nd + h->rlist;
    for (uint32_t t = lane_id(); t < h->nRset; t += 32) dst[t] = r_orig ? r_orig[rl[t]] : rl[t];
}

// R list of the child record of x_i (ranks): the parent's list, x_i, the
// absorbed.  Warp-collective.
__device__ __noinline__ void write_child_rlist(const uint32_t* nd, uint32_t xcand, const uint32_t* abs,
                                               uint32_t nabs, uint32_t* dst) {
    const uint32_t nrec = ((const NodeHdr*)nd)->nRset;
    copy_rlist(nd, dst, nullptr);
    if (lane_id() == 0) dst[nrec] = xcand;
    for (uint32_t t = lane_id(); t < nabs; t += 32) dst[nrec + 1 + t] = abs[t];
}

// x and the candidates of root x absorbed into R (count d = |N(x)|), as
// ranks, or as file ids when r_orig is given.  Warp-collective.
__device__ void root_rlist(uint32_t x, const uint32_t* cl, const uint32_t* cntA, uint32_t n, uint32_t d,
                           uint32_t* dst, const uint32_t* r_orig) {
    const unsigned lane = lane_id();
    if (lane == 0) dst[0] = r_orig ? r_orig[x] : x;
    uint32_t m = 1;
    for (uint32_t base = 0; base < n; base += 32) {
        const uint32_t i = base + lane;
        const uint32_t v = i < n ? cl[i] : 0u;
        const bool ab = i < n && v > x && cntA[i] == d;
        const unsigned b = __ballot_sync(kFull, ab);
        if (ab) dst[m + __popc(b & lanemask_lt())] = r_orig ? r_orig[v] : v;
        m += __popc(b);
    }
}

// ---------------------------------------------------------------------------
// Phase A: root expansion

// L0 (the root's neighbour list) staged in shared memory (dynamic, a.stage_words
// words per block) when its 16-byte rounded span fits.
constexpr uint32_t kStageWords = 4096;
// The two scatters over the neighbours' lists give a warp a whole list; a
// list longer than kLongList (a hub's) is scanned by the whole block
// instead, so that one warp's hub list does not keep the other seven
// waiting at the next barrier.  Up to kLongCap such lists per root are
// noted (with many long lists the warps' shares even out by themselves);
// any beyond stay with their warp.  The notes take 260 bytes, so that two
// root-expansion blocks still fit beside a server slot's three DFS blocks
// in the DFS kernel's 64 KB carveout.
constexpr uint32_t kLongList = 128;
constexpr uint32_t kLongCap = 64;

// kShareSM: the instance capped (server) contexts launch.  Their kernels
// share SMs with other slots' persistent DFS blocks, so this instance stages
// nothing and prefers the DFS kernel's shared-memory carveout: a block can
// then join an SM the other slot's DFS blocks hold (a kernel that prefers
// another carveout waits for the SM to drain, which kept light requests
// behind a heavy one for the heavy one's whole run).
template <bool kShareSM>
__global__ void __launch_bounds__(kThreadsA) expand_roots_kernel(const __grid_constant__ EngineArgs a) {
    extern __shared__ __align__(16) uint32_t s_L0[];
    __shared__ unsigned long long s_bar;
    __shared__ uint32_t s_idx, s_stop, s_ncand, s_nq, s_np, s_nabs, s_nonmax, s_counted;
    __shared__ uint32_t s_kept[32], s_nk, s_p1, s_wsum[32];
    __shared__ unsigned long long s_sabs, s_sl, s_rec, s_scan;
    __shared__ unsigned long long s_keys[2048];
    __shared__ uint32_t s_long[kLongCap], s_nlong;  // positions in L0 of the long lists
    int* cmap = a.cmap + (size_t)blockIdx.x * a.maxNR;
    uint32_t* cl = a.a_cl + (size_t)blockIdx.x * a.maxNR;
    uint32_t* cntA = a.a_cnt + (size_t)blockIdx.x * a.maxNR;
    unsigned long long* gkeys = a.a_keys + (size_t)blockIdx.x * a.keys_cap;
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u, nwarps = blockDim.x >> 5;
    const bool rs = a.variant != MBE_NORS;
    if (threadIdx.x == 0) mbar_init(&s_bar, 1);
    __syncthreads();
    uint32_t stage_parity = 0;  // phase of s_bar the next staged copy completes

    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            s_stop = 0;
            if (ld_volatile(a.error))
                s_stop = 1;
            else if (ld_volatile(a.pool_top) > a.pool_watermark)
                s_stop = 1;
            else {
                uint32_t i = atomicAdd(a.root_next, 1u);
                if (i >= a.n_roots)
                    s_stop = 1;
                else
                    s_idx = i;
            }
            s_ncand = 0;
            s_nlong = 0;
            s_nq = s_np = s_nabs = s_nonmax = s_counted = 0;
            s_sabs = s_sl = s_scan = 0;
        }
        __syncthreads();
        if (s_stop) break;
#ifdef MBE_PROFILE
        long long pa_t = clock64();
        const long long pa_root0 = pa_t;
#endif
        const uint2 rt = a.roots[s_idx];
        const GraphView G = a.graphs[rt.x];
        const uint32_t x = rt.y;
        const uint32_t d = G.r_ptr[x + 1] - G.r_ptr[x];
        if (d == 0 || d < G.minL) continue;  // uniform across the block
        const uint32_t* L0 = G.r_adj + G.r_ptr[x];
        const uint32_t W = (d + 31) / 32;
        {
            // Stream L0 into shared memory with one asynchronous bulk copy
            // (every pass below reads it, and the candidate-side count of
            // noRS binary-searches it per neighbour).  The span is rounded
            // out to 16-byte boundaries and copied only when that stays
            // inside the adjacency array (its allocated slack included).
            const uintptr_t beg = (uintptr_t)L0 & ~(uintptr_t)15;
            const uintptr_t end = ((uintptr_t)(L0 + d) + 15) & ~(uintptr_t)15;
            const uintptr_t lim = (uintptr_t)(G.r_adj + G.r_ptr[G.nR] + G.r_adj_slack);
            if (!kShareSM && end - beg <= sizeof(uint32_t) * a.stage_words && beg >= (uintptr_t)G.r_adj &&
                end <= lim) {
                if (threadIdx.x == 0) bulk_load(s_L0, (const void*)beg, (uint32_t)(end - beg), &s_bar);
                bool ok = mbar_wait(&s_bar, stage_parity, 1000000000ull);
                if (!ok) {
                    set_error(a, kErrTimeout, 0xB0000000ull | x);
                    ok = mbar_wait(&s_bar, stage_parity, 1000000000ull);  // let the copy land before leaving
                }
                stage_parity ^= 1u;
                if (__syncthreads_or(!ok)) break;
                L0 = s_L0 + ((uintptr_t)L0 - beg) / sizeof(uint32_t);
            }
        }

        // 1. candidates C = N(N(x)) \ {x}: first toucher claims a slot.  With
        // the reverse scan the same scatter also counts |N(v) n L0|
        // (src/mbe_cuMBE.cuh:215-227): the per-block map holds touches - 1.
        unsigned long long scan = 0;  // list entries read (lane 0 / thread 0 counts)
        for (uint32_t j = warp; j < d; j += nwarps) {
            uint32_t u = L0[j], b = G.l_ptr[u], e = G.l_ptr[u + 1];
            if (e - b > kLongList) {  // noted for the whole block, unless the notes are full
                uint32_t slot = 0;
                if (lane == 0) slot = atomicAdd(&s_nlong, 1u);
                slot = __shfl_sync(kFull, slot, 0);
                if (slot < kLongCap) {
                    if (lane == 0) s_long[slot] = j;
                    continue;
                }
            }
            if (lane == 0) scan += e - b;
            for (uint32_t k = b + lane; k < e; k += 32) {
                uint32_t v = G.l_adj[k];
                if (v == x) continue;
                const int old = rs ? atomicAdd(&cmap[v], 1) : atomicCAS(&cmap[v], -1, -2);
                if (old == -1) cl[atomicAdd(&s_ncand, 1u)] = v;
            }
        }
        __syncthreads();
        const uint32_t nlong = min(s_nlong, kLongCap);
        for (uint32_t h = 0; h < nlong; h++) {
            const uint32_t u = L0[s_long[h]], b = G.l_ptr[u], e = G.l_ptr[u + 1];
            if (threadIdx.x == 0) scan += e - b;
            for (uint32_t k = b + threadIdx.x; k < e; k += blockDim.x) {
                uint32_t v = G.l_adj[k];
                if (v == x) continue;
                const int old = rs ? atomicAdd(&cmap[v], 1) : atomicCAS(&cmap[v], -1, -2);
                if (old == -1) cl[atomicAdd(&s_ncand, 1u)] = v;
            }
        }
        __syncthreads();
        const uint32_t n = s_ncand;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            const uint32_t v = cl[i];
            cntA[i] = rs ? (uint32_t)(cmap[v] + 1) : 0u;
            cmap[v] = (int)i;
        }
        __syncthreads();
        // 2. |N(v) n L0| per candidate (already counted by the reverse scan)
        if (!rs) {
            // forward scan: each candidate's own list against sorted L0
            // (src/mbe_noRS.cuh:274-283)
            for (uint32_t i = warp; i < n; i += nwarps) {
                uint32_t v = cl[i], b = G.r_ptr[v], e = G.r_ptr[v + 1];
                uint32_t c = 0;
                for (uint32_t k = b + lane; k < e; k += 32) {
                    uint32_t u = G.r_adj[k], lo = 0, hi = d;
                    while (lo < hi) {
                        uint32_t mid = (lo + hi) >> 1;
                        if (L0[mid] < u)
                            lo = mid + 1;
                        else
                            hi = mid;
                    }
                    c += (lo < d && L0[lo] == u);
                }
                if (lane == 0) scan += e - b;
                c = warp_sum(c);
                if (lane == 0) cntA[i] = c;
            }
        }
        __syncthreads();
        PA_MARK(0);
        // 3. classify: Q part (lower rank), absorbed, P part
        unsigned long long sabs = 0;
        uint32_t nabs = 0, nq = 0, np = 0, nonmax = 0;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            uint32_t v = cl[i], c = cntA[i];
            if (v < x) {
                nonmax |= (c == d);
                nq++;
            } else if (c == d) {
                sabs += G.eR[v];
                nabs++;
                cmap[v] = -3;
            } else {
                np++;
            }
        }
        sabs = warp_sum(sabs);
        nabs = warp_sum(nabs);
        nq = warp_sum(nq);
        np = warp_sum(np);
        nonmax = __any_sync(kFull, nonmax != 0);
        scan = warp_sum(scan);
        unsigned long long sl = 0;
        for (uint32_t j = threadIdx.x; j < d; j += blockDim.x) sl += G.eL[L0[j]];
        sl = warp_sum(sl);
        if (lane == 0) {
            atomicAdd(&s_sabs, sabs);
            atomicAdd(&s_nabs, nabs);
            atomicAdd(&s_nq, nq);
            atomicAdd(&s_np, np);
            if (nonmax) s_nonmax = 1;
            atomicAdd(&s_sl, sl);
            atomicAdd(&s_scan, scan);
        }
        __syncthreads();
        const uint32_t nRset = 1 + s_nabs;
        const uint32_t n2 = s_nq + s_np;
        const bool emit_task = !s_nonmax && s_np > 0 && nRset + s_np >= G.minR;
        const uint64_t rw = a.emit ? record_words_r(W, n2, false, nRset) : record_words(W, n2);
        if (threadIdx.x == 0) {
            s_rec = ~0ull;
            bool ok = true;
            if (emit_task) {
                unsigned long long off = pool_alloc(a, rw);
                if (off == ~0ull) {
                    // does not fit this chunk: retry in a later chunk, count nothing now
                    ok = false;
                    uint32_t r = atomicAdd(a.n_retry, 1u);
                    if (r < a.retry_cap)
                        a.retry[r] = s_idx;
                    else
                        set_error(a, kErrPool, rw);
                }
                s_rec = off;
            }
            if (ok) {
                ResultAcc* r = &a.results[rt.x];
                unsigned long long words = s_scan * 2 + d;
                atomicAdd(&r->nodes, 1ull);
                atomicAdd(&r->words_expand, words);
                if (!s_nonmax && nRset >= G.minR) {
                    unsigned long long sR = G.eR[x] + s_sabs;
                    atomicAdd(&r->count, 1ull);
                    atomicAdd(&r->hash, (unsigned long long)side_hash(G, s_sl, d, sR, nRset));
                    s_counted = 1;
                }
            }
        }
        __syncthreads();
        PA_MARK(1);
        if (a.emit && s_counted && warp == 0) {
            // the root biclique: R = x + the absorbed, L = N(x)
            const unsigned long long o = emit_reserve(a, nRset, d, G.swapped);
            if (o != ~0ull) {
                uint32_t* dr = a.emit_ids + o + (G.swapped ? d : 0);
                uint32_t* dl = a.emit_ids + o + (G.swapped ? 0 : nRset);
                root_rlist(x, cl, cntA, n, d, dr, G.r_orig);
                for (uint32_t t = lane; t < d; t += 32) dl[t] = L0[t];
            }
        }
        if (emit_task && s_rec != ~0ull) {
            // 4. order: Q part by count descending, then P part by count
            // ascending (the min-count child order), by a counting sort over
            // 2d buckets: a Q count c goes to bucket d - c, a P count c to
            // bucket d + c.  Candidates of equal count keep no fixed order.
            uint32_t* hist = 2 * d <= 4096 ? (uint32_t*)s_keys : (uint32_t*)gkeys;
            for (uint32_t b = threadIdx.x; b < 2 * d; b += blockDim.x) hist[b] = 0;
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                const uint32_t v = cl[i], c = cntA[i];
                if (v < x)
                    atomicAdd(&hist[d - c], 1u);
                else if (c != d)
                    atomicAdd(&hist[d + c], 1u);
            }
            __syncthreads();
            block_exclusive_scan(hist, 2 * d, s_wsum);
#ifdef MBE_PROFILE
            PA_MARK(2);
#endif
            {
                uint32_t* rec = a.pool + s_rec;
                uint32_t* wmap = rec + kHdrWords;
                uint32_t* Lm = wmap + pad4(W);
                uint32_t* cand = Lm + pad4(W);
                uint32_t* cnt = cand + pad4(n2);
                uint32_t* M = cnt + pad4(n2);
                if (threadIdx.x == 0) {
                    atomicMax(a.max_n, n2);
                    NodeHdr* h = (NodeHdr*)rec;
                    h->graph = rt.x;
                    h->root = x;
                    h->W = W;
                    h->n = n2;
                    h->nq = s_nq;
                    h->l = d;
                    h->nRset = nRset;
                    h->depth = 1;
                    h->sR = G.eR[x] + s_sabs;
                    h->words = (uint32_t)rw;
                    h->rlist = 0;
                    h->flags = 0;
                }
                for (uint32_t w = threadIdx.x; w < W; w += blockDim.x) {
                    wmap[w] = w;
                    uint32_t rem = d - w * 32;
                    Lm[w] = rem >= 32 ? 0xFFFFFFFFu : ((1u << rem) - 1u);
                }
                for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                    const uint32_t v = cl[i], c = cntA[i];
                    const bool q = v < x;
                    if (!q && c == d) continue;  // absorbed
                    const uint32_t p = atomicAdd(&hist[q ? d - c : d + c], 1u);
                    cand[p] = v;
                    cnt[p] = q ? 0u : c;
                    cmap[v] = (int)p;
                }
                uint64_t mw = (uint64_t)W * n2;
                for (uint64_t i = threadIdx.x; i < mw; i += blockDim.x) M[i] = 0;
                __syncthreads();
                // 6. bit rows: bit j of candidate p set iff (L0[j], cand[p]) is an edge
                if (rs) {
                    // the long lists noted by the first scatter are scanned
                    // by the whole block (all of them, when none was left
                    // with its warp), the rest by a warp each
                    const bool split = s_nlong <= kLongCap;
                    for (uint32_t j = warp; j < d; j += nwarps) {
                        uint32_t u = L0[j], b = G.l_ptr[u], e = G.l_ptr[u + 1];
                        if (split && e - b > kLongList) continue;
                        uint32_t* Mw = M + (size_t)(j >> 5) * n2;
                        uint32_t bit = 1u << (j & 31);
                        for (uint32_t k = b + lane; k < e; k += 32) {
                            int p = cmap[G.l_adj[k]];
                            if (p >= 0) atomicOr(&Mw[p], bit);
                        }
                    }
                    for (uint32_t h = 0; split && h < s_nlong; h++) {
                        const uint32_t j = s_long[h];
                        const uint32_t u = L0[j], b = G.l_ptr[u], e = G.l_ptr[u + 1];
                        uint32_t* Mw = M + (size_t)(j >> 5) * n2;
                        const uint32_t bit = 1u << (j & 31);
                        for (uint32_t k = b + threadIdx.x; k < e; k += blockDim.x) {
                            int p = cmap[G.l_adj[k]];
                            if (p >= 0) atomicOr(&Mw[p], bit);
                        }
                    }
                } else {
                    for (uint32_t p = warp; p < n2; p += nwarps) {
                        uint32_t v = cand[p], b = G.r_ptr[v], e = G.r_ptr[v + 1];
                        for (uint32_t k = b + lane; k < e; k += 32) {
                            uint32_t u = G.r_adj[k], lo = 0, hi = d;
                            while (lo < hi) {
                                uint32_t mid = (lo + hi) >> 1;
                                if (L0[mid] < u)
                                    lo = mid + 1;
                                else
                                    hi = mid;
                            }
                            if (lo < d && L0[lo] == u) atomicOr(&M[(size_t)(lo >> 5) * n2 + p], 1u << (lo & 31));
                        }
                    }
                }
                __syncthreads();
                PA_MARK(3);
                // 7. Q reduction: a Q row contained in one of the first
                // kKeepWindow kept rows (Q is in count-descending order) is
                // dropped; the record is then compacted in place.
                uint32_t* flag = s_nq <= 4096 ? (uint32_t*)s_keys : (uint32_t*)gkeys;  // keep flags
                if (warp == 0) {
                    // kept window: greedy in row order, 32 rows per step.  Each
                    // lane tests its row against the window; survivors are
                    // taken in order and each one kept is tested against by
                    // the later lanes (same result as one row at a time).
                    uint32_t kept_p = 0, nk = 0, pos = 0;
                    while (pos < s_nq && nk < kKeepWindow) {
                        const uint32_t p = pos + lane;
                        const bool valid = p < s_nq;
                        const SparseRow r = sparse_row(M, n2, W, valid ? p : pos);
                        bool dom = !valid;
                        for (uint32_t j = 0; j < nk; j++) {
                            const uint32_t kp = __shfl_sync(kFull, kept_p, j);
                            dom = dom || row_subset(r, M, n2, W, p, kp);
                        }
                        unsigned pending = __ballot_sync(kFull, !dom), keepm = 0;
                        uint32_t upto = 32;  // lanes whose row this step decides
                        while (pending) {
                            const uint32_t j = __ffs(pending) - 1;
                            pending &= pending - 1;
                            if (nk == kKeepWindow) {  // window full: the rest go to the parallel pass
                                upto = j;
                                break;
                            }
                            keepm |= 1u << j;
                            if (lane == nk) kept_p = pos + j;
                            nk++;
                            pending &= ~__ballot_sync(kFull, lane > j && ((pending >> lane) & 1u) &&
                                                                 row_subset(r, M, n2, W, p, pos + j));
                        }
                        if (valid && lane < upto) flag[p] = (keepm >> lane) & 1u;
                        pos += upto;
                    }
                    if (lane < nk) s_kept[lane] = kept_p;
                    if (lane == 0) {
                        s_nk = nk;
                        s_p1 = min(pos, s_nq);
                    }
                }
                __syncthreads();
                for (uint32_t p = s_p1 + threadIdx.x; p < s_nq; p += blockDim.x) {
                    const SparseRow r = sparse_row(M, n2, W, p);
                    bool keep = true;
                    for (uint32_t j = 0; j < s_nk && keep; j++)
                        if (row_subset(r, M, n2, W, p, s_kept[j])) keep = false;
                    flag[p] = keep;
                }
                __syncthreads();
                PA_MARK(4);
                // new positions of kept Q rows (block scan in chunks, one
                // barrier each: every thread keeps the running total, and
                // the warp counts alternate between two halves of s_wsum, so
                // a chunk's counts never overwrite ones still being read)
                static_assert(kThreadsA / 32 <= 16, "two halves of s_wsum hold the warp counts");
                uint32_t nq2 = 0;
                for (uint32_t b0 = 0, it = 0; b0 < s_nq; b0 += blockDim.x, it++) {
                    uint32_t* ws = s_wsum + (it & 1u) * 16u;
                    uint32_t p = b0 + threadIdx.x;
                    uint32_t f = p < s_nq ? flag[p] : 0u;
                    unsigned bal = __ballot_sync(kFull, f);
                    if (lane == 0) ws[warp] = __popc(bal);
                    __syncthreads();
                    uint32_t before = nq2, tot = 0;
                    for (uint32_t ww = 0; ww < nwarps; ww++) {
                        const uint32_t c = ws[ww];
                        if (ww < warp) before += c;
                        tot += c;
                    }
                    if (p < s_nq) flag[p] = f ? (before + __popc(bal & lanemask_lt())) : 0xFFFFFFFFu;
                    nq2 += tot;
                }
                __syncthreads();  // the new positions are read by other threads below
                if (nq2 < s_nq) {
                    const uint32_t n3 = nq2 + s_np;
                    // every move goes to a lower address: process arrays in
                    // address order, each in chunks read-all-then-write-all
                    auto newpos = [&](uint32_t p) -> uint32_t {
                        return p < s_nq ? flag[p] : p - s_nq + nq2;
                    };
                    uint32_t* cand3 = Lm + pad4(W);
                    uint32_t* cnt3 = cand3 + pad4(n3);
                    uint32_t* M3 = cnt3 + pad4(n3);
                    for (int arr = 0; arr < 2 + (int)W; arr++) {
                        const uint32_t* src = arr == 0 ? cand : arr == 1 ? cnt : M + (size_t)(arr - 2) * n2;
                        uint32_t* dst = arr == 0 ? cand3 : arr == 1 ? cnt3 : M3 + (size_t)(arr - 2) * n3;
                        for (uint32_t b0 = 0; b0 < n2; b0 += 4 * blockDim.x) {
                            uint32_t vals[4], dpos[4];
#pragma unroll
                            for (int q = 0; q < 4; q++) {
                                uint32_t p = b0 + q * blockDim.x + threadIdx.x;
                                dpos[q] = 0xFFFFFFFFu;
                                if (p < n2) {
                                    uint32_t np_ = newpos(p);
                                    if (np_ != 0xFFFFFFFFu) {
                                        dpos[q] = np_;
                                        vals[q] = src[p];
                                    }
                                }
                            }
                            __syncthreads();
                            // a write lands below its own source, so it can
                            // only meet sources of lower positions (read by
                            // now) or of the previous array (done): the next
                            // chunk's reads need no barrier after the writes
#pragma unroll
                            for (int q = 0; q < 4; q++)
                                if (dpos[q] != 0xFFFFFFFFu) dst[dpos[q]] = vals[q];
                        }
                    }
                    __syncthreads();
                    if (threadIdx.x == 0) {
                        NodeHdr* h = (NodeHdr*)rec;
                        h->n = n3;
                        h->nq = nq2;
                        h->words = (uint32_t)record_words(W, n3);
                    }
                }
                if (a.emit) {
                    // R list after the (compacted) rows: x + the absorbed, as ranks
                    const uint32_t nfin = nq2 < s_nq ? nq2 + s_np : n2;
                    const uint32_t rl = (uint32_t)record_words(W, nfin);
                    __syncthreads();
                    if (warp == 0) root_rlist(x, cl, cntA, n, d, rec + rl, nullptr);
                    if (threadIdx.x == 0) {
                        ((NodeHdr*)rec)->rlist = rl;
                        ((NodeHdr*)rec)->words = rl + pad4(nRset);
                    }
                }
                __threadfence();
                __syncthreads();
                if (threadIdx.x == 0) {
                    Task t{};
                    t.node = (unsigned long long)(rec);
                    t.begin = 0;
                    t.end = s_np;
                    t.plen = 0;  // pool record: shared by pointer
                    push_task(a, t);
                }
            }
        }
        __syncthreads();
        PA_MARK(5);
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) cmap[cl[i]] = -1;
        __syncthreads();
#ifdef MBE_PROFILE
        if (threadIdx.x == 0 && a.prof_a) {
            unsigned long long tot = (unsigned long long)(clock64() - pa_root0);
            atomicAdd(&a.prof_a[12], tot);
            atomicAdd(&a.prof_a[13], 1ull);
            if (tot > atomicMax(&a.prof_a[14], tot)) a.prof_a[15] = d;
        }
#endif
    }
}

// ---------------------------------------------------------------------------
// Phase B: warp DFS with donation

// Per-warp state of the DFS kernel.  It is warp-uniform, so it lives in
// shared memory, one copy per warp: kept in local memory it would be held
// once per lane (local memory is per thread) and compete with the record
// scans for L1.  Lane 0 writes it (at kernel start, and slab_* when
// donating); every lane reads it.
struct WarpCtx {
    uint32_t* arena;       // this warp's DFS arena (a.arena_words words)
    uint32_t* scrLi;
    uint32_t* scrNz;
    uint32_t* scrQcnt;
    unsigned long long* scrKeysP;
    unsigned long long* scrKeysQ;
    uint32_t* scrPack;     // 2 x kc words: srow, spos of a packed build too large for shared memory
    uint32_t* scrHist;     // 32 maxW + 32 words: count histogram of a wide child's sorts
    uint32_t* scrAbs;      // scr_n words: ranks absorbed by the child being evaluated (output stream only)
    uint32_t scr_kc;       // key-array capacity of this launch's scratch layout
    unsigned long long slab_off, slab_end;  // this warp's slab of the node pool (donation copies)
#ifdef MBE_PROFILE
    long long prof[kProfSlots];    // section cycles and events (lane 0 adds)
    unsigned long long last_busy;  // globaltimer when the warp last finished a task
    unsigned long long t_start;    // globaltimer at kernel start
#endif
};

// Shared memory of the DFS kernel, per warp (file scope, so that the
// out-of-line helpers address it directly).
__shared__ WarpCtx s_wc[kWarpsB];
__shared__ uint32_t s_Li[kWarpsB][kSmemW];        // L_i words (when W <= kSmemW)
__shared__ uint32_t s_Nz[kWarpsB][kSmemW];        // their record word indices
__shared__ uint32_t s_Bucket[kWarpsB][64];        // Q' then P' count buckets of a packed build
__shared__ uint32_t s_Row[kWarpsB][kShRows];      // Q' rows of a packed build
__shared__ uint32_t s_Pos[kWarpsB][kShRows];      // their parent positions
__shared__ unsigned long long s_Keys[kWarpsB][kShRows];  // P' keys of a packed child
__shared__ SolveLevel s_Solve[kWarpsB][kSolveRows + 1];  // saved levels of the register search
__shared__ GraphView s_G[kWarpsB];                // the graph of the warp's current task
__shared__ ResultAcc s_acc[kWarpsB];              // the current task's counts (flushed per task)

__device__ __forceinline__ uint32_t warp_in_block() { return threadIdx.x >> 5; }
__device__ __forceinline__ WarpCtx& my_wc() { return s_wc[warp_in_block()]; }

// Adds one evaluation's counts (kept in registers while it runs) to the
// warp's accumulator in shared memory: lane 0 writes, so nothing of it stays
// live in registers across the search loop's out-of-line calls.
__device__ __forceinline__ void acc_commit(const ResultAcc& v) {
    if (lane_id() == 0) {
        ResultAcc& s = s_acc[warp_in_block()];
        s.count += v.count;
        s.hash += v.hash;
        s.nodes += v.nodes;
        s.words += v.words;
    }
}

// Adds v to an evaluation's set-word counter when the build keeps it.
template <class Acc>
__device__ __forceinline__ void count_words(Acc& acc, unsigned long long v) {
    if (kCountWords) acc.words += v;
}

// Ticket queue: an idle warp takes the next slot index with one atomicAdd
// and then watches only that slot's ready flag, so waiting warps never
// contend on a shared word.  Slot h is filled by the h-th push.  Waiting
// ends when the slot is ready, or when pending == 0 (no queued and no
// running task: nothing can be pushed any more), or on an error, or when
// no warp has made progress for timeout_ns.
struct Popped {
    unsigned long long node;   // 0 when no task was taken (done, error)
    uint32_t begin, end, plen;
    uint32_t path;             // lane j holds path[j]
};

__device__ __noinline__ Popped pop_task(const EngineArgs& a) {
    unsigned lane = lane_id();
    Popped t{0ull, 0u, 0u, 0u, 0u};
    int state = 0;  // 1 = got, 2 = done
    uint32_t h = 0;
    if (lane == 0) {
        h = atomicAdd(a.q_head, 1u);
        unsigned long long t0 = globaltimer_ns();
        unsigned long long last_prog = ld_volatile(a.progress);
        unsigned sleep_ns = 32;
        const uint32_t slot = h % a.task_cap;
        for (;;) {
            if (ld_volatile(&a.ready[slot]) == h + 1u) {
                state = 1;
                break;
            }
            if (ld_volatile(a.error) || ld_volatile(a.pending) == 0) {
                state = 2;
                break;
            }
            __nanosleep(sleep_ns);
            if (sleep_ns < kPopSleepMax) sleep_ns <<= 1;
            unsigned long long now = globaltimer_ns();
            unsigned long long prog = ld_volatile(a.progress);
            if (prog != last_prog) {
                last_prog = prog;
                t0 = now;
            } else if (now - t0 > a.timeout_ns) {
                set_error(a, kErrTimeout, h);
                state = 2;
                break;
            }
        }
        __threadfence();
    }
    state = __shfl_sync(kFull, state, 0);
    h = __shfl_sync(kFull, h, 0);
    if (state != 1) return t;
    const uint32_t slot = h % a.task_cap;
    volatile Task* src = (volatile Task*)&a.tasks[slot];
    t.node = src->node;
    t.begin = src->begin;
    t.end = src->end;
    t.plen = src->plen;
    t.path = lane < t.plen ? src->path[lane] : 0u;
    __syncwarp();
    if (lane == 0) {
        __threadfence();
        atomicExch(&a.ready[slot], 0u);
        atomicAdd(a.q_done, 1u);
    }
    return t;
}

struct ChildOut {
    uint32_t* rec;
    uint32_t nchild;
    uint32_t size;   // words taken from the arena (0 when in the pool)
    unsigned long long words;  // set words the out-of-line wide build streamed (added by its caller)
};


// row(c) n L_i is a subset of row(k) (both within the non-zero words of L_i)
__device__ __forceinline__ bool row_subset(const uint32_t* M, uint32_t n, const uint32_t* Nz, const uint32_t* Li,
                                           uint32_t nnz, uint32_t c, uint32_t k) {
    for (uint32_t j = 0; j < nnz; j++) {
        const uint32_t* Mw = M + (size_t)Nz[j] * n;
        if (Mw[c] & Li[j] & ~Mw[k]) return false;
    }
    return true;
}

struct RecView {
    uint32_t W, n, nq, flags;
    const uint32_t* map;   // wmap[W], or lmap[32] when packed
    const uint32_t* Lm;
    const uint32_t* cand;
    const uint32_t* cnt;   // nullptr when packed: a count is the row's popcount
    const uint32_t* M;
};

__device__ __forceinline__ RecView rec_view(const uint32_t* nd) {
    const NodeHdr* h = (const NodeHdr*)nd;
    RecView v;
    v.W = h->W;
    v.n = h->n;
    v.nq = h->nq;
    v.flags = h->flags;
    v.map = nd + kHdrWords;
    v.Lm = v.map + ((v.flags & kRecPacked) ? 32u : pad4(v.W));
    v.cand = v.Lm + pad4(v.W);
    const bool packed = (v.flags & kRecPacked) != 0;
    v.cnt = packed ? nullptr : v.cand + pad4(v.n);
    v.M = v.cand + (packed ? 1u : 2u) * pad4(v.n);
    return v;
}

// Writes the L members of L_i (words Li[0..nnz) at record words Nz[]) of
// record R (root nd) to dst in bit order.  Warp-collective.
__device__ __forceinline__ void write_lset(const GraphView& G, const uint32_t* nd, const RecView& R,
                                           const uint32_t* Li, const uint32_t* Nz, uint32_t nnz, uint32_t* dst) {
    const unsigned lane = lane_id();
    if (R.flags & kRecPacked) {  // packed maps hold L vertices
        const uint32_t bits = Li[0];
        if ((bits >> lane) & 1u) dst[__popc(bits & lanemask_lt())] = R.map[lane];
        return;
    }
    const uint32_t* L0 = G.r_adj + G.r_ptr[((const NodeHdr*)nd)->root];
    uint32_t before = 0;
    for (uint32_t k = 0; k < nnz; k++) {
        const uint32_t w = Li[k];
        if ((w >> lane) & 1u) dst[before + __popc(w & lanemask_lt())] = L0[R.map[Nz[k]] * 32 + lane];
        before += __popc(w);
    }
}

// Child x_i of record nd is a counted maximal biclique: R = the record's R
// list + x_i + the absorbed ranks abs[0..nabs), L = L_i.  Warp-collective.
__device__ __noinline__ void emit_child(const EngineArgs& a, const GraphView& G, const uint32_t* nd, uint32_t xi,
                                        const uint32_t* Li, const uint32_t* Nz, uint32_t nnz, uint32_t li,
                                        const uint32_t* abs, uint32_t nabs) {
    const RecView R = rec_view(nd);
    const uint32_t nrec = ((const NodeHdr*)nd)->nRset, nr = nrec + 1 + nabs;
    const unsigned long long o = emit_reserve(a, nr, li, G.swapped);
    if (o == ~0ull) return;
    uint32_t* dr = a.emit_ids + o + (G.swapped ? li : 0);
    uint32_t* dl = a.emit_ids + o + (G.swapped ? 0 : nr);
    copy_rlist(nd, dr, G.r_orig);
    if (lane_id() == 0) dr[nrec] = G.r_orig[R.cand[xi]];
    for (uint32_t t = lane_id(); t < nabs; t += 32) dr[nrec + 1 + t] = G.r_orig[abs[t]];
    write_lset(G, nd, R, Li, Nz, nnz, dl);
}

// A counted biclique of the register-resident search below packed record
// nd: R = the record's R list + the candidates of rows in Rm, L = the bits
// of L2 (over the record's L bits).  Warp-collective.
__device__ __noinline__ void emit_solved(const EngineArgs& a, const GraphView& G, const uint32_t* nd, uint32_t Rm,
                                         uint32_t L2) {
    const unsigned lane = lane_id();
    const RecView R = rec_view(nd);
    const uint32_t nrec = ((const NodeHdr*)nd)->nRset, nr = nrec + __popc(Rm), nl = __popc(L2);
    const unsigned long long o = emit_reserve(a, nr, nl, G.swapped);
    if (o == ~0ull) return;
    uint32_t* dr = a.emit_ids + o + (G.swapped ? nl : 0);
    uint32_t* dl = a.emit_ids + o + (G.swapped ? 0 : nr);
    copy_rlist(nd, dr, G.r_orig);
    if ((Rm >> lane) & 1u) dr[nrec + __popc(Rm & lanemask_lt())] = G.r_orig[R.cand[lane]];
    if ((L2 >> lane) & 1u) dl[__popc(L2 & lanemask_lt())] = R.map[lane];
}

// bits of x selected by m, packed to the low end in order
__device__ __forceinline__ uint32_t pext32(uint32_t x, uint32_t m) {
    uint32_t r = 0, bit = 1;
    while (m) {
        uint32_t low = m & (0u - m);
        if (x & low) r |= bit;
        bit <<= 1;
        m &= m - 1;
    }
    return r;
}


// Bit compress with a fixed mask (Warren, Hacker's Delight, 2nd ed., 7-4):
// the five shift masks depend on the mask only, so a build that packs many
// rows against the same L_i computes them once and then packs each row in
// five shift/mask steps.
struct CompressPlan {
    uint32_t mask, mv[5];
};

__device__ __forceinline__ CompressPlan compress_plan(uint32_t m) {
    CompressPlan p;
    p.mask = m;
    uint32_t mk = ~m << 1;
#pragma unroll
    for (int i = 0; i < 5; i++) {
        uint32_t mp = mk ^ (mk << 1);
        mp ^= mp << 2;
        mp ^= mp << 4;
        mp ^= mp << 8;
        mp ^= mp << 16;
        uint32_t mv = mp & m;
        p.mv[i] = mv;
        m = (m ^ mv) | (mv >> (1u << i));
        mk &= ~mp;
    }
    return p;
}

__device__ __forceinline__ uint32_t compress32(uint32_t x, const CompressPlan& p) {
    x &= p.mask;
#pragma unroll
    for (int i = 0; i < 5; i++) {
        uint32_t t = x & p.mv[i];
        x = (x ^ t) | (t >> (1u << i));
    }
    return x;
}

// L_i-restricted row of candidate c, packed to one word (|L_i| <= 32);
// plan0 is the compress plan of Li[0], used when L_i spans one word.
__device__ __forceinline__ uint32_t packed_row(const uint32_t* M, uint32_t n, const uint32_t* Nz,
                                               const uint32_t* Li, uint32_t nnz, uint32_t c,
                                               const CompressPlan& plan0) {
    if (nnz == 1) return compress32(M[(size_t)Nz[0] * n + c], plan0);
    uint32_t row = 0, sh = 0;
    for (uint32_t k = 0; k < nnz; k++) {
        row |= pext32(M[(size_t)Nz[k] * n + c], Li[k]) << sh;
        sh += __popc(Li[k]);
    }
    return row;
}

// Row of candidate c restricted to L_i, as the Q' gather and reduction use
// it: raw (M & Li[0]) when L_i spans one word, since counts and subset tests
// are the same on raw and packed masks; packed otherwise.  A raw row is
// packed (compress32 with plan0) only if it is kept.  M0 is the row strip of
// L_i's one word.
__device__ __forceinline__ uint32_t gather_row(const uint32_t* M, const uint32_t* M0, uint32_t n,
                                               const uint32_t* Nz, const uint32_t* Li, uint32_t nnz, uint32_t c,
                                               const CompressPlan& plan0) {
    if (nnz == 1) return M0[c] & plan0.mask;
    return packed_row(M, n, Nz, Li, nnz, c, plan0);
}

// Position of the k-th (0-based) set bit of x (k < popc(x)), by halving.
__device__ __forceinline__ uint32_t select32(uint32_t x, uint32_t k) {
    uint32_t pos = 0, c;
    c = __popc(x & 0xFFFFu);
    if (k >= c) { k -= c; x >>= 16; pos += 16; }
    c = __popc(x & 0xFFu);
    if (k >= c) { k -= c; x >>= 8; pos += 8; }
    c = __popc(x & 0xFu);
    if (k >= c) { k -= c; x >>= 4; pos += 4; }
    c = __popc(x & 0x3u);
    if (k >= c) { k -= c; x >>= 2; pos += 2; }
    if (k >= (x & 1u)) pos += 1;
    return pos;
}

// Turns per-key counts sb[0..32) into exclusive offsets; returns the total.
__device__ __forceinline__ uint32_t bucket_offsets(uint32_t* sb) {
    const unsigned lane = lane_id();
    __syncwarp();
    uint32_t cnt = sb[lane], inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, inc, o);
        if (lane >= (unsigned)o) inc += y;
    }
    __syncwarp();
    sb[lane] = inc - cnt;
    __syncwarp();
    return __shfl_sync(kFull, inc, 31);
}

// Child record construction when |L_i| <= 32: rows are packed to one word,
// so ordering is a counting sort over at most 31 counts and the Q reduction
// compares single words held in lane registers.  The Q' rows are gathered
// twice (a count histogram, then a scatter straight to their sorted slots,
// in shared memory when they fit); the P' histogram was taken during the
// expansion scan, so P' rows are written straight to their record slots.
// Produces the same record (same order, same reduction) as the general
// path would with packed rows.
__device__ ChildOut build_packed(const EngineArgs& a, const RecView& R, const NodeHdr* h, uint32_t xi, uint32_t li,
                                 uint32_t nnz, const uint32_t* Li, const uint32_t* Nz, uint32_t npp, uint32_t nR2,
                                 unsigned long long sR2, const unsigned long long* keysP, const GraphView& G,
                                 uint32_t arena_top, ResultAcc& acc) {
    const unsigned lane = lane_id();
    const uint32_t wb = warp_in_block();
    WarpCtx& wc = my_wc();
    const uint32_t n = R.n, nq = R.nq;
    const uint32_t* M = R.M;
    const CompressPlan plan0 = compress_plan(Li[0]);
    const uint32_t* M0 = M + (size_t)Nz[0] * n;
    ChildOut out{nullptr, 0, 0, 0ull};
    PROF_T0();
    // Q' = rows of Q u P[0..i) meeting L_i, by count descending (key li -
    // count in 1..31), parent order within a count
    uint32_t* sb = s_Bucket[wb];
    sb[lane] = 0;
    __syncwarp();
    for (uint32_t base = 0; base < xi; base += 32 * kUnrollG) {  // kUnrollG chunks per step: independent loads
        uint32_t r[kUnrollG];
#pragma unroll
        for (int q = 0; q < kUnrollG; q++) {
            uint32_t c = base + 32 * q + lane;
            r[q] = c < xi ? gather_row(M, M0, n, Nz, Li, nnz, c, plan0) : 0u;
        }
#pragma unroll
        for (int q = 0; q < kUnrollG; q++) {
            if (base + 32 * q >= xi) break;  // uniform: no rows left
            uint32_t key = r[q] ? li - __popc(r[q]) : 32u;
            unsigned grp = __match_any_sync(kFull, key);
            if (r[q] && (grp & lanemask_lt()) == 0) atomicAdd(&sb[key], (uint32_t)__popc(grp));
        }
    }
    const uint32_t m = bucket_offsets(sb);
    const bool shq = m <= kShRows;
    uint32_t* srow = shq ? s_Row[wb] : wc.scrPack;
    uint32_t* spos = shq ? s_Pos[wb] : wc.scrPack + wc.scr_kc;
    for (uint32_t base = 0; base < xi; base += 32 * kUnrollG) {
        uint32_t r[kUnrollG];
#pragma unroll
        for (int q = 0; q < kUnrollG; q++) {
            uint32_t c = base + 32 * q + lane;
            r[q] = c < xi ? gather_row(M, M0, n, Nz, Li, nnz, c, plan0) : 0u;
        }
#pragma unroll
        for (int q = 0; q < kUnrollG; q++) {
            if (base + 32 * q >= xi) break;  // uniform: no rows left
            uint32_t key = r[q] ? li - __popc(r[q]) : 32u;
            unsigned grp = __match_any_sync(kFull, key);
            uint32_t off = r[q] ? sb[key] : 0u;
            if (r[q]) {
                uint32_t p = off + __popc(grp & lanemask_lt());
                srow[p] = r[q];
                spos[p] = base + 32 * q + lane;
            }
            __syncwarp();
            if (r[q] && (grp & lanemask_lt()) == 0) sb[key] = off + __popc(grp);
            __syncwarp();
        }
    }
    count_words(acc, (unsigned long long)xi * nnz);
    PROF_ADD(wc.prof, kProfBGather);
    PROF_ADD(wc.prof, kProfBSort);
    // reduction, 32 candidates per step: every lane tests its row against the
    // window (the first kKeepWindow kept rows, in lane registers); the
    // survivors are then taken in order, and each one that joins the window
    // is tested against by all later lanes at once.  Same result as the
    // one-by-one greedy.
    uint32_t kept_row = 0, nk = 0, nq2 = 0;
    for (uint32_t base = 0; base < m; base += 32) {
        uint32_t idx = base + lane;
        bool valid = idx < m;
        uint32_t r = valid ? srow[idx] : 0u, p = valid ? spos[idx] : 0u;
        // lanes >= nk hold 0, which dominates no valid (non-zero) row
        bool dom = !valid;
        for (uint32_t j = 0; j < nk; j += 4) {
#pragma unroll
            for (uint32_t u = 0; u < 4; u++) {
                uint32_t kr = __shfl_sync(kFull, kept_row, j + u);
                dom = dom || (r & ~kr) == 0;
            }
            if (__all_sync(kFull, dom)) break;
        }
        unsigned pending = __ballot_sync(kFull, !dom), keep = 0;
        while (pending) {
            uint32_t j = __ffs(pending) - 1;
            pending &= pending - 1;
            keep |= 1u << j;
            if (nk < kKeepWindow) {
                uint32_t rj = __shfl_sync(kFull, r, j);
                if (lane == nk) kept_row = rj;
                nk++;
                pending &= ~__ballot_sync(kFull, lane > j && (r & ~rj) == 0);
            }
        }
        __syncwarp();  // all reads of this chunk precede the compacting writes
        if ((keep >> lane) & 1u) {
            uint32_t q = nq2 + __popc(keep & lanemask_lt());
            srow[q] = r;
            spos[q] = p;
        }
        nq2 += __popc(keep);
        __syncwarp();
    }
    PROF_ADD(wc.prof, kProfBReduce);
    // P' by count ascending, parent order within a count (keys in scan order)
    uint32_t* sbp = s_Bucket[wb] + 32;
    bucket_offsets(sbp);
    // allocate and write
    const uint32_t n2 = nq2 + npp;
    const uint64_t rw = a.emit ? record_words_r(1, n2, true, nR2) : record_words(1, n2, true);
    uint32_t* rec;
    if ((uint64_t)arena_top + rw <= a.arena_words) {
        rec = wc.arena + arena_top;
        out.size = (uint32_t)rw;
    } else {
        unsigned long long off = 0;
        if (lane == 0) {
            off = pool_alloc(a, rw);
            if (off == ~0ull) set_error(a, kErrPool, rw);
        }
        off = __shfl_sync(kFull, off, 0);
        if (off == ~0ull) return out;
        rec = a.pool + off;
        out.size = 0;
    }
    uint32_t* map2 = rec + kHdrWords;
    uint32_t* Lm2 = map2 + 32;
    uint32_t* cand2 = Lm2 + 4;
    uint32_t* M2 = cand2 + pad4(n2);  // no count array: counts are row popcounts
    if (lane == 0) {
        NodeHdr* h2 = (NodeHdr*)rec;
        h2->graph = h->graph;
        h2->root = h->root;
        h2->W = 1;
        h2->n = n2;
        h2->nq = nq2;
        h2->l = li;
        h2->nRset = nR2;
        h2->depth = h->depth + 1;
        h2->sR = sR2;
        h2->words = (uint32_t)rw;
        h2->rlist = a.emit ? (uint32_t)record_words(1, n2, true) : 0u;
        h2->flags = kRecPacked;
        Lm2[0] = li == 32 ? 0xFFFFFFFFu : ((1u << li) - 1u);
    }
    if (a.emit)
        write_child_rlist((const uint32_t*)h, R.cand[xi], wc.scrAbs, nR2 - h->nRset - 1,
                          rec + record_words(1, n2, true));
    // lane t < li: L vertex of the t-th set bit of L_i (words in order)
    if (lane < li) {
        uint32_t vtx;
        if (R.flags & kRecPacked) {
            vtx = R.map[select32(Li[0], lane)];
        } else {
            uint32_t before = 0, k = 0;
            for (; k + 1 < nnz; k++) {
                uint32_t c = __popc(Li[k]);
                if (lane < before + c) break;
                before += c;
            }
            const uint32_t* L0 = G.r_adj + G.r_ptr[h->root];
            vtx = L0[R.map[Nz[k]] * 32 + select32(Li[k], lane - before)];
        }
        map2[lane] = vtx;
    }
    for (uint32_t t = lane; t < nq2; t += 32) {
        cand2[t] = R.cand[spos[t]];
        M2[t] = nnz == 1 ? compress32(srow[t], plan0) : srow[t];
    }
    for (uint32_t base = 0; base < npp; base += 32) {
        uint32_t t = base + lane;
        bool v = t < npp;
        unsigned long long key = v ? keysP[t] : 0ull;
        uint32_t cc = v ? (uint32_t)(key >> 32) : 32u;
        unsigned grp = __match_any_sync(kFull, cc);
        uint32_t off = v ? sbp[cc] : 0u;
        if (v) {
            uint32_t dst = nq2 + off + __popc(grp & lanemask_lt());
            uint32_t c = nq + (uint32_t)key;
            cand2[dst] = R.cand[c];
            M2[dst] = nnz == 1 ? compress32(M0[c], plan0) : packed_row(M, n, Nz, Li, nnz, c, plan0);
        }
        __syncwarp();
        if (v && (grp & lanemask_lt()) == 0) sbp[cc] = off + __popc(grp);
        __syncwarp();
    }
    count_words(acc, (unsigned long long)n2 + (unsigned long long)npp * nnz);
    __syncwarp();
    PROF_ADD(wc.prof, kProfBWrite);
    PROF_VAL(wc.prof, kProfSumXi, xi);
    PROF_VAL(wc.prof, kProfSumM, m);
    PROF_VAL(wc.prof, kProfSumNq2, nq2);
    PROF_VAL(wc.prof, kProfSumNpp, npp);
    out.rec = rec;
    out.nchild = npp;
    return out;
}

// Stable counting sort of n 64-bit keys by their high word (in [0, B)),
// through tmp[n]; hist holds B words.  Replaces a bitonic sort of the same
// keys when the high words are small counts: the order is the same.
// Warp-collective.
__device__ void warp_count_sort(unsigned long long* keys, uint32_t n, uint32_t B, uint32_t* hist,
                                unsigned long long* tmp) {
    const unsigned lane = lane_id();
    for (uint32_t b = lane; b < B; b += 32) hist[b] = 0;
    __syncwarp();
    for (uint32_t base = 0; base < n; base += 32) {
        const uint32_t i = base + lane;
        const bool v = i < n;
        const uint32_t k = v ? (uint32_t)(keys[i] >> 32) : 0xFFFFFFFFu;
        const unsigned grp = __match_any_sync(kFull, k);
        if (v && (grp & lanemask_lt()) == 0) atomicAdd(&hist[k], (uint32_t)__popc(grp));
    }
    __syncwarp();
    uint32_t carry = 0;
    for (uint32_t base = 0; base < B; base += 32) {
        const uint32_t b = base + lane;
        const uint32_t c = b < B ? hist[b] : 0u;
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, inc, o);
            if (lane >= (unsigned)o) inc += y;
        }
        if (b < B) hist[b] = carry + inc - c;
        carry += __shfl_sync(kFull, inc, 31);
    }
    __syncwarp();
    for (uint32_t base = 0; base < n; base += 32) {
        const uint32_t i = base + lane;
        const bool v = i < n;
        const unsigned long long key = v ? keys[i] : 0ull;
        const uint32_t k = v ? (uint32_t)(key >> 32) : 0xFFFFFFFFu;
        const unsigned grp = __match_any_sync(kFull, k);
        const uint32_t off = v ? hist[k] : 0u;
        if (v) tmp[off + __popc(grp & lanemask_lt())] = key;
        __syncwarp();
        if (v && (grp & lanemask_lt()) == 0) hist[k] = off + __popc(grp);
        __syncwarp();
    }
    for (uint32_t i = lane; i < n; i += 32) keys[i] = tmp[i];
    __syncwarp();
}

// Child record construction when |L_i| > 32 (rows stay word-sliced): the
// Q part is sorted by count descending and reduced against a window of kept
// rows, the P part sorted by count ascending.  Kept out of line: it is rare
// next to packed builds and large.
__device__ __noinline__ ChildOut build_general(const EngineArgs& a, const GraphView& G, const uint32_t* nd,
                                               uint32_t xi, uint32_t li, uint32_t nnz, const uint32_t* Li,
                                               const uint32_t* Nz, uint32_t npp, uint32_t nR2,
                                               unsigned long long sR2, bool known_max, uint32_t arena_top) {
    const unsigned lane = lane_id();
    WarpCtx& wc = my_wc();
    struct { unsigned long long words; } acc{0ull};  // set words streamed, returned in ChildOut
    PROF_T0();
    const NodeHdr* h = (const NodeHdr*)nd;
    const RecView R = rec_view(nd);
    const uint32_t n = R.n, nq = R.nq;
    const uint32_t* M = R.M;
    const uint32_t* cand = R.cand;
    ChildOut out{nullptr, 0, 0, 0ull};
    if (known_max) {
        // the prefilter only settled maximality: count Q u P[0..i) now
        for (uint32_t base = 0; base < xi; base += 32) {
            uint32_t c = base + lane;
            if (c < xi) {
                uint32_t cc = 0;
                for (uint32_t k = 0; k < nnz; k++) cc += __popc(M[(size_t)Nz[k] * n + c] & Li[k]);
                wc.scrQcnt[c] = cc;
            }
        }
        count_words(acc, (unsigned long long)nnz * xi);
        __syncwarp();
    }

    // 5a. Q' = Q u P[0..i) restricted to rows meeting L_i, by count descending
    uint32_t m = 0;
    for (uint32_t base = 0; base < xi; base += 32) {
        uint32_t c = base + lane;
        uint32_t cc = c < xi ? wc.scrQcnt[c] : 0u;
        unsigned bal = __ballot_sync(kFull, cc > 0);
        if (cc > 0) wc.scrKeysQ[m + __popc(bal & lanemask_lt())] = ((unsigned long long)(li - cc) << 32) | c;
        m += __popc(bal);
    }
    __syncwarp();
    if (m <= 32) {
        unsigned long long k = lane < m ? wc.scrKeysQ[lane] : kInvalidKey;
        k = warp_sort_reg(k);
        if (lane < m) wc.scrKeysQ[lane] = k;
    } else {
        // count descending (key li - count), parent order within a count
        warp_count_sort(wc.scrKeysQ, m, li + 1, wc.scrHist, (unsigned long long*)wc.scrPack);
    }
    __syncwarp();
    // 5b. reduction, 32 candidates per step (same scheme as build_packed):
    // test against the window of kept rows in parallel, then take the
    // survivors in order, each row joining the window tested by later lanes
    uint32_t kept_c = 0, nk = 0, nq2 = 0;  // lane j holds the j-th kept candidate
    for (uint32_t base = 0; base < m; base += 32) {
        uint32_t idx = base + lane;
        bool valid = idx < m;
        uint32_t c = valid ? (uint32_t)wc.scrKeysQ[idx] : 0u;
        bool dom = !valid;
        for (uint32_t j = 0; j < nk; j++) {
            uint32_t kc = __shfl_sync(kFull, kept_c, j);
            if (!dom && row_subset(M, n, Nz, Li, nnz, c, kc)) dom = true;
        }
        unsigned pending = __ballot_sync(kFull, !dom), keep = 0;
        while (pending) {
            uint32_t j = __ffs(pending) - 1;
            pending &= pending - 1;
            keep |= 1u << j;
            if (nk < kKeepWindow) {
                uint32_t cj = __shfl_sync(kFull, c, j);
                if (lane == nk) kept_c = cj;
                nk++;
                bool d = ((pending >> lane) & 1u) && row_subset(M, n, Nz, Li, nnz, c, cj);
                pending &= ~__ballot_sync(kFull, d);
            }
        }
        __syncwarp();  // all reads of this chunk precede the compacting writes
        if ((keep >> lane) & 1u) wc.scrKeysQ[nq2 + __popc(keep & lanemask_lt())] = c;
        nq2 += __popc(keep);
        __syncwarp();
    }
    count_words(acc, (unsigned long long)m * nnz);
    // 5c. P' by (count ascending, parent order)
    if (npp <= 32) {
        unsigned long long k = lane < npp ? wc.scrKeysP[lane] : kInvalidKey;
        k = warp_sort_reg(k);
        if (lane < npp) wc.scrKeysP[lane] = k;
    } else {
        // count ascending, parent order within a count (keys in scan order)
        warp_count_sort(wc.scrKeysP, npp, li + 1, wc.scrHist, (unsigned long long*)wc.scrPack);
    }
    __syncwarp();

    // 5d. allocate and write the record
    const uint32_t n2 = nq2 + npp, W2 = nnz;  // |L_i| > 32 here: an unpacked child
    const uint64_t rw = a.emit ? record_words_r(W2, n2, false, nR2) : record_words(W2, n2, false);
    uint32_t* rec;
    if ((uint64_t)arena_top + rw <= a.arena_words) {
        rec = wc.arena + arena_top;
        out.size = (uint32_t)rw;
    } else {
        unsigned long long off = 0;
        if (lane == 0) {
            off = pool_alloc(a, rw);
            if (off == ~0ull) set_error(a, kErrPool, rw);
        }
        off = __shfl_sync(kFull, off, 0);
        if (off == ~0ull) {
            out.words = acc.words;
            return out;
        }
        rec = a.pool + off;
        out.size = 0;
    }
    uint32_t* map2 = rec + kHdrWords;
    uint32_t* Lm2 = map2 + pad4(W2);
    uint32_t* cand2 = Lm2 + pad4(W2);
    uint32_t* cnt2 = cand2 + pad4(n2);
    uint32_t* M2 = cnt2 + pad4(n2);
    if (lane == 0) {
        NodeHdr* h2 = (NodeHdr*)rec;
        h2->graph = h->graph;
        h2->root = h->root;
        h2->W = W2;
        h2->n = n2;
        h2->nq = nq2;
        h2->l = li;
        h2->nRset = nR2;
        h2->depth = h->depth + 1;
        h2->sR = sR2;
        h2->words = (uint32_t)rw;
        h2->rlist = a.emit ? (uint32_t)record_words(W2, n2, false) : 0u;
        h2->flags = 0u;
    }
    if (a.emit)
        write_child_rlist(nd, cand[xi], wc.scrAbs, nR2 - h->nRset - 1, rec + record_words(W2, n2, false));
    for (uint32_t k = lane; k < W2; k += 32) {
        map2[k] = R.map[Nz[k]];
        Lm2[k] = Li[k];
    }
    for (uint32_t t = lane; t < n2; t += 32) {
        uint32_t c, cntv;
        if (t < nq2) {
            c = (uint32_t)wc.scrKeysQ[t];
            cntv = 0;
        } else {
            unsigned long long key = wc.scrKeysP[t - nq2];
            c = nq + (uint32_t)key;
            cntv = (uint32_t)(key >> 32);
        }
        cand2[t] = cand[c];
        cnt2[t] = cntv;
        for (uint32_t k = 0; k < W2; k++) M2[(size_t)k * n2 + t] = M[(size_t)Nz[k] * n + c] & Li[k];
    }
    count_words(acc, (unsigned long long)W2 * n2);
    __syncwarp();
    PROF_ADD(wc.prof, kProfBuild);
    out.rec = rec;
    out.nchild = npp;
    out.words = acc.words;
    return out;
}

// Evaluates child i of the node record `nd` (one tree node).  Counts and
// hashes the biclique when maximal; materialises the child record when it
// has candidates.  Warp-collective.  known_max: the caller has already
// established that no row of Q u P[0..i) covers L_i (batch prefilter).
//
// The child's Q part is ordered by |N(v) n L_i| descending and reduced:
// a Q row contained in one of the first kKeepWindow kept rows is dropped,
// since whatever it covers in the subtree the containing row covers too.
// Large rows first make the first covering row of a non-maximal
// descendant appear within the first few candidates.  A child with
// |L_i| <= 32 is written packed: one word per row, L bits dense.
#ifdef MBE_EVAL_NOINLINE
__device__ __noinline__
#else
__device__
#endif
ChildOut eval_child_impl(const EngineArgs& a, const GraphView& G, const uint32_t* nd, uint32_t i, uint32_t arena_top,
                         ResultAcc& acc, bool replay, bool known_max) {
    const unsigned lane = lane_id();
    const uint32_t wb = warp_in_block();
    WarpCtx& wc = my_wc();
    PROF_T0();
    const NodeHdr* h = (const NodeHdr*)nd;
    const RecView R = rec_view(nd);
    const uint32_t W = R.W, n = R.n, nq = R.nq;
    const bool packed = (R.flags & kRecPacked) != 0;
    const uint32_t* M = R.M;
    const uint32_t* cand = R.cand;
    const uint32_t xi = nq + i;
    const uint32_t li = packed ? __popc(M[xi]) : R.cnt[xi];
    uint32_t* Li = W <= kSmemW ? s_Li[wb] : wc.scrLi;
    uint32_t* Nz = W <= kSmemW ? s_Nz[wb] : wc.scrNz;
    ChildOut out{nullptr, 0, 0, 0ull};

    // 1. L_i = L n N(x_i), keeping only non-zero words
    uint32_t nnz = 0;
    for (uint32_t base = 0; base < W; base += 32) {
        uint32_t w = base + lane;
        uint32_t v = w < W ? (R.Lm[w] & M[(size_t)w * n + xi]) : 0u;
        unsigned bal = __ballot_sync(kFull, v != 0);
        if (v) {
            uint32_t pos = nnz + __popc(bal & lanemask_lt());
            Li[pos] = v;
            Nz[pos] = w;
        }
        nnz += __popc(bal);
    }
    __syncwarp();
    if (!known_max) acc.nodes++;
    count_words(acc, W);
    // one-word L_i (the common case): its row strip and mask in registers,
    // since the scans below store to shared memory and the compiler would
    // otherwise reload Nz[0] and Li[0] before every chunk
    const uint32_t* M0 = M + (size_t)(nnz ? Nz[0] : 0u) * n;
    const uint32_t L0 = Li[0];

    // 2. maximality against Q u P[0..i); counts kept for Q' of a wide child
    // (a packed child, |L_i| <= 32, regathers its rows and never reads them)
    if (!known_max) {
        const bool es = a.variant != MBE_NOES;
        const bool keep_counts = li > 32;
        bool maximal = true;
        for (uint32_t base = 0; base < xi; base += 32) {
            uint32_t c = base + lane;
            uint32_t cc = 0;
            if (c < xi) {
                if (nnz == 1)
                    cc = __popc(M0[c] & L0);
                else
                    for (uint32_t k = 0; k < nnz; k++) cc += __popc(M[(size_t)Nz[k] * n + c] & Li[k]);
                if (keep_counts) wc.scrQcnt[c] = cc;
            }
            unsigned full = __ballot_sync(kFull, c < xi && cc == li);
            count_words(acc, (unsigned long long)nnz * min(32u, xi - base));
            if (full) {
                maximal = false;
                if (es) break;
            }
        }
        __syncwarp();
        PROF_ADD(wc.prof, kProfQscan);
        if (!maximal) return out;
    }

    // 3. expansion over P(i..], two chunks per step (independent loads).
    // For a packed child (|L_i| <= 32) the P' count histogram is taken here
    // and the keys stay in shared memory when they fit.
    const bool packed_child = li <= 32;
    unsigned long long* keysP = packed_child && n - xi - 1 <= kShRows ? s_Keys[wb] : wc.scrKeysP;
    if (packed_child) s_Bucket[wb][32 + lane] = 0;
    __syncwarp();
    uint32_t npp = 0, nabs = 0;
    unsigned long long sabs = 0;
    for (uint32_t base = xi + 1; base < n; base += 32 * kUnrollE) {
        uint32_t cc2[kUnrollE];
#pragma unroll
        for (int h2 = 0; h2 < kUnrollE; h2++) {
            uint32_t c = base + 32 * h2 + lane;
            uint32_t cc = 0;
            if (c < n) {
                if (nnz == 1)
                    cc = __popc(M0[c] & L0);
                else
                    for (uint32_t k = 0; k < nnz; k++) cc += __popc(M[(size_t)Nz[k] * n + c] & Li[k]);
            }
            cc2[h2] = cc;
        }
#pragma unroll
        for (int h2 = 0; h2 < kUnrollE; h2++) {
            if (base + 32 * h2 >= n) break;  // uniform: no rows left
            uint32_t c = base + 32 * h2 + lane;
            bool valid = c < n;
            uint32_t cc = cc2[h2];
            bool absorbed = valid && cc == li;
            bool partial = valid && cc > 0 && cc < li;
            if (absorbed) sabs += G.eR[cand[c]];
            unsigned pb = __ballot_sync(kFull, partial), ab = __ballot_sync(kFull, absorbed);
            if (partial) keysP[npp + __popc(pb & lanemask_lt())] = ((unsigned long long)cc << 32) | (c - nq);
            if (a.emit && absorbed) wc.scrAbs[nabs + __popc(ab & lanemask_lt())] = cand[c];
            if (packed_child && pb) {
                unsigned grp = __match_any_sync(kFull, partial ? cc : 32u);
                if (partial && (grp & lanemask_lt()) == 0) atomicAdd(&s_Bucket[wb][32 + cc], (uint32_t)__popc(grp));
            }
            npp += __popc(pb);
            nabs += __popc(ab);
        }
        count_words(acc, (unsigned long long)nnz * min(32u * kUnrollE, n - base));
    }
    __syncwarp();
    sabs = warp_sum(sabs);
    const uint32_t nR2 = h->nRset + 1 + nabs;
    const unsigned long long sR2 = h->sR + G.eR[cand[xi]] + sabs;

    // 4. count + canonical hash
    if (li >= G.minL && nR2 >= G.minR) {
        unsigned long long sl = 0;
        if (packed) {
            if ((Li[0] >> lane) & 1u) sl = G.eL[R.map[lane]];  // packed maps hold L vertices
        } else {
            const uint32_t* L0 = G.r_adj + G.r_ptr[h->root];
            for (uint32_t k = lane; k < nnz; k += 32) {
                uint32_t bits = Li[k], b0 = R.map[Nz[k]] * 32;
                while (bits) {
                    uint32_t t = __ffs(bits) - 1;
                    bits &= bits - 1;
                    sl += G.eL[L0[b0 + t]];
                }
            }
        }
        sl = warp_sum(sl);
        acc.count++;
        acc.hash += side_hash(G, sl, li, sR2, nR2);
        if (a.emit && !replay) emit_child(a, G, nd, xi, Li, Nz, nnz, li, wc.scrAbs, nabs);
    }

    // 5. child record
    PROF_ADD(wc.prof, kProfExpand);
    if (npp == 0 || li < G.minL || nR2 + npp < G.minR) return out;
    if (packed_child) {
        out = build_packed(a, R, h, xi, li, nnz, Li, Nz, npp, nR2, sR2, keysP, G, arena_top, acc);
        PROF_ADD(wc.prof, kProfBuild);
        return out;
    }
#ifdef MBE_PROFILE
    const long long c0g = clock64();
#endif
    out = build_general(a, G, nd, xi, li, nnz, Li, Nz, npp, nR2, sR2, known_max, arena_top);
    acc.words += out.words;
#ifdef MBE_PROFILE
    PROF_VAL(wc.prof, kProfGeneral, clock64() - c0g);
#endif
    return out;
}

// eval_child_impl with its counts committed to the warp's accumulator; a
// replayed evaluation re-derives a donated node, and its counts belong to
// the donor: they are dropped.
__device__ __forceinline__ ChildOut eval_child(const EngineArgs& a, const GraphView& G, const uint32_t* nd,
                                               uint32_t i, uint32_t arena_top, bool replay, bool known_max) {
    ResultAcc acc{};
    const ChildOut o = eval_child_impl(a, G, nd, i, arena_top, acc, replay, known_max);
    if (!replay) acc_commit(acc);
    return o;
}

// Maximality of up to 32 consecutive children of a record with one-word
// rows, one lane per child: lane j takes child base + j and walks the rows
// of Q u P[0..i) that can cover L_i, in order, until one does.  At every
// step all lanes read the same row (one broadcast load), eight rows per
// step.  Returns the children no row covers.  Exact: the same test
// eval_child makes, skipping only rows whose count rules them out.
__device__ uint32_t prefilter_w1(const RecView& R, uint32_t base, uint32_t nb) {
    const unsigned lane = lane_id();
    const bool active = lane < nb;
    const uint32_t nq = R.nq;
    const uint32_t xi = nq + base + lane;
    const uint32_t Li = active ? (R.Lm[0] & R.M[xi]) : 0u;
    const uint32_t lim = active ? xi : 0u;
    // A row covering L_i holds at least |L_i| of L's bits.  P rows are in
    // ascending count order, so none of P[0..i) has more than |L_i| and only
    // the run with exactly |L_i| can cover L_i: the lane scans all of Q,
    // then P from the first row of that run (found by binary search).
    uint32_t plo = lim;
    if (active) {
        const uint32_t li = __popc(Li);
        // counts: the record's count array, or the row popcounts of a
        // packed record (which stores none)
        const bool packed = (R.flags & kRecPacked) != 0;
        const uint32_t* cs = packed ? R.M : R.cnt;
        uint32_t lo = nq, hi = xi;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            const uint32_t v = cs[mid];
            if ((packed ? (uint32_t)__popc(v) : v) < li)
                lo = mid + 1;
            else
                hi = mid;
        }
        plo = lo;
    }
    bool covered = !active;
    uint32_t seen = 0;  // rows this lane tested
    const uint32_t qlim = min(nq, lim);
    for (uint32_t c = 0; __any_sync(kFull, !covered && c < qlim); c += kUnrollP) {
#pragma unroll
        for (uint32_t u = 0; u < (uint32_t)kUnrollP; u++) {
            const uint32_t cc = c + u;
            if (!covered && cc < qlim) {
                const uint32_t r = R.M[cc];
                covered = (r & Li) == Li;
                if (kCountWords) seen++;
            }
        }
    }
    const uint32_t p0 = __reduce_min_sync(kFull, covered ? 0xFFFFFFFFu : plo);
    for (uint32_t c = p0; __any_sync(kFull, !covered && c < lim); c += kUnrollP) {
#pragma unroll
        for (uint32_t u = 0; u < (uint32_t)kUnrollP; u++) {
            const uint32_t cc = c + u;
            if (!covered && cc >= plo && cc < lim) {
                const uint32_t r = R.M[cc];
                covered = (r & Li) == Li;
                if (kCountWords) seen++;
            }
        }
    }
    const unsigned long long scanned = kCountWords ? warp_sum((unsigned long long)seen) : 0ull;
    if (lane == 0) {
        if (kCountWords) s_acc[warp_in_block()].words += scanned + nb;
        s_acc[warp_in_block()].nodes += nb;
    }
    return __ballot_sync(kFull, active && !covered);
}

// Splits the remaining children of the shallowest frame with at least
// donate_min of them among the donor and up to 31 waiting warps (one task
// per lane, equal shares; the donor keeps the lowest indices).  Children the
// batch prefilter found maximal and that still wait in a frame's pmask count
// too, and go first: a frame with two or more of them gives its highest ones
// away as one-child tasks (the receiver re-tests their maximality).  Without
// this a warp holding a batch of up to 31 heavy children could not share them
// (bench graph 287 -> 256 ms, all of it in the closing phase).  A frame whose
// record is in the node pool is shared by pointer.  A frame whose record lives
// in this warp's arena is copied once into the pool when it fits (pool below
// 60%: small records into this warp's slab, larger ones by a direct
// allocation) and shared by pointer; otherwise it is described by the
// child-index path from frame 0 (always a pool record), which each receiver
// replays.  Warp-collective.
__device__ __noinline__ void try_donate(const EngineArgs& a, Frame* frames, int depth, uint32_t waiters) {
    unsigned lane = lane_id();
    WarpCtx& wc = my_wc();
    int k = -1;
    for (int base = 0; base <= depth && k < 0; base += 32) {
        int f = base + (int)lane;
        bool ok = false;
        if (f <= depth) {
            Frame fr = frames[f];
            uint32_t* nd = (uint32_t*)fr.node;
            bool in_arena = nd >= wc.arena && nd < wc.arena + a.arena_words;
            ok = ((fr.end > fr.next && fr.end - fr.next >= a.donate_min) || __popc(fr.pmask) >= 2) &&
                 (!in_arena || f <= (int)kMaxPath);
        }
        unsigned bal = __ballot_sync(kFull, ok);
        if (bal) k = base + __ffs(bal) - 1;
    }
    if (k < 0) return;
    Frame fr = frames[k];
    // children the batch prefilter found maximal and that wait in pmask go
    // first (they precede [next, end)); each one given away is its own task
    const uint32_t npend = __popc(fr.pmask);
    const bool from_mask = npend >= 2;
    const uint32_t rem = from_mask ? npend : fr.end - fr.next;
    const uint32_t pieces = min(min(waiters, 31u), rem - 1);  // tasks given away
    if (pieces == 0) return;
    const uint32_t share = rem / (pieces + 1);
    const uint32_t mid = fr.end - pieces * share;
    uint32_t* nd = (uint32_t*)fr.node;
    bool in_arena = nd >= wc.arena && nd < wc.arena + a.arena_words;
    unsigned long long copy_off = ~0ull;
    if (in_arena && a.donate_copy) {
        const uint32_t words = ((const NodeHdr*)nd)->words;
        const unsigned long long need = (words + 31ull) & ~31ull;  // whole 128-byte lines
        const unsigned long long limit = a.pool_words / 10 * 6;
        if (words <= kDonateSlabMax) {
            unsigned long long so = wc.slab_off, se = wc.slab_end;  // the warp's slab (uniform)
            if (so + need > se) {
                unsigned long long base = ~0ull;
                if (lane == 0 && ld_volatile(a.pool_top) + kSlabWords < limit)
                    base = atomicAdd(a.pool_top, (unsigned long long)kSlabWords);
                base = __shfl_sync(kFull, base, 0);
                if (base != ~0ull && base + kSlabWords <= a.pool_words) {
                    so = base;
                    se = base + kSlabWords;
                }
            }
            if (so + need <= se) {
                copy_off = so;
                so += need;
            }
            __syncwarp();
            if (lane == 0) {
                wc.slab_off = so;
                wc.slab_end = se;
            }
            __syncwarp();
        } else if (words <= kDonateCopyMax) {
            unsigned long long base = ~0ull;
            if (lane == 0 && ld_volatile(a.pool_top) + need < limit) base = atomicAdd(a.pool_top, need);
            base = __shfl_sync(kFull, base, 0);
            if (base != ~0ull && base + need <= a.pool_words) copy_off = base;
        }
        if (copy_off != ~0ull) {
            const uint4* s4 = (const uint4*)nd;
            uint4* d4 = (uint4*)(a.pool + copy_off);
            const uint32_t n4 = words / 4;
            uint32_t w = lane;
            for (; w + 96 < n4; w += 128) {  // four independent lines in flight
                uint4 v0 = s4[w], v1 = s4[w + 32], v2 = s4[w + 64], v3 = s4[w + 96];
                d4[w] = v0;
                d4[w + 32] = v1;
                d4[w + 64] = v2;
                d4[w + 96] = v3;
            }
            for (; w < n4; w += 32) d4[w] = s4[w];
            __threadfence();
            __syncwarp();
        }
    }
    // path element j = the child of frame j that frame j+1 expands (k <= kMaxPath <= 31)
    uint32_t pe = ((int)lane < k) ? frames[lane].cur : 0u;
    Task t{};
    if (!in_arena) {
        t.node = fr.node;
        t.plen = 0;
    } else if (copy_off != ~0ull) {
        t.node = (unsigned long long)(a.pool + copy_off);
        t.plen = 0;
    } else {
        t.node = frames[0].node;
        t.plen = (uint32_t)k;
    }
    for (int j = 0; j < (int)t.plen; j++) t.path[j] = __shfl_sync(kFull, pe, j);
    if (from_mask) {
        // the highest `pieces` pending children leave; the donor keeps the
        // lower ones (select32 gives the position of a set bit by rank)
        const uint32_t first = select32(fr.pmask, npend - pieces);
        if (lane == 0) frames[k].pmask = fr.pmask & ((1u << first) - 1u);
        if (lane < pieces) {
            t.begin = fr.mbase + select32(fr.pmask, npend - pieces + lane);
            t.end = t.begin + 1;
            push_task(a, t);
        }
    } else {
        if (lane == 0) frames[k].end = mid;
        if (lane < pieces) {
            t.begin = mid + lane * share;
            t.end = t.begin + share;
            push_task(a, t);
        }
    }
    __syncwarp();
}

// Adds the warp's accumulated counts to graph's result and clears them.
__device__ __noinline__ void flush_acc(const EngineArgs& a, uint32_t graph) {
    __syncwarp();
    if (lane_id() == 0) {
        ResultAcc& acc = s_acc[warp_in_block()];
        ResultAcc* r = &a.results[graph];
        if (acc.count) atomicAdd(&r->count, acc.count);
        if (acc.hash) atomicAdd(&r->hash, acc.hash);
        if (acc.nodes) atomicAdd(&r->nodes, acc.nodes);
        if (acc.words) atomicAdd(&r->words, acc.words);
        acc = ResultAcc{};
    }
    __syncwarp();
}

// 32 x 32 bit transpose across the warp: lane i holds row i on entry, lane
// b holds column b (bit i = bit b of row i) on return.  Five rounds swap the
// off-diagonal blocks of width 16, 8, 4, 2 and 1 with the partner lane i ^ s
// (each round exchanges one bit of the row index with the same bit of the
// column index); five shuffles instead of 32 ballots.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x) {
    const unsigned lane = lane_id();
    constexpr uint32_t kMask[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const uint32_t sh = 16u >> k, m = kMask[k];
        const uint32_t y = __shfl_xor_sync(kFull, x, sh);
        x = (lane & sh) ? ((x & ~m) | ((y >> sh) & m)) : ((x & m) | ((y & m) << sh));
    }
    return x;
}

// Children (lanes in `kids`) of a small-record node (L, Q, P) that no row of
// Q, nor an earlier row of P, covers.  One lane per child x: its coverers are
// the rows holding every bit of L_x = L & row_x, i.e. the AND over those bits
// b of col_b (col_b = the rows holding bit b: lane b's `col`, the transpose
// of the record's rows, fixed for the whole record).  Starting from the rows
// x may be covered by (Q, and P before x) and ANDing col_b bit by bit, x is
// maximal iff nothing is left; the loop takes popc(L_x) steps at most and
// ends as soon as no lane has a candidate coverer left.  Warp-collective.
__device__ __forceinline__ uint32_t solve_maximal(uint32_t row, uint32_t col, uint32_t L, uint32_t Q, uint32_t P,
                                                  uint32_t kids) {
    const unsigned lane = lane_id();
    const bool mine = (kids >> lane) & 1u;
    uint32_t rem = mine ? (L & row) : 0u;
    uint32_t cover = mine ? (Q | (P & ((1u << lane) - 1u))) : 0u;
    while (__any_sync(kFull, rem != 0 && cover != 0)) {
        const uint32_t b = rem ? __ffs(rem) - 1 : 0u;
        const uint32_t cb = __shfl_sync(kFull, col, b);
        if (rem) {
            cover &= cb;
            rem &= rem - 1;
        }
    }
    return __ballot_sync(kFull, mine && cover == 0);
}

// Enumerates the subtree below the children [next, end) of frame `fdepth`,
// whose record is packed with at most kSolveRows rows, without building
// child records: lane j holds row j (a mask over the record's L bits), and
// a tree node is (L, Q, P) with Q and P masks over the lanes.  Child x of a
// node takes L' = L & row_x; rows of P after x meeting all of L' join R,
// those meeting part of it form P', rows of Q or of P before x meeting it
// form Q'.  Rows are never reduced, so every check is one pass of shuffles.
// Q rows always precede the children of their node in row order.  The
// frame mirrors level 0 (next = one past the child in progress), so a donor
// may split the remaining level-0 children off as an ordinary task; the
// search then drops those it no longer owns.  Inlined into the search
// loop: as a call it made the loop save and restore its live registers in
// local memory on every small record (bench graph 236.8 -> 232.6 ms when
// inlined).  Warp-collective.
__device__ __forceinline__ void solve_small(const EngineArgs& a, const GraphView& G, const uint32_t* nd, Frame* frames,
                                         int fdepth, bool donate) {
    const unsigned lane = lane_id();
    ResultAcc acc{};  // in registers; committed to the warp's accumulator at the end
    const NodeHdr* h = (const NodeHdr*)nd;
    const RecView R = rec_view(nd);
    const uint32_t n = R.n, nq = R.nq;
    const uint32_t row = lane < n ? R.M[lane] : 0u;
    // transpose: lane b holds the rows that contain bit b of the record's L
    const uint32_t col = warp_transpose32(row);
    const unsigned long long eR = lane < n ? G.eR[R.cand[lane]] : 0ull;
    const uint32_t Lroot = R.Lm[0];
    const unsigned long long eL = ((Lroot >> lane) & 1u) ? G.eL[R.map[lane]] : 0ull;  // packed maps hold L vertices
    SolveLevel* st = s_Solve[warp_in_block()];
    const uint32_t all = n >= 32 ? ~0u : ((1u << n) - 1u);
    const uint32_t Qroot = (1u << nq) - 1u;  // nq < n <= 32
    const uint32_t lo = nq + frames[fdepth].next, hi = nq + frames[fdepth].end;
    const uint32_t kids0 = (hi >= 32 ? ~0u : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
    uint32_t L = Lroot, Q = Qroot, P = all & ~Qroot, nR = h->nRset, Rm = 0;
    unsigned long long sR = h->sR;
    uint32_t pend = solve_maximal(row, col, L, Q, P, kids0);
    acc.nodes += __popc(kids0);
    count_words(acc, n + 32);
    int depth = 0;
    uint32_t iter = 0;
    for (;;) {
        if (pend == 0) {
            if (depth == 0) break;
            depth--;
            const SolveLevel sv = st[depth];
            L = sv.L;
            Q = sv.Q;
            P = sv.P;
            pend = sv.pend;
            nR = sv.nR;
            Rm = sv.Rm;
            sR = sv.sR;
            continue;
        }
        const uint32_t x = __ffs(pend) - 1;
        pend &= pend - 1;
        if (depth == 0 && lane == 0) {
            frames[fdepth].next = x - nq + 1;
            frames[fdepth].cur = x - nq;
        }
        const uint32_t L2 = L & __shfl_sync(kFull, row, x);
        const uint32_t l2 = __popc(L2);
        const uint32_t c = __popc(row & L2);
        const bool inA = ((P >> lane) & 1u) && lane > x;
        const bool inQ = ((Q >> lane) & 1u) || (((P >> lane) & 1u) && lane < x);
        const uint32_t absorbed = __ballot_sync(kFull, inA && c == l2);
        const uint32_t P2 = __ballot_sync(kFull, inA && c > 0 && c < l2);
        const uint32_t Q2 = __ballot_sync(kFull, inQ && c > 0);
        const uint32_t nR2 = nR + 1 + __popc(absorbed);
        unsigned long long sR2 = sR + __shfl_sync(kFull, eR, x);
        if (absorbed) sR2 += warp_sum(((absorbed >> lane) & 1u) ? eR : 0ull);
        if (l2 >= G.minL && nR2 >= G.minR) {
            const unsigned long long sl = warp_sum(((L2 >> lane) & 1u) ? eL : 0ull);
            acc.count++;
            acc.hash += side_hash(G, sl, l2, sR2, nR2);
            if (a.emit) emit_solved(a, G, nd, Rm | (1u << x) | absorbed, L2);
        }
        if (P2 && l2 >= G.minL && nR2 + __popc(P2) >= G.minR) {
            const uint32_t pend2 = solve_maximal(row, col, L2, Q2, P2, P2);
            acc.nodes += __popc(P2);
            if (pend2) {
                if (lane == 0) st[depth] = SolveLevel{L, Q, P, pend, nR, Rm, sR};
                __syncwarp();
                depth++;
                Rm |= (1u << x) | absorbed;
                L = L2;
                Q = Q2;
                P = P2;
                pend = pend2;
                nR = nR2;
                sR = sR2;
            }
        }
        if ((++iter & 63u) == 0) {
            if (lane == 0 && (iter & 1023u) == 0) atomicAdd(a.progress, 1ull);
            if (ld_volatile(a.error)) break;
            if (donate) {
                uint32_t qh = ld_volatile(a.q_head), qt = ld_volatile(a.q_tail), qd = ld_volatile(a.q_done);
                if ((int)(qh - qt) > 0 && (qt - qd) + a.q_margin < a.task_cap) {
                    try_donate(a, frames, fdepth, qh - qt);
                    const uint32_t hi2 = nq + frames[fdepth].end;  // lowered when level 0 was split
                    const uint32_t keep = hi2 >= 32 ? ~0u : ((1u << hi2) - 1u);
                    if (depth == 0)
                        pend &= keep;
                    else if (lane == 0)
                        st[0].pend &= keep;
                    __syncwarp();
                }
            }
        }
    }
    if (lane == 0) frames[fdepth].next = frames[fdepth].end;
    acc_commit(acc);
    __syncwarp();
}

#ifdef MBE_PROFILE
// Spreads one idle interval [w0, w1) over the 4 ms bins of the kernel-time
// histogram (idle ns per bin, then waits ending per bin).
__device__ void prof_idle(const EngineArgs& a, unsigned long long t0, unsigned long long w0, unsigned long long w1) {
    unsigned long long* hist = a.prof + kProfSlots + a.prof_warps;
    unsigned long long s = w0 - t0, e = w1 - t0;
    for (unsigned long long b = s / kProfBinNs; b < kProfBins && b * kProfBinNs < e; b++) {
        unsigned long long lo = max(s, b * kProfBinNs), hi = min(e, (b + 1) * kProfBinNs);
        atomicAdd(&hist[b], hi - lo);
    }
    unsigned long long be = e / kProfBinNs;
    if (be < kProfBins) atomicAdd(&hist[kProfBins + be], 1ull);
}
#endif

__global__ void __launch_bounds__(kThreadsB, MBE_DFS_MIN_BLOCKS) dfs_kernel(const __grid_constant__ EngineArgs a) {
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const size_t gw = (size_t)blockIdx.x * kWarpsB + warp;
    Frame* frames = a.frames + gw * a.frame_stride + (a.frame_skew ? frame_skew((uint32_t)gw) : 0u);
    WarpCtx& wc = s_wc[warp];
    uint32_t arena_top = 0;  // words of this warp's arena in use (warp-uniform)
    if (lane == 0) {
        wc.arena = a.arena + gw * a.arena_stride + arena_skew((uint32_t)gw, a.arena_stride);
        // scratch layout (scratch_words): scr_n from the largest root record
        // of the chunk, kc the power of two >= scr_n
        uint32_t scr_n = a.scr_n, kc = a.scr_kc;
        size_t sw = a.scratch_words;
        if (a.scratch_dyn) {
            scr_n = max(*(const volatile uint32_t*)a.max_n, 32u);
            kc = 32;
            while (kc < scr_n) kc <<= 1;
            sw = scratch_words(a.max_W, scr_n, kc, a.emit != 0);
        }
        uint32_t* scr = a.scratch + gw * sw;
        wc.scrLi = scr;
        wc.scrNz = scr + a.max_W;
        wc.scrQcnt = scr + 2 * (size_t)a.max_W;
        const size_t koff = (2 * (size_t)a.max_W + scr_n + 1) & ~(size_t)1;
        wc.scrKeysP = (unsigned long long*)(scr + koff);
        wc.scrKeysQ = wc.scrKeysP + kc;
        wc.scrPack = (uint32_t*)(wc.scrKeysQ + kc);
        wc.scrHist = wc.scrPack + 2 * (size_t)kc;
        wc.scrAbs = wc.scrHist + 32 * (size_t)a.max_W + 32;
        wc.scr_kc = kc;
        wc.slab_off = wc.slab_end = 0;
#ifdef MBE_PROFILE
        for (int q = 0; q < kProfSlots; q++) wc.prof[q] = 0;
        wc.last_busy = globaltimer_ns();
        wc.t_start = wc.last_busy;
#endif
    }
    __syncwarp();
#ifdef MBE_PROFILE
    __shared__ unsigned long long sTab[kProfTB * kProfTC * 2];
    for (int i = threadIdx.x; i < kProfTB * kProfTC * 2; i += blockDim.x) sTab[i] = 0;
    __syncthreads();
#endif
    const bool donate = a.variant != MBE_NOWS;
    const bool prefilter = a.variant != MBE_NOES;
    if (lane == 0) s_acc[warp] = ResultAcc{};
    __syncwarp();
    uint32_t evals = 0, evals_reported = 0;
    uint32_t last_poll = kPollCycles ? (uint32_t)clock() - kPollCycles : 0u;  // SM clock of the last counter read
    for (;;) {
        Popped t;
        {
            PROF_T0();
#ifdef MBE_PROFILE
            unsigned long long w0 = globaltimer_ns();
#endif
            t = pop_task(a);
            PROF_ADD(wc.prof, kProfPop);
#ifdef MBE_PROFILE
            if (lane == 0 && a.prof) prof_idle(a, wc.t_start, w0, globaltimer_ns());
#endif
            if (!t.node) break;
        }
        PROF_T0();
        const uint32_t my_path = t.path;
        const uint32_t graph = ((const NodeHdr*)t.node)->graph;
        if (lane == 0) s_G[warp] = a.graphs[graph];
        __syncwarp();
        const GraphView& G = s_G[warp];
        arena_top = 0;
        int depth = 0;
        {
            uint32_t p0 = __shfl_sync(kFull, my_path, 0);
            if (lane == 0) {
                Frame f0;
                f0.node = t.node;
                f0.next = t.plen ? p0 + 1 : t.begin;
                f0.end = t.plen ? p0 + 1 : t.end;
                f0.arena_mark = 0;
                f0.cur = p0;
                f0.mbase = 0;
                f0.pmask = 0;
                frames[0] = f0;
            }
        }
        __syncwarp();
        // re-derive the donated node along its path (uncounted)
        bool replay_ok = true;
        for (uint32_t j = 0; j < t.plen; j++) {
            uint32_t idx = __shfl_sync(kFull, my_path, j);
            uint32_t nxt = __shfl_sync(kFull, my_path, (j + 1) & 31);
            uint32_t mark = arena_top;
#ifdef MBE_PROFILE
            long long c0r = clock64();
#endif
            ChildOut co = eval_child(a, G, (const uint32_t*)frames[j].node, idx, arena_top, true, false);
#ifdef MBE_PROFILE
            PROF_TAB(8, c0r, clock64() - c0r);
#endif
            if (!co.rec) {
                if (lane == 0) set_error(a, kErrReplay, j);
                replay_ok = false;
                break;
            }
            arena_top += co.size;
            depth = (int)j + 1;
            if (lane == 0) {
                Frame nf;
                nf.node = (unsigned long long)co.rec;
                bool last = j + 1 == t.plen;
                nf.next = last ? t.begin : nxt + 1;
                nf.end = last ? t.end : nxt + 1;
                nf.arena_mark = mark;
                nf.cur = nxt;
                nf.mbase = 0;
                nf.pmask = 0;
                frames[depth] = nf;
            }
            __syncwarp();
        }
        if (!replay_ok) depth = -1;
        PROF_ADD(wc.prof, kProfReplay);
        while (depth >= 0) {
            Frame f = frames[depth];
            uint32_t child;
            bool known_max = false;
            if (f.pmask) {
                // a child the batch prefilter found maximal
                child = f.mbase + __ffs(f.pmask) - 1;
                known_max = true;
                if (lane == 0) {
                    frames[depth].pmask = f.pmask & (f.pmask - 1);
                    frames[depth].cur = child;
                }
                __syncwarp();
            } else {
                if (f.next >= f.end) {
                    arena_top = f.arena_mark;
                    depth--;
                    continue;
                }
                // Waiting warps = tickets taken beyond the tasks pushed.  Read
                // every iteration by default: reading them at most every 4,096
                // or 16,384 SM cycles measured slower (bench graph 232.6 ->
                // 235.8 / 235.1 ms), prompt donation being worth more than the
                // counters' L2 round trip.  The frame is reloaded only after a
                // donation changed it (232.6 -> 231.4 ms).
                if (donate && (kPollCycles == 0 || (uint32_t)(clock() - last_poll) >= kPollCycles)) {
                    if (kPollCycles) last_poll = (uint32_t)clock();
                    uint32_t qh = ld_volatile(a.q_head), qt = ld_volatile(a.q_tail), qd = ld_volatile(a.q_done);
                    if ((int)(qh - qt) > 0 && (qt - qd) + a.q_margin < a.task_cap) {
                        PROF_T0();
                        try_donate(a, frames, depth, qh - qt);
                        PROF_ADD(wc.prof, kProfDonate);
                        f = frames[depth];
                        if (f.next >= f.end) continue;
                    }
                }
                const uint32_t* nd = (const uint32_t*)f.node;
                if (prefilter && (((const NodeHdr*)nd)->flags & kRecPacked) && ((const NodeHdr*)nd)->n <= a.solve_rows) {
                    PROF_T0();
                    solve_small(a, G, nd, frames, depth, donate);
                    PROF_ADD(wc.prof, kProfSolve);
                    continue;
                }
                if (prefilter && ((const NodeHdr*)nd)->W == 1) {
                    PROF_T0();
                    const RecView R = rec_view(nd);
                    uint32_t nb = min(32u, f.end - f.next);
#ifdef MBE_PROFILE
                    long long c0p = clock64();
#endif
                    uint32_t mask = prefilter_w1(R, f.next, nb);
#ifdef MBE_PROFILE
                    PROF_TAB(9, c0p, clock64() - c0p);
            if ((R.flags & kRecPacked) && R.n <= 32) PROF_VAL(wc.prof, kProfSmallPre, clock64() - c0p);
#endif
                    PROF_ADD(wc.prof, kProfPrefilter);
                    evals += nb;
                    if (lane == 0) {
                        frames[depth].next = f.next + nb;
                        frames[depth].mbase = f.next;
                        frames[depth].pmask = mask;
                    }
                    __syncwarp();
                    if (evals - evals_reported >= 1024) {
                        evals_reported = evals;
                        if (lane == 0) atomicAdd(a.progress, 1ull);
                    }
                    continue;
                }
                child = f.next;
                if (lane == 0) {
                    frames[depth].next = f.next + 1;
                    frames[depth].cur = child;
                }
                __syncwarp();
            }
            uint32_t mark = arena_top;
#ifdef MBE_PROFILE
            long long c0e = clock64();
            const uint32_t pW = ((const NodeHdr*)f.node)->W;
#endif
            ChildOut co = eval_child(a, G, (const uint32_t*)f.node, child, arena_top, false, known_max);
#ifdef MBE_PROFILE
            PROF_TAB(min(7, 31 - __clz(pW)), c0e, clock64() - c0e);
            if ((((const NodeHdr*)f.node)->flags & kRecPacked) && ((const NodeHdr*)f.node)->n <= 32)
                PROF_VAL(wc.prof, kProfSmallEval, clock64() - c0e);
            else if (co.rec && (((const NodeHdr*)co.rec)->flags & kRecPacked) && ((const NodeHdr*)co.rec)->n <= 32)
                PROF_VAL(wc.prof, kProfSmallBuild, clock64() - c0e);
            PROF_TAB(10, 0, depth);
#endif
            evals++;
            if (evals - evals_reported >= 1024) {
                evals_reported = evals;
                if (lane == 0) atomicAdd(a.progress, 1ull);
            }
            if (co.rec) {
                if (depth + 1 >= (int)a.max_frames) {
                    if (lane == 0) set_error(a, kErrFrames, depth);
                    break;
                }
                arena_top += co.size;
                depth++;
                if (lane == 0) {
                    Frame nf;
                    nf.node = (unsigned long long)co.rec;
                    nf.next = 0;
                    nf.end = co.nchild;
                    nf.arena_mark = mark;
                    nf.cur = 0;
                    nf.mbase = 0;
                    nf.pmask = 0;
                    frames[depth] = nf;
                }
                __syncwarp();
            }
            if ((evals & 7u) == 0 && ld_volatile(a.error)) break;
        }
        flush_acc(a, graph);
        if (lane == 0) {
            __threadfence();
            atomicSub(a.pending, 1);
            atomicAdd(a.progress, 1ull);
        }
        __syncwarp();
#ifdef MBE_PROFILE
        wc.last_busy = globaltimer_ns();
#endif
    }
#ifdef MBE_PROFILE
    __syncthreads();
    for (int i = threadIdx.x; i < kProfTB * kProfTC * 2 && a.prof; i += blockDim.x)
        if (sTab[i]) atomicAdd(&a.prof[kProfSlots + a.prof_warps + 2 * kProfBins + i], sTab[i]);
    if (lane == 0 && a.prof) {
        for (int q = 0; q < kProfSlots; q++) atomicAdd(&a.prof[q], (unsigned long long)wc.prof[q]);
        a.prof[kProfSlots + gw] = wc.last_busy;
    }
#endif
}

}  // namespace

// ---------------------------------------------------------------------------
// host driver

size_t EngineBuffers::bytes() const {
    size_t t = 0;
    for (const DevBuf* b : {&graphs, &roots, &ctrl, &tasks, &ready, &cmap, &a_cl, &a_cnt, &a_keys, &pool, &arena, &frames,
                            &scratch, &results, &retry_in, &retry_list, &e_ids, &e_start, &e_nrows, &e_ncols, &e_ctl})
        t += b->bytes;
    return t;
}

void EngineBuffers::release() {
    for (DevBuf* b : {&graphs, &roots, &ctrl, &tasks, &ready, &cmap, &a_cl, &a_cnt, &a_keys, &pool, &arena, &frames,
                      &scratch, &results, &retry_in, &retry_list, &e_ids, &e_start, &e_nrows, &e_ncols, &e_ctl})
        b->free();
    for (cudaEvent_t& e : ev)
        if (e) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    pin_in.free();
    pin_out.free();
    pin_retry.free();
    cmap_clean = ready_clean = 0;
}

mbe_status HostBuf::ensure(size_t need) {
    if (need <= bytes) return MBE_OK;
    free();
    const size_t want = std::max<size_t>(need, 4096);
    if (cudaMallocHost(&ptr, want) != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        cudaGetLastError();
        return fail(MBE_ERR_OUT_OF_MEMORY, "pinned host allocation of " + std::to_string(want) + " bytes failed");
    }
    bytes = want;
    return MBE_OK;
}

void HostBuf::free() {
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    bytes = 0;
}

mbe_status DevBuf::ensure(size_t need) {
    if (need <= bytes) return MBE_OK;
    free();
    size_t want = std::max(need, (size_t)256);
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        cudaGetLastError();
        return fail(MBE_ERR_OUT_OF_MEMORY, "device allocation of " + std::to_string(want) + " bytes failed");
    }
    bytes = want;
    return MBE_OK;
}

void DevBuf::free() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

// Control block layout (words): see offsets below.
namespace {
struct Ctrl {
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

// Device-driven chunk loop (graph mode): runs before each chunk's root
// expansion in the captured sequence and resets what the host resets
// between chunks -- the node pool and the task ring's counters (the ring's
// flags and the candidate maps are clean after a chunk that ended without
// an error).  The root cursor carries over, so each chunk resumes where the
// previous one stopped; once it is past the last root, the chunk's kernels
// find nothing to do.  A root whose record did not fit the pool would need
// the host's re-queueing: it is reported as pool exhaustion, and the host
// runs the batch again with its own chunk loop.
__global__ void chunk_prep_kernel(Ctrl* c) {
    if (threadIdx.x != 0 || c->error) return;
    if (c->n_retry) {
        c->error = kErrPool;
        c->error_info = c->n_retry;
        return;
    }
    c->pool_top = 0;
    c->q_tail = c->q_head = c->q_done = 0;
    c->pending = 0;
    __threadfence();
}
}  // namespace

// Shared-memory carveout for the DFS kernel: the smallest share of the SM's
// unified memory that holds MBE_DFS_MIN_BLOCKS blocks, raised until the
// occupancy query confirms that many.  The rest stays L1, which the record
// scans run from: 64 KB of shared memory measured faster than the default
// carveout (bench graph 303.9 -> 294.9 ms, 588-graph batch 737 -> 696 ms).
static cudaError_t set_dfs_carveout() {
    cudaFuncAttributes fa{};
    cudaError_t e = cudaFuncGetAttributes(&fa, dfs_kernel);
    if (e != cudaSuccess) return e;
    int dev = 0, per_sm = 0, reserved = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess) return e;
    if (per_sm <= 0) return cudaSuccess;
    const size_t need = (size_t)MBE_DFS_MIN_BLOCKS * (fa.sharedSizeBytes + (size_t)reserved);
    for (int pct = (int)std::min<size_t>(100, (need * 100 + per_sm - 1) / per_sm); pct <= 100; pct++) {
        if ((e = cudaFuncSetAttribute(dfs_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct)) != cudaSuccess)
            return e;
        int occ = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dfs_kernel, kThreadsB, 0)) != cudaSuccess) return e;
        if (occ >= MBE_DFS_MIN_BLOCKS)  // the server's root expansion prefers the same split
            return cudaFuncSetAttribute(expand_roots_kernel<true>, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    }
    return cudaFuncSetAttribute(dfs_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, -1);
}

// The carveout is a hint, applied once per device (the attribute belongs to
// the device's context and persists): if the device refuses it, the default
// stands and only the error the refusal recorded is cleared.  An error that
// was already pending when this is called (an earlier launch nobody checked)
// is returned, not swallowed.
static cudaError_t try_dfs_carveout() {
    const cudaError_t before = cudaGetLastError();
    if (before != cudaSuccess) return before;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    constexpr int kMaxDev = 128;
    static std::mutex mu;
    static bool done[kMaxDev] = {};
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < kMaxDev && done[dev]) return cudaSuccess;
    if (set_dfs_carveout() != cudaSuccess) (void)cudaGetLastError();
    if (dev >= 0 && dev < kMaxDev) done[dev] = true;
    return cudaSuccess;
}

// SM count and the two kernels' resident blocks per SM (after the DFS
// carveout is applied), looked up once per device: they do not change, and
// the queries cost host time on every small request otherwise.
static cudaError_t device_facts(int dev, int* n_sm, int* occA, int* occB) {
    constexpr int kMaxDev = 128;
    static std::mutex mu;
    static int facts[kMaxDev][3];
    static bool known[kMaxDev] = {};
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 0 || dev >= kMaxDev || !known[dev]) {
        int f[3] = {0, 0, 0};
        cudaError_t e = cudaDeviceGetAttribute(&f[0], cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f[1], expand_roots_kernel<false>, kThreadsA,
                                                              sizeof(uint32_t) * kStageWords);
        if (e == cudaSuccess) e = try_dfs_carveout();
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f[2], dfs_kernel, kThreadsB, 0);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < kMaxDev) {
            std::memcpy(facts[dev], f, sizeof f);
            known[dev] = true;
        }
        *n_sm = f[0];
        *occA = f[1];
        *occB = f[2];
        return cudaSuccess;
    }
    *n_sm = facts[dev][0];
    *occA = facts[dev][1];
    *occB = facts[dev][2];
    return cudaSuccess;
}

// Sets aside the device's persisting L2 share once (per device and
// process: a context limit, released with the context): the largest the
// device allows, capped at want bytes.  Returns the share and the largest
// access-policy window the device takes.
static cudaError_t l2_persist_setup(int dev, size_t want, size_t* persist, size_t* max_window) {
    constexpr int kMaxDev = 128;
    static std::mutex mu;
    static size_t set_to[kMaxDev] = {};
    int pmax = 0, wmax = 0;
    cudaError_t e = cudaDeviceGetAttribute(&pmax, cudaDevAttrMaxPersistingL2CacheSize, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&wmax, cudaDevAttrMaxAccessPolicyWindowSize, dev);
    if (e != cudaSuccess) return e;
    const size_t share = std::min<size_t>((size_t)std::max(pmax, 0), want);
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < kMaxDev && share > set_to[dev]) {
        if ((e = cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, share)) != cudaSuccess) return e;
        set_to[dev] = share;
    }
    *persist = dev >= 0 && dev < kMaxDev ? set_to[dev] : 0;
    *max_window = (size_t)std::max(wmax, 0);
    return cudaSuccess;
}

cudaError_t dfs_blocks_per_sm(int dev, int* occ) {
    int n_sm = 0, occA = 0;
    return device_facts(dev, &n_sm, &occA, occ);
}

// The status and message for the error a chunk's kernels recorded.
static mbe_status kernel_error(const Ctrl& hc) {
    static const char* names[] = {"none",
                                  "node pool exhausted",
                                  "task queue full",
                                  "device wait timed out",
                                  "search deeper than the frame stack",
                                  "scratch too small",
                                  "donated path did not re-derive"};
    const mbe_status code = hc.error == kErrTimeout ? MBE_ERR_DEVICE_TIMEOUT
                            : hc.error == kErrPool  ? MBE_ERR_OUT_OF_MEMORY
                                                    : MBE_ERR_CAPACITY;
    return fail(code, std::string("enumeration kernel: ") + names[hc.error > 0 && hc.error < 7 ? hc.error : 0] +
                          " (info " + std::to_string(hc.error_info) + ")");
}

// engine_run's chunk loop in graph mode (EngineConfig::graph_chunks): every
// root of a's list, chunk after chunk, with the chunks' kernels (prep, root
// expansion, DFS; per_launch chunks) captured once into a CUDA graph that
// is launched until the root cursor has passed the last root.  The scratch
// must be laid out by the kernels (a.scratch_dyn).  *fall_back is set when
// a record did not fit the pool (the host-driven loop re-queues such roots
// and grows the pool); the caller then runs that loop instead.
static mbe_status run_graph_chunks(EngineBuffers& eb, cudaStream_t s, EngineArgs a, Ctrl* ctrl, Ctrl* pin_ctrl,
                                   uint32_t n_roots, uint32_t task_cap, uint32_t gridA, uint32_t gridB,
                                   uint32_t per_launch, cudaEvent_t e0, cudaEvent_t e1, float* ms, uint32_t* chunks,
                                   bool* fall_back, IoCounters* io) {
    *fall_back = false;
    *ms = 0;
    *chunks = 0;
    a.roots = (const uint2*)eb.roots.ptr;
    a.n_roots = n_roots;
    MBE_CUDA_TRY(cudaMemsetAsync(ctrl, 0, sizeof(Ctrl), s));
    if (eb.ready_clean < sizeof(uint32_t) * (size_t)task_cap)
        MBE_CUDA_TRY(cudaMemsetAsync(eb.ready.ptr, 0, sizeof(uint32_t) * (size_t)task_cap, s));
    eb.ready_clean = 0;  // unknown while the kernels run (the caller restores it after a clean run)
    eb.cmap_clean = 0;
    struct Graph {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t x = nullptr;
        ~Graph() {
            if (x) cudaGraphExecDestroy(x);
            if (g) cudaGraphDestroy(g);
        }
    } gr;
    // nothing between begin and end returns early: a failed capture must
    // still end, or the stream would stay in capture mode
    MBE_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (uint32_t k = 0; k < per_launch; k++) {
        chunk_prep_kernel<<<1, 32, 0, s>>>(ctrl);
        expand_roots_kernel<false><<<gridA, kThreadsA, sizeof(uint32_t) * a.stage_words, s>>>(a);
        dfs_kernel<<<gridB, kThreadsB, 0, s>>>(a);
    }
    cudaError_t ce = cudaStreamEndCapture(s, &gr.g);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    MBE_CUDA_TRY(ce);
    MBE_CUDA_TRY(cudaGraphInstantiate(&gr.x, gr.g, 0));
    uint32_t last_next = 0;
    for (;;) {
        MBE_CUDA_TRY(cudaEventRecord(e0, s));
        MBE_CUDA_TRY(cudaGraphLaunch(gr.x, s));
        MBE_CUDA_TRY(cudaEventRecord(e1, s));
        MBE_CUDA_TRY(cudaMemcpyAsync(pin_ctrl, ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
        MBE_CUDA_TRY(cudaStreamSynchronize(s));
        const Ctrl hc = *pin_ctrl;
        io->launches += 3 * per_launch;
        io->d2h += sizeof(Ctrl);
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        *ms += t;
        *chunks += per_launch;
        // a record that did not fit (whether or not a later chunk's prep
        // saw it), or no root claimed in a whole launch: the host loop
        if (hc.error == kErrPool || hc.n_retry ||
            (!hc.error && hc.root_next < n_roots && hc.root_next == last_next)) {
            *fall_back = true;
            return MBE_OK;
        }
        if (hc.error) return kernel_error(hc);
        if (hc.root_next >= n_roots) return MBE_OK;
        last_next = hc.root_next;
    }
}

mbe_status engine_run(EngineBuffers& eb, cudaStream_t s, const EngineConfig& cfg,
                      const std::vector<const DeviceGraph*>& gs, const std::vector<uint2>& roots,
                      std::vector<ResultAcc>& results, EngineStats* stats, IoCounters* io) {
    const uint32_t ng = (uint32_t)gs.size();
    results.assign(ng, ResultAcc{});
    // the per-graph results are read with each chunk's control block when
    // they are small (the last chunk's copy is the final one)
    const bool results_with_ctrl = sizeof(ResultAcc) * ng <= 4096;
    if (ng == 0 || roots.empty()) return MBE_OK;
    uint32_t maxNR = 1, maxW = 1, maxRD = 1;
    for (const DeviceGraph* g : gs) {
        maxNR = std::max(maxNR, g->nR);
        maxW = std::max(maxW, (g->max_rdeg + 31) / 32);
        maxRD = std::max(maxRD, g->max_rdeg);
    }
    // per-block root scratch: keep flags (u32 per candidate) and the count
    // histogram (2 x degree u32), as u64 words
    const uint32_t keys_cap = (uint32_t)std::max<size_t>(std::max<size_t>(2048, maxRD + 1), [&] {
        size_t p = 1;
        while (p < maxNR) p <<= 1;
        return p;
    }());
    int dev = 0;
    MBE_CUDA_TRY(cudaGetDevice(&dev));
    int n_sm = 0, occA = 0, occB = 0;
    MBE_CUDA_TRY(device_facts(dev, &n_sm, &occA, &occB));
    // root expansion at full occupancy (4 blocks per SM measured 23 -> 15 ms
    // on the 94k x 30k graph against 2), or within the share of the GPU a
    // caller asked for (server slots that run side by side)
    const int capA = cfg.blocks_per_sm ? (int)cfg.blocks_per_sm : occA;
    uint32_t gridA = (uint32_t)n_sm * (uint32_t)std::max(1, std::min(occA, capA));
    uint32_t bpsm = cfg.blocks_per_sm ? cfg.blocks_per_sm : (uint32_t)std::max(1, occB);
    bpsm = std::min<uint32_t>(bpsm, (uint32_t)std::max(1, occB));
    uint32_t gridB = (uint32_t)n_sm * bpsm;
    uint32_t nwarpsB = gridB * kWarpsB;
    const uint32_t q_margin = 32 * nwarpsB + 1024;  // a donor pushes up to 31 tasks after its check
    const uint32_t task_cap = (uint32_t)std::min<size_t>(roots.size() + q_margin + (size_t)cfg.extra_tasks, 0x7FFFFFFF);
    const uint32_t max_frames = cfg.max_frames;
    // Per-warp DFS arenas default to 4 MiB each (at most 30% of free device
    // memory in total); the shared node pool starts at 8 GiB and is doubled
    // (up to 60% of free memory) whenever a run exhausts it.
    if (!eb.arena_words) {
        size_t free_b = 0, tot_b = 0;
        MBE_CUDA_TRY(cudaMemGetInfo(&free_b, &tot_b));
        uint64_t cap = (uint64_t)(free_b * 0.30) / nwarpsB / 4;
        uint64_t want = 1u << 20;
        if (const char* env = std::getenv("MBE_ARENA_WORDS")) want = std::strtoull(env, nullptr, 10);
        eb.arena_words = (uint32_t)std::max<uint64_t>(std::min(want, cap), 1u << 14) & ~31u;
    }
    if (!eb.pool_words) {
        eb.pool_words = 1ull << 31;
        if (const char* e = std::getenv("MBE_POOL_INIT_MB")) {  // tuning: first pool size
            const unsigned long long mb = std::strtoull(e, nullptr, 10);
            if (mb) eb.pool_words = mb * (1ull << 20) / 4;
        }
    }
    uint32_t arena_words = cfg.arena_words ? std::min(cfg.arena_words, eb.arena_words) : eb.arena_words;
    const uint32_t retry_cap = 1u << 16;
    // Under a memory cap the arenas take at most a quarter of it, and the
    // node pool what the other buffers (as they will be held after this
    // call: DevBuf only grows) leave.
    uint64_t pool_cap_words = ~0ull;
    if (cfg.mem_cap) {
        arena_words = (uint32_t)std::max<uint64_t>(std::min<uint64_t>(arena_words, cfg.mem_cap / 4 / nwarpsB / 4),
                                                   1u << 12) & ~31u;
        const uint32_t scr_b = std::max<uint32_t>(maxNR, 32);
        size_t kc_b = 32;
        while (kc_b < scr_b) kc_b <<= 1;
        auto held = [](const DevBuf& b, size_t need) { return std::max(b.bytes, std::max(need, (size_t)256)); };
        const size_t fixed =
            held(eb.graphs, sizeof(GraphView) * ng) + held(eb.roots, sizeof(uint2) * roots.size()) +
            held(eb.ctrl, sizeof(Ctrl)) + held(eb.tasks, sizeof(Task) * (size_t)task_cap) +
            held(eb.ready, sizeof(uint32_t) * (size_t)task_cap) + held(eb.cmap, sizeof(int) * (size_t)gridA * maxNR) +
            held(eb.a_cl, sizeof(uint32_t) * (size_t)gridA * maxNR) +
            held(eb.a_cnt, sizeof(uint32_t) * (size_t)gridA * maxNR) +
            held(eb.a_keys, sizeof(unsigned long long) * (size_t)gridA * keys_cap) +
            held(eb.arena, sizeof(uint32_t) * (size_t)nwarpsB * arena_words) +
            held(eb.frames, sizeof(Frame) * (size_t)nwarpsB * (max_frames + kFrameSlack)) + held(eb.results, sizeof(ResultAcc) * ng) +
            held(eb.retry_in, sizeof(uint32_t) * (size_t)retry_cap) +
            held(eb.retry_list, sizeof(uint2) * roots.size()) +
            held(eb.scratch, sizeof(uint32_t) * (size_t)nwarpsB * scratch_words(maxW, scr_b, kc_b, cfg.emit != nullptr));
        const size_t min_pool = 16u << 20;
        if (fixed + min_pool > cfg.mem_cap)
            return fail(MBE_ERR_OUT_OF_MEMORY, "memory cap of " + std::to_string(cfg.mem_cap) + " bytes is below the " +
                                                   std::to_string(fixed + min_pool) + " bytes this run needs");
        pool_cap_words = ((cfg.mem_cap - fixed) / 4) & ~31ull;
        eb.pool_words = std::min<uint64_t>(eb.pool_words, pool_cap_words);
        if (eb.pool.bytes > sizeof(uint32_t) * pool_cap_words) eb.pool.free();  // reallocated below, smaller
        // The scratch is allocated for its bound now (it is counted in the
        // cap anyway), not grown per chunk: a capped context serves requests
        // next to other streams, and growing a buffer (cudaFree) would wait
        // for every kernel on the device, theirs included.
        mbe_status sst = eb.scratch.ensure(sizeof(uint32_t) * (size_t)nwarpsB *
                                           scratch_words(maxW, scr_b, kc_b, cfg.emit != nullptr));
        if (sst) return sst;
    }

    mbe_status st;
    // thresholds per entry (the same graph may appear with different ones),
    // given in file orientation (rows, cols) and stored in L/R orientation
    std::vector<GraphView> views;
    for (uint32_t i = 0; i < ng; i++) {
        GraphView v = view_of(*gs[i]);
        const uint2 t = cfg.entry_thr ? (*cfg.entry_thr)[i] : make_uint2(cfg.min_rows, cfg.min_cols);
        v.minL = gs[i]->swapped ? t.x : t.y;
        v.minR = gs[i]->swapped ? t.y : t.x;
        views.push_back(v);
    }
    if ((st = eb.graphs.ensure(sizeof(GraphView) * ng))) return st;
    if ((st = eb.roots.ensure(sizeof(uint2) * roots.size()))) return st;
    if ((st = eb.ctrl.ensure(sizeof(Ctrl)))) return st;
    if ((st = eb.tasks.ensure(sizeof(Task) * (size_t)task_cap))) return st;
    if ((st = eb.ready.ensure(sizeof(uint32_t) * (size_t)task_cap))) return st;
    size_t cmap_bytes = sizeof(int) * (size_t)gridA * maxNR;
    if ((st = eb.cmap.ensure(cmap_bytes))) return st;
    if ((st = eb.a_cl.ensure(sizeof(uint32_t) * (size_t)gridA * maxNR))) return st;
    if ((st = eb.a_cnt.ensure(sizeof(uint32_t) * (size_t)gridA * maxNR))) return st;
    if ((st = eb.a_keys.ensure(sizeof(unsigned long long) * (size_t)gridA * keys_cap))) return st;
    if ((st = eb.arena.ensure(sizeof(uint32_t) * (size_t)nwarpsB * arena_words))) return st;
    if ((st = eb.frames.ensure(sizeof(Frame) * (size_t)nwarpsB * (max_frames + kFrameSlack)))) return st;
    if ((st = eb.results.ensure(sizeof(ResultAcc) * ng))) return st;
    if ((st = eb.retry_in.ensure(sizeof(uint32_t) * (size_t)retry_cap))) return st;
    // inputs and readbacks through pinned staging (see HostBuf)
    const size_t in_views = sizeof(GraphView) * ng, in_roots = sizeof(uint2) * roots.size();
    const size_t out_res_off = (sizeof(Ctrl) + 15) & ~(size_t)15;
    const size_t out_retry_off = (out_res_off + sizeof(ResultAcc) * ng + 15) & ~(size_t)15;
    if ((st = eb.pin_in.ensure(in_views + in_roots))) return st;
    if ((st = eb.pin_out.ensure(out_retry_off + sizeof(uint32_t) * (size_t)retry_cap))) return st;
    std::memcpy(eb.pin_in.ptr, views.data(), in_views);
    std::memcpy((char*)eb.pin_in.ptr + in_views, roots.data(), in_roots);
    MBE_CUDA_TRY(cudaMemcpyAsync(eb.graphs.ptr, eb.pin_in.ptr, in_views, cudaMemcpyHostToDevice, s));
    MBE_CUDA_TRY(cudaMemcpyAsync(eb.roots.ptr, (char*)eb.pin_in.ptr + in_views, in_roots, cudaMemcpyHostToDevice, s));
    Ctrl* const pin_ctrl = (Ctrl*)eb.pin_out.ptr;
    ResultAcc* const pin_res = (ResultAcc*)((char*)eb.pin_out.ptr + out_res_off);
    uint32_t* const pin_retry_idx = (uint32_t*)((char*)eb.pin_out.ptr + out_retry_off);
    io->h2d += sizeof(GraphView) * ng + sizeof(uint2) * roots.size();

    Ctrl* ctrl = (Ctrl*)eb.ctrl.ptr;
    EngineArgs a;
    std::memset(&a, 0, sizeof a);
    a.graphs = (const GraphView*)eb.graphs.ptr;
    a.n_graphs = ng;
    a.variant = cfg.variant;
        a.donate_min = std::max(2u, cfg.donate_min);
    a.donate_copy = 1;
    a.solve_rows = std::min<uint32_t>(cfg.solve_rows, kSolveRows);
    if (const char* e = std::getenv("MBE_SOLVE_ROWS")) a.solve_rows = std::min<uint32_t>((uint32_t)std::atoi(e), kSolveRows);
    if (const char* e = std::getenv("MBE_DONATE_COPY")) a.donate_copy = (uint32_t)std::atoi(e);
    a.root_next = &ctrl->root_next;
    a.retry = (uint32_t*)eb.retry_in.ptr;
    a.n_retry = &ctrl->n_retry;
    a.retry_cap = retry_cap;
    a.pool_top = &ctrl->pool_top;
    a.tasks = (Task*)eb.tasks.ptr;
    a.ready = (uint32_t*)eb.ready.ptr;
    a.task_cap = task_cap;
    a.q_tail = &ctrl->q_tail;
    a.q_head = &ctrl->q_head;
    a.q_done = &ctrl->q_done;
    a.q_margin = q_margin;
    a.pending = &ctrl->pending;
    a.progress = &ctrl->progress;
    a.cmap = (int*)eb.cmap.ptr;
    a.a_cl = (uint32_t*)eb.a_cl.ptr;
    a.a_cnt = (uint32_t*)eb.a_cnt.ptr;
    a.a_keys = (unsigned long long*)eb.a_keys.ptr;
    a.maxNR = maxNR;
    a.keys_cap = keys_cap;
    a.max_n = &ctrl->max_n;
    a.arena = (uint32_t*)eb.arena.ptr;
    a.arena_stride = arena_words;
    a.arena_words = arena_usable_words(arena_words);
    a.frames = (Frame*)eb.frames.ptr;
    a.max_frames = max_frames;
    a.frame_stride = max_frames + kFrameSlack;
    a.frame_skew = 1;
    a.max_W = maxW;
    a.results = (ResultAcc*)eb.results.ptr;
    a.error = &ctrl->error;
    a.error_info = &ctrl->error_info;
    a.timeout_ns = cfg.timeout_ns;
    // L0 staging buffer of the root expansion: none on capped (server)
    // contexts, whose kernels share SMs with other slots' persistent DFS
    // blocks -- with 16 KB more shared memory an expansion block no longer
    // fits beside them and would wait for them to finish.
    a.stage_words = cfg.mem_cap ? 0u : kStageWords;
    if (cfg.emit) {
        a.emit = 1;
        a.emit_ids = cfg.emit->ids;
        a.emit_cap_ids = cfg.emit->cap_ids;
        a.emit_start = cfg.emit->start;
        a.emit_nrows = cfg.emit->nrows;
        a.emit_ncols = cfg.emit->ncols;
        a.emit_cap_b = cfg.emit->cap_b;
        a.emit_ctl = cfg.emit->ctl;
    }
#ifdef MBE_PROFILE
    static unsigned long long* prof_dev = nullptr;
    static size_t prof_n = 0;
    if (prof_n < kProfSlots + nwarpsB + 2 * kProfBins + 2 * kProfTB * kProfTC + 16) {
        if (prof_dev) cudaFree(prof_dev);
        prof_n = kProfSlots + nwarpsB + 2 * kProfBins + 2 * kProfTB * kProfTC + 16;
        MBE_CUDA_TRY(cudaMalloc(&prof_dev, sizeof(unsigned long long) * prof_n));
    }
    MBE_CUDA_TRY(cudaMemsetAsync(prof_dev, 0, sizeof(unsigned long long) * prof_n, s));
    a.prof = prof_dev;
    a.prof_warps = nwarpsB;
    a.prof_a = prof_dev + prof_n - 16;
#endif

    {
        // One graph: no readback between the kernels when the scratch can be
        // sized for the bound on any record (fewer than |R| candidates)
        // within 4 GiB (small requests 0.191 -> 0.176 ms).  Many graphs keep
        // the readback: measured faster for batches and server slots.
        const uint32_t scr_b = std::max<uint32_t>(maxNR, 32);
        size_t kc = 32;
        while (kc < scr_b) kc <<= 1;
        const size_t bytes = sizeof(uint32_t) * (size_t)nwarpsB * scratch_words(maxW, scr_b, kc, cfg.emit != nullptr);
        // (graph mode needs it too: no host step between the kernels)
        const bool want_graph = cfg.graph_chunks && ng > 1 && !cfg.emit && !cfg.mem_cap;
        if ((ng == 1 || want_graph) && bytes <= (4ull << 30)) {
            if ((st = eb.scratch.ensure(bytes))) return st;
            a.scratch = (uint32_t*)eb.scratch.ptr;
            a.scratch_dyn = 1;
        }
    }
    // High-degree adjacency pinned in L2: on a single-graph run the L-side
    // lists, which the root expansion's reverse scan streams (a hub's list
    // once per root next to it), get an access-policy window of persisting
    // lines on the stream for the run, so the node records streaming through
    // L2 do not evict them.  The L2 share is set aside once per device (the
    // largest the device allows, up to the window); the window is cleared and
    // the persisting lines released after the run.  Multi-graph runs and
    // capped (server) contexts share the L2 with other work: no window.
    // Measured on this engine: neutral to 1-2% slower (bench graph 239.6 vs
    // 239.7 ms; full-size stress sample 2,540 vs 2,488 ms), both graphs'
    // adjacency being L2-resident anyway (1.2 and 32 MB of a 126 MB L2), so
    // it is off unless asked for (MBE_OPT_L2_PIN).
    bool l2_window = ng == 1 && !cfg.mem_cap && cfg.l2_pin && gs[0]->nE;
    if (l2_window) {
        const size_t bytes = sizeof(uint32_t) * (size_t)gs[0]->nE;
        size_t persist = 0, max_window = 0;
        MBE_CUDA_TRY(l2_persist_setup(dev, bytes, &persist, &max_window));
        if (persist && max_window) {
            cudaStreamAttrValue v{};
            v.accessPolicyWindow.base_ptr = (void*)gs[0]->l_adj;
            v.accessPolicyWindow.num_bytes = std::min(bytes, max_window);
            v.accessPolicyWindow.hitRatio =
                (float)std::min(1.0, (double)persist / (double)v.accessPolicyWindow.num_bytes);
            v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
            v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
            MBE_CUDA_TRY(cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &v));
        } else {
            l2_window = false;
        }
    }
    struct L2Release {  // clears the window and demotes the lines however the run ends
        bool on;
        cudaStream_t s;
        ~L2Release() {
            if (!on) return;
            cudaStreamAttrValue v{};
            v.accessPolicyWindow.num_bytes = 0;
            cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &v);
            cudaCtxResetPersistingL2Cache();
        }
    } l2_release{l2_window, s};
    for (cudaEvent_t& e : eb.ev)
        if (!e) MBE_CUDA_TRY(cudaEventCreate(&e));
    cudaEvent_t e0 = eb.ev[0], e1 = eb.ev[1], e2 = eb.ev[2];
    // a buffer that was (re)allocated since the last clean run starts unknown
    if (eb.cmap.bytes < eb.cmap_clean) eb.cmap_clean = 0;
    if (eb.ready.bytes < eb.ready_clean) eb.ready_clean = 0;
    float ms_a = 0, ms_b = 0;
    uint32_t chunks = 0;
    mbe_status result = MBE_OK;
    // graph mode: multi-graph runs whose scratch is laid out by the kernels
    bool use_graph = cfg.graph_chunks && ng > 1 && !cfg.emit && !cfg.mem_cap && a.scratch_dyn;
    for (int attempt = 0;; attempt++) {
        // The node pool grows by doubling when a run exhausts it (up to 60% of
        // free device memory); a fixed cap (cfg.pool_words) disables growth.
        const uint64_t pool_words = cfg.pool_words ? std::min<uint64_t>(cfg.pool_words, eb.pool_words) : eb.pool_words;
        if ((st = eb.pool.ensure(sizeof(uint32_t) * eb.pool_words))) {
            result = st;
            break;
        }
        a.pool = (uint32_t*)eb.pool.ptr;
        a.pool_words = pool_words;
        a.pool_watermark = cfg.chunk_words ? std::min<uint64_t>(cfg.chunk_words, pool_words / 2) : pool_words / 2;
        if (eb.cmap_clean < cmap_bytes) {  // the kernels restore -1 after each root
            MBE_CUDA_TRY(cudaMemsetAsync(eb.cmap.ptr, 0xFF, cmap_bytes, s));
            eb.cmap_clean = cmap_bytes;
        }
        const size_t cmap_known = eb.cmap_clean;
        MBE_CUDA_TRY(cudaMemsetAsync(eb.results.ptr, 0, sizeof(ResultAcc) * ng, s));
        if (cfg.emit) MBE_CUDA_TRY(cudaMemsetAsync(cfg.emit->ctl, 0, 3 * sizeof(unsigned long long), s));
        ms_a = ms_b = 0;
        chunks = 0;
        result = MBE_OK;
        bool pool_exhausted = false;
        // Roots that did not fit the pool in one chunk are retried first in
        // the next chunk (from a host copy), then the main list resumes.
        std::vector<uint2> pending_roots;
        uint32_t main_next = 0;
        if (use_graph) {
            // The chunk loop runs on the device: graph_chunks chunks (prep,
            // root expansion, DFS) captured once into a CUDA graph, launched
            // until the root cursor has passed every root, with one host
            // synchronisation per launch instead of two per chunk.
            bool fall_back = false;
            result = run_graph_chunks(eb, s, a, ctrl, pin_ctrl, (uint32_t)roots.size(), task_cap, gridA, gridB,
                                      cfg.graph_chunks, e0, e2, &ms_b, &chunks, &fall_back, io);
            if (fall_back) {  // a record did not fit the pool: the host loop re-queues it
                use_graph = false;
                continue;
            }
            if (result != MBE_OK) break;
            if (results_with_ctrl) {
                MBE_CUDA_TRY(cudaMemcpyAsync(pin_res, eb.results.ptr, sizeof(ResultAcc) * ng,
                                             cudaMemcpyDeviceToHost, s));
                MBE_CUDA_TRY(cudaStreamSynchronize(s));
                std::memcpy(results.data(), pin_res, sizeof(ResultAcc) * ng);
                io->d2h += sizeof(ResultAcc) * ng;
            }
            eb.ready_clean = sizeof(uint32_t) * (size_t)task_cap;
            eb.cmap_clean = cmap_known;
            break;
        }
        while (main_next < roots.size() || !pending_roots.empty()) {
            chunks++;
            const uint2* list;
            uint32_t list_n;
            std::vector<uint2> chunk_list;
            if (!pending_roots.empty()) {
                chunk_list = pending_roots;
                list_n = (uint32_t)chunk_list.size();
                if ((st = eb.retry_list.ensure(sizeof(uint2) * list_n))) return st;
                if ((st = eb.pin_retry.ensure(sizeof(uint2) * list_n))) return st;
                std::memcpy(eb.pin_retry.ptr, chunk_list.data(), sizeof(uint2) * list_n);
                MBE_CUDA_TRY(cudaMemcpyAsync(eb.retry_list.ptr, eb.pin_retry.ptr, sizeof(uint2) * list_n,
                                             cudaMemcpyHostToDevice, s));
                io->h2d += sizeof(uint2) * list_n;
                list = (const uint2*)eb.retry_list.ptr;
            } else {
                list = (const uint2*)eb.roots.ptr + main_next;
                list_n = (uint32_t)roots.size() - main_next;
            }
            a.roots = list;
            a.n_roots = list_n;
            MBE_CUDA_TRY(cudaMemsetAsync(ctrl, 0, sizeof(Ctrl), s));
            if (eb.ready_clean < sizeof(uint32_t) * (size_t)task_cap) {
                MBE_CUDA_TRY(cudaMemsetAsync(eb.ready.ptr, 0, sizeof(uint32_t) * (size_t)task_cap, s));
                eb.ready_clean = sizeof(uint32_t) * (size_t)task_cap;
            }
            // unknown while the kernels run; clean again only after a chunk
            // that ended without an error
            const size_t ready_known = eb.ready_clean;
            eb.ready_clean = 0;
            eb.cmap_clean = 0;
            MBE_CUDA_TRY(cudaEventRecord(e0, s));
            if (cfg.mem_cap)
                expand_roots_kernel<true><<<gridA, kThreadsA, 0, s>>>(a);
            else
                expand_roots_kernel<false><<<gridA, kThreadsA, sizeof(uint32_t) * a.stage_words, s>>>(a);
            MBE_CUDA_TRY(cudaGetLastError());
            MBE_CUDA_TRY(cudaEventRecord(e1, s));
            // DFS scratch is laid out for the largest record this chunk made:
            // by the kernel itself when the scratch is sized for the bound,
            // else from a readback of that size
            if (!a.scratch_dyn) {
                MBE_CUDA_TRY(cudaMemcpyAsync(&pin_ctrl->max_n, &ctrl->max_n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
                MBE_CUDA_TRY(cudaStreamSynchronize(s));
                const uint32_t max_n = pin_ctrl->max_n;
                io->d2h += sizeof max_n;
                uint32_t scr_n = std::max<uint32_t>(max_n, 32);
                size_t kc = 32;
                while (kc < scr_n) kc <<= 1;
                size_t sw = scratch_words(maxW, scr_n, kc, cfg.emit != nullptr);
                if ((st = eb.scratch.ensure(sizeof(uint32_t) * (size_t)nwarpsB * sw))) return st;
                a.scratch = (uint32_t*)eb.scratch.ptr;
                a.scratch_words = (uint32_t)sw;
                a.scr_n = scr_n;
                a.scr_kc = (uint32_t)kc;
            }
            dfs_kernel<<<gridB, kThreadsB, 0, s>>>(a);
            MBE_CUDA_TRY(cudaGetLastError());
            MBE_CUDA_TRY(cudaEventRecord(e2, s));
            io->launches += 2;
            MBE_CUDA_TRY(cudaMemcpyAsync(pin_ctrl, ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
            if (results_with_ctrl) {  // small result sets ride along: one synchronisation per chunk
                MBE_CUDA_TRY(cudaMemcpyAsync(pin_res, eb.results.ptr, sizeof(ResultAcc) * ng, cudaMemcpyDeviceToHost, s));
                io->d2h += sizeof(ResultAcc) * ng;
            }
            MBE_CUDA_TRY(cudaStreamSynchronize(s));
            const Ctrl hc = *pin_ctrl;
            if (results_with_ctrl) std::memcpy(results.data(), pin_res, sizeof(ResultAcc) * ng);
            io->d2h += sizeof(Ctrl);
            float t1 = 0, t2 = 0;
            cudaEventElapsedTime(&t1, e0, e1);
            cudaEventElapsedTime(&t2, e1, e2);
            ms_a += t1;
            ms_b += t2;
            if (!hc.error) {
                eb.ready_clean = ready_known;
                eb.cmap_clean = cmap_known;
            }
            if (hc.error) {
                if (hc.error == kErrPool) pool_exhausted = true;
                result = kernel_error(hc);
                break;
            }
            uint32_t consumed = std::min(hc.root_next, list_n);
            std::vector<uint32_t> retry_idx(std::min(hc.n_retry, retry_cap));
            if (!retry_idx.empty()) {
                MBE_CUDA_TRY(cudaMemcpyAsync(pin_retry_idx, a.retry, sizeof(uint32_t) * retry_idx.size(),
                                             cudaMemcpyDeviceToHost, s));
                MBE_CUDA_TRY(cudaStreamSynchronize(s));
                std::memcpy(retry_idx.data(), pin_retry_idx, sizeof(uint32_t) * retry_idx.size());
                io->d2h += sizeof(uint32_t) * retry_idx.size();
            }
            if (hc.n_retry > retry_cap || consumed == 0 || consumed == (uint32_t)retry_idx.size()) {
                // nothing fitted an empty pool: more chunks would not help
                pool_exhausted = true;
                result = fail(MBE_ERR_OUT_OF_MEMORY, "a root's search record does not fit the node pool");
                break;
            }
            std::vector<uint2> next_pending;
            const uint2* host_list = pending_roots.empty() ? roots.data() + main_next : chunk_list.data();
            for (uint32_t r : retry_idx) next_pending.push_back(host_list[r]);
            if (!pending_roots.empty()) {
                for (uint32_t r = consumed; r < list_n; r++) next_pending.push_back(chunk_list[r]);
            } else {
                main_next += consumed;
            }
            pending_roots.swap(next_pending);
        }
        if (pool_exhausted && !cfg.pool_words) {
            size_t fr = 0, tt = 0;
            MBE_CUDA_TRY(cudaMemGetInfo(&fr, &tt));
            uint64_t limit_words = std::min<uint64_t>((uint64_t)((fr + eb.pool.bytes) * 0.60) / 4, pool_cap_words);
            if (eb.pool_words * 2 <= limit_words) {
                eb.pool_words *= 2;
                continue;
            }
        }
        break;
    }
    if (result != MBE_OK) {
        // an error can stop the kernels with tasks still queued in the ring
        eb.ready_clean = 0;
        return result;
    }
    if (!results_with_ctrl) {
        MBE_CUDA_TRY(cudaMemcpyAsync(pin_res, eb.results.ptr, sizeof(ResultAcc) * ng, cudaMemcpyDeviceToHost, s));
        MBE_CUDA_TRY(cudaStreamSynchronize(s));
        std::memcpy(results.data(), pin_res, sizeof(ResultAcc) * ng);
        io->d2h += sizeof(ResultAcc) * ng;
    }
#ifdef MBE_PROFILE
    {
        unsigned long long hp[kProfSlots];
        MBE_CUDA_TRY(cudaMemcpy(hp, a.prof, sizeof hp, cudaMemcpyDeviceToHost));
        static const char* names[] = {"pop", "replay", "donate", "prefilter", "qscan", "expand", "build", "solve",
                                      "b.gather", "b.sort", "b.reduce", "b.write", "sum xi", "sum m", "sum nq2", "sum npp",
                                      "small eval", "small pre", "small bld", "general"};
        unsigned long long tot = 0;
        for (int q = 0; q < kProfMain; q++) tot += hp[2 * q];
        for (int q = 0; q < kProfSections; q++)
            std::fprintf(stderr, "prof %-10s cycles %14llu (%5.1f%%) events %12llu avg %.1f\n", names[q], hp[2 * q],
                         tot ? 100.0 * hp[2 * q] / tot : 0.0, hp[2 * q + 1],
                         hp[2 * q + 1] ? (double)hp[2 * q] / hp[2 * q + 1] : 0.0);
        std::vector<unsigned long long> ex(nwarpsB);
        MBE_CUDA_TRY(cudaMemcpy(ex.data(), a.prof + kProfSlots, sizeof(unsigned long long) * nwarpsB,
                                cudaMemcpyDeviceToHost));
        std::sort(ex.begin(), ex.end());
        unsigned long long t0 = ex.front();
        std::fprintf(stderr, "prof warps last busy after the first (ms): p10 %.3f p50 %.3f p90 %.3f p99 %.3f max %.3f\n",
                     (ex[nwarpsB / 10] - t0) / 1e6, (ex[nwarpsB / 2] - t0) / 1e6, (ex[nwarpsB * 9 / 10] - t0) / 1e6,
                     (ex[nwarpsB * 99 / 100] - t0) / 1e6, (ex.back() - t0) / 1e6);
        std::vector<unsigned long long> hist(2 * kProfBins);
        MBE_CUDA_TRY(cudaMemcpy(hist.data(), a.prof + kProfSlots + nwarpsB, sizeof(unsigned long long) * 2 * kProfBins,
                                cudaMemcpyDeviceToHost));
        std::fprintf(stderr, "prof chunks %u; idle %% of warp time per 20 ms (pops ending):", chunks);
        for (int b = 0; b < kProfBins; b += 5) {
            unsigned long long idle = 0, pops = 0;
            for (int q = b; q < b + 5 && q < kProfBins; q++) idle += hist[q], pops += hist[kProfBins + q];
            if (!idle && !pops) continue;
            std::fprintf(stderr, " [%d] %.0f%% (%llu)", b * 4, 100.0 * idle / (5.0 * kProfBinNs * nwarpsB), pops);
        }
        std::fprintf(stderr, "\n");
        std::vector<unsigned long long> tab(2 * kProfTB * kProfTC);
        MBE_CUDA_TRY(cudaMemcpy(tab.data(), a.prof + kProfSlots + nwarpsB + 2 * kProfBins,
                                sizeof(unsigned long long) * tab.size(), cudaMemcpyDeviceToHost));
        {
            unsigned long long pa[16];
            MBE_CUDA_TRY(cudaMemcpy(pa, a.prof_a, sizeof pa, cudaMemcpyDeviceToHost));
            static const char* an[] = {"discover+count", "classify", "sort", "rows", "reduce", "compact+push"};
            std::fprintf(stderr, "profA roots %llu total Gcycles %.2f; max root %.2f Mcycles (degree %llu)\n", pa[13],
                         pa[12] / 1e9, pa[14] / 1e6, pa[15]);
            for (int q = 0; q < 6; q++)
                std::fprintf(stderr, "profA %-15s Gcycles %8.3f (%5.1f%%) events %llu\n", an[q], pa[2 * q] / 1e9,
                             pa[12] ? 100.0 * pa[2 * q] / pa[12] : 0.0, pa[2 * q + 1]);
        }
        std::fprintf(stderr, "prof eval table: per 64 ms, class W1 W2 W4 W8 W16 W32 W64 W128+ replay prefilter: "
                             "Gcycles/evals; avg depth\n");
        for (int b = 0; b < kProfTB; b++) {
            unsigned long long any = 0;
            for (int c = 0; c < kProfTC; c++) any += tab[(b * kProfTC + c) * 2 + 1];
            if (!any) continue;
            std::fprintf(stderr, "  t%4d", b * 64);
            for (int c = 0; c < 10; c++)
                std::fprintf(stderr, " %.1f/%llu", tab[(b * kProfTC + c) * 2] / 1e9, tab[(b * kProfTC + c) * 2 + 1]);
            unsigned long long dn = tab[(b * kProfTC + 10) * 2 + 1];
            std::fprintf(stderr, " d%.1f\n", dn ? (double)tab[(b * kProfTC + 10) * 2] / dn : 0.0);
        }
    }
#endif
    if (stats) {
        stats->ms_expand = ms_a;
        stats->ms_dfs = ms_b;
        stats->chunks = chunks;
        stats->grid_a = gridA;
        stats->grid_b = gridB;
    }
    if (std::getenv("MBE_VERBOSE"))
        std::fprintf(stderr,
                     "engine: %u graphs, %zu roots, %u chunks, pool %.1f GiB, expand %.2f ms (%u blocks, occupancy %d), "
                     "dfs %.2f ms (%u blocks)\n",
                     ng, roots.size(), chunks, eb.pool_words * 4.0 / (1u << 30), ms_a, gridA, occA, ms_b, gridB);
    return MBE_OK;
}

// Launchers for callers outside this file that lay out EngineArgs
// themselves (the static-scratch entry point in capi_static.cu).
cudaError_t launch_expand_roots(const EngineArgs& a, unsigned grid, cudaStream_t s) {
    expand_roots_kernel<false><<<grid, kThreadsA, sizeof(uint32_t) * a.stage_words, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_dfs(const EngineArgs& a, unsigned grid, cudaStream_t s) {
    const cudaError_t e = try_dfs_carveout();
    if (e != cudaSuccess) return e;
    dfs_kernel<<<grid, kThreadsB, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mbe
