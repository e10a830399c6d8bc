// Enumeration engine: device data structures shared by the root-expansion
// kernel, the DFS kernel and the host driver.
//
// Search semantics (same result set as src/mbe_cuMBE.cuh):
//   root x (a rank of the R side):  L0 = N(x); candidates C = N(N(x)) \ {x};
//     Q0 = candidates of lower rank (processed before x), P0 = higher rank.
//     The root is non-maximal iff some v in Q0 is adjacent to all of L0.
//   node (L, R, P, Q), children x_i = P[i] in order:
//     L_i = L n N(x_i); non-maximal iff some v in Q u P[0..i) covers L_i;
//     absorbed  = {v in P(i..] : N(v) covers L_i}  -> R_i;
//     P_i       = {v in P(i..] : 0 < |N(v) n L_i| < |L_i|}, stably sorted by
//                 that count (the reference's min-count pivot order);
//     Q_i       = {v in Q u P[0..i) : |N(v) n L_i| > 0}.
//
// Every internal node is a self-contained RECORD: its L is a set of bit
// positions of the root universe (bit j <-> L0[j]); each candidate holds a
// bit row over the node's words; rows are stored word-major so that a warp
// reading 32 consecutive candidates of one word issues one 128-byte load.
// A child record keeps only the words where L_i is non-zero, with rows
// pre-masked by L_i.
#pragma once
#include <stdint.h>

#include "graph_dev.cuh"

namespace mbe {

// Shape of the DFS kernel: warps per block and the resident blocks per SM
// it is compiled for (the register budget).  4 x 7 = 28 warps per SM at 72
// registers measured fastest, with the shared arrays trimmed so that seven
// blocks fit a 64 KB carveout (bench graph: 6 blocks at 80 registers
// 233.7 ms, 7 blocks 229.0 ms, 8 blocks at 64 registers 239.4 ms; 600-graph
// batch 2,972 / 2,796 / 2,890 ms).
#ifndef MBE_DFS_WARPS
#define MBE_DFS_WARPS 4
#endif
#ifndef MBE_DFS_MIN_BLOCKS
#define MBE_DFS_MIN_BLOCKS 7
#endif
constexpr int kDfsWarps = MBE_DFS_WARPS;

constexpr uint32_t kHdrWords = 16;
constexpr uint32_t kMaxPath = 27;

__host__ __device__ inline uint32_t pad4(uint32_t x) { return (x + 3u) & ~3u; }

// Per-warp DFS arenas sit at a fixed stride (a multiple of 4 MiB by
// default), so without an offset every warp's hot stack top would fall on
// the same cache sets.  Warp gw's arena starts arena_skew(gw, stride) words
// into its region: one of up to 32 128-byte line offsets, chosen by a
// multiplicative hash of gw (warps of blocks resident on one SM differ in
// gw by multiples of the grid's block count).  The slack the largest offset
// takes is at most a sixteenth of the stride.
__host__ __device__ inline uint32_t arena_skew_lines(uint32_t stride) {
    const uint32_t l = stride / 512u;
    return l < 32u ? l : 32u;
}
__host__ __device__ inline uint32_t arena_usable_words(uint32_t stride) {
    const uint32_t l = arena_skew_lines(stride);
    return l ? stride - (l - 1u) * 32u : stride;
}
__host__ __device__ inline uint32_t arena_skew(uint32_t gw, uint32_t stride) {
    const uint32_t l = arena_skew_lines(stride);
    return l ? (((gw * 2654435761u) >> 16) % l) * 32u : 0u;
}
// The same for the per-warp frame stacks (512 frames of 32 bytes, a 16 KB
// stride): one of 32 line offsets (4 frames each), so the region of a warp
// holds kFrameSlack frames more than its stack.
constexpr uint32_t kFrameSlack = 31u * 4u;
__host__ __device__ inline uint32_t frame_skew(uint32_t gw) { return (((gw * 2654435761u) >> 16) % 32u) * 4u; }

// record layout (32-bit words):
//   [0,16)      header
//   wmap[W]     root word index of each word (lmap[32] when packed)
//   Lm[W]       L as bits per word
//   cand[n]     candidate ranks; [0,nq) = Q part, [nq,n) = P part
//   cnt[n]      |N(v) n L| (P part); absent when packed, where a row is one
//               word holding only L's bits and its count is the row's popcount
//   M[W*n]      word-major bit rows
struct NodeHdr {
    uint32_t graph;
    uint32_t root;
    uint32_t W;
    uint32_t n;
    uint32_t nq;
    uint32_t l;
    uint32_t nRset;
    uint32_t depth;
    unsigned long long sR;
    uint32_t words;
    uint32_t rlist;   // word offset (from record start) of the R list, 0 if absent
    uint32_t flags;   // kRecPacked: W == 1 and bit t of L is root bit lmap[t]
    uint32_t pad[3];
};
static_assert(sizeof(NodeHdr) == kHdrWords * 4, "header size");

constexpr uint32_t kRecPacked = 1;

// Section buckets of the optional cycle profile (-DMBE_PROFILE): cycles
// spent and events counted per section, summed over warps.
enum : int {
    kProfPop = 0,        // waiting for / taking a task
    kProfReplay,         // re-deriving donated paths
    kProfDonate,         // donating
    kProfPrefilter,      // batch maximality prefilter (one-word rows)
    kProfQscan,          // L_i + maximality scan of single evaluations
    kProfExpand,         // expansion (P scan) + hash of maximal children
    kProfBuild,          // child record construction
    kProfSolve,          // register-resident enumeration of small packed records
    kProfMain,           // sections above partition the warp time; below: detail of packed builds
    kProfBGather = kProfMain,  // Q' gather
    kProfBSort,          // Q' bucket sort and permutation
    kProfBReduce,        // Q' reduction
    kProfBWrite,         // P' sort, record write
    kProfSumXi,          // value sums (cycles field) per packed build (events field)
    kProfSumM,
    kProfSumNq2,
    kProfSumNpp,
    kProfSmallEval,      // evaluations (cycles) of children of packed records with <= 32 rows
    kProfSmallPre,       // prefilter batches (cycles) on such records
    kProfSmallBuild,     // builds of packed records with <= 32 rows (cycles)
    kProfGeneral,        // builds of unpacked (|L| > 32) child records (cycles, events)
    kProfSections,
    kProfSlots = 2 * kProfSections,
    kProfBins = 512,           // idle-time histogram over kernel time
    kProfBinNs = 4000000,      // 4 ms per bin
    kProfTB = 16,              // eval table: time bins of 64 ms ...
    kProfTC = 11,              // ... x classes: parent W bucket 0..7, replay, prefilter, depth sum
    kProfTabNs = 64000000
};

// A packed record (|L| <= 32) keeps its L bits dense in one word and maps
// bit t to root bit lmap[t] (32 words); otherwise word k of a row is root
// word wmap[k].  A packed record stores no count array: its counts are the
// popcounts of its one-word rows.
__host__ __device__ inline uint64_t record_words(uint32_t W, uint32_t n, bool packed = false) {
    return kHdrWords + (packed ? 32ull : pad4(W)) + pad4(W) + (packed ? 1ull : 2ull) * pad4(n) +
           (((uint64_t)W * n + 3) & ~3ull);
}

// Words of a record that also carries its R list (nr ranks; output stream
// only), stored right after the bit rows at word offset record_words().
__host__ __device__ inline uint64_t record_words_r(uint32_t W, uint32_t n, bool packed, uint32_t nr) {
    return record_words(W, n, packed) + pad4(nr);
}

// Words of one DFS warp's scratch for records of up to scr_n candidates
// (kc = the power of two >= scr_n, maxW = the widest L in words):
//   Li[maxW] Nz[maxW] qcnt[scr_n] (padded to even) | keysP[kc] keysQ[kc]
//   (u64) | pack[2 kc] | hist[32 maxW + 32] | absorbed[scr_n] (output stream)
// The DFS kernel lays it out the same way.
__host__ __device__ inline size_t scratch_words(uint32_t maxW, uint32_t scr_n, size_t kc, bool emit) {
    const size_t w = ((2 * (size_t)maxW + scr_n + 1) & ~(size_t)1) + 6 * kc + 32 * (size_t)maxW + 32 +
                     (emit ? scr_n : 0);
    return (w + 31) & ~(size_t)31;
}

// A unit of work: children [begin, end) of the node reached from the pool
// record `node` by following child indices path[0..plen).  The receiver
// re-derives the nodes on the path (deterministic), so donating a node that
// lives in the donor's private arena copies nothing.
struct Task {
    unsigned long long node;     // device pointer of a node-pool record
    uint32_t begin, end;         // child range (P-part indices)
    uint32_t plen;
    uint32_t path[kMaxPath];
};
static_assert(sizeof(Task) == 128, "task size");

struct Frame {
    unsigned long long node;
    uint32_t next, end;       // children [next, end) not yet looked at
    uint32_t arena_mark;      // arena top to restore when the frame pops
    uint32_t cur;             // child the next frame expands (donation paths)
    uint32_t mbase, pmask;    // children mbase + bit of pmask: known maximal, pending
};
static_assert(sizeof(Frame) == 32, "frame size");

struct ResultAcc {
    unsigned long long count, hash, nodes, words, words_expand;
};

enum : int {
    kErrNone = 0,
    kErrPool = 1,       // node pool exhausted
    kErrQueue = 2,      // task queue capacity
    kErrTimeout = 3,    // a bounded wait ran out
    kErrFrames = 4,     // DFS deeper than the frame stack
    kErrScratch = 5,    // per-warp scratch too small
    kErrReplay = 6,     // a donated path did not re-derive
};

struct EngineArgs {
    const GraphView* graphs;
    uint32_t n_graphs;
    uint32_t variant;
    uint32_t donate_min;
    uint32_t donate_copy;      // 1: donate small arena records by copy into the pool
    uint32_t solve_rows;       // packed records with at most this many rows (<= 32) are solved in registers
    // root list: (graph, rank) pairs, processed from index 0
    const uint2* roots;
    uint32_t n_roots;
    uint32_t* root_next;       // next root index to expand
    uint32_t* retry;           // roots whose record did not fit the pool
    uint32_t* n_retry;
    uint32_t retry_cap;
    // node pool (bump allocator, reset per chunk)
    uint32_t* pool;
    unsigned long long pool_words;
    unsigned long long* pool_top;
    unsigned long long pool_watermark;
    // task queue
    Task* tasks;
    uint32_t* ready;           // per slot: ticket+1 of the task stored, 0 = free
    uint32_t task_cap;         // ring capacity
    uint32_t* q_tail;          // tickets handed to producers
    uint32_t* q_head;          // tickets handed to consumers
    uint32_t* q_done;          // tasks read out of their slot
    uint32_t q_margin;         // free slots a donor leaves untouched
    int* pending;
    unsigned long long* progress;
    // phase A per-block scratch
    int* cmap;                 // [gridA][maxNR]  vertex -> candidate slot, -1 when free
    uint32_t* a_cl;            // [gridA][maxNR]
    uint32_t* a_cnt;           // [gridA][maxNR]
    unsigned long long* a_keys;// [gridA][pow2(maxNR)]
    uint32_t maxNR;
    uint32_t keys_cap;
    uint32_t stage_words;      // dynamic shared words per root-expansion block for staging L0 (0 = none)
    uint32_t* max_n;           // largest candidate count of any root record
    // phase B per-warp memory
    uint32_t* arena;
    uint32_t arena_words;      // usable words of one warp's arena
    uint32_t arena_stride;     // words between consecutive warps' arena regions
    Frame* frames;
    uint32_t max_frames;
    uint32_t frame_stride;     // frames between consecutive warps' stacks (>= max_frames)
    uint32_t frame_skew;       // 1: stacks start at hashed line offsets (frame_stride >= max_frames + kFrameSlack)
    uint32_t* scratch;
    uint32_t scratch_words;
    uint32_t scr_n;            // candidate bound the scratch is laid out for
    uint32_t scr_kc;           // key-array capacity (power of two >= scr_n)
    uint32_t scratch_dyn;      // 1: the DFS kernel lays its scratch out from *max_n itself
                               //    (scratch sized for the bound; scr_n / scr_kc / scratch_words unused)
    uint32_t max_W;            // largest universe word count
    // section cycle counters (builds with -DMBE_PROFILE only; else null)
    unsigned long long* prof;  // [kProfSlots + warps + 2 * kProfBins]
    uint32_t prof_warps;
    unsigned long long* prof_a;  // [16] root-expansion sections (profile builds)
    // output stream (MBE_OPT_EMIT; emit == 0 otherwise): each counted
    // biclique reserves room for its file rows then its file cols
    uint32_t emit;
    uint32_t* emit_ids;                 // [emit_cap_ids]
    unsigned long long emit_cap_ids;
    unsigned long long* emit_start;     // [emit_cap_b] id offset of each biclique
    uint32_t* emit_nrows;               // [emit_cap_b] |A| (file rows)
    uint32_t* emit_ncols;               // [emit_cap_b] |B| (file cols)
    unsigned long long emit_cap_b;
    unsigned long long* emit_ctl;       // [0] ids reserved, [1] bicliques reserved, [2] overflow
    // results
    ResultAcc* results;        // [n_graphs]
    int* error;
    unsigned long long* error_info;
    unsigned long long timeout_ns;
};

}  // namespace mbe
