/*
 * mbe.h - C ABI of libmbe, a GB300-native (sm_103a) maximal biclique
 * enumeration engine that is a drop-in for the cuMBE enumeration path.
 *
 * The reference (NTUDDSNLab/cuMBE) has no library API: its boundary is the
 * `mbe <graph.bi> [cuMBE|noRS|noES|noWS]` command (src/main.cu:9,121-122),
 * the `.bi` text format it parses (src/main.cu:38-48), the orientation swap
 * (src/main.cu:65-70), the CSR transpose kernel (src/transpose.cuh:1-52),
 * the host root ordering (src/header.cuh:55-63) and the cooperative launch
 * of CUDA_MBE_<variant> (src/main.cu:190-199) whose only result is the
 * int32 count in `num_mb` (src/main.cu:207).  Each entry point below names
 * the reference interface it replaces.
 *
 * Conventions
 *  - Every call returns an mbe_status; nothing calls exit().  A failing call
 *    leaves a message retrievable with mbe_last_error().
 *  - Vertex ids are uint32, CSR offsets uint64.  Orientation is the file's:
 *    "rows" are the first header field of a `.bi` file, "cols" the second.
 *  - A context owns one CUDA stream on one device.  Calls on different
 *    contexts may run from different host threads; calls on one context
 *    must not overlap.
 *  - Counts are uint64 (the reference counts in int32 and wraps past 2^31).
 */
#ifndef MBE_H_
#define MBE_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define MBE_API __attribute__((visibility("default")))
#else
#define MBE_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mbe_status {
    MBE_OK = 0,
    MBE_ERR_INVALID_ARG = 1,
    MBE_ERR_IO = 2,
    MBE_ERR_FORMAT = 3,          /* malformed .bi text or CSR arrays        */
    MBE_ERR_CUDA = 4,            /* a CUDA runtime call failed              */
    MBE_ERR_OUT_OF_MEMORY = 5,   /* device pool / arena exhausted           */
    MBE_ERR_DEVICE_TIMEOUT = 6,  /* a bounded device-side wait ran out      */
    MBE_ERR_CAPACITY = 7,        /* a fixed-size device structure overflowed */
    MBE_ERR_NO_DEVICE = 8,       /* no CUDA device / driver available       */
    MBE_ERR_BUSY = 9             /* server: admission queue full            */
} mbe_status;

/* The four algorithm names the reference's CLI accepts
 * (src/header.cuh:12, src/main.cu:121-122).  All four return the same
 * count and hash; they differ in how the engine counts and schedules:
 *   MBE_CUMBE  reverse scanning (L-side scatter) + early stop + stealing
 *   MBE_NORS   candidate-side (forward) counting in the root expansion
 *   MBE_NOES   no early exit in the maximality and count loops
 *   MBE_NOWS   no work donation between warps (static root ownership)   */
typedef enum mbe_variant {
    MBE_CUMBE = 0,
    MBE_NORS = 1,
    MBE_NOES = 2,
    MBE_NOWS = 3
} mbe_variant;

typedef struct mbe_graph mbe_graph;
typedef struct mbe_ctx mbe_ctx;

typedef struct mbe_graph_info {
    uint32_t n_rows;
    uint32_t n_cols;
    uint64_t n_edges;
    uint32_t max_row_deg;
    uint32_t max_col_deg;
    uint32_t n_dup_dropped;      /* duplicate entries removed on ingest    */
    uint32_t swapped;            /* 1 when rows > cols: rows become the
                                    L side (src/main.cu:65-70)             */
} mbe_graph_info;

/* Synthetic bipartite Chung-Lu generator (replaces the reference's
 * KONECT download + data/gen_bi.cpp conversion, which needs network).
 * Weights w_i = (i+1)^(-1/(gamma-1)) per side, scaled to n_edges and capped
 * at max_deg; endpoints drawn with a splitmix64 stream seeded by `seed`;
 * duplicates rejected until n_edges distinct edges exist (or 64*n_edges
 * draws were made).  `planted` adds near-bicliques K_{planted_rows,
 * planted_cols} at edge density planted_density, half of each side drawn
 * from the 1% highest-weight vertices (hubs) and half uniformly.
 * gamma <= 0 on a side selects uniform endpoints (Erdos-Renyi G(n,m)). */
typedef struct mbe_gen_params {
    uint32_t n_rows;
    uint32_t n_cols;
    uint64_t n_edges;
    double gamma_rows;
    double gamma_cols;
    uint32_t max_deg;            /* 0 = uncapped                           */
    uint64_t seed;
    uint32_t planted;            /* number of planted blocks               */
    uint32_t planted_rows;
    uint32_t planted_cols;
    double planted_density;
} mbe_gen_params;

/* Enumeration options. */
enum {
    MBE_OPT_NO_HASH = 1u << 0,   /* skip the per-biclique canonical hash    */
    MBE_OPT_EMIT = 1u << 1,      /* materialise bicliques into emit buffers */
    MBE_OPT_TIMING = 1u << 2,    /* fill mbe_result.ms with device time     */
    MBE_OPT_L2_PIN = 1u << 3,    /* one-graph runs: keep the graph's L-side
                                    adjacency (the lists the root expansion
                                    streams, hubs' included) persisting in
                                    L2 for the run (access-policy window)   */
    MBE_OPT_HOST_CHUNKS = 1u << 4 /* mbe_batch_run: drive the chunk loop
                                    from the host (two synchronisations per
                                    chunk) instead of launching the chunks
                                    as a captured CUDA graph, the default  */
};

typedef struct mbe_opts {
    uint32_t flags;
    uint32_t min_rows;           /* thresholded enumeration: |A| >= min_rows */
    uint32_t min_cols;           /*                          |B| >= min_cols */
    /* tuning (0 = engine default) */
    uint32_t warps_per_block;    /* 0 or MBE_DFS_WARPS_PER_BLOCK: the DFS
                                    block shape is compiled in; any other
                                    value returns MBE_ERR_INVALID_ARG      */
    uint32_t blocks_per_sm;
    uint32_t donate_min;         /* min remaining children to donate       */
    uint32_t stack_words;        /* per-warp DFS arena size, 32-bit words  */
    /* Optional output stream (MBE_OPT_EMIT; mbe_enumerate only).  The
     * reference only counts (src/main.cu:207); this materialises each
     * counted biclique k into the caller's host buffers:
     *   emit_ids[emit_offsets[k] .. +emit_nrows[k]]     its rows (A),
     *   emit_ids[.. emit_offsets[k+1]]                  its cols (B),
     * in file ids, sides in no particular order, bicliques in no particular
     * order; mbe_result.emitted = bicliques written.  When the capacities
     * are too small the call returns MBE_ERR_CAPACITY with the result
     * filled (count and hash still cover every biclique) and the buffers
     * holding the first emitted ones.  emit_cap_ids must be < 2^32. */
    uint32_t* emit_offsets;      /* [emit_cap_bicliques+1] into emit_ids    */
    uint32_t* emit_ids;          /* rows of a biclique, then its cols       */
    uint32_t* emit_nrows;        /* [emit_cap_bicliques] |A| per biclique   */
    uint64_t emit_cap_bicliques;
    uint64_t emit_cap_ids;
    /* Root sample (all zero = every root).  The reference grabs roots
     * lowest degree first (src/mbe_cuMBE.cuh:57-64,125-133); here the
     * processing order is the branching side's vertices with at least one
     * edge by degree ascending, then id ascending.  Only the roots at
     * positions p of that order with root_begin <= p < root_end (root_end 0:
     * no upper bound) and (p - root_begin) % root_stride == 0 (root_stride
     * 0: 1) are expanded.  A sampled root still excludes every root before
     * it, so the result covers exactly the maximal bicliques whose
     * earliest branching-side member is a sampled root.  Used to measure a
     * fixed share of graphs whose full enumeration is out of reach. */
    uint32_t root_begin;
    uint32_t root_end;
    uint32_t root_stride;
    uint32_t reserved0;          /* must be 0                              */
    /* Longest time, in nanoseconds, that a device-side wait of the
     * enumeration kernels may last while no warp on the device makes
     * progress; past it the kernels stop and the call returns
     * MBE_ERR_DEVICE_TIMEOUT, leaving the context usable (0 = 60 s). */
    uint64_t wait_timeout_ns;
} mbe_opts;

/* Warps per block of the compiled DFS kernel (mbe_opts.warps_per_block). */
#define MBE_DFS_WARPS_PER_BLOCK 4u

typedef struct mbe_result {
    uint64_t count;              /* maximal bicliques (thresholds applied)  */
    uint64_t hash;               /* sum over bicliques of mbe_biclique_hash */
    uint64_t nodes;              /* search-tree nodes evaluated             */
    uint64_t words;              /* 32-bit words of set data streamed by
                                    the DFS kernel; a diagnostic counted
                                    only by builds with MBE_COUNT_WORDS=1
                                    or MBE_PROFILE=1, else 0               */
    uint64_t words_expand;       /* words streamed by the root expansion    */
    uint64_t emitted;            /* bicliques written to emit buffers       */
    float ms;                    /* device time of the enumeration kernels  */
    float ms_prep;               /* device time of the root expansion       */
} mbe_result;

/* ---- graphs (host side; no device needed) ------------------------------ */

/* Parses a `.bi` file: header "R L E", R lines "start length", E lines
 * "nbr x" with the second token ignored (src/main.cu:38-48).  Row lists
 * are sorted and deduplicated (the reference's own files hold unsorted
 * lists, data/gen_bi.cpp:78).  Replaces the ifstream reader at
 * src/main.cu:38-48; large files are parsed and normalised on all host
 * threads. */
MBE_API mbe_status mbe_graph_load_bi(const char* path, mbe_graph** out);

/* Builds a graph from a host CSR in file orientation.  Lists may be
 * unsorted and hold duplicates; both are normalised on ingest.  Replaces
 * the managed-memory CSR of src/main.cu:41-47. */
MBE_API mbe_status mbe_graph_from_csr(uint32_t n_rows, uint32_t n_cols,
                              const uint64_t* row_ptr, const uint32_t* col_idx,
                              mbe_graph** out);

MBE_API mbe_status mbe_graph_generate(const mbe_gen_params* params, mbe_graph** out);

/* Writes the `.bi` layout data/gen_bi.cpp:72-79 writes. */
MBE_API mbe_status mbe_graph_write_bi(const mbe_graph* g, const char* path);

/* Binary graph image: the normalised CSR (row_ptr, col_idx) behind a
 * checksummed header, loaded without parsing or normalising.  No reference
 * counterpart: the reference re-parses its text file on every run
 * (src/main.cu:38-48).  Loading verifies the checksum, the sizes and the
 * CSR invariants (monotone offsets, sorted unique ids in range) and
 * returns MBE_ERR_FORMAT otherwise. */
MBE_API mbe_status mbe_graph_write_bin(const mbe_graph* g, const char* path);
MBE_API mbe_status mbe_graph_load_bin(const char* path, mbe_graph** out);

/* Loads the `.bi` file bi_path through a binary cache at cache_path: the
 * cache is used when it is at least as new as bi_path and intact;
 * otherwise bi_path is parsed and the cache (re)written, best effort. */
MBE_API mbe_status mbe_graph_load_cached(const char* bi_path, const char* cache_path, mbe_graph** out);

/* Builds a graph from a KONECT edge-pair file the way data/gen_bi.cpp:14-60
 * does: skip_words leading tokens are skipped (the "%" header lines), then
 * "source target" pairs are read, each followed by skip_per_edge ignored
 * tokens (weights, timestamps), until the text ends or a pair is not two
 * integers.  Rows are sources, cols targets, each numbered by first
 * appearance; repeated pairs count once.  mbe_graph_write_bi then writes
 * the same `.bi` graph gen_bi writes (row lists sorted here). */
MBE_API mbe_status mbe_graph_load_konect(const char* path, uint32_t skip_words, uint32_t skip_per_edge,
                                         mbe_graph** out);

MBE_API mbe_status mbe_graph_info_get(const mbe_graph* g, mbe_graph_info* out);

/* Copies the normalised CSR out: row_ptr[n_rows+1], col_idx[n_edges]. */
MBE_API mbe_status mbe_graph_copy_csr(const mbe_graph* g, uint64_t* row_ptr,
                              uint32_t* col_idx);

MBE_API void mbe_graph_free(mbe_graph* g);

/* ---- contexts ------------------------------------------------------------ */

MBE_API mbe_status mbe_ctx_create(int device, mbe_ctx** out);
MBE_API void mbe_ctx_destroy(mbe_ctx* ctx);

/* Message of the last failing call on this host thread. */
MBE_API const char* mbe_last_error(void);

/* ---- device-resident graph -------------------------------------------- */

/* Copies the graph to the device, builds the transposed CSR with the
 * transpose kernels (replaces CUDA_TRANSPOSE, src/transpose.cuh:1-52) and
 * the root order (replaces my_memset_sort, src/header.cuh:55-63).  The
 * device copy stays resident in the context until mbe_graph_release or
 * mbe_ctx_destroy; repeated calls with the same graph are no-ops. */
MBE_API mbe_status mbe_graph_upload(mbe_ctx* ctx, const mbe_graph* g);
MBE_API mbe_status mbe_graph_release(mbe_ctx* ctx, const mbe_graph* g);

/* ---- enumeration -------------------------------------------------------- */

/* Counts (and hashes, and optionally emits) the maximal bicliques of g.
 * Replaces the cooperative launch of CUDA_MBE_<variant>
 * (src/main.cu:190-207, src/mbe_cuMBE.cuh:1-8).  Uploads g first when it
 * is not resident. */
MBE_API mbe_status mbe_enumerate(mbe_ctx* ctx, const mbe_graph* g, mbe_variant variant,
                         const mbe_opts* opts, mbe_result* out);

/* Batched enumeration: n graphs in one call.  Their roots are expanded in
 * chunks of ~128 MiB of node records, each chunk enumerated by one
 * persistent DFS launch; the chunks' launches run as a captured CUDA graph
 * (8 chunks per graph launch) unless opts->flags has MBE_OPT_HOST_CHUNKS.
 * Per-graph results go to out[i]; *total_ms (may be NULL) receives the
 * device time.  No reference counterpart: the reference runs one graph per
 * process (src/main.cu:9). */
MBE_API mbe_status mbe_batch_run(mbe_ctx* ctx, const mbe_graph* const* graphs, uint32_t n,
                         mbe_variant variant, const mbe_opts* opts,
                         mbe_result* out, float* total_ms);

/* ---- batched mode: autotuning ------------------------------------------ */

/* One size bucket's tuning.  No reference counterpart (the reference has one
 * fixed launch shape, src/main.cu:50-63).  A graph's bucket is
 * 4 * (|R| class) + (degree class), with |R| the branching side's vertices
 * with edges (classes < 256, < 1024, < 4096, larger) and the degree E/|R|
 * (classes < 4, < 16, < 64, larger). */
typedef struct mbe_tune_choice {
    uint32_t bucket;
    uint32_t n_graphs;           /* graphs of the tuned batch in the bucket  */
    uint32_t sample_graphs;      /* graphs the sweep timed                   */
    uint32_t blocks_per_sm;      /* DFS blocks per SM (0 = all that fit)     */
    uint32_t donate_min;         /* donation granularity (0 = default 2)     */
    uint32_t solve_rows;         /* register-search row limit (0 = off)      */
    uint32_t chunk_mwords;       /* root records per chunk, Mi 32-bit words  */
    uint32_t trials;             /* configurations timed                     */
    float ms_default;            /* the sample's device time, defaults       */
    float ms_tuned;              /* ... with this choice                     */
} mbe_tune_choice;

/* Tunes the engine for the buckets of the graphs given: for each bucket, a
 * sample of its graphs (up to 32, spread over its edge counts) is timed
 * with CUDA events under a coordinate descent over DFS blocks per SM,
 * donation granularity, register-search row limit and root chunk size (a
 * change is kept when it is 3% faster).  The choices are cached for the
 * process per (device, variant, bucket); mbe_batch_run then runs each group
 * of graphs that share a choice as one launch pair with it (when opts sets
 * no tuning field itself).  Up to cap choices are written to out. */
MBE_API mbe_status mbe_batch_tune(mbe_ctx* ctx, const mbe_graph* const* graphs, uint32_t n, mbe_variant variant,
                                  const mbe_opts* opts, mbe_tune_choice* out, uint32_t cap, uint32_t* n_out);
/* Forgets the cached choices of ctx's device. */
MBE_API mbe_status mbe_batch_tune_reset(mbe_ctx* ctx);

/* Canonical per-biclique hash: rows A and cols B in file orientation, in
 * any order.  The graph hash is the wrapping sum of this over bicliques. */
MBE_API uint64_t mbe_biclique_hash(const uint32_t* rows, uint32_t n_rows,
                           const uint32_t* cols, uint32_t n_cols);

MBE_API const char* mbe_variant_name(mbe_variant v);
/* Maps a CLI algorithm string to a variant; unknown strings map to
 * MBE_CUMBE as src/main.cu:122 does. */
MBE_API mbe_variant mbe_variant_from_name(const char* name);

/* ---- serving: continuous batching of enumeration requests -------------- */

/* No reference counterpart (the reference runs one graph per process).
 * Graphs are added once and stay resident; requests name a graph and
 * optional thresholds and are answered asynchronously.  `slots` worker
 * threads each own a stream and engine buffers and run on a share of the
 * GPU (`blocks_per_sm` DFS blocks per SM), so batches of different slots
 * overlap on the device.  A free slot takes the oldest waiting request
 * plus later waiting requests (whatever their thresholds: one launch applies
 * each request's own), up to `max_batch`, while the estimated root-record
 * memory of the batch fits
 * half the slot's share of `mem_budget` (a larger request runs alone).
 * `mem_budget` bounds the device memory of the search: it is divided among
 * the slots up front, and a slot's buffers never outgrow its share (its
 * node pool stops growing there and larger work runs in root chunks). */
typedef struct mbe_server mbe_server;

typedef struct mbe_server_config {
    uint32_t slots;              /* default 2                               */
    uint32_t max_batch;          /* default 256 (1 = one request per launch) */
    uint32_t blocks_per_sm;      /* default 3; 0 = the whole GPU per slot   */
    uint32_t variant;            /* mbe_variant                             */
    uint64_t mem_budget;         /* default 120 GB                          */
    uint64_t heavy_bytes;        /* requests whose estimated search memory
                                    exceeds this run on slot 0 only, alone
                                    (default 32 MiB)                        */
} mbe_server_config;

typedef struct mbe_request_result {
    uint64_t request;
    uint32_t graph;
    uint32_t status;             /* mbe_status of the request               */
    uint64_t count;
    uint64_t hash;
    double submit_s, start_s, done_s;  /* server clock, seconds            */
    uint32_t batch_size;         /* requests in the launch that served it   */
    uint32_t slot;
} mbe_request_result;

MBE_API mbe_status mbe_server_start(int device, const mbe_server_config* cfg, mbe_server** out);
/* Uploads g (device-resident for the server's lifetime); *graph_id names it. */
MBE_API mbe_status mbe_server_add_graph(mbe_server* s, const mbe_graph* g, uint32_t* graph_id);
/* Estimated bytes of search memory of a request on graph_id. */
MBE_API mbe_status mbe_server_estimate(mbe_server* s, uint32_t graph_id, uint64_t* bytes);
/* Queues a request (thresholds |A| >= min_rows, |B| >= min_cols); never blocks. */
MBE_API mbe_status mbe_server_submit(mbe_server* s, uint32_t graph_id, uint32_t min_rows, uint32_t min_cols,
                                     uint64_t* request_id);
/* Moves up to cap finished requests into out, oldest first. */
MBE_API mbe_status mbe_server_poll(mbe_server* s, mbe_request_result* out, uint32_t cap, uint32_t* n_out);
/* Seconds since the server started (the clock of mbe_request_result). */
MBE_API double mbe_server_clock(mbe_server* s);
/* Sizes every slot's device buffers for the graphs added so far and
 * returns when all slots are done, so that the requests that follow pay for
 * no device allocation (cudaMalloc and cudaFree synchronise the device, which
 * would stall the other slots' work). */
MBE_API mbe_status mbe_server_warmup(mbe_server* s);
/* Device memory the server holds: search_bytes = the slots' engine buffers
 * (never above mem_budget: each slot holds at most slot_cap =
 * min(mem_budget, 85% of the memory free at start) / slots), graph_bytes =
 * the resident graphs. */
MBE_API mbe_status mbe_server_memory(mbe_server* s, uint64_t* search_bytes, uint64_t* graph_bytes,
                                     uint64_t* slot_cap);
/* Finishes every queued request, stops the workers and frees the server. */
MBE_API mbe_status mbe_server_stop(mbe_server* s);

/* ---- allocation-free enumeration --------------------------------------- */

/* Working memory of mbe_enumerate_static: one array compiled into the
 * library, held on every GPU that loads it until the process exits. */
#define MBE_STATIC_SCRATCH_BYTES (64u << 20)
/* Largest side mbe_enumerate_static accepts. */
#define MBE_STATIC_MAX_VERTICES 4096u

/* Counts and hashes the maximal bicliques of a small graph without
 * allocating any device memory.  No counterpart in the reference: it is for
 * callers that may not allocate device memory while they run (hosts that
 * own the device through their own pool allocator, latency-bound serving
 * loops, plugin runtimes without an allocation budget).  The caller passes
 * the graph as two sorted, duplicate-free device CSRs with 32-bit offsets,
 * d_row_ptr[n_rows+1]/d_row_idx (rows -> cols) and its transpose
 * d_col_ptr[n_cols+1]/d_col_idx (cols -> rows), and a device buffer
 * d_result[2] that receives {count, hash} in stream order.  All working
 * memory comes from a fixed 64 MiB array inside the library: no cudaMalloc
 * or cudaFree is called.  Limits: at most MBE_STATIC_MAX_VERTICES per side
 * (MBE_ERR_CAPACITY beyond), and the search must fit the array
 * (MBE_ERR_OUT_OF_MEMORY otherwise).  The first call on a device, with that
 * device current, looks the array's address up; make it before any stream
 * capture.  The call synchronises `stream` to read the device status.
 * Every call reuses the same array: calls that overlap on the GPU race, so
 * serialise them.  `stream` is a cudaStream_t (NULL = default stream). */
MBE_API mbe_status mbe_enumerate_static(uint32_t n_rows, uint32_t n_cols, const uint32_t* d_row_ptr,
                                        const uint32_t* d_row_idx, const uint32_t* d_col_ptr,
                                        const uint32_t* d_col_idx, mbe_variant variant, uint64_t* d_result,
                                        void* stream);

/* Cumulative accounting of ctx since creation: kernels of this library
 * launched, bytes copied host->device and device->host. */
MBE_API mbe_status mbe_ctx_counters(mbe_ctx* ctx, uint64_t* launches, uint64_t* h2d_bytes, uint64_t* d2h_bytes);

/* Launch geometry of the last enumeration on ctx (the CLI's grid_size line). */
MBE_API mbe_status mbe_ctx_last_grid(mbe_ctx* ctx, uint32_t* grid_expand, uint32_t* grid_dfs, uint32_t* block);

#ifdef __cplusplus
}
#endif

#endif /* MBE_H_ */
