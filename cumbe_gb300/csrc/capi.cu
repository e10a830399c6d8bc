// C ABI of libmbe: contexts, device residency, enumeration, batching.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <new>
#include <unordered_map>
#include <vector>

#include "dev_common.cuh"
#include "engine_host.h"
#include "graph_dev.cuh"
#include "mbe_internal.h"

using namespace mbe;

struct mbe_ctx {
    int device = 0;
    int n_sm = 0;
    cudaStream_t stream = nullptr;
    std::unordered_map<uint64_t, DeviceGraph> resident;
    EngineBuffers eb;
    EngineStats last_stats;
    IoCounters io;
    std::mutex mu;
};

namespace {

mbe_status check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return MBE_OK;
    cudaGetLastError();
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return fail(MBE_ERR_NO_DEVICE, std::string(what) + ": " + cudaGetErrorString(e));
    return fail(e == cudaErrorMemoryAllocation ? MBE_ERR_OUT_OF_MEMORY : MBE_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

mbe_status ensure_resident(mbe_ctx* ctx, const mbe_graph* g, const DeviceGraph** out) {
    auto it = ctx->resident.find(g->uid);
    if (it != ctx->resident.end()) {
        *out = &it->second;
        return MBE_OK;
    }
    DeviceGraph d;
    mbe_status st = build_device_graph(g, ctx->stream, ctx->n_sm, &d, &ctx->io);
    if (st != MBE_OK) return st;
    auto res = ctx->resident.emplace(g->uid, std::move(d));
    *out = &res.first->second;
    return MBE_OK;
}

EngineConfig make_config(mbe_variant v, const mbe_opts* o) {
    EngineConfig c;
    c.variant = (uint32_t)v;
    // multi-graph runs launch their chunks as a captured CUDA graph, 8 chunks
    // per launch, unless the caller asks for the host-driven loop
    c.graph_chunks = 8;
    if (const char* env = std::getenv("MBE_GRAPH_CHUNKS"))
        c.graph_chunks = (uint32_t)std::max(1ul, std::strtoul(env, nullptr, 10));
    if (o && (o->flags & MBE_OPT_HOST_CHUNKS)) c.graph_chunks = 0;
    if (o) {
        c.min_rows = o->min_rows;  // file orientation; each entry maps them to its own
        c.min_cols = o->min_cols;
        if (o->donate_min) c.donate_min = o->donate_min;
        if (o->blocks_per_sm) c.blocks_per_sm = o->blocks_per_sm;
        if (o->stack_words) c.arena_words = (o->stack_words + 3u) & ~3u;
        if (o->wait_timeout_ns) c.timeout_ns = o->wait_timeout_ns;
        c.l2_pin = (o->flags & MBE_OPT_L2_PIN) != 0;
    }
    if (const char* env = std::getenv("MBE_POOL_MB")) {
        unsigned long long mb = std::strtoull(env, nullptr, 10);
        if (mb) c.pool_words = mb * (1ull << 20) / 4;
    }
    return c;
}

// Rejects option values the engine cannot honour.
mbe_status check_opts(const mbe_opts* o) {
    if (!o) return MBE_OK;
    if (o->warps_per_block && o->warps_per_block != (uint32_t)kDfsWarps)
        return fail(MBE_ERR_INVALID_ARG, "warps_per_block must be 0 or " + std::to_string(kDfsWarps) +
                                             " (the DFS kernel's compiled block shape)");
    if (o->root_end && o->root_end <= o->root_begin)
        return fail(MBE_ERR_INVALID_ARG, "root_end must be 0 or greater than root_begin");
    if (o->reserved0) return fail(MBE_ERR_INVALID_ARG, "mbe_opts.reserved0 must be 0");
    return MBE_OK;
}

}  // namespace

extern "C" mbe_status mbe_ctx_create(int device, mbe_ctx** out) {
    clear_error();
    if (!out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    int n = 0;
    mbe_status st = check_cuda(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (st != MBE_OK) return st;
    if (device < 0 || device >= n) return fail(MBE_ERR_NO_DEVICE, "device index out of range");
    if ((st = check_cuda(cudaSetDevice(device), "cudaSetDevice"))) return st;
    auto* c = new (std::nothrow) mbe_ctx();
    if (!c) return fail(MBE_ERR_OUT_OF_MEMORY, "host allocation failed");
    c->device = device;
    if ((st = check_cuda(cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, device), "attr")) ||
        (st = check_cuda(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate"))) {
        delete c;
        return st;
    }
    *out = c;
    return MBE_OK;
}

extern "C" void mbe_ctx_destroy(mbe_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->resident) kv.second.release();
    ctx->eb.release();
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" mbe_status mbe_graph_upload(mbe_ctx* ctx, const mbe_graph* g) {
    clear_error();
    if (!ctx || !g) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    mbe_status st = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (st) return st;
    const DeviceGraph* d;
    return ensure_resident(ctx, g, &d);
}

extern "C" mbe_status mbe_graph_release(mbe_ctx* ctx, const mbe_graph* g) {
    clear_error();
    if (!ctx || !g) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->resident.find(g->uid);
    if (it != ctx->resident.end()) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        it->second.release();
        ctx->resident.erase(it);
    }
    return MBE_OK;
}

namespace mbe {

// Enumerates the maximal bicliques of the resident graphs `devs` (one
// result per entry; an entry may repeat a graph).  Roots of all graphs are
// expanded heaviest first in one launch pair.  Thresholds are stated in
// file orientation, so a list mixing orientations with thresholds runs
// once per orientation group.
mbe_status run_devs(EngineBuffers& eb, cudaStream_t s, IoCounters* io, const std::vector<const DeviceGraph*>& devs,
                    mbe_variant variant, const mbe_opts* opts, std::vector<ResultAcc>& acc, EngineStats& stats,
                    const EmitTarget* emit, uint64_t mem_cap, const BatchKnobs* knobs,
                    const std::vector<uint2>* entry_thr) {
    const uint32_t n = (uint32_t)devs.size();
    std::vector<uint2> roots;
    size_t total = 0;
    for (uint32_t i = 0; i < n; i++) total += devs[i]->nR - devs[i]->n_isolated;
    roots.reserve(total);
    // root sample: positions p = rank - n_isolated of the processing order
    const uint32_t s_begin = opts ? opts->root_begin : 0u, s_end = opts && opts->root_end ? opts->root_end : ~0u;
    const uint32_t s_stride = opts && opts->root_stride > 1 ? opts->root_stride : 1u;
    for (uint32_t i = 0; i < n; i++)
        for (uint32_t r = devs[i]->nR; r-- > devs[i]->n_isolated;) {
            const uint32_t p = r - devs[i]->n_isolated;
            if (p < s_begin || p >= s_end || (p - s_begin) % s_stride) continue;
            roots.push_back(make_uint2(i, r));
        }
    if (n > 1)
        std::stable_sort(roots.begin(), roots.end(), [&](const uint2& a, const uint2& b) {
            return devs[a.x]->deg_by_rank[a.y] > devs[b.x]->deg_by_rank[b.y];
        });
    acc.assign(n, ResultAcc{});
    stats = EngineStats{};
    EngineConfig cfg = make_config(variant, opts);
    cfg.emit = emit;
    cfg.mem_cap = mem_cap;
    cfg.entry_thr = entry_thr;
    // Many graphs: chunks of ~128 MiB of root records, so that the DFS
    // reads each chunk's records while they are still in L2 (measured:
    // 4,096 mixed graphs 19.4 s -> 17.2 s).  One graph keeps one chunk:
    // every chunk ends in a load-imbalance tail, which costs more there.
    if (n > 1 && !cfg.pool_words) cfg.chunk_words = 32ull << 20;
    if (knobs) {
        if (knobs->blocks_per_sm) cfg.blocks_per_sm = knobs->blocks_per_sm;
        if (knobs->donate_min) cfg.donate_min = knobs->donate_min;
        cfg.solve_rows = knobs->solve_rows;
        if (knobs->chunk_words && !cfg.pool_words) cfg.chunk_words = knobs->chunk_words;
    }
    return engine_run(eb, s, cfg, devs, roots, acc, &stats, io);
}

}  // namespace mbe

// Output stream of one enumeration: device buffers sized by the caller's
// capacities, then compacted into the caller's host buffers in
// reservation order (offsets[k]..offsets[k+1] = rows then cols of
// biclique k).
struct EmitRun {
    EmitTarget t;
    mbe_status setup(mbe_ctx* ctx, const mbe_opts* o) {
        if (!o->emit_offsets || !o->emit_ids || !o->emit_nrows || !o->emit_cap_bicliques)
            return fail(MBE_ERR_INVALID_ARG, "MBE_OPT_EMIT needs emit_offsets, emit_ids, emit_nrows and capacities");
        if (o->emit_cap_ids >= (1ull << 32))
            return fail(MBE_ERR_INVALID_ARG, "emit_cap_ids must be below 2^32 (offsets are 32-bit)");
        EngineBuffers& eb = ctx->eb;
        mbe_status st;
        const size_t capb = (size_t)o->emit_cap_bicliques, capi = std::max<size_t>(1, (size_t)o->emit_cap_ids);
        if ((st = eb.e_ids.ensure(4 * capi)) || (st = eb.e_start.ensure(8 * capb)) ||
            (st = eb.e_nrows.ensure(4 * capb)) || (st = eb.e_ncols.ensure(4 * capb)) ||
            (st = eb.e_ctl.ensure(3 * sizeof(unsigned long long))))
            return st;
        t.ids = (uint32_t*)eb.e_ids.ptr;
        t.cap_ids = o->emit_cap_ids;
        t.start = (unsigned long long*)eb.e_start.ptr;
        t.nrows = (uint32_t*)eb.e_nrows.ptr;
        t.ncols = (uint32_t*)eb.e_ncols.ptr;
        t.cap_b = o->emit_cap_bicliques;
        t.ctl = (unsigned long long*)eb.e_ctl.ptr;
        return MBE_OK;
    }
    // Copies the stream to the caller's buffers; *emitted = bicliques
    // written; MBE_ERR_CAPACITY when some did not fit.
    mbe_status finish(mbe_ctx* ctx, const mbe_opts* o, uint64_t* emitted) {
        unsigned long long ctl[3];
        mbe_status st = check_cuda(cudaMemcpy(ctl, t.ctl, sizeof ctl, cudaMemcpyDeviceToHost), "emit readback");
        if (st) return st;
        const size_t K = (size_t)std::min<unsigned long long>(ctl[1], t.cap_b);
        const size_t used = (size_t)std::min<unsigned long long>(ctl[0], t.cap_ids);
        std::vector<unsigned long long> start(K);
        std::vector<uint32_t> nr(K), nc(K), ids(used);
        if (K && ((st = check_cuda(cudaMemcpy(start.data(), t.start, 8 * K, cudaMemcpyDeviceToHost), "emit")) ||
                  (st = check_cuda(cudaMemcpy(nr.data(), t.nrows, 4 * K, cudaMemcpyDeviceToHost), "emit")) ||
                  (st = check_cuda(cudaMemcpy(nc.data(), t.ncols, 4 * K, cudaMemcpyDeviceToHost), "emit"))))
            return st;
        if (used && (st = check_cuda(cudaMemcpy(ids.data(), t.ids, 4 * used, cudaMemcpyDeviceToHost), "emit")))
            return st;
        ctx->io.d2h += sizeof ctl + 16 * K + 4 * used;
        uint64_t off = 0;
        for (size_t k = 0; k < K; k++) {
            const uint32_t sz = nr[k] + nc[k];
            o->emit_offsets[k] = (uint32_t)off;
            o->emit_nrows[k] = nr[k];
            std::memcpy(o->emit_ids + off, ids.data() + start[k], 4ull * sz);
            off += sz;
        }
        o->emit_offsets[K] = (uint32_t)off;
        *emitted = K;
        if (ctl[2])
            return fail(MBE_ERR_CAPACITY, "emit buffers full: " + std::to_string(K) +
                                              " bicliques written (count and hash cover all)");
        return MBE_OK;
    }
};

// ---------------------------------------------------------------------------
// Batched mode: autotuning of the engine knobs per graph-size bucket.
//
// A graph's bucket is its branching side's size class (|R| < 256, < 1024,
// < 4096, larger) and its average degree class (E/|R| < 4, < 16, < 64,
// larger).  mbe_batch_tune times, for each bucket present in a batch, a
// sample of the bucket's graphs (up to 32, spread over the bucket's range of
// edge counts) under a coordinate descent over four knobs -- DFS blocks per
// SM (block count), donation granularity (steal granularity), the register
// search's row limit (bitmap search in registers vs records in memory) and
// the root-record chunk (how much search state is live at once) -- keeping
// a change only when it is 3% faster, and caches the choice per (device,
// variant, bucket) for the process.  mbe_batch_run applies cached choices.
namespace {

constexpr uint32_t kTuneSample = 32;

uint32_t tune_bucket(const DeviceGraph& d) {
    const uint32_t nR = d.nR - d.n_isolated;
    const double deg = nR ? (double)d.nE / nR : 0.0;
    const uint32_t rc = nR < 256 ? 0 : nR < 1024 ? 1 : nR < 4096 ? 2 : 3;
    const uint32_t dc = deg < 4 ? 0 : deg < 16 ? 1 : deg < 64 ? 2 : 3;
    return 4 * rc + dc;
}

struct TuneKey {
    int device;
    uint32_t variant, bucket;
    bool operator<(const TuneKey& o) const {
        return std::tie(device, variant, bucket) < std::tie(o.device, o.variant, o.bucket);
    }
};

std::mutex g_tune_mu;
std::map<TuneKey, mbe_tune_choice> g_tune;

bool explicit_tuning(const mbe_opts* o) { return o && (o->blocks_per_sm || o->donate_min || o->stack_words); }

BatchKnobs knobs_of(const mbe_tune_choice& c) {
    BatchKnobs k;
    k.blocks_per_sm = c.blocks_per_sm;
    k.donate_min = c.donate_min;
    k.solve_rows = c.solve_rows;
    k.chunk_words = (uint64_t)c.chunk_mwords << 20;
    return k;
}

}  // namespace

extern "C" mbe_status mbe_batch_tune(mbe_ctx* ctx, const mbe_graph* const* graphs, uint32_t n, mbe_variant variant,
                                     const mbe_opts* opts, mbe_tune_choice* out, uint32_t cap, uint32_t* n_out) {
    clear_error();
    if (!ctx || (!graphs && n) || (!out && cap)) return fail(MBE_ERR_INVALID_ARG, "null argument");
    if (explicit_tuning(opts)) return fail(MBE_ERR_INVALID_ARG, "mbe_batch_tune chooses the tuning fields itself");
    std::lock_guard<std::mutex> lk(ctx->mu);
    mbe_status st = check_opts(opts);
    if (st) return st;
    if ((st = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice"))) return st;
    std::map<uint32_t, std::vector<const DeviceGraph*>> buckets;
    for (uint32_t i = 0; i < n; i++) {
        if (!graphs[i]) return fail(MBE_ERR_INVALID_ARG, "null graph");
        const DeviceGraph* d;
        if ((st = ensure_resident(ctx, graphs[i], &d))) return st;
        buckets[tune_bucket(*d)].push_back(d);
    }
    int occB = 0;
    if ((st = check_cuda(dfs_blocks_per_sm(ctx->device, &occB), "occupancy"))) return st;
    uint32_t k_out = 0;
    for (auto& kv : buckets) {
        std::vector<const DeviceGraph*>& all = kv.second;
        std::stable_sort(all.begin(), all.end(), [](const DeviceGraph* a, const DeviceGraph* b) { return a->nE > b->nE; });
        std::vector<const DeviceGraph*> sample;
        const size_t m = std::min<size_t>(all.size(), kTuneSample);
        for (size_t j = 0; j < m; j++) sample.push_back(all[j * all.size() / m]);
        uint32_t trials = 0;
        uint64_t ref_count = 0;
        bool have_ref = false;
        auto measure = [&](const BatchKnobs& k, float* ms) -> mbe_status {
            float best = 0;
            for (int rep = 0; rep < 2; rep++) {
                std::vector<ResultAcc> acc;
                EngineStats stats;
                mbe_status s2 = run_devs(ctx->eb, ctx->stream, &ctx->io, sample, variant, opts, acc, stats, nullptr, 0, &k);
                if (s2) return s2;
                uint64_t c = 0;
                for (const ResultAcc& r : acc) c += r.count;
                if (have_ref && c != ref_count) return fail(MBE_ERR_CUDA, "autotuner: results differ between configurations");
                ref_count = c;
                have_ref = true;
                const float t = stats.ms_expand + stats.ms_dfs;
                if (rep == 0 || t < best) best = t;
                if (t > 200.0f) break;  // heavy samples: one timing is enough
            }
            trials++;
            *ms = best;
            return MBE_OK;
        };
        BatchKnobs cur;  // engine defaults
        cur.chunk_words = 32ull << 20;
        float best = 0, ms_default = 0;
        if ((st = measure(cur, &best))) return st;
        // heavy buckets: thin the sample (every other graph) until a run
        // takes under ~400 ms, so that the sweep stays short
        while (best > 400.0f && sample.size() > 2) {
            std::vector<const DeviceGraph*> thin;
            for (size_t j = 0; j < sample.size(); j += 2) thin.push_back(sample[j]);
            sample.swap(thin);
            have_ref = false;
            if ((st = measure(cur, &best))) return st;
        }
        ms_default = best;
        const uint32_t b_alt[2] = {(uint32_t)std::max(1, occB - 2), (uint32_t)std::max(1, occB / 2)};
        const uint32_t d_alt[2] = {3, 4};
        const uint32_t s_alt[2] = {16, 0};
        const uint64_t c_alt[2] = {8ull << 20, 128ull << 20};
        for (int knob = 0; knob < 4; knob++)
            for (int j = 0; j < 2; j++) {
                BatchKnobs k2 = cur;
                if (knob == 0) k2.blocks_per_sm = b_alt[j];
                if (knob == 1) k2.donate_min = d_alt[j];
                if (knob == 2) k2.solve_rows = s_alt[j];
                if (knob == 3) k2.chunk_words = c_alt[j];
                float t = 0;
                if ((st = measure(k2, &t))) return st;
                if (t < 0.97f * best) {
                    best = t;
                    cur = k2;
                }
            }
        mbe_tune_choice c;
        std::memset(&c, 0, sizeof c);
        c.bucket = kv.first;
        c.n_graphs = (uint32_t)all.size();
        c.sample_graphs = (uint32_t)sample.size();
        c.blocks_per_sm = cur.blocks_per_sm;
        c.donate_min = cur.donate_min;
        c.solve_rows = cur.solve_rows;
        c.chunk_mwords = (uint32_t)(cur.chunk_words >> 20);
        c.trials = trials;
        c.ms_default = ms_default;
        c.ms_tuned = best;
        {
            std::lock_guard<std::mutex> tl(g_tune_mu);
            g_tune[TuneKey{ctx->device, (uint32_t)variant, kv.first}] = c;
        }
        if (k_out < cap) out[k_out] = c;
        k_out++;
    }
    if (n_out) *n_out = std::min(k_out, cap);
    return MBE_OK;
}

extern "C" mbe_status mbe_batch_tune_reset(mbe_ctx* ctx) {
    clear_error();
    if (!ctx) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> tl(g_tune_mu);
    for (auto it = g_tune.begin(); it != g_tune.end();)
        it = it->first.device == ctx->device ? g_tune.erase(it) : std::next(it);
    return MBE_OK;
}

static mbe_status run_graphs(mbe_ctx* ctx, const mbe_graph* const* graphs, uint32_t n, mbe_variant variant,
                             const mbe_opts* opts, mbe_result* out, float* total_ms) {
    const bool emit = opts && (opts->flags & MBE_OPT_EMIT);
    if (emit && n != 1) return fail(MBE_ERR_INVALID_ARG, "MBE_OPT_EMIT takes one graph (mbe_enumerate)");
    mbe_status st = check_opts(opts);
    if (st) return st;
    st = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (st) return st;
    std::vector<const DeviceGraph*> devs(n);
    for (uint32_t i = 0; i < n; i++) {
        if (!graphs[i]) return fail(MBE_ERR_INVALID_ARG, "null graph");
        if ((st = ensure_resident(ctx, graphs[i], &devs[i]))) return st;
    }
    EmitRun er;
    if (emit && (st = er.setup(ctx, opts))) return st;
    std::vector<ResultAcc> acc;
    EngineStats stats;
    // graphs whose bucket mbe_batch_tune has tuned on this device run with
    // the cached choice, one launch pair per distinct choice
    std::map<std::tuple<uint32_t, uint32_t, uint32_t, uint32_t>, std::vector<uint32_t>> groups;
    std::map<std::tuple<uint32_t, uint32_t, uint32_t, uint32_t>, BatchKnobs> group_knobs;
    if (n > 1 && !explicit_tuning(opts)) {
        std::lock_guard<std::mutex> tl(g_tune_mu);
        if (!g_tune.empty())
            for (uint32_t i = 0; i < n; i++) {
                auto it = g_tune.find(TuneKey{ctx->device, (uint32_t)variant, tune_bucket(*devs[i])});
                BatchKnobs k;
                k.chunk_words = 32ull << 20;
                if (it != g_tune.end()) k = knobs_of(it->second);
                const auto key = std::make_tuple(k.blocks_per_sm, k.donate_min, k.solve_rows, (uint32_t)(k.chunk_words >> 20));
                groups[key].push_back(i);
                group_knobs[key] = k;
            }
    }
    if (!groups.empty()) {
        acc.assign(n, ResultAcc{});
        for (auto& kv : groups) {
            std::vector<const DeviceGraph*> sub;
            for (uint32_t i : kv.second) sub.push_back(devs[i]);
            std::vector<ResultAcc> part;
            EngineStats ps;
            if ((st = run_devs(ctx->eb, ctx->stream, &ctx->io, sub, variant, opts, part, ps, nullptr, 0,
                               &group_knobs[kv.first])))
                return st;
            for (size_t j = 0; j < kv.second.size(); j++) acc[kv.second[j]] = part[j];
            stats.ms_expand += ps.ms_expand;
            stats.ms_dfs += ps.ms_dfs;
            stats.chunks += ps.chunks;
            stats.grid_a = ps.grid_a;
            stats.grid_b = ps.grid_b;
        }
    } else if ((st = run_devs(ctx->eb, ctx->stream, &ctx->io, devs, variant, opts, acc, stats,
                              emit ? &er.t : nullptr))) {
        return st;
    }
    ctx->last_stats = stats;
    for (uint32_t i = 0; i < n; i++) {
        mbe_result& r = out[i];
        std::memset(&r, 0, sizeof r);
        r.count = acc[i].count;
        r.hash = (opts && (opts->flags & MBE_OPT_NO_HASH)) ? 0 : acc[i].hash;
        r.nodes = acc[i].nodes;
        r.words = acc[i].words;
        r.words_expand = acc[i].words_expand;
        r.ms = stats.ms_expand + stats.ms_dfs;
        r.ms_prep = stats.ms_expand;
    }
    if (total_ms) *total_ms = stats.ms_expand + stats.ms_dfs;
    if (emit) return er.finish(ctx, opts, &out[0].emitted);
    return MBE_OK;
}

extern "C" mbe_status mbe_enumerate(mbe_ctx* ctx, const mbe_graph* g, mbe_variant variant, const mbe_opts* opts,
                                    mbe_result* out) {
    clear_error();
    if (!ctx || !g || !out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return run_graphs(ctx, &g, 1, variant, opts, out, nullptr);
}

extern "C" mbe_status mbe_batch_run(mbe_ctx* ctx, const mbe_graph* const* graphs, uint32_t n, mbe_variant variant,
                                    const mbe_opts* opts, mbe_result* out, float* total_ms) {
    clear_error();
    if (!ctx || (!graphs && n) || (!out && n)) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return run_graphs(ctx, graphs, n, variant, opts, out, total_ms);
}

extern "C" mbe_status mbe_ctx_counters(mbe_ctx* ctx, uint64_t* launches, uint64_t* h2d, uint64_t* d2h) {
    clear_error();
    if (!ctx) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (launches) *launches = ctx->io.launches;
    if (h2d) *h2d = ctx->io.h2d;
    if (d2h) *d2h = ctx->io.d2h;
    return MBE_OK;
}

// Launch geometry of the last enumeration (CLI "grid_size" line).
extern "C" mbe_status mbe_ctx_last_grid(mbe_ctx* ctx, uint32_t* grid_expand, uint32_t* grid_dfs, uint32_t* block) {
    clear_error();
    if (!ctx) return fail(MBE_ERR_INVALID_ARG, "null argument");
    if (grid_expand) *grid_expand = ctx->last_stats.grid_a;
    if (grid_dfs) *grid_dfs = ctx->last_stats.grid_b;
    if (block) *block = 32u * kDfsWarps;  // the enumeration (DFS) kernel's block
    return MBE_OK;
}
