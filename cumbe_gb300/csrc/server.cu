// Serving: continuous batching of enumeration requests over a pool of
// device-resident graphs (no reference counterpart; see include/mbe.h).
//
// Each worker ("slot") owns a CUDA stream and its own engine buffers and
// runs the root-expansion and DFS kernels on `blocks_per_sm` blocks per SM,
// so launches of different slots share the GPU at the same time.  A slot
// that becomes free takes, under the queue lock, the oldest waiting request
// and later waiting requests (each keeps its own thresholds: the engine
// applies them per entry, so one launch mixes them) up to max_batch, while
// the estimated search memory of the batch fits the slot's node-pool share;
// requests arriving while others run join the next batch of the next free
// slot.  Heavy requests (estimated search memory above heavy_bytes) are
// taken by slot 0 only and run alone, so the other slots always serve the
// light ones.  Latency = done - submit on one steady clock.
//
// Memory: mem_budget is divided among the slots up front.  A slot's engine
// buffers (node pool, per-warp arenas, scratch, task ring, root-expansion
// maps) never hold more than its share: the arenas shrink to fit, the pool
// gets what the other buffers leave and stops growing at the share, and a
// batch larger than the pool is enumerated in root chunks that fit.  So the
// search memory the server holds is bounded by mem_budget whatever the
// requests; mbe_server_memory reports what it holds.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "dev_common.cuh"
#include "engine_host.h"
#include "graph_dev.cuh"
#include "mbe_internal.h"

using namespace mbe;

namespace {

struct Req {
    uint64_t id;
    uint32_t graph;
    uint32_t min_rows, min_cols;
    double submit_s;
    uint64_t est;
};

// Bytes of root records the search of g will materialise, an upper
// estimate: sum over R vertices x of ceil(deg(x)/32) words per candidate
// times min(2-hop volume, |R|) candidates, plus the candidate arrays.
uint64_t estimate_bytes(const mbe_graph* g) {
    bool swapped = g->n_rows > g->n_cols;
    uint32_t nR = swapped ? g->n_cols : g->n_rows, nL = swapped ? g->n_rows : g->n_cols;
    std::vector<uint32_t> degL(nL, 0), degR(nR, 0);
    std::vector<uint64_t> vol(nR, 0);
    for (uint32_t r = 0; r < g->n_rows; r++)
        for (uint64_t e = g->row_ptr[r]; e < g->row_ptr[r + 1]; e++) {
            uint32_t c = g->col_idx[e];
            if (!swapped) {
                degR[r]++;
                degL[c]++;
            } else {
                degR[c]++;
                degL[r]++;
            }
        }
    for (uint32_t r = 0; r < g->n_rows; r++)
        for (uint64_t e = g->row_ptr[r]; e < g->row_ptr[r + 1]; e++) {
            uint32_t c = g->col_idx[e];
            uint32_t x = swapped ? c : r, u = swapped ? r : c;
            vol[x] += degL[u];
        }
    uint64_t words = 0;
    for (uint32_t x = 0; x < nR; x++) {
        uint64_t n = std::min<uint64_t>(vol[x], nR);
        words += (uint64_t)((degR[x] + 31) / 32 + 2) * n + 64;
    }
    return words * 4;
}

}  // namespace

struct mbe_server {
    int device = 0;
    mbe_server_config cfg{};
    cudaStream_t upload_stream = nullptr;
    int n_sm = 0;
    std::deque<DeviceGraph> graphs;      // stable addresses
    std::vector<uint64_t> graph_est;
    uint64_t graph_bytes = 0;            // device bytes of the resident graphs
    uint64_t slot_cap = 0;               // device bytes one slot's engine buffers may hold
    std::mutex mu;                       // queue, results, admission, memory figures
    std::condition_variable cv;
    std::deque<Req> queue;
    std::deque<mbe_request_result> done;
    std::vector<uint64_t> slot_bytes;    // device bytes each slot holds (after its last launch)
    std::vector<uint32_t> slot_warm;     // warm-up epoch each slot has completed
    uint32_t warm_epoch = 0;
    uint64_t next_id = 1;
    bool stopping = false;
    std::vector<std::thread> workers;
    std::mutex graph_mu;                 // graph list growth
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    IoCounters io_upload;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    // Sizes a slot's buffers for every resident graph at once (largest
    // side, widest row, all roots in one task ring) without expanding any
    // root (thresholds no root meets), so that requests do not pay for
    // device allocations and the synchronisation they cause.
    void warm(uint32_t slot, EngineBuffers& eb, cudaStream_t stream, IoCounters& io) {
        std::vector<const DeviceGraph*> devs;
        {
            std::lock_guard<std::mutex> glk(graph_mu);
            for (const DeviceGraph& d : graphs) devs.push_back(&d);
        }
        if (!devs.empty()) {
            mbe_opts opts;
            std::memset(&opts, 0, sizeof opts);
            opts.min_rows = opts.min_cols = 0xFFFFFFFFu;
            opts.blocks_per_sm = cfg.blocks_per_sm;
            std::vector<ResultAcc> acc;
            EngineStats stats;
            run_devs(eb, stream, &io, devs, (mbe_variant)cfg.variant, &opts, acc, stats, nullptr, slot_cap);
        }
        std::lock_guard<std::mutex> lk(mu);
        slot_bytes[slot] = eb.bytes();
    }

    void worker(uint32_t slot) {
        cudaSetDevice(device);
        cudaStream_t stream = nullptr;
        cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        EngineBuffers eb;
        IoCounters io;
        // a batch's estimated root-record bytes should fit half the slot's
        // share (the node pool); a request larger than that runs alone
        const uint64_t batch_bytes = slot_cap / 2;
        // Heavy requests (estimated search memory above heavy_bytes) run on
        // slot 0 only, one per launch: the other slots keep serving light
        // requests while a heavy one holds slot 0, so light requests never
        // queue behind heavy ones (with one slot, everything shares it).
        const uint64_t heavy = cfg.heavy_bytes;
        const bool light_only = slot > 0;
        for (;;) {
            std::vector<Req> batch;
            bool do_warm = false;
            uint32_t epoch = 0;
            {
                std::unique_lock<std::mutex> lk(mu);
                for (;;) {
                    if (slot_warm[slot] != warm_epoch) {
                        do_warm = true;
                        epoch = warm_epoch;
                        break;
                    }
                    // the oldest request this slot may take: slot 0 any,
                    // the others light ones only
                    auto first = queue.begin();
                    while (first != queue.end() && light_only && first->est > heavy) ++first;
                    if (first == queue.end()) {
                        if (stopping && queue.empty()) break;
                        cv.wait(lk);
                        continue;
                    }
                    const Req r0 = *first;
                    const bool r0_heavy = r0.est > heavy;
                    uint64_t admitted = 0;
                    // thresholds travel per request, so one launch mixes them
                    for (auto it = first; it != queue.end() && batch.size() < cfg.max_batch;) {
                        bool same = (it->est > heavy) == r0_heavy && (batch.empty() || !r0_heavy);
                        bool fits = batch.empty() || admitted + it->est <= batch_bytes;
                        if (same && fits) {
                            admitted += it->est;
                            batch.push_back(*it);
                            it = queue.erase(it);
                        } else {
                            ++it;
                        }
                    }
                    break;
                }
                if (!do_warm && batch.empty()) break;  // stopping and drained
            }
            if (do_warm) {
                warm(slot, eb, stream, io);
                std::lock_guard<std::mutex> lk(mu);
                slot_warm[slot] = epoch;
                cv.notify_all();
                continue;
            }
            double t_start = now();
            std::vector<const DeviceGraph*> devs;
            {
                std::lock_guard<std::mutex> glk(graph_mu);
                for (const Req& r : batch) devs.push_back(&graphs[r.graph]);
            }
            mbe_opts opts;
            std::memset(&opts, 0, sizeof opts);
            opts.blocks_per_sm = cfg.blocks_per_sm;
            std::vector<uint2> thr;
            for (const Req& r : batch) thr.push_back(make_uint2(r.min_rows, r.min_cols));
            std::vector<ResultAcc> acc;
            EngineStats stats;
            mbe_status st = run_devs(eb, stream, &io, devs, (mbe_variant)cfg.variant, &opts, acc, stats, nullptr,
                                     slot_cap, nullptr, &thr);
            double t_done = now();
            std::lock_guard<std::mutex> lk(mu);
            slot_bytes[slot] = eb.bytes();
            for (size_t i = 0; i < batch.size(); i++) {
                mbe_request_result rr;
                std::memset(&rr, 0, sizeof rr);
                rr.request = batch[i].id;
                rr.graph = batch[i].graph;
                rr.status = (uint32_t)st;
                rr.count = st == MBE_OK ? acc[i].count : 0;
                rr.hash = st == MBE_OK ? acc[i].hash : 0;
                rr.submit_s = batch[i].submit_s;
                rr.start_s = t_start;
                rr.done_s = t_done;
                rr.batch_size = (uint32_t)batch.size();
                rr.slot = slot;
                done.push_back(rr);
            }
            cv.notify_all();
        }
        cudaStreamSynchronize(stream);
        eb.release();
        cudaStreamDestroy(stream);
    }
};

extern "C" mbe_status mbe_server_start(int device, const mbe_server_config* cfg, mbe_server** out) {
    clear_error();
    if (!out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return fail(MBE_ERR_NO_DEVICE, "no such CUDA device");
    }
    auto* s = new (std::nothrow) mbe_server();
    if (!s) return fail(MBE_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->device = device;
    if (cfg) s->cfg = *cfg;
    if (!s->cfg.slots) s->cfg.slots = 2;
    if (!s->cfg.max_batch) s->cfg.max_batch = 256;
    if (!s->cfg.mem_budget) s->cfg.mem_budget = 120ull << 30;
    if (!s->cfg.heavy_bytes) s->cfg.heavy_bytes = 32ull << 20;
    if (!cfg) s->cfg.blocks_per_sm = 3;
    cudaSetDevice(device);
    cudaDeviceGetAttribute(&s->n_sm, cudaDevAttrMultiProcessorCount, device);
    // each slot's share of the budget, and of 85% of the memory free now
    size_t free_b = 0, tot_b = 0;
    cudaMemGetInfo(&free_b, &tot_b);
    s->slot_cap = std::min<uint64_t>(s->cfg.mem_budget, (uint64_t)(free_b * 0.85)) / s->cfg.slots;
    s->slot_bytes.assign(s->cfg.slots, 0);
    s->slot_warm.assign(s->cfg.slots, 0);
    if (cudaStreamCreateWithFlags(&s->upload_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return fail(MBE_ERR_CUDA, "cudaStreamCreate failed");
    }
    for (uint32_t i = 0; i < s->cfg.slots; i++) s->workers.emplace_back([s, i] { s->worker(i); });
    *out = s;
    return MBE_OK;
}

extern "C" mbe_status mbe_server_add_graph(mbe_server* s, const mbe_graph* g, uint32_t* graph_id) {
    clear_error();
    if (!s || !g || !graph_id) return fail(MBE_ERR_INVALID_ARG, "null argument");
    cudaSetDevice(s->device);
    DeviceGraph d;
    mbe_status st = build_device_graph(g, s->upload_stream, s->n_sm, &d, &s->io_upload);
    if (st != MBE_OK) return st;
    uint64_t est = estimate_bytes(g);
    const uint64_t gbytes = 4ull * (d.nR + 1) + 4ull * (d.nL + 1) + 8ull * d.nE + 12ull * d.nR + 8ull * d.nL;
    std::lock_guard<std::mutex> glk(s->graph_mu);
    *graph_id = (uint32_t)s->graphs.size();
    s->graphs.push_back(std::move(d));
    std::lock_guard<std::mutex> lk(s->mu);
    s->graph_est.push_back(est);
    s->graph_bytes += gbytes;
    return MBE_OK;
}

extern "C" mbe_status mbe_server_warmup(mbe_server* s) {
    clear_error();
    if (!s) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stopping) return fail(MBE_ERR_BUSY, "server is stopping");
    const uint32_t epoch = ++s->warm_epoch;
    s->cv.notify_all();
    s->cv.wait(lk, [&] {
        for (uint32_t w : s->slot_warm)
            if (w != epoch) return false;
        return true;
    });
    return MBE_OK;
}

extern "C" mbe_status mbe_server_memory(mbe_server* s, uint64_t* search_bytes, uint64_t* graph_bytes,
                                        uint64_t* slot_cap) {
    clear_error();
    if (!s) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    uint64_t t = 0;
    for (uint64_t b : s->slot_bytes) t += b;
    if (search_bytes) *search_bytes = t;
    if (graph_bytes) *graph_bytes = s->graph_bytes;
    if (slot_cap) *slot_cap = s->slot_cap;
    return MBE_OK;
}

extern "C" mbe_status mbe_server_estimate(mbe_server* s, uint32_t graph_id, uint64_t* bytes) {
    clear_error();
    if (!s || !bytes) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (graph_id >= s->graph_est.size()) return fail(MBE_ERR_INVALID_ARG, "unknown graph id");
    *bytes = s->graph_est[graph_id];
    return MBE_OK;
}

extern "C" mbe_status mbe_server_submit(mbe_server* s, uint32_t graph_id, uint32_t min_rows, uint32_t min_cols,
                                        uint64_t* request_id) {
    clear_error();
    if (!s) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return fail(MBE_ERR_BUSY, "server is stopping");
    if (graph_id >= s->graph_est.size()) return fail(MBE_ERR_INVALID_ARG, "unknown graph id");
    Req r{s->next_id++, graph_id, min_rows, min_cols, s->now(), s->graph_est[graph_id]};
    s->queue.push_back(r);
    if (request_id) *request_id = r.id;
    s->cv.notify_one();
    return MBE_OK;
}

extern "C" mbe_status mbe_server_poll(mbe_server* s, mbe_request_result* out, uint32_t cap, uint32_t* n_out) {
    clear_error();
    if (!s || (!out && cap) || !n_out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    uint32_t n = 0;
    while (n < cap && !s->done.empty()) {
        out[n++] = s->done.front();
        s->done.pop_front();
    }
    *n_out = n;
    return MBE_OK;
}

extern "C" double mbe_server_clock(mbe_server* s) { return s ? s->now() : 0.0; }

extern "C" mbe_status mbe_server_stop(mbe_server* s) {
    clear_error();
    if (!s) return MBE_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        s->cv.notify_all();
    }
    for (auto& t : s->workers) t.join();
    cudaSetDevice(s->device);
    for (auto& d : s->graphs) d.release();
    cudaStreamDestroy(s->upload_stream);
    delete s;
    return MBE_OK;
}
