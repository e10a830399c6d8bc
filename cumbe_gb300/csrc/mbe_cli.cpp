// `mbe <graph.bi> [cuMBE|noRS|noES|noWS]` - drop-in for the reference's
// command (src/main.cu:9-234).  Same arguments, same stdout lines and the
// same result/<dataset>_<algo> file (written when ./result exists, as the
// reference's ofstream silently does nothing otherwise); three lines are
// added after the reference's: the canonical hash, bicliques/sec and the
// device time split.  Exit status is non-zero on any error (the reference
// ignores errors and prints a count of 0, src/main.cu:185-207).
//
// The graph may also be a binary graph image (mbe_graph_write_bin),
// recognised by its magic.
//
// `--emit FILE` (no reference counterpart; the reference only counts) also
// writes every maximal biclique to FILE, one per line: its rows, " | ",
// its cols, each side in ascending file ids.  stdout is unchanged.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "mbe.h"

static int die(const char* what, mbe_status st) {
    std::fprintf(stderr, "mbe: %s failed (status %d): %s\n", what, (int)st, mbe_last_error());
    return 1;
}

// Runs the enumeration again with the output stream on (buffers sized from
// the count, the id buffer grown until it fits) and writes FILE.
static int write_bicliques(mbe_ctx* ctx, const mbe_graph* g, mbe_variant var, uint64_t count, const char* path) {
    std::vector<uint32_t> offs(count + 1), nrows(std::max<uint64_t>(count, 1));
    uint64_t cap_ids = std::max<uint64_t>(1024, 16 * count);
    std::vector<uint32_t> ids;
    mbe_result res;
    for (;;) {
        ids.assign(cap_ids, 0);
        mbe_opts o;
        std::memset(&o, 0, sizeof o);
        o.flags = MBE_OPT_EMIT;
        o.emit_offsets = offs.data();
        o.emit_nrows = nrows.data();
        o.emit_ids = ids.data();
        o.emit_cap_bicliques = std::max<uint64_t>(count, 1);
        o.emit_cap_ids = cap_ids;
        mbe_status st = mbe_enumerate(ctx, g, var, &o, &res);
        if (st == MBE_OK) break;
        if (st != MBE_ERR_CAPACITY || cap_ids >= 0xFFFFFFFFull) return die("emitting the bicliques", st);
        cap_ids = std::min<uint64_t>(0xFFFFFFFFull, 2 * cap_ids);
    }
    FILE* f = std::fopen(path, "w");
    if (!f) {
        std::fprintf(stderr, "mbe: cannot write %s\n", path);
        return 1;
    }
    std::vector<uint32_t> side;
    for (uint64_t k = 0; k < res.emitted; k++) {
        const uint32_t* p = ids.data() + offs[k];
        const uint32_t nr = nrows[k], nc = offs[k + 1] - offs[k] - nr;
        for (int s = 0; s < 2; s++) {
            side.assign(p + (s ? nr : 0), p + (s ? nr + nc : nr));
            std::sort(side.begin(), side.end());
            for (size_t i = 0; i < side.size(); i++) std::fprintf(f, i ? " %u" : "%u", side[i]);
            std::fputs(s ? "\n" : " | ", f);
        }
    }
    std::fclose(f);
    std::fprintf(stderr, "mbe: %llu bicliques written to %s\n", (unsigned long long)res.emitted, path);
    return 0;
}

int main(int argc, char** argv) {
    const char* emit_path = nullptr;
    std::vector<const char*> pos;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--emit") && i + 1 < argc)
            emit_path = argv[++i];
        else
            pos.push_back(argv[i]);
    }
    if (pos.empty()) {
        std::fprintf(stderr, "usage: %s <graph.bi> [cuMBE|noRS|noES|noWS] [--emit FILE]\n", argv[0]);
        return 2;
    }
    std::time_t now = std::time(nullptr);
    std::string dataset = pos[0];
    size_t slash = dataset.rfind('/');
    if (slash != std::string::npos) dataset = dataset.substr(slash + 1);
    mbe_variant var = mbe_variant_from_name(pos.size() > 1 ? pos[1] : "cuMBE");
    std::string algo = mbe_variant_name(var);
    std::string stem = dataset.substr(0, dataset.rfind('.'));

    mbe_graph* g = nullptr;
    // a binary graph image (mbe_graph_write_bin) is taken in place of the text
    bool image = false;
    if (FILE* f = std::fopen(pos[0], "rb")) {
        char magic[8] = {0};
        image = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "MBEGRAPH", 8) == 0;
        std::fclose(f);
    }
    mbe_status st = image ? mbe_graph_load_bin(pos[0], &g) : mbe_graph_load_bi(pos[0], &g);
    if (st != MBE_OK) return die("loading the graph", st);
    mbe_graph_info info;
    mbe_graph_info_get(g, &info);
    uint32_t nR = info.swapped ? info.n_cols : info.n_rows;
    uint32_t nL = info.swapped ? info.n_rows : info.n_cols;

    mbe_ctx* ctx = nullptr;
    if ((st = mbe_ctx_create(0, &ctx)) != MBE_OK) return die("creating the device context", st);
    if ((st = mbe_graph_upload(ctx, g)) != MBE_OK) return die("uploading the graph", st);
    mbe_opts opts;
    std::memset(&opts, 0, sizeof opts);
    opts.flags = MBE_OPT_TIMING;
    mbe_result res;
    if ((st = mbe_enumerate(ctx, g, var, &opts, &res)) != MBE_OK) return die("enumerating", st);
    uint32_t grid_a = 0, grid_b = 0, block = 0;
    mbe_ctx_last_grid(ctx, &grid_a, &grid_b, &block);

    char head[512];
    std::snprintf(head, sizeof head,
                  "date/time: %salgorithm: %s\ndataset: %s\n|R|: %u, |L|: %u, |E|: %llu\n"
                  "grid_size: %u, block_size: %u\n",
                  std::ctime(&now), algo.c_str(), dataset.c_str(), nR, nL, (unsigned long long)info.n_edges, grid_b,
                  block);
    double secs = res.ms / 1000.0;
    char tail[512];
    std::snprintf(tail, sizeof tail, "maximal bicliques: %llu\nruntime (s): %g\n", (unsigned long long)res.count,
                  secs);
    char extra[512];
    std::snprintf(extra, sizeof extra, "hash: 0x%016llx\nbicliques/sec: %.6g\ndevice ms (expand, total): %.3f, %.3f\n",
                  (unsigned long long)res.hash, secs > 0 ? (double)res.count / secs : 0.0, res.ms_prep, res.ms);
    std::fputs(head, stdout);
    std::fputs(tail, stdout);
    std::fputs(extra, stdout);
    std::string path = "result/" + stem + "_" + algo;
    if (FILE* f = std::fopen(path.c_str(), "w")) {
        std::fputs(head, f);
        std::fputs(tail, f);
        std::fclose(f);
    }
    int rc = emit_path ? write_bicliques(ctx, g, var, res.count, emit_path) : 0;
    mbe_ctx_destroy(ctx);
    mbe_graph_free(g);
    return rc;
}
