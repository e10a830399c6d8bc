// `mbe <graph.bi> [cuMBE|noRS|noES|noWS]` - drop-in for the reference's
// command (src/main.cu:9-234).  Same arguments, same stdout lines and the
// same result/<dataset>_<algo> file (written when ./result exists, as the
// reference's ofstream silently does nothing otherwise); three lines are
// added after the reference's: the canonical hash, bicliques/sec and the
// device time split.  Exit status is non-zero on any error (the reference
// ignores errors and prints a count of 0, src/main.cu:185-207).
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>

#include "mbe.h"

static int die(const char* what, mbe_status st) {
    std::fprintf(stderr, "mbe: %s failed (status %d): %s\n", what, (int)st, mbe_last_error());
    return 1;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <graph.bi> [cuMBE|noRS|noES|noWS]\n", argv[0]);
        return 2;
    }
    std::time_t now = std::time(nullptr);
    std::string dataset = argv[1];
    size_t slash = dataset.rfind('/');
    if (slash != std::string::npos) dataset = dataset.substr(slash + 1);
    mbe_variant var = mbe_variant_from_name(argc > 2 ? argv[2] : "cuMBE");
    std::string algo = mbe_variant_name(var);
    std::string stem = dataset.substr(0, dataset.rfind('.'));

    mbe_graph* g = nullptr;
    mbe_status st = mbe_graph_load_bi(argv[1], &g);
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
    mbe_ctx_destroy(ctx);
    mbe_graph_free(g);
    return 0;
}
