// Host-side graph handling of libmbe: `.bi` reader and writer, CSR ingest,
// the binary graph image and cache, and the synthetic bipartite generator.
// No CUDA calls here, so every function works on a machine without a GPU.
// Large inputs are parsed and normalised on all host threads.
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "mbe_hash.h"
#include "mbe_internal.h"

namespace mbe {

static thread_local std::string g_last_error;

mbe_status fail(mbe_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

void clear_error() { g_last_error.clear(); }

uint64_t next_graph_uid() {
    static std::atomic<uint64_t> ctr{1};
    return ctr.fetch_add(1);
}

namespace {

// Host threads for a job over `work` items (1 below `min_work`).
unsigned worker_count(uint64_t work, uint64_t min_work) {
    if (work < min_work) return 1;
    unsigned hw = std::thread::hardware_concurrency();
    return std::max(1u, std::min(hw ? hw : 1u, 32u));
}

// Runs f(t) for t in [0, n) on n threads (the calling thread takes t = 0).
template <class F>
void run_threads(unsigned n, F f) {
    std::vector<std::thread> th;
    for (unsigned t = 1; t < n; t++) th.emplace_back(f, t);
    f(0u);
    for (auto& x : th) x.join();
}

// Row ranges [cut[t], cut[t+1]) holding about equal numbers of edges.
std::vector<uint32_t> row_cuts(const std::vector<uint64_t>& row_ptr, uint32_t n_rows, unsigned T) {
    std::vector<uint32_t> cut(T + 1, n_rows);
    cut[0] = 0;
    const uint64_t E = row_ptr[n_rows];
    for (unsigned t = 1; t < T; t++) {
        const uint64_t target = E * t / T;
        cut[t] = (uint32_t)(std::lower_bound(row_ptr.begin(), row_ptr.begin() + n_rows + 1, target) - row_ptr.begin());
        cut[t] = std::max(cut[t], cut[t - 1]);
    }
    return cut;
}

}  // namespace

// Sorts and dedupes every row, checks column ids, fills the degree maxima.
// Rows are processed on all host threads for large graphs; the first row
// (in row order) holding a bad id is the one reported.
mbe_status normalise(mbe_graph* g) {
    const uint32_t nr = g->n_rows, nc = g->n_cols;
    const unsigned T = worker_count(g->col_idx.size(), 1u << 20);
    const std::vector<uint32_t> cut = row_cuts(g->row_ptr, nr, T);
    std::vector<uint64_t> newlen((size_t)nr + 1, 0);
    std::vector<uint32_t> bad_row(T, UINT32_MAX);
    run_threads(T, [&](unsigned t) {
        for (uint32_t r = cut[t]; r < cut[t + 1]; r++) {
            auto first = g->col_idx.begin() + (ptrdiff_t)g->row_ptr[r];
            auto last = g->col_idx.begin() + (ptrdiff_t)g->row_ptr[r + 1];
            for (auto it = first; it != last; ++it)
                if (*it >= nc) {
                    bad_row[t] = r;
                    return;
                }
            std::sort(first, last);
            newlen[r] = (uint64_t)(std::unique(first, last) - first);
        }
    });
    for (unsigned t = 0; t < T; t++)
        if (bad_row[t] != UINT32_MAX) {
            const uint32_t r = bad_row[t];
            uint32_t c = 0;
            for (uint64_t i = g->row_ptr[r]; i < g->row_ptr[r + 1]; i++)
                if (g->col_idx[i] >= nc) {
                    c = g->col_idx[i];
                    break;
                }
            return fail(MBE_ERR_FORMAT, "column id " + std::to_string(c) + " out of range in row " + std::to_string(r));
        }
    // new offsets (serial prefix over rows), then compaction and column
    // degrees per thread
    std::vector<uint64_t> np((size_t)nr + 1, 0);
    uint64_t w = 0, dup = 0;
    uint32_t maxr = 0;
    for (uint32_t r = 0; r < nr; r++) {
        np[r] = w;
        w += newlen[r];
        dup += (g->row_ptr[r + 1] - g->row_ptr[r]) - newlen[r];
        maxr = std::max<uint32_t>(maxr, (uint32_t)newlen[r]);
    }
    np[nr] = w;
    std::vector<uint32_t> out(w);
    std::vector<std::vector<uint32_t>> deg(T);
    run_threads(T, [&](unsigned t) {
        deg[t].assign(nc, 0);
        for (uint32_t r = cut[t]; r < cut[t + 1]; r++) {
            const uint32_t* src = g->col_idx.data() + g->row_ptr[r];
            if (newlen[r]) std::memcpy(out.data() + np[r], src, sizeof(uint32_t) * newlen[r]);
            for (uint64_t i = 0; i < newlen[r]; i++) deg[t][src[i]]++;
        }
    });
    uint32_t maxc = 0;
    for (uint32_t c = 0; c < nc; c++) {
        uint32_t d = 0;
        for (unsigned t = 0; t < T; t++) d += deg[t][c];
        maxc = std::max(maxc, d);
    }
    g->row_ptr.swap(np);
    g->col_idx.swap(out);
    g->n_dup = (uint32_t)std::min<uint64_t>(dup, UINT32_MAX);
    g->max_row_deg = maxr;
    g->max_col_deg = maxc;
    return MBE_OK;
}

// ---------------------------------------------------------------------------
// `.bi` text parsing

namespace {

struct Scanner {
    const char* p;
    const char* end;
    // Reads one decimal integer (optional sign); false at EOF or on junk.
    bool next(long long* out) {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) p++;
        if (p >= end) return false;
        bool neg = false;
        if (*p == '-' || *p == '+') {
            neg = (*p == '-');
            p++;
        }
        if (p >= end || *p < '0' || *p > '9') return false;
        long long v = 0;
        while (p < end && *p >= '0' && *p <= '9') {
            v = v * 10 + (*p - '0');
            if (v > (1LL << 40)) return false;
            p++;
        }
        *out = neg ? -v : v;
        return true;
    }
};

inline bool is_ws(char c) { return c == ' ' || c == '\n' || c == '\r' || c == '\t'; }

// One whitespace-delimited token [b, e) read like Scanner::next: optional
// sign, decimal digits, at most 2^40.
inline bool parse_token(const char* b, const char* e, long long* out) {
    bool neg = false;
    if (b < e && (*b == '-' || *b == '+')) {
        neg = *b == '-';
        b++;
    }
    if (b >= e) return false;
    long long v = 0;
    for (; b < e; b++) {
        if (*b < '0' || *b > '9') return false;
        v = v * 10 + (*b - '0');
        if (v > (1LL << 40)) return false;
    }
    *out = neg ? -v : v;
    return true;
}

// Parses a `.bi` image (src/main.cu:38-48 reads the same layout: header
// "R L E", R lines "start len", E lines "neighbour ignored") into a
// normalised graph.  After the header, the text is cut at whitespace into
// one chunk per host thread; a first pass counts each chunk's tokens, a
// second parses every token straight into its slot (row table or edge
// list).  Errors name the same row / edge as a sequential read would.
mbe_status parse_bi(const char* data, size_t size, mbe_graph** out) {
    Scanner sc{data, data + size};
    long long nr, nl, ne;
    if (!sc.next(&nr) || !sc.next(&nl) || !sc.next(&ne)) return fail(MBE_ERR_FORMAT, "missing header 'R L E'");
    if (nr < 0 || nl < 0 || ne < 0 || nr > 0xFFFFFFFFLL || nl > 0xFFFFFFFFLL)
        return fail(MBE_ERR_FORMAT, "bad header values");
    const char* p0 = sc.p;
    const char* end = data + size;
    const uint64_t want = 2ull * (uint64_t)nr + 2ull * (uint64_t)ne;  // tokens after the header
    const unsigned T = worker_count((uint64_t)(end - p0), 8u << 20);
    std::vector<const char*> cut(T + 1);
    cut[0] = p0;
    cut[T] = end;
    for (unsigned k = 1; k < T; k++) {
        const char* c = p0 + (size_t)(end - p0) * k / T;
        while (c < end && !is_ws(*c)) c++;
        cut[k] = std::max(c, cut[k - 1]);
    }
    // pass 1: tokens per chunk (a chunk starts at whitespace, or right after the header)
    std::vector<uint64_t> first(T + 1, 0);
    run_threads(T, [&](unsigned t) {
        uint64_t n = 0;
        bool in = false;
        for (const char* c = cut[t]; c < cut[t + 1]; c++) {
            const bool w = is_ws(*c);
            n += (!w && !in);
            in = !w;
        }
        first[t + 1] = n;
    });
    for (unsigned t = 0; t < T; t++) first[t + 1] += first[t];
    const uint64_t total = first[T];
    std::vector<long long> start((size_t)nr), len((size_t)nr);
    std::vector<uint32_t> edges((size_t)ne);
    std::vector<uint64_t> bad_tok(T, UINT64_MAX), bad_nbr(T, UINT64_MAX);
    // pass 2: every token into its slot
    run_threads(T, [&](unsigned t) {
        uint64_t idx = first[t];
        const char* c = cut[t];
        const char* ce = cut[t + 1];
        while (c < ce && idx < want) {
            while (c < ce && is_ws(*c)) c++;
            if (c >= ce) break;
            const char* b = c;
            while (c < ce && !is_ws(*c)) c++;
            long long v;
            if (!parse_token(b, c, &v)) {
                bad_tok[t] = idx;
                return;
            }
            if (idx < 2ull * (uint64_t)nr) {
                (idx & 1 ? len : start)[(size_t)(idx >> 1)] = v;
            } else {
                const uint64_t u = idx - 2ull * (uint64_t)nr;
                if (!(u & 1)) {
                    if (v < 0 || v >= nl) {
                        if (bad_nbr[t] == UINT64_MAX) bad_nbr[t] = u >> 1;
                    } else {
                        edges[(size_t)(u >> 1)] = (uint32_t)v;
                    }
                }
            }
            idx++;
        }
    });
    uint64_t tok_err = total < want ? total : UINT64_MAX, nbr_err = UINT64_MAX;
    for (unsigned t = 0; t < T; t++) {
        tok_err = std::min(tok_err, bad_tok[t]);
        nbr_err = std::min(nbr_err, bad_nbr[t]);
    }
    // the row table, in the order a sequential read reports problems
    const uint64_t rows_ok = tok_err < 2ull * (uint64_t)nr ? tok_err / 2 : (uint64_t)nr;
    for (uint64_t i = 0; i < rows_ok; i++)
        if (start[i] < 0 || len[i] < 0 || start[i] + len[i] > ne)
            return fail(MBE_ERR_FORMAT, "row " + std::to_string(i) + " range outside edge list");
    if (tok_err < 2ull * (uint64_t)nr)
        return fail(MBE_ERR_FORMAT, "truncated row table at row " + std::to_string(tok_err / 2));
    const uint64_t edge_tok_err = tok_err == UINT64_MAX ? UINT64_MAX : (tok_err - 2ull * (uint64_t)nr) / 2;
    if (edge_tok_err != UINT64_MAX && edge_tok_err <= nbr_err)
        return fail(MBE_ERR_FORMAT, "truncated edge list at edge " + std::to_string(edge_tok_err));
    if (nbr_err != UINT64_MAX)
        return fail(MBE_ERR_FORMAT, "neighbour id out of range at edge " + std::to_string(nbr_err));
    auto* g = new (std::nothrow) mbe_graph();
    if (!g) return fail(MBE_ERR_OUT_OF_MEMORY, "host allocation failed");
    g->n_rows = (uint32_t)nr;
    g->n_cols = (uint32_t)nl;
    g->row_ptr.assign((size_t)nr + 1, 0);
    uint64_t tot = 0;
    for (long long i = 0; i < nr; i++) {
        g->row_ptr[(size_t)i] = tot;
        tot += (uint64_t)len[(size_t)i];
    }
    g->row_ptr[(size_t)nr] = tot;
    g->col_idx.resize(tot);
    const std::vector<uint32_t> rc = row_cuts(g->row_ptr, (uint32_t)nr, worker_count(tot, 1u << 20));
    run_threads((unsigned)rc.size() - 1, [&](unsigned t) {
        for (uint32_t i = rc[t]; i < rc[t + 1]; i++)
            if (len[i])
                std::memcpy(g->col_idx.data() + g->row_ptr[i], edges.data() + start[i], sizeof(uint32_t) * (size_t)len[i]);
    });
    mbe_status st = normalise(g);
    if (st != MBE_OK) {
        delete g;
        return st;
    }
    g->uid = next_graph_uid();
    *out = g;
    return MBE_OK;
}

mbe_status read_file(const char* path, std::vector<char>& buf) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(MBE_ERR_IO, std::string("cannot open ") + path);
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 0) {
        std::fclose(f);
        return fail(MBE_ERR_IO, "cannot size file");
    }
    buf.resize((size_t)sz);
    size_t got = sz ? std::fread(buf.data(), 1, (size_t)sz, f) : 0;
    std::fclose(f);
    if (got != (size_t)sz) return fail(MBE_ERR_IO, "short read");
    return MBE_OK;
}

// Binary graph image: this header, then row_ptr (u64 x (n_rows + 1)), then
// col_idx (u32 x n_edges), little-endian, rows already normalised.
struct BinHeader {
    char magic[8];
    uint32_t n_rows, n_cols;
    uint64_t n_edges;
    uint32_t max_row_deg, max_col_deg, n_dup, version;
    uint64_t checksum;
};
static_assert(sizeof(BinHeader) == 48, "binary header size");
constexpr char kBinMagic[8] = {'M', 'B', 'E', 'G', 'R', 'A', 'P', 'H'};
constexpr uint32_t kBinVersion = 1;

// Order-independent checksum of the two arrays (wrapping sum of mixed
// (position, value) pairs), computed on all host threads.
uint64_t image_checksum(const std::vector<uint64_t>& rp, const std::vector<uint32_t>& ci) {
    const unsigned T = worker_count(rp.size() + ci.size(), 1u << 20);
    std::vector<uint64_t> part(T, 0);
    run_threads(T, [&](unsigned t) {
        uint64_t h = 0;
        for (size_t i = rp.size() * t / T; i < rp.size() * (t + 1) / T; i++)
            h += mbe_fmix64(rp[i] ^ (0x9E3779B97F4A7C15ull * (i + 1)));
        for (size_t i = ci.size() * t / T; i < ci.size() * (t + 1) / T; i++)
            h += mbe_fmix64(((uint64_t)ci[i] << 1) ^ (0xD1B54A32D192ED03ull * (i + 1)));
        part[t] = h;
    });
    uint64_t h = 0;
    for (uint64_t x : part) h += x;
    return h;
}

}  // namespace
}  // namespace mbe

using namespace mbe;

extern "C" mbe_status mbe_graph_load_bi(const char* path, mbe_graph** out) {
    clear_error();
    if (!path || !out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    std::vector<char> buf;
    mbe_status st = read_file(path, buf);
    if (st != MBE_OK) return st;
    return parse_bi(buf.data(), buf.size(), out);
}

extern "C" mbe_status mbe_graph_write_bin(const mbe_graph* g, const char* path) {
    clear_error();
    if (!g || !path) return fail(MBE_ERR_INVALID_ARG, "null argument");
    BinHeader h;
    std::memcpy(h.magic, kBinMagic, 8);
    h.n_rows = g->n_rows;
    h.n_cols = g->n_cols;
    h.n_edges = g->col_idx.size();
    h.max_row_deg = g->max_row_deg;
    h.max_col_deg = g->max_col_deg;
    h.n_dup = g->n_dup;
    h.version = kBinVersion;
    h.checksum = image_checksum(g->row_ptr, g->col_idx);
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return fail(MBE_ERR_IO, std::string("cannot open ") + tmp);
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 &&
              std::fwrite(g->row_ptr.data(), sizeof(uint64_t), g->row_ptr.size(), f) == g->row_ptr.size() &&
              (g->col_idx.empty() ||
               std::fwrite(g->col_idx.data(), sizeof(uint32_t), g->col_idx.size(), f) == g->col_idx.size());
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return fail(MBE_ERR_IO, std::string("cannot write ") + path);
    }
    return MBE_OK;
}

extern "C" mbe_status mbe_graph_load_bin(const char* path, mbe_graph** out) {
    clear_error();
    if (!path || !out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    std::vector<char> buf;
    mbe_status st = read_file(path, buf);
    if (st != MBE_OK) return st;
    BinHeader h;
    if (buf.size() < sizeof h) return fail(MBE_ERR_FORMAT, "not a binary graph image (too short)");
    std::memcpy(&h, buf.data(), sizeof h);
    if (std::memcmp(h.magic, kBinMagic, 8) != 0) return fail(MBE_ERR_FORMAT, "not a binary graph image");
    if (h.version != kBinVersion) return fail(MBE_ERR_FORMAT, "unsupported binary graph version");
    const uint64_t need = sizeof h + 8ull * ((uint64_t)h.n_rows + 1) + 4ull * h.n_edges;
    if (buf.size() != need) return fail(MBE_ERR_FORMAT, "binary graph image has the wrong size");
    auto* g = new (std::nothrow) mbe_graph();
    if (!g) return fail(MBE_ERR_OUT_OF_MEMORY, "host allocation failed");
    g->n_rows = h.n_rows;
    g->n_cols = h.n_cols;
    g->row_ptr.resize((size_t)h.n_rows + 1);
    g->col_idx.resize((size_t)h.n_edges);
    std::memcpy(g->row_ptr.data(), buf.data() + sizeof h, 8 * g->row_ptr.size());
    if (h.n_edges) std::memcpy(g->col_idx.data(), buf.data() + sizeof h + 8 * g->row_ptr.size(), 4 * g->col_idx.size());
    // checksum, then the CSR invariants the kernels rely on
    bool ok = image_checksum(g->row_ptr, g->col_idx) == h.checksum && g->row_ptr[0] == 0 &&
              g->row_ptr[h.n_rows] == h.n_edges;
    for (uint32_t r = 0; ok && r < h.n_rows; r++) ok = g->row_ptr[r] <= g->row_ptr[r + 1];
    if (ok) {
        const unsigned T = worker_count(h.n_edges, 1u << 20);
        const std::vector<uint32_t> cut = row_cuts(g->row_ptr, h.n_rows, T);
        std::vector<char> good(T, 1);
        run_threads(T, [&](unsigned t) {
            for (uint32_t r = cut[t]; r < cut[t + 1] && good[t]; r++)
                for (uint64_t i = g->row_ptr[r]; i < g->row_ptr[r + 1]; i++)
                    if (g->col_idx[i] >= h.n_cols || (i > g->row_ptr[r] && g->col_idx[i] <= g->col_idx[i - 1])) {
                        good[t] = 0;
                        break;
                    }
        });
        for (char c : good) ok = ok && c;
    }
    if (!ok) {
        delete g;
        return fail(MBE_ERR_FORMAT, "binary graph image is corrupt");
    }
    g->max_row_deg = h.max_row_deg;
    g->max_col_deg = h.max_col_deg;
    g->n_dup = h.n_dup;
    g->uid = next_graph_uid();
    *out = g;
    return MBE_OK;
}

extern "C" mbe_status mbe_graph_load_cached(const char* bi_path, const char* cache_path, mbe_graph** out) {
    clear_error();
    if (!bi_path || !cache_path || !out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    struct stat sb, sc;
    if (stat(bi_path, &sb) != 0) return fail(MBE_ERR_IO, std::string("cannot open ") + bi_path);
    if (stat(cache_path, &sc) == 0 && sc.st_mtime >= sb.st_mtime && mbe_graph_load_bin(cache_path, out) == MBE_OK)
        return MBE_OK;
    mbe_status st = mbe_graph_load_bi(bi_path, out);
    if (st != MBE_OK) return st;
    mbe_graph_write_bin(*out, cache_path);  // best effort: the graph is loaded either way
    clear_error();
    return MBE_OK;
}

// KONECT edge-pair text -> bipartite graph, as data/gen_bi.cpp builds it:
// skip `skip_words` leading tokens, then read "source target" pairs each
// followed by `skip_per_edge` ignored tokens until the text ends or a pair
// does not parse as integers; rows are sources and cols targets, each
// numbered by first appearance; repeated pairs count once.
extern "C" mbe_status mbe_graph_load_konect(const char* path, uint32_t skip_words, uint32_t skip_per_edge,
                                            mbe_graph** out) {
    clear_error();
    if (!path || !out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    std::vector<char> buf;
    mbe_status st = read_file(path, buf);
    if (st != MBE_OK) return st;
    const char* c = buf.data();
    const char* end = c + buf.size();
    auto token = [&](const char** b, const char** e) -> bool {
        while (c < end && is_ws(*c)) c++;
        if (c >= end) return false;
        *b = c;
        while (c < end && !is_ws(*c)) c++;
        *e = c;
        return true;
    };
    // an int32 like `istream >> int`: optional sign, digits, no overflow
    auto as_int = [](const char* b, const char* e, int* v) -> bool {
        long long x;
        if (!parse_token(b, e, &x) || x < INT32_MIN || x > INT32_MAX) return false;
        *v = (int)x;
        return true;
    };
    const char *b, *e;
    for (uint32_t i = 0; i < skip_words; i++)
        if (!token(&b, &e)) break;
    std::unordered_map<int, uint32_t> rid, cid;
    std::vector<std::pair<uint32_t, uint32_t>> pairs;
    for (;;) {
        int r, l;
        if (!token(&b, &e) || !as_int(b, e, &r)) break;
        if (!token(&b, &e) || !as_int(b, e, &l)) break;
        for (uint32_t i = 0; i < skip_per_edge; i++)
            if (!token(&b, &e)) break;
        auto ir = rid.emplace(r, (uint32_t)rid.size()).first->second;
        auto il = cid.emplace(l, (uint32_t)cid.size()).first->second;
        pairs.emplace_back(ir, il);
    }
    auto* g = new (std::nothrow) mbe_graph();
    if (!g) return fail(MBE_ERR_OUT_OF_MEMORY, "host allocation failed");
    g->n_rows = (uint32_t)rid.size();
    g->n_cols = (uint32_t)cid.size();
    g->row_ptr.assign((size_t)g->n_rows + 1, 0);
    for (auto& pr : pairs) g->row_ptr[pr.first + 1]++;
    for (uint32_t r = 0; r < g->n_rows; r++) g->row_ptr[r + 1] += g->row_ptr[r];
    g->col_idx.resize(pairs.size());
    std::vector<uint64_t> fill(g->row_ptr.begin(), g->row_ptr.end() - 1);
    for (auto& pr : pairs) g->col_idx[fill[pr.first]++] = pr.second;
    st = normalise(g);
    if (st != MBE_OK) {
        delete g;
        return st;
    }
    g->uid = next_graph_uid();
    *out = g;
    return MBE_OK;
}

extern "C" mbe_status mbe_graph_from_csr(uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr,
                                         const uint32_t* col_idx, mbe_graph** out) {
    clear_error();
    if (!out || (!row_ptr && n_rows)) return fail(MBE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (n_rows && row_ptr[0] != 0) return fail(MBE_ERR_FORMAT, "row_ptr[0] must be 0");
    for (uint32_t r = 0; r < n_rows; r++)
        if (row_ptr[r + 1] < row_ptr[r]) return fail(MBE_ERR_FORMAT, "row_ptr not monotone");
    uint64_t ne = n_rows ? row_ptr[n_rows] : 0;
    if (ne && !col_idx) return fail(MBE_ERR_INVALID_ARG, "null col_idx");
    auto* g = new (std::nothrow) mbe_graph();
    if (!g) return fail(MBE_ERR_OUT_OF_MEMORY, "host allocation failed");
    g->n_rows = n_rows;
    g->n_cols = n_cols;
    g->row_ptr.assign(row_ptr, row_ptr + n_rows + 1);
    if (!n_rows) g->row_ptr.assign(1, 0);
    g->col_idx.assign(col_idx, col_idx + ne);
    mbe_status st = normalise(g);
    if (st != MBE_OK) {
        delete g;
        return st;
    }
    g->uid = next_graph_uid();
    *out = g;
    return MBE_OK;
}

extern "C" mbe_status mbe_graph_write_bi(const mbe_graph* g, const char* path) {
    clear_error();
    if (!g || !path) return fail(MBE_ERR_INVALID_ARG, "null argument");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(MBE_ERR_IO, std::string("cannot open ") + path);
    std::string s;
    s.reserve(1 << 20);
    char tmp[64];
    auto flush = [&]() {
        if (!s.empty()) std::fwrite(s.data(), 1, s.size(), f);
        s.clear();
    };
    std::snprintf(tmp, sizeof tmp, "%u %u %llu\n\n", g->n_rows, g->n_cols, (unsigned long long)g->col_idx.size());
    s += tmp;
    for (uint32_t r = 0; r < g->n_rows; r++) {
        std::snprintf(tmp, sizeof tmp, "%llu %llu\n", (unsigned long long)g->row_ptr[r],
                      (unsigned long long)(g->row_ptr[r + 1] - g->row_ptr[r]));
        s += tmp;
        if (s.size() > (1u << 20)) flush();
    }
    for (uint32_t c : g->col_idx) {
        std::snprintf(tmp, sizeof tmp, "\n%u 1", c);
        s += tmp;
        if (s.size() > (1u << 20)) flush();
    }
    flush();
    bool ok = std::fclose(f) == 0;
    return ok ? MBE_OK : fail(MBE_ERR_IO, "write failed");
}

extern "C" mbe_status mbe_graph_info_get(const mbe_graph* g, mbe_graph_info* out) {
    clear_error();
    if (!g || !out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    out->n_rows = g->n_rows;
    out->n_cols = g->n_cols;
    out->n_edges = g->col_idx.size();
    out->max_row_deg = g->max_row_deg;
    out->max_col_deg = g->max_col_deg;
    out->n_dup_dropped = g->n_dup;
    out->swapped = g->n_rows > g->n_cols ? 1u : 0u;
    return MBE_OK;
}

extern "C" mbe_status mbe_graph_copy_csr(const mbe_graph* g, uint64_t* row_ptr, uint32_t* col_idx) {
    clear_error();
    if (!g || !row_ptr || (!col_idx && !g->col_idx.empty())) return fail(MBE_ERR_INVALID_ARG, "null argument");
    std::memcpy(row_ptr, g->row_ptr.data(), sizeof(uint64_t) * (g->n_rows + 1));
    if (!g->col_idx.empty()) std::memcpy(col_idx, g->col_idx.data(), sizeof(uint32_t) * g->col_idx.size());
    return MBE_OK;
}

extern "C" void mbe_graph_free(mbe_graph* g) { delete g; }

extern "C" const char* mbe_last_error(void) { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// Synthetic generator

namespace {

struct SplitMix {
    uint64_t s;
    uint64_t next() {
        s += 0x9E3779B97F4A7C15ULL;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    uint32_t below(uint32_t n) { return (uint32_t)(((unsigned __int128)next() * n) >> 64); }
};

// Power-law weights with a cap on the expected degree, as a CDF.
struct Side {
    uint32_t n;
    bool uniform;
    std::vector<double> cdf;
    void build(uint32_t n_, double gamma, double n_edges, uint32_t cap) {
        n = n_;
        uniform = gamma <= 0.0 || n == 0;
        if (uniform) return;
        std::vector<double> w(n);
        double ex = -1.0 / (gamma - 1.0);
        for (uint32_t i = 0; i < n; i++) w[i] = std::pow((double)i + 1.0, ex);
        for (int it = 0; it < 32 && cap; it++) {
            double tot = 0;
            for (double x : w) tot += x;
            double lim = (double)cap * tot / n_edges;
            bool clipped = false;
            for (double& x : w)
                if (x > lim * (1 + 1e-12)) {
                    x = lim;
                    clipped = true;
                }
            if (!clipped) break;
        }
        cdf.resize(n);
        double acc = 0;
        for (uint32_t i = 0; i < n; i++) {
            acc += w[i];
            cdf[i] = acc;
        }
    }
    uint32_t draw(SplitMix& rng) const {
        if (uniform) return rng.below(n);
        double r = rng.u01() * cdf.back();
        uint32_t i = (uint32_t)(std::upper_bound(cdf.begin(), cdf.end(), r) - cdf.begin());
        return i < n ? i : n - 1;
    }
};

struct EdgeSet {
    std::vector<uint64_t> slots;
    uint64_t mask = 0, used = 0;
    explicit EdgeSet(uint64_t want) {
        uint64_t cap = 1024;
        while (cap < want * 2) cap <<= 1;
        slots.assign(cap, ~0ULL);
        mask = cap - 1;
    }
    bool insert(uint64_t key) {
        if ((used + 1) * 10 > slots.size() * 7) grow();
        uint64_t h = mbe_fmix64(key) & mask;
        while (true) {
            if (slots[h] == ~0ULL) {
                slots[h] = key;
                used++;
                return true;
            }
            if (slots[h] == key) return false;
            h = (h + 1) & mask;
        }
    }
    void grow() {
        std::vector<uint64_t> old;
        old.swap(slots);
        slots.assign(old.size() * 2, ~0ULL);
        mask = slots.size() - 1;
        used = 0;
        for (uint64_t k : old)
            if (k != ~0ULL) insert(k);
    }
};

}  // namespace

extern "C" mbe_status mbe_graph_generate(const mbe_gen_params* p, mbe_graph** out) {
    clear_error();
    if (!p || !out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if ((p->n_rows == 0 || p->n_cols == 0) && p->n_edges)
        return fail(MBE_ERR_INVALID_ARG, "edges requested on an empty side");
    uint64_t maxe = (uint64_t)p->n_rows * p->n_cols;
    uint64_t target = std::min<uint64_t>(p->n_edges, maxe);
    SplitMix rng{p->seed};
    Side rs, cs;
    rs.build(p->n_rows, p->gamma_rows, (double)std::max<uint64_t>(target, 1), p->max_deg);
    cs.build(p->n_cols, p->gamma_cols, (double)std::max<uint64_t>(target, 1), p->max_deg);
    EdgeSet set(target + (uint64_t)p->planted * p->planted_rows * p->planted_cols + 16);
    std::vector<uint64_t> keys;
    keys.reserve(target);
    std::vector<uint32_t> rdeg(p->n_rows, 0), cdeg(p->n_cols, 0);
    uint64_t draws = 0, max_draws = 64 * target + 1024;
    while (keys.size() < target && draws < max_draws) {
        draws++;
        uint32_t r = rs.draw(rng), c = cs.draw(rng);
        if (p->max_deg && (rdeg[r] >= p->max_deg || cdeg[c] >= p->max_deg)) continue;
        uint64_t k = ((uint64_t)r << 32) | c;
        if (set.insert(k)) {
            keys.push_back(k);
            rdeg[r]++;
            cdeg[c]++;
        }
    }
    // planted near-bicliques overlapping hubs
    if (p->planted && p->n_rows && p->n_cols) {
        uint32_t hub_r = std::max<uint32_t>(1, p->n_rows / 100), hub_c = std::max<uint32_t>(1, p->n_cols / 100);
        uint32_t pr = std::min(p->planted_rows, p->n_rows), pc = std::min(p->planted_cols, p->n_cols);
        std::vector<uint32_t> rows, cols;
        for (uint32_t b = 0; b < p->planted; b++) {
            auto pick = [&](uint32_t count, uint32_t n, uint32_t hubs, std::vector<uint32_t>& dst) {
                dst.clear();
                uint32_t tries = 0;
                while (dst.size() < count && tries < 1000u * count) {
                    tries++;
                    uint32_t v = (dst.size() * 2 < count) ? rng.below(hubs) : rng.below(n);
                    if (std::find(dst.begin(), dst.end(), v) == dst.end()) dst.push_back(v);
                }
            };
            pick(pr, p->n_rows, hub_r, rows);
            pick(pc, p->n_cols, hub_c, cols);
            for (uint32_t r : rows)
                for (uint32_t c : cols)
                    if (rng.u01() < p->planted_density) {
                        uint64_t k = ((uint64_t)r << 32) | c;
                        if (set.insert(k)) keys.push_back(k);
                    }
        }
    }
    std::sort(keys.begin(), keys.end());
    auto* g = new (std::nothrow) mbe_graph();
    if (!g) return fail(MBE_ERR_OUT_OF_MEMORY, "host allocation failed");
    g->n_rows = p->n_rows;
    g->n_cols = p->n_cols;
    g->row_ptr.assign((size_t)p->n_rows + 1, 0);
    g->col_idx.resize(keys.size());
    for (size_t i = 0; i < keys.size(); i++) {
        g->row_ptr[(keys[i] >> 32) + 1]++;
        g->col_idx[i] = (uint32_t)keys[i];
    }
    for (uint32_t r = 0; r < p->n_rows; r++) g->row_ptr[r + 1] += g->row_ptr[r];
    mbe_status st = normalise(g);
    if (st != MBE_OK) {
        delete g;
        return st;
    }
    g->uid = next_graph_uid();
    *out = g;
    return MBE_OK;
}

extern "C" uint64_t mbe_biclique_hash(const uint32_t* rows, uint32_t n_rows, const uint32_t* cols,
                                      uint32_t n_cols) {
    uint64_t sa = 0, sb = 0;
    for (uint32_t i = 0; i < n_rows; i++) sa += mbe_elem_row(rows[i]);
    for (uint32_t i = 0; i < n_cols; i++) sb += mbe_elem_col(cols[i]);
    return mbe_pair_hash(sa, n_rows, sb, n_cols);
}

extern "C" const char* mbe_variant_name(mbe_variant v) {
    switch (v) {
        case MBE_NORS: return "noRS";
        case MBE_NOES: return "noES";
        case MBE_NOWS: return "noWS";
        default: return "cuMBE";
    }
}

extern "C" mbe_variant mbe_variant_from_name(const char* name) {
    if (!name) return MBE_CUMBE;
    if (!std::strcmp(name, "noRS")) return MBE_NORS;
    if (!std::strcmp(name, "noES")) return MBE_NOES;
    if (!std::strcmp(name, "noWS")) return MBE_NOWS;
    return MBE_CUMBE;
}
