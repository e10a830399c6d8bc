// Host-side graph handling of libmbe: `.bi` reader and writer, CSR ingest,
// and the synthetic bipartite generator.  No CUDA calls here, so every
// function works on a machine without a GPU.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
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

mbe_status normalise(mbe_graph* g) {
    g->n_dup = 0;
    g->max_row_deg = 0;
    std::vector<uint32_t> col_deg(g->n_cols, 0);
    uint64_t w = 0;
    for (uint32_t r = 0; r < g->n_rows; r++) {
        uint64_t b = g->row_ptr[r], e = g->row_ptr[r + 1];
        auto first = g->col_idx.begin() + (ptrdiff_t)b;
        auto last = g->col_idx.begin() + (ptrdiff_t)e;
        for (auto it = first; it != last; ++it)
            if (*it >= g->n_cols)
                return fail(MBE_ERR_FORMAT, "column id " + std::to_string(*it) + " out of range in row " +
                                                std::to_string(r));
        std::sort(first, last);
        auto uend = std::unique(first, last);
        uint64_t len = (uint64_t)(uend - first);
        g->n_dup += (uint32_t)((e - b) - len);
        // compact in place (w <= b always holds)
        for (uint64_t i = 0; i < len; i++) {
            uint32_t c = g->col_idx[b + i];
            g->col_idx[w + i] = c;
            col_deg[c]++;
        }
        g->row_ptr[r] = w;
        w += len;
        if (len > g->max_row_deg) g->max_row_deg = (uint32_t)len;
    }
    g->row_ptr[g->n_rows] = w;
    g->col_idx.resize(w);
    g->col_idx.shrink_to_fit();
    g->max_col_deg = 0;
    for (uint32_t c : col_deg) g->max_col_deg = std::max(g->max_col_deg, c);
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

}  // namespace
}  // namespace mbe

using namespace mbe;

extern "C" mbe_status mbe_graph_load_bi(const char* path, mbe_graph** out) {
    clear_error();
    if (!path || !out) return fail(MBE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(MBE_ERR_IO, std::string("cannot open ") + path);
    std::vector<char> buf;
    {
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
    }
    Scanner sc{buf.data(), buf.data() + buf.size()};
    long long nr, nl, ne;
    if (!sc.next(&nr) || !sc.next(&nl) || !sc.next(&ne))
        return fail(MBE_ERR_FORMAT, "missing header 'R L E'");
    if (nr < 0 || nl < 0 || ne < 0 || nr > 0xFFFFFFFFLL || nl > 0xFFFFFFFFLL)
        return fail(MBE_ERR_FORMAT, "bad header values");
    std::vector<long long> start((size_t)nr), len((size_t)nr);
    for (long long i = 0; i < nr; i++) {
        if (!sc.next(&start[(size_t)i]) || !sc.next(&len[(size_t)i]))
            return fail(MBE_ERR_FORMAT, "truncated row table at row " + std::to_string(i));
        if (start[(size_t)i] < 0 || len[(size_t)i] < 0 || start[(size_t)i] + len[(size_t)i] > ne)
            return fail(MBE_ERR_FORMAT, "row " + std::to_string(i) + " range outside edge list");
    }
    std::vector<uint32_t> edges((size_t)ne);
    for (long long i = 0; i < ne; i++) {
        long long nbr, ignored;
        if (!sc.next(&nbr) || !sc.next(&ignored))
            return fail(MBE_ERR_FORMAT, "truncated edge list at edge " + std::to_string(i));
        if (nbr < 0 || nbr >= nl) return fail(MBE_ERR_FORMAT, "neighbour id out of range at edge " + std::to_string(i));
        edges[(size_t)i] = (uint32_t)nbr;
    }
    auto* g = new (std::nothrow) mbe_graph();
    if (!g) return fail(MBE_ERR_OUT_OF_MEMORY, "host allocation failed");
    g->n_rows = (uint32_t)nr;
    g->n_cols = (uint32_t)nl;
    g->row_ptr.assign((size_t)nr + 1, 0);
    uint64_t tot = 0;
    for (long long i = 0; i < nr; i++) tot += (uint64_t)len[(size_t)i];
    g->col_idx.resize(tot);
    uint64_t w = 0;
    for (long long i = 0; i < nr; i++) {
        g->row_ptr[(size_t)i] = w;
        std::memcpy(g->col_idx.data() + w, edges.data() + start[(size_t)i], sizeof(uint32_t) * (size_t)len[(size_t)i]);
        w += (uint64_t)len[(size_t)i];
    }
    g->row_ptr[(size_t)nr] = w;
    mbe_status st = normalise(g);
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
