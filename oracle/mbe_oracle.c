/*
 * mbe_oracle.c - CPU oracle for maximal biclique enumeration.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (libmbe, the `mbe`
 * CLI, the Python package) links or calls this file; only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg do, as the
 * checker or the timed CPU baseline.
 *
 * Two independent oracles:
 *
 *  1. oracle_ref_enumerate: a sequential restatement of the reference's
 *     block-level backtracking (NTUDDSNLab/cuMBE src/mbe_cuMBE.cuh phase 1,
 *     which is also the whole of src/mbe_noWS.cuh).  It keeps the
 *     reference's index-prefix sets (L/u2L, P/v2P, Q/v2Q with swap
 *     maintenance), per-level arrays x/L_lp/R_lp/P_lp/Q_lp/pre_min, the
 *     root order (src/header.cuh:55-63) grabbed from the tail
 *     (src/mbe_cuMBE.cuh:57-64,125-133), the reverse-scan maximality test
 *     (:215-238), the expansion (:242-291), the min-count pivot with early
 *     stop and the per-level pre_min carry-over (:345-390), and the
 *     noRS/noES deltas (src/mbe_noRS.cuh:234-256,274-283;
 *     src/mbe_noES.cuh:352,365-366).  With n_threads > 1 each thread plays
 *     one reference block of phase 1, grabbing roots from one shared
 *     counter (the reference's P_ptr).  It also counts the adjacency
 *     entries the algorithm streams (the roofline numerator) and the
 *     tree nodes it evaluates.
 *
 *  2. oracle_brute: subset enumeration of the smaller side (<= 24
 *     vertices, the other side <= 64) straight from the definition of a
 *     maximal biclique.
 *
 * Parity pinning: (2) checks (1) on random tiny graphs; (1) is checked on
 * the synthetic workloads against counts printed by the reference's own
 * CUDA_MBE_* kernels (built from its sources by oracle/build_ref.sh and
 * driven by oracle/ref_runner.cpp on a GPU).
 *
 * Hash: per biclique h(A,B) = fmix64(SA ^ fmix64(SB + (|A|<<32 | |B|))),
 * SA = sum fmix64(a + 0x9E3779B97F4A7C15) over rows a, SB = sum
 * fmix64(b + 0xD1B54A32D192ED03) over cols b; graph hash = sum of h.
 * fmix64 is the splitmix64 output mixer.
 */
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_API __attribute__((visibility("default")))

typedef struct {
    uint64_t count;
    uint64_t hash;
    uint64_t nodes;    /* tree nodes evaluated (x picks)               */
    uint64_t scanned;  /* adjacency entries streamed                    */
} oracle_result;

/* Optional canonical output (single-thread runs only). */
typedef struct {
    uint64_t cap_bicliques;
    uint64_t cap_ids;
    uint64_t n_bicliques;
    uint64_t n_ids;
    uint32_t* offsets; /* [cap_bicliques + 1]                            */
    uint32_t* nrows;   /* [cap_bicliques]                                */
    uint32_t* ids;     /* rows (sorted) then cols (sorted) per biclique  */
    int overflow;
} oracle_emit;

static inline uint64_t fmix64(uint64_t z) {
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ULL;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return z;
}
static inline uint64_t e_row(uint32_t a) { return fmix64((uint64_t)a + 0x9E3779B97F4A7C15ULL); }
static inline uint64_t e_col(uint32_t b) { return fmix64((uint64_t)b + 0xD1B54A32D192ED03ULL); }
static inline uint64_t pair_hash(uint64_t sa, uint32_t na, uint64_t sb, uint32_t nb) {
    uint64_t sizes = ((uint64_t)na << 32) | (uint64_t)nb;
    return fmix64(sa ^ fmix64(sb + sizes));
}

ORACLE_API uint64_t oracle_biclique_hash(const uint32_t* rows, uint32_t nr, const uint32_t* cols, uint32_t nc) {
    uint64_t sa = 0, sb = 0;
    for (uint32_t i = 0; i < nr; i++) sa += e_row(rows[i]);
    for (uint32_t i = 0; i < nc; i++) sb += e_col(cols[i]);
    return pair_hash(sa, nr, sb, nc);
}

/* ------------------------------------------------------------------------ */
/* Oriented graph: R = smaller side (branching), L = larger side
 * (src/main.cu:65-70: swap when NUM_R > NUM_L).                            */

typedef struct {
    int nR, nL;
    int swapped;          /* 1: R = file cols, L = file rows               */
    int64_t* rptr;        /* R vertex -> L neighbours                      */
    int32_t* radj;
    int64_t* lptr;        /* L vertex -> R neighbours                      */
    int32_t* ladj;
} ograph;

static void csr_transpose(int n_src, int n_dst, const uint64_t* ptr, const uint32_t* adj, int64_t** optr,
                          int32_t** oadj) {
    uint64_t ne = ptr[n_src];
    int64_t* p = (int64_t*)calloc((size_t)n_dst + 1, sizeof(int64_t));
    int32_t* a = (int32_t*)malloc(sizeof(int32_t) * (ne ? ne : 1));
    for (uint64_t e = 0; e < ne; e++) p[adj[e] + 1]++;
    for (int i = 0; i < n_dst; i++) p[i + 1] += p[i];
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n_dst + 1));
    memcpy(cur, p, sizeof(int64_t) * ((size_t)n_dst + 1));
    for (int s = 0; s < n_src; s++)
        for (uint64_t e = ptr[s]; e < ptr[s + 1]; e++) a[cur[adj[e]]++] = s;
    free(cur);
    *optr = p;
    *oadj = a;
}

static void csr_copy(int n, const uint64_t* ptr, const uint32_t* adj, int64_t** optr, int32_t** oadj) {
    uint64_t ne = ptr[n];
    int64_t* p = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
    int32_t* a = (int32_t*)malloc(sizeof(int32_t) * (ne ? ne : 1));
    for (int i = 0; i <= n; i++) p[i] = (int64_t)ptr[i];
    for (uint64_t e = 0; e < ne; e++) a[e] = (int32_t)adj[e];
    *optr = p;
    *oadj = a;
}

static void ograph_build(ograph* g, uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr,
                         const uint32_t* col_idx) {
    g->swapped = n_rows > n_cols;
    if (!g->swapped) {
        g->nR = (int)n_rows;
        g->nL = (int)n_cols;
        csr_copy(g->nR, row_ptr, col_idx, &g->rptr, &g->radj);
        csr_transpose(g->nR, g->nL, row_ptr, col_idx, &g->lptr, &g->ladj);
    } else {
        g->nR = (int)n_cols;
        g->nL = (int)n_rows;
        csr_copy(g->nL, row_ptr, col_idx, &g->lptr, &g->ladj);
        csr_transpose(g->nL, g->nR, row_ptr, col_idx, &g->rptr, &g->radj);
    }
}

static void ograph_free(ograph* g) {
    free(g->rptr);
    free(g->radj);
    free(g->lptr);
    free(g->ladj);
}

/* ------------------------------------------------------------------------ */
/* Restatement of the reference's per-block state machine.                   */

enum { V_CUMBE = 0, V_NORS = 1, V_NOES = 2, V_NOWS = 3 };
#define ORACLE_INF 1073741824 /* src/header.cuh:8 */

typedef struct {
    const ograph* g;
    const int* ori_P;
    atomic_int* P_ptr;
    int variant;
    uint32_t min_rows, min_cols;
    int k_lo;                 /* only roots with ori_P index >= k_lo      */
    int stride;               /* only every stride-th root (1 = all)       */
    int last;                 /* index of the first root in processing order */
    oracle_emit* emit;
    /* per-thread ("per-block") state, src/main.cu:72-86 */
    int *u2L, *L, *v2P, *P, *v2Q, *Q, *R, *x, *L_lp, *R_lp, *P_lp, *Q_lp, *pre_min;
    int *num_N_u, *L_buf, *touched;
    oracle_result res;
} ostate;

static void q_add(ostate* s, int lvl, int v) {
    /* Q <- Q u {v}: swap v into the prefix (src/mbe_cuMBE.cuh:318-333) */
    int q = s->v2Q[v];
    int t = s->Q[s->Q_lp[lvl]];
    s->Q[s->Q_lp[lvl]] = v;
    s->Q[q] = t;
    s->v2Q[v] = s->Q_lp[lvl]++;
    s->v2Q[t] = q;
}

static int cmp_u32(const void* a, const void* b) {
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return x < y ? -1 : x > y;
}

static void report(ostate* s, int nl, int nr) {
    const ograph* g = s->g;
    uint32_t na = (uint32_t)(g->swapped ? nl : nr); /* rows */
    uint32_t nb = (uint32_t)(g->swapped ? nr : nl); /* cols */
    if (na < s->min_rows || nb < s->min_cols) return;
    uint64_t sl = 0, sr = 0;
    for (int i = 0; i < nl; i++) sl += g->swapped ? e_row((uint32_t)s->L[i]) : e_col((uint32_t)s->L[i]);
    for (int i = 0; i < nr; i++) sr += g->swapped ? e_col((uint32_t)s->R[i]) : e_row((uint32_t)s->R[i]);
    uint64_t sa = g->swapped ? sl : sr, sb = g->swapped ? sr : sl;
    s->res.count++;
    s->res.hash += pair_hash(sa, na, sb, nb);
    oracle_emit* em = s->emit;
    if (em) {
        if (em->n_bicliques >= em->cap_bicliques || em->n_ids + na + nb > em->cap_ids) {
            em->overflow = 1;
            return;
        }
        uint32_t* dst = em->ids + em->n_ids;
        const int* a_src = g->swapped ? s->L : s->R;
        const int* b_src = g->swapped ? s->R : s->L;
        for (uint32_t i = 0; i < na; i++) dst[i] = (uint32_t)a_src[i];
        for (uint32_t i = 0; i < nb; i++) dst[na + i] = (uint32_t)b_src[i];
        qsort(dst, na, sizeof(uint32_t), cmp_u32);
        qsort(dst + na, nb, sizeof(uint32_t), cmp_u32);
        em->offsets[em->n_bicliques] = (uint32_t)em->n_ids;
        em->nrows[em->n_bicliques] = na;
        em->n_bicliques++;
        em->n_ids += na + nb;
        em->offsets[em->n_bicliques] = (uint32_t)em->n_ids;
    }
}

/* Evaluates tree node (lvl, xv): L', maximality against Q, expansion,
 * count.  Returns 1 when the node must recurse (P' non-empty).
 * src/mbe_cuMBE.cuh:160-314 (level 0) and :396-550 (levels >= 1). */
static int eval_node(ostate* s, int lvl, int xv) {
    const ograph* g = s->g;
    s->res.nodes++;
    /* R' <- R u {x}; P' <- {}; Q' <- Q; L' <- {} */
    s->R_lp[lvl + 1] = s->R_lp[lvl];
    s->R[s->R_lp[lvl + 1]++] = xv;
    s->P_lp[lvl + 1] = 0;
    s->Q_lp[lvl + 1] = s->Q_lp[lvl];
    s->L_lp[lvl + 1] = 0;
    /* L' <- {u in L | (u,x) in E}, then swap them into the prefix (:187-211) */
    int nl = 0;
    for (int64_t e = g->rptr[xv]; e < g->rptr[xv + 1]; e++) {
        int u = g->radj[e];
        if (s->u2L[u] < s->L_lp[lvl]) s->L_buf[nl++] = u;
    }
    s->res.scanned += (uint64_t)(g->rptr[xv + 1] - g->rptr[xv]);
    for (int i = 0; i < nl; i++) {
        int u = s->L_buf[i];
        int l = s->u2L[u];
        int pos = s->L_lp[lvl + 1]++;
        int t = s->L[pos];
        s->L[pos] = s->L[l];
        s->L[l] = t;
        int ut = s->u2L[s->L[l]];
        s->u2L[s->L[l]] = s->u2L[u];
        s->u2L[u] = ut;
    }
    /* maximality: exists v in Q with |N(v) n L'| = |L'| (:215-238) */
    int nt = 0;
    for (int i = 0; i < nl; i++) {
        int u = s->L[i];
        for (int64_t e = g->lptr[u]; e < g->lptr[u + 1]; e++) {
            int v = g->ladj[e];
            if (s->v2Q[v] < s->Q_lp[lvl] && s->num_N_u[v]++ == 0) s->touched[nt++] = v;
        }
        s->res.scanned += (uint64_t)(g->lptr[u + 1] - g->lptr[u]);
    }
    if (s->variant == V_NORS) {
        /* noRS recounts each touched Q vertex by a forward scan of N(v)
         * (src/mbe_noRS.cuh:234-256) */
        for (int i = 0; i < nt; i++) {
            int v = s->touched[i];
            int c = 0;
            for (int64_t e = g->rptr[v]; e < g->rptr[v + 1]; e++)
                if (s->u2L[g->radj[e]] < nl) c++;
            s->res.scanned += (uint64_t)(g->rptr[v + 1] - g->rptr[v]);
            s->num_N_u[v] = c;
        }
    }
    int maximal = 1;
    for (int i = 0; i < nt; i++) {
        int v = s->touched[i];
        if (s->num_N_u[v] == nl) maximal = 0;
        s->num_N_u[v] = 0;
    }
    if (!maximal) return 0;
    /* expansion over P (:242-291; noRS: forward scan over P, src/mbe_noRS.cuh:274-283) */
    nt = 0;
    if (s->variant != V_NORS) {
        for (int i = 0; i < nl; i++) {
            int u = s->L[i];
            for (int64_t e = g->lptr[u]; e < g->lptr[u + 1]; e++) {
                int v = g->ladj[e];
                if (s->v2P[v] < s->P_lp[lvl] && s->num_N_u[v]++ == 0) s->touched[nt++] = v;
            }
            s->res.scanned += (uint64_t)(g->lptr[u + 1] - g->lptr[u]);
        }
    } else {
        for (int i = 0; i < s->P_lp[lvl]; i++) {
            int v = s->P[i];
            for (int64_t e = g->rptr[v]; e < g->rptr[v + 1]; e++)
                if (s->u2L[g->radj[e]] < nl && s->num_N_u[v]++ == 0) s->touched[nt++] = v;
            s->res.scanned += (uint64_t)(g->rptr[v + 1] - g->rptr[v]);
        }
    }
    for (int i = 0; i < nt; i++) {
        int v = s->touched[i];
        if (s->num_N_u[v] == nl) s->R[s->R_lp[lvl + 1]++] = v;
    }
    for (int i = 0; i < nt; i++) {
        int v = s->touched[i];
        if (s->num_N_u[v] != nl) {
            int p = s->v2P[v];
            int pos = s->P_lp[lvl + 1]++;
            int t = s->P[pos];
            s->P[pos] = v;
            s->P[p] = t;
            s->v2P[v] = pos;
            s->v2P[t] = p;
        }
        s->num_N_u[v] = 0;
    }
    report(s, nl, s->R_lp[lvl + 1]);
    return s->P_lp[lvl + 1] != 0;
}

/* Pivot: argmin_{v in P} |N(v) n L| scanning P from its tail, strict
 * improvement only, stopping early once the minimum equals pre_min[lvl];
 * the chosen vertex is swapped to P[P_lp-1] (src/mbe_cuMBE.cuh:345-390). */
static void pick_pivot(ostate* s, int lvl) {
    const ograph* g = s->g;
    int es = s->variant != V_NOES;
    int best = ORACLE_INF, i_min = s->P_lp[lvl] - 1;
    for (int i = s->P_lp[lvl]; i-- > 0 && (!es || best != s->pre_min[lvl]);) {
        int v = s->P[i];
        int c = 0;
        int64_t e = g->rptr[v], end = g->rptr[v + 1];
        for (; e < end; e++) {
            if (s->u2L[g->radj[e]] < s->L_lp[lvl]) {
                c++;
                if (es && c > best) {
                    e++;
                    break;
                }
            }
        }
        s->res.scanned += (uint64_t)(e - g->rptr[v]);
        if (c < best) {
            best = c;
            i_min = i;
        }
    }
    s->pre_min[lvl] = best;
    int last = s->P_lp[lvl] - 1;
    int t = s->P[last];
    s->P[last] = s->P[i_min];
    s->P[i_min] = t;
    s->v2P[s->P[last]] = last;
    s->v2P[t] = i_min;
}

static void* run_block(void* arg) {
    ostate* s = (ostate*)arg;
    const ograph* g = s->g;
    int nR = g->nR;
    s->P_lp[0] = nR;
    int lvl = 0;
    while (lvl >= 0) {
        int rec = 0;
        if (lvl == 0) {
            for (;;) {
                int before = s->P_lp[0];
                int k = atomic_fetch_sub(s->P_ptr, 1);
                if (k < s->k_lo) k = -1;
                /* a stride sample skips roots but keeps their Q semantics:
                 * the next processed root adds every skipped root to Q */
                while (k >= 0 && s->stride > 1 && (s->last - k) % s->stride != 0) k = atomic_fetch_sub(s->P_ptr, 1);
                if (k < s->k_lo) k = -1;
                s->P_lp[0] = k;
                if (k < 0) break;
                /* Q gains the roots skipped since this block's previous root (:135-150) */
                for (int i = k + 1; i < before; i++) q_add(s, 0, s->ori_P[i]);
                /* P reset to ori_P[0..before) (:153-154) */
                for (int i = 0; i < before; i++) {
                    s->P[i] = s->ori_P[i];
                    s->v2P[s->P[i]] = i;
                }
                int xv = s->ori_P[k];
                s->x[0] = xv;
                if (eval_node(s, 0, xv)) {
                    rec = 1;
                    break;
                }
                q_add(s, 0, xv);
            }
        } else {
            while (s->P_lp[lvl] != 0) {
                pick_pivot(s, lvl);
                int xv = s->P[--s->P_lp[lvl]];
                s->x[lvl] = xv;
                if (eval_node(s, lvl, xv)) {
                    rec = 1;
                    break;
                }
                q_add(s, lvl, xv);
            }
        }
        /* level transitions (:584-611) */
        if (rec)
            lvl++;
        else if (lvl-- > 0)
            q_add(s, lvl, s->x[lvl]);
    }
    return NULL;
}

typedef struct {
    const uint64_t* deg;
} sort_ctx;

static const int64_t* g_sort_ptr; /* only used inside ref_order (single-threaded) */
static int cmp_root(const void* a, const void* b) {
    int x = *(const int*)a, y = *(const int*)b;
    int64_t dx = g_sort_ptr[x + 1] - g_sort_ptr[x], dy = g_sort_ptr[y + 1] - g_sort_ptr[y];
    if (dx != dy) return dx > dy ? -1 : 1; /* degree descending */
    return x < y ? -1 : x > y;             /* ties: id ascending */
}

/* ori_P: R ids by degree descending (src/header.cuh:55-63).  The
 * reference's std::sort leaves ties in a libstdc++-defined order; the
 * count does not depend on it, so ties go by id here. */
static void ref_order(const ograph* g, int* ori_P) {
    for (int i = 0; i < g->nR; i++) ori_P[i] = i;
    g_sort_ptr = g->rptr;
    qsort(ori_P, (size_t)g->nR, sizeof(int), cmp_root);
}

static int alloc_state(ostate* s, int nR, int nL) {
    size_t r = (size_t)nR + 2, l = (size_t)nL + 2;
    s->u2L = malloc(sizeof(int) * l);
    s->L = malloc(sizeof(int) * l);
    s->L_buf = malloc(sizeof(int) * l);
    s->v2P = malloc(sizeof(int) * r);
    s->P = malloc(sizeof(int) * r);
    s->v2Q = malloc(sizeof(int) * r);
    s->Q = malloc(sizeof(int) * r);
    s->R = malloc(sizeof(int) * r);
    s->x = malloc(sizeof(int) * r);
    s->L_lp = malloc(sizeof(int) * r);
    s->R_lp = malloc(sizeof(int) * r);
    s->P_lp = malloc(sizeof(int) * r);
    s->Q_lp = malloc(sizeof(int) * r);
    s->pre_min = malloc(sizeof(int) * r);
    s->num_N_u = calloc(r, sizeof(int));
    s->touched = malloc(sizeof(int) * r);
    if (!s->u2L || !s->L || !s->L_buf || !s->v2P || !s->P || !s->v2Q || !s->Q || !s->R || !s->x || !s->L_lp ||
        !s->R_lp || !s->P_lp || !s->Q_lp || !s->pre_min || !s->num_N_u || !s->touched)
        return -1;
    /* initial values, src/main.cu:72-86 */
    for (int i = 0; i < nL; i++) s->u2L[i] = s->L[i] = i;
    for (int i = 0; i < nR; i++) s->v2P[i] = s->P[i] = s->v2Q[i] = s->Q[i] = s->R[i] = i;
    for (size_t i = 0; i < r; i++) {
        s->x[i] = -1;
        s->L_lp[i] = nL;
        s->R_lp[i] = 0;
        s->P_lp[i] = nR;
        s->Q_lp[i] = 0;
        s->pre_min[i] = 1;
    }
    memset(&s->res, 0, sizeof s->res);
    return 0;
}

static void free_state(ostate* s) {
    free(s->u2L);
    free(s->L);
    free(s->L_buf);
    free(s->v2P);
    free(s->P);
    free(s->v2Q);
    free(s->Q);
    free(s->R);
    free(s->x);
    free(s->L_lp);
    free(s->R_lp);
    free(s->P_lp);
    free(s->Q_lp);
    free(s->pre_min);
    free(s->num_N_u);
    free(s->touched);
}

/* Enumerates the maximal bicliques of the file-orientation CSR.
 * root_lo/root_hi (fractions in [0,1] of the non-isolated roots, taken
 * from the processing tail) bound a sample; 0/1 runs everything.  Returns
 * 0 on success, -1 on allocation failure, -2 on emit overflow. */
static int ref_enumerate_impl(uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr, const uint32_t* col_idx,
                              int variant, int n_threads, uint32_t min_rows, uint32_t min_cols, double root_frac,
                              int stride, oracle_result* out, oracle_emit* emit);

ORACLE_API int oracle_ref_enumerate(uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr,
                                    const uint32_t* col_idx, int variant, int n_threads, uint32_t min_rows,
                                    uint32_t min_cols, double root_frac, oracle_result* out, oracle_emit* emit) {
    return ref_enumerate_impl(n_rows, n_cols, row_ptr, col_idx, variant, n_threads, min_rows, min_cols, root_frac, 1,
                              out, emit);
}

/* Bounded sample for timing: only every stride-th root in processing
 * order is expanded (with the full Q of everything processed before it),
 * so the sample spans all degrees.  The count is that of the sampled
 * roots' subtrees. */
ORACLE_API int oracle_ref_enumerate_sampled(uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr,
                                            const uint32_t* col_idx, int variant, int n_threads, int stride,
                                            oracle_result* out) {
    return ref_enumerate_impl(n_rows, n_cols, row_ptr, col_idx, variant, n_threads, 0, 0, 0.0,
                              stride < 1 ? 1 : stride, out, NULL);
}

static int ref_enumerate_impl(uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr, const uint32_t* col_idx,
                              int variant, int n_threads, uint32_t min_rows, uint32_t min_cols, double root_frac,
                              int stride, oracle_result* out, oracle_emit* emit) {
    memset(out, 0, sizeof *out);
    ograph g;
    ograph_build(&g, n_rows, n_cols, row_ptr, col_idx);
    if (n_threads < 1) n_threads = 1;
    if (emit) n_threads = 1;
    int* ori_P = (int*)malloc(sizeof(int) * ((size_t)g.nR + 1));
    ref_order(&g, ori_P);
    /* P_ptr = last index of ori_P with a non-zero degree (:57-64) */
    int last = -1;
    for (int i = g.nR - 1; i >= 0; i--)
        if (g.rptr[ori_P[i] + 1] > g.rptr[ori_P[i]]) {
            last = i;
            break;
        }
    atomic_int P_ptr;
    atomic_init(&P_ptr, last);
    int k_lo = 0;
    if (root_frac > 0.0 && root_frac < 1.0 && last >= 0) {
        int n = last + 1;
        int take = (int)(root_frac * n);
        if (take < 1) take = 1;
        k_lo = n - take;
    }
    int rc = 0;
    ostate* st = (ostate*)calloc((size_t)n_threads, sizeof(ostate));
    pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
    for (int t = 0; t < n_threads; t++) {
        st[t].g = &g;
        st[t].ori_P = ori_P;
        st[t].P_ptr = &P_ptr;
        st[t].variant = variant;
        st[t].min_rows = min_rows;
        st[t].min_cols = min_cols;
        st[t].k_lo = k_lo;
        st[t].stride = stride;
        st[t].last = last;
        st[t].emit = emit;
        if (alloc_state(&st[t], g.nR, g.nL)) rc = -1;
    }
    if (rc == 0 && last >= 0) {
        if (n_threads == 1) {
            run_block(&st[0]);
        } else {
            for (int t = 0; t < n_threads; t++) pthread_create(&th[t], NULL, run_block, &st[t]);
            for (int t = 0; t < n_threads; t++) pthread_join(th[t], NULL);
        }
    }
    for (int t = 0; t < n_threads; t++) {
        out->count += st[t].res.count;
        out->hash += st[t].res.hash;
        out->nodes += st[t].res.nodes;
        out->scanned += st[t].res.scanned;
        free_state(&st[t]);
    }
    free(st);
    free(th);
    free(ori_P);
    ograph_free(&g);
    if (rc == 0 && emit && emit->overflow) rc = -2;
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Brute force from the definition: for every non-empty subset S of the
 * smaller side, A = common neighbours of S; (A, S) is maximal iff A is
 * non-empty and S equals the set of vertices adjacent to all of A. */
ORACLE_API int oracle_brute(uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr, const uint32_t* col_idx,
                            uint32_t min_rows, uint32_t min_cols, oracle_result* out, oracle_emit* emit) {
    memset(out, 0, sizeof *out);
    int swapped = n_rows > n_cols;
    int ns = (int)(swapped ? n_cols : n_rows), nb = (int)(swapped ? n_rows : n_cols);
    if (ns > 24 || nb > 64) return -1;
    uint64_t* nbr = (uint64_t*)calloc((size_t)ns + 1, sizeof(uint64_t));
    for (uint32_t r = 0; r < n_rows; r++)
        for (uint64_t e = row_ptr[r]; e < row_ptr[r + 1]; e++) {
            uint32_t c = col_idx[e];
            if (!swapped)
                nbr[r] |= 1ULL << c;
            else
                nbr[c] |= 1ULL << r;
        }
    uint64_t full = nb == 64 ? ~0ULL : ((1ULL << nb) - 1);
    uint32_t a_ids[64], b_ids[64];
    for (uint64_t mask = 1; mask < (1ULL << ns); mask++) {
        uint64_t A = full;
        for (int v = 0; v < ns; v++)
            if (mask >> v & 1) A &= nbr[v];
        if (!A) continue;
        uint64_t closure = 0;
        for (int v = 0; v < ns; v++)
            if ((nbr[v] & A) == A) closure |= 1ULL << v;
        if (closure != mask) continue;
        uint32_t ns_cnt = 0, nb_cnt = 0;
        for (int v = 0; v < ns; v++)
            if (mask >> v & 1) a_ids[ns_cnt++] = (uint32_t)v;
        for (int u = 0; u < nb; u++)
            if (A >> u & 1) b_ids[nb_cnt++] = (uint32_t)u;
        const uint32_t* rows = swapped ? b_ids : a_ids;
        const uint32_t* cols = swapped ? a_ids : b_ids;
        uint32_t nr = swapped ? nb_cnt : ns_cnt, nc = swapped ? ns_cnt : nb_cnt;
        if (nr < min_rows || nc < min_cols) continue;
        out->count++;
        out->hash += oracle_biclique_hash(rows, nr, cols, nc);
        if (emit) {
            if (emit->n_bicliques >= emit->cap_bicliques || emit->n_ids + nr + nc > emit->cap_ids) {
                emit->overflow = 1;
                continue;
            }
            uint32_t* dst = emit->ids + emit->n_ids;
            memcpy(dst, rows, sizeof(uint32_t) * nr);
            memcpy(dst + nr, cols, sizeof(uint32_t) * nc);
            emit->offsets[emit->n_bicliques] = (uint32_t)emit->n_ids;
            emit->nrows[emit->n_bicliques] = nr;
            emit->n_bicliques++;
            emit->n_ids += nr + nc;
            emit->offsets[emit->n_bicliques] = (uint32_t)emit->n_ids;
        }
    }
    free(nbr);
    return emit && emit->overflow ? -2 : 0;
}
