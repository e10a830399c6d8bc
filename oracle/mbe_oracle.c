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
 * CUDA_MBE_* kernels (built from its sources by oracle/build_ref.py and
 * driven by oracle/ref_runner.cpp on a GPU).
 *
 * Hash: per biclique h(A,B) = fmix64(SA ^ fmix64(SB + (|A|<<32 | |B|))),
 * SA = sum fmix64(a + 0x9E3779B97F4A7C15) over rows a, SB = sum
 * fmix64(b + 0xD1B54A32D192ED03) over cols b; graph hash = sum of h.
 * fmix64 is the splitmix64 output mixer.
 */
#include <math.h>
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
    int p_begin, p_end;       /* root sample: processing positions [p_begin, p_end) ... */
    int stride;               /* ... every stride-th one from p_begin (1 = all) */
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
                /* a root sample skips roots but keeps their Q semantics:
                 * the next processed root adds every skipped root to Q.
                 * Position j = last - k in processing order. */
                int k = atomic_fetch_sub(s->P_ptr, 1);
                while (k >= 0 && s->last - k < s->p_end &&
                       (s->last - k < s->p_begin || (s->last - k - s->p_begin) % s->stride != 0))
                    k = atomic_fetch_sub(s->P_ptr, 1);
                if (k >= 0 && s->last - k >= s->p_end) k = -1;
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
    return x > y ? -1 : x < y;             /* ties: id descending */
}

/* ori_P: R ids by degree descending (src/header.cuh:55-63).  The
 * reference's std::sort leaves ties in a libstdc++-defined order; the
 * count does not depend on it, so ties go by id descending here: roots are
 * processed from the tail, so the processing order is degree ascending,
 * id ascending, the order the GPU engine ranks roots in (root samples of
 * the two then cover the same roots). */
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
                              int p_begin, int p_end, int stride, oracle_result* out, oracle_emit* emit);

ORACLE_API int oracle_ref_enumerate(uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr,
                                    const uint32_t* col_idx, int variant, int n_threads, uint32_t min_rows,
                                    uint32_t min_cols, double root_frac, oracle_result* out, oracle_emit* emit) {
    return ref_enumerate_impl(n_rows, n_cols, row_ptr, col_idx, variant, n_threads, min_rows, min_cols, root_frac, 0,
                              -1, 1, out, emit);
}

/* Bounded sample for timing: only every stride-th root in processing
 * order is expanded (with the full Q of everything processed before it),
 * so the sample spans all degrees.  The count is that of the sampled
 * roots' subtrees. */
ORACLE_API int oracle_ref_enumerate_sampled(uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr,
                                            const uint32_t* col_idx, int variant, int n_threads, int stride,
                                            oracle_result* out) {
    return ref_enumerate_impl(n_rows, n_cols, row_ptr, col_idx, variant, n_threads, 0, 0, 0.0, 0, -1,
                              stride < 1 ? 1 : stride, out, NULL);
}

/* Root sample as the GPU engine's mbe_opts takes it: the roots at
 * processing positions p (degree ascending, id ascending, vertices with
 * edges only) with p_begin <= p < p_end (p_end < 0: no bound) and
 * (p - p_begin) % stride == 0.  Each sampled root keeps every earlier root
 * in its Q, so the result is the maximal bicliques whose earliest member
 * of the branching side is sampled. */
ORACLE_API int oracle_ref_enumerate_roots(uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr,
                                          const uint32_t* col_idx, int variant, int n_threads, uint32_t min_rows,
                                          uint32_t min_cols, int p_begin, int p_end, int stride,
                                          oracle_result* out) {
    return ref_enumerate_impl(n_rows, n_cols, row_ptr, col_idx, variant, n_threads, min_rows, min_cols, 0.0,
                              p_begin < 0 ? 0 : p_begin, p_end, stride < 1 ? 1 : stride, out, NULL);
}

static int ref_enumerate_impl(uint32_t n_rows, uint32_t n_cols, const uint64_t* row_ptr, const uint32_t* col_idx,
                              int variant, int n_threads, uint32_t min_rows, uint32_t min_cols, double root_frac,
                              int p_begin, int p_end, int stride, oracle_result* out, oracle_emit* emit) {
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
    if (p_end < 0 || p_end > last + 1) p_end = last + 1;
    if (root_frac > 0.0 && root_frac < 1.0 && last >= 0) {
        /* the first root_frac of the roots in processing order */
        int take = (int)(root_frac * (last + 1));
        p_end = take < 1 ? 1 : take;
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
        st[t].p_begin = p_begin;
        st[t].p_end = p_end;
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

/* ------------------------------------------------------------------------ */
/* Synthetic Chung-Lu generator, restated from the product's generator
 * (mbe_graph_generate) so that the timed CPU baseline can build its input
 * without loading the product library.  Same published recipe, same
 * stream: splitmix64 (Steele, Lea & Flood 2014) seeded by `seed`; weights
 * w_i = (i+1)^(-1/(gamma-1)) capped at max_deg expected degree by repeated
 * clipping; endpoints drawn by inverse CDF (first cdf entry above u * total);
 * duplicates and endpoints at max_deg rejected until n_edges distinct edges
 * exist or 64 n_edges + 1024 draws were made; then `planted` blocks of
 * planted_rows x planted_cols at planted_density, half of each side from
 * the 1% lowest ids (the hubs) and half uniform.  The CSR is sorted by
 * (row, col).  tests/ checks it equal to the product's on several shapes. */

typedef struct {
    uint32_t n_rows, n_cols;
    uint64_t n_edges;
    double gamma_rows, gamma_cols;
    uint32_t max_deg;
    uint64_t seed;
    uint32_t planted, planted_rows, planted_cols;
    double planted_density;
} oracle_gen;

typedef struct {
    uint64_t s;
} gen_rng;

static uint64_t gen_next(gen_rng* r) {
    r->s += 0x9E3779B97F4A7C15ULL;
    return fmix64(r->s);
}
static double gen_u01(gen_rng* r) { return (double)(gen_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static uint32_t gen_below(gen_rng* r, uint32_t n) {
    return (uint32_t)(((unsigned __int128)gen_next(r) * n) >> 64);
}

typedef struct {
    uint32_t n;
    int uniform;
    double* cdf;
} gen_side;

static int gen_side_build(gen_side* sd, uint32_t n, double gamma, double n_edges, uint32_t cap) {
    sd->n = n;
    sd->cdf = NULL;
    sd->uniform = gamma <= 0.0 || n == 0;
    if (sd->uniform) return 0;
    double* w = (double*)malloc(sizeof(double) * n);
    if (!w) return -1;
    const double ex = -1.0 / (gamma - 1.0);
    for (uint32_t i = 0; i < n; i++) w[i] = pow((double)i + 1.0, ex);
    for (int it = 0; it < 32 && cap; it++) {
        double tot = 0;
        for (uint32_t i = 0; i < n; i++) tot += w[i];
        const double lim = (double)cap * tot / n_edges;
        int clipped = 0;
        for (uint32_t i = 0; i < n; i++)
            if (w[i] > lim * (1 + 1e-12)) {
                w[i] = lim;
                clipped = 1;
            }
        if (!clipped) break;
    }
    double acc = 0;
    for (uint32_t i = 0; i < n; i++) {
        acc += w[i];
        w[i] = acc;
    }
    sd->cdf = w;
    return 0;
}

static uint32_t gen_side_draw(const gen_side* sd, gen_rng* r) {
    if (sd->uniform) return gen_below(r, sd->n);
    const double u = gen_u01(r) * sd->cdf[sd->n - 1];
    uint32_t lo = 0, hi = sd->n; /* first index with cdf > u */
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (sd->cdf[mid] > u)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo < sd->n ? lo : sd->n - 1;
}

/* open-addressing set of (row << 32 | col) keys */
typedef struct {
    uint64_t* slot;
    uint64_t mask, used;
} gen_set;

static int gen_set_init(gen_set* st, uint64_t want) {
    uint64_t cap = 1024;
    while (cap < want * 2) cap <<= 1;
    st->slot = (uint64_t*)malloc(sizeof(uint64_t) * cap);
    if (!st->slot) return -1;
    memset(st->slot, 0xFF, sizeof(uint64_t) * cap);
    st->mask = cap - 1;
    st->used = 0;
    return 0;
}

static int gen_set_insert(gen_set* st, uint64_t key);

static int gen_set_grow(gen_set* st) {
    uint64_t* old = st->slot;
    const uint64_t n = st->mask + 1;
    st->slot = (uint64_t*)malloc(sizeof(uint64_t) * n * 2);
    if (!st->slot) {
        st->slot = old;
        return -1;
    }
    memset(st->slot, 0xFF, sizeof(uint64_t) * n * 2);
    st->mask = n * 2 - 1;
    st->used = 0;
    for (uint64_t i = 0; i < n; i++)
        if (old[i] != ~0ULL) gen_set_insert(st, old[i]);
    free(old);
    return 0;
}

/* 1 = inserted, 0 = present */
static int gen_set_insert(gen_set* st, uint64_t key) {
    if ((st->used + 1) * 10 > (st->mask + 1) * 7) gen_set_grow(st);
    uint64_t h = fmix64(key) & st->mask;
    for (;;) {
        if (st->slot[h] == ~0ULL) {
            st->slot[h] = key;
            st->used++;
            return 1;
        }
        if (st->slot[h] == key) return 0;
        h = (h + 1) & st->mask;
    }
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

typedef struct {
    uint64_t* v;
    uint64_t n, cap;
} gen_vec;

static int gen_push(gen_vec* v, uint64_t x) {
    if (v->n == v->cap) {
        uint64_t nc = v->cap ? v->cap * 2 : 1024;
        uint64_t* p = (uint64_t*)realloc(v->v, sizeof(uint64_t) * nc);
        if (!p) return -1;
        v->v = p;
        v->cap = nc;
    }
    v->v[v->n++] = x;
    return 0;
}

static void gen_pick(gen_rng* r, uint32_t count, uint32_t n, uint32_t hubs, uint32_t* dst, uint32_t* m) {
    uint32_t tries = 0;
    *m = 0;
    while (*m < count && tries < 1000u * count) {
        tries++;
        const uint32_t v = ((uint64_t)*m * 2 < count) ? gen_below(r, hubs) : gen_below(r, n);
        int seen = 0;
        for (uint32_t i = 0; i < *m; i++)
            if (dst[i] == v) seen = 1;
        if (!seen) dst[(*m)++] = v;
    }
}

/* Returns 0 and malloc'd arrays row_ptr[n_rows+1], col_idx[*n_edges]
 * (free with oracle_free), -1 on bad arguments or allocation failure. */
ORACLE_API int oracle_generate(const oracle_gen* p, uint64_t** row_ptr, uint32_t** col_idx, uint64_t* n_edges) {
    *row_ptr = NULL;
    *col_idx = NULL;
    *n_edges = 0;
    if ((p->n_rows == 0 || p->n_cols == 0) && p->n_edges) return -1;
    const uint64_t maxe = (uint64_t)p->n_rows * p->n_cols;
    const uint64_t target = p->n_edges < maxe ? p->n_edges : maxe;
    gen_rng rng = {p->seed};
    gen_side rs, cs;
    const double te = (double)(target > 1 ? target : 1);
    if (gen_side_build(&rs, p->n_rows, p->gamma_rows, te, p->max_deg) ||
        gen_side_build(&cs, p->n_cols, p->gamma_cols, te, p->max_deg))
        return -1;
    gen_set set;
    if (gen_set_init(&set, target + (uint64_t)p->planted * p->planted_rows * p->planted_cols + 16)) return -1;
    gen_vec keys = {NULL, 0, 0};
    uint32_t* rdeg = (uint32_t*)calloc((size_t)p->n_rows + 1, sizeof(uint32_t));
    uint32_t* cdeg = (uint32_t*)calloc((size_t)p->n_cols + 1, sizeof(uint32_t));
    int rc = (rdeg && cdeg) ? 0 : -1;
    uint64_t draws = 0;
    const uint64_t max_draws = 64 * target + 1024;
    while (rc == 0 && keys.n < target && draws < max_draws) {
        draws++;
        const uint32_t r = gen_side_draw(&rs, &rng);
        const uint32_t c = gen_side_draw(&cs, &rng);
        if (p->max_deg && (rdeg[r] >= p->max_deg || cdeg[c] >= p->max_deg)) continue;
        const uint64_t k = ((uint64_t)r << 32) | c;
        if (gen_set_insert(&set, k)) {
            rc = gen_push(&keys, k);
            rdeg[r]++;
            cdeg[c]++;
        }
    }
    if (rc == 0 && p->planted && p->n_rows && p->n_cols) {
        const uint32_t hub_r = p->n_rows / 100 ? p->n_rows / 100 : 1, hub_c = p->n_cols / 100 ? p->n_cols / 100 : 1;
        const uint32_t pr = p->planted_rows < p->n_rows ? p->planted_rows : p->n_rows;
        const uint32_t pc = p->planted_cols < p->n_cols ? p->planted_cols : p->n_cols;
        uint32_t* rows = (uint32_t*)malloc(sizeof(uint32_t) * (pr + 1));
        uint32_t* cols = (uint32_t*)malloc(sizeof(uint32_t) * (pc + 1));
        if (!rows || !cols) rc = -1;
        for (uint32_t b = 0; rc == 0 && b < p->planted; b++) {
            uint32_t nr = 0, nc = 0;
            gen_pick(&rng, pr, p->n_rows, hub_r, rows, &nr);
            gen_pick(&rng, pc, p->n_cols, hub_c, cols, &nc);
            for (uint32_t i = 0; i < nr && rc == 0; i++)
                for (uint32_t j = 0; j < nc && rc == 0; j++)
                    if (gen_u01(&rng) < p->planted_density) {
                        const uint64_t k = ((uint64_t)rows[i] << 32) | cols[j];
                        if (gen_set_insert(&set, k)) rc = gen_push(&keys, k);
                    }
        }
        free(rows);
        free(cols);
    }
    free(rdeg);
    free(cdeg);
    free(set.slot);
    free(rs.cdf);
    free(cs.cdf);
    if (rc) {
        free(keys.v);
        return -1;
    }
    qsort(keys.v, keys.n, sizeof(uint64_t), cmp_u64);
    uint64_t* rp = (uint64_t*)calloc((size_t)p->n_rows + 1, sizeof(uint64_t));
    uint32_t* ci = (uint32_t*)malloc(sizeof(uint32_t) * (keys.n ? keys.n : 1));
    if (!rp || !ci) {
        free(rp);
        free(ci);
        free(keys.v);
        return -1;
    }
    for (uint64_t i = 0; i < keys.n; i++) {
        rp[(keys.v[i] >> 32) + 1]++;
        ci[i] = (uint32_t)keys.v[i];
    }
    for (uint32_t r = 0; r < p->n_rows; r++) rp[r + 1] += rp[r];
    free(keys.v);
    *row_ptr = rp;
    *col_idx = ci;
    *n_edges = rp[p->n_rows];
    return 0;
}

ORACLE_API void oracle_free(void* ptr) { free(ptr); }
