/*
 * oracle/sparsity.c -- TEST INFRASTRUCTURE ONLY (the parity oracle).  Nothing
 * in the pyop2_gb300 product links or calls this file; tests and the CPU
 * baseline of bench.py do.
 *
 * Sequential CPU restatement of PyOP2's sparsity construction:
 *   pyop2/sparsity.pyx:178-405 (fill_with_zeros) walks, for every map pair
 *   and every iterated entity (and layer, when extruded), the block
 *   rmap[e,:] x cmap[e,:] and inserts it into a PETSc MATPREALLOCATOR; the
 *   diagonal is inserted first for i < min(nrow, ncol) (:214-219); composed
 *   maps are resolved innermost-last and skipped when negative (:249-281);
 *   extruded rows are rmap + roffset * ((layer + k + q) % nl - q % nl)
 *   (:361-374).  PETSc ignores negative indices and keeps, per row, the set
 *   of distinct columns: that set, sorted, is what this file produces.
 *
 * Build: oracle/build.py compiles it with gcc into oracle/_ref/liboracle.so.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    const int32_t *rmap, *cmap;   /* [nent_total, arity] of the outermost maps */
    int32_t rarity, carity;
    int64_t nent;                 /* entities iterated                         */
    int32_t region;               /* 1 bottom, 2 top, 3 interior facets, 4 all */
    int32_t nrc, ncc;             /* composed chain lengths                    */
    const int32_t *rc[8], *cc[8]; /* arity-1 inner maps, outermost first       */
    const int32_t *roff, *coff;   /* extruded offsets or NULL                  */
    const int32_t *rq, *cq;       /* offset quotients or NULL                  */
} oracle_pair;

typedef struct {
    int64_t nrows, ncols;
    int32_t set_diag, extruded, constant_layers, periodic;
    const int32_t *layers;
    int32_t npairs;
    const oracle_pair *pairs;
} oracle_sparsity;

/* Calls emit(row, col) for every inserted entry, in the reference's order. */
typedef void (*emit_fn)(void *ctx, int64_t r, int64_t c);

static int mod_term(int layer, int k, int q, int nl) {
    int eff = layer + k + q;
    return nl > 0 ? (eff % nl - q % nl) : (eff - q);
}

static int walk(const oracle_sparsity *S, emit_fn emit, void *ctx) {
    if (S->set_diag) {
        int64_t n = S->nrows < S->ncols ? S->nrows : S->ncols;
        for (int64_t i = 0; i < n; ++i) emit(ctx, i, i);
    }
    int32_t rv[512], cv[512];
    for (int p = 0; p < S->npairs; ++p) {
        const oracle_pair *P = &S->pairs[p];
        if (P->rarity * 2 > 512 || P->carity * 2 > 512) return -1;
        for (int64_t e = 0; e < P->nent; ++e) {
            int64_t re = e, ce = e;
            int skip = 0;
            for (int i = 0; i < P->nrc && !skip; ++i) {
                re = P->rc[P->nrc - 1 - i][re];
                if (re < 0) skip = 1;
            }
            for (int i = 0; i < P->ncc && !skip; ++i) {
                ce = P->cc[P->ncc - 1 - i][ce];
                if (ce < 0) skip = 1;
            }
            if (skip) continue;
            if (!S->extruded) {
                for (int i = 0; i < P->rarity; ++i)
                    for (int j = 0; j < P->carity; ++j) {
                        int64_t r = P->rmap[re * P->rarity + i], c = P->cmap[ce * P->carity + j];
                        if (r >= 0 && c >= 0) emit(ctx, r, c);
                    }
                continue;
            }
            const int32_t *L = S->constant_layers ? S->layers : S->layers + 2 * e;
            int ls = L[0], le = L[1] - 1;
            const int nl = le - ls;
            int tr = P->rarity, tc = P->carity;
            if (P->region == 1) le = ls + 1;
            else if (P->region == 2) ls = le - 1;
            else if (P->region == 3) {
                tr *= 2;
                tc *= 2;
                if (!S->periodic) le = le - 1;
            }
            for (int layer = ls; layer < le; ++layer) {
                for (int i = 0; i < tr; ++i) {
                    int k = i / P->rarity, ir = i % P->rarity;
                    int q = P->rq ? P->rq[ir] : 0;
                    rv[i] = P->rmap[re * P->rarity + ir] + P->roff[ir] * mod_term(layer, k, q, nl);
                }
                for (int j = 0; j < tc; ++j) {
                    int k = j / P->carity, jr = j % P->carity;
                    int q = P->cq ? P->cq[jr] : 0;
                    cv[j] = P->cmap[ce * P->carity + jr] + P->coff[jr] * mod_term(layer, k, q, nl);
                }
                for (int i = 0; i < tr; ++i)
                    for (int j = 0; j < tc; ++j)
                        if (rv[i] >= 0 && cv[j] >= 0) emit(ctx, rv[i], cv[j]);
            }
        }
    }
    return 0;
}

typedef struct {
    int64_t nrows, ncols;
    int64_t *count;   /* per-row candidate count or fill cursor */
    int32_t *buf;     /* candidates, row-major by start offsets  */
    const int64_t *start;
    int bad;
} ctx_t;

static void emit_count(void *v, int64_t r, int64_t c) {
    ctx_t *x = (ctx_t *)v;
    if (r >= x->nrows || c >= x->ncols) { x->bad = 1; return; }
    x->count[r]++;
}

static void emit_fill(void *v, int64_t r, int64_t c) {
    ctx_t *x = (ctx_t *)v;
    if (r >= x->nrows || c >= x->ncols) { x->bad = 1; return; }
    x->buf[x->start[r] + x->count[r]++] = (int32_t)c;
}

static int cmp_i32(const void *a, const void *b) {
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* Build the pattern.  rowptr[nrows+1] is written; *colidx is malloc'ed and
 * must be freed with oracle_free.  Returns 0, -1 (arity too large) or -2
 * (index out of range). */
int oracle_sparsity_build(const oracle_sparsity *S, int64_t *rowptr, int32_t **colidx,
                          int64_t *nnz) {
    ctx_t x;
    memset(&x, 0, sizeof x);
    x.nrows = S->nrows;
    x.ncols = S->ncols;
    x.count = (int64_t *)calloc((size_t)S->nrows + 1, sizeof(int64_t));
    if (walk(S, emit_count, &x) != 0) { free(x.count); return -1; }
    if (x.bad) { free(x.count); return -2; }
    int64_t *start = (int64_t *)malloc(sizeof(int64_t) * ((size_t)S->nrows + 1));
    start[0] = 0;
    for (int64_t r = 0; r < S->nrows; ++r) start[r + 1] = start[r] + x.count[r];
    x.buf = (int32_t *)malloc(sizeof(int32_t) * (size_t)(start[S->nrows] + 1));
    x.start = start;
    memset(x.count, 0, sizeof(int64_t) * ((size_t)S->nrows + 1));
    walk(S, emit_fill, &x);
    int64_t out = 0;
    rowptr[0] = 0;
    for (int64_t r = 0; r < S->nrows; ++r) {
        int32_t *row = x.buf + start[r];
        int64_t n = start[r + 1] - start[r];
        qsort(row, (size_t)n, sizeof(int32_t), cmp_i32);
        for (int64_t i = 0; i < n; ++i)
            if (i == 0 || row[i] != row[i - 1]) x.buf[out++] = row[i];
        rowptr[r + 1] = out;
    }
    *colidx = x.buf;
    *nnz = out;
    free(start);
    free(x.count);
    return 0;
}

void oracle_free(void *p) { free(p); }
