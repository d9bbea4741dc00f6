/*
 * oracle.c -- CPU oracle for the delta-stepping SSSP path.  TEST INFRASTRUCTURE
 * ONLY: loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg as the checker.  The product library never links or calls it.
 *
 * What is restated here (reference paths relative to the GRAPHBENCH tree):
 *   - or_delta_stepping_{u32,f32}: the serial array delta-stepping of
 *     sssp/csr_sspath_array.c:149-363 (run_sspath_arr without USE_OMP) with
 *     its helpers request_arr_single (:941-961), remember_arr_single
 *     (:1019-1042) and relax_arr_single (:403-449), over the light/heavy split
 *     of graph/csr.c:74-130 (separate_csr: light iff w <= delta).  Buckets are
 *     tombstoned arrays with a per-vertex (bucket, position) index
 *     (include/array.h:3-10).  Defects D1 (vidx rewritten when the vertex does
 *     not move, :445-446), D2 (b_total not re-incremented when a vertex that
 *     was already moved to S is re-inserted, :426-434) and D4 (S/R sized by
 *     the edge count, :202-204) are fixed; D3 (uninitialised degrees) does not
 *     arise because the split is computed directly.  The distance type is the
 *     reference's double for uint32 weights (every path sum < 2^53 is exact)
 *     and float for float32 weights (fl32(d[u] + w) per relaxation).
 *   - or_dijkstra_{u32,f32}: binary-heap Dijkstra in the weight's own type, an
 *     independent cross-check of the same least fixpoint (the reference's own
 *     Dijkstra is sssp/csr_sspath.c:5-36, a list priority queue).
 *   - or_min_tight_pred_*: predecessor = smallest tight in-neighbour, i.e. the
 *     one edge the product's packed (dist<<32 | pred) atomicMin keeps.
 *   - or_count_tight_preds_* / or_fill_tight_preds_*: all tight predecessors,
 *     the set the list path keeps (sssp/csr_sspath.c:116-118) for betweenness.
 *
 * CSR convention: row[v]..row[v+1] (exclusive offsets, uint64), col uint32.
 * Unreached vertices: dist = UINT32_MAX (u32) / +inf (f32), pred = -1.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#define OR_UNREACHED_U32 0xFFFFFFFFu

/* ------------------------------------------------------------------ heap */
typedef struct { double key; uint32_t v; } or_hent;

typedef struct {
    or_hent *a;
    size_t n, cap;
} or_heap;

static int heap_push(or_heap *h, double key, uint32_t v) {
    if (h->n == h->cap) {
        size_t nc = h->cap ? h->cap * 2 : 1024;
        or_hent *na = (or_hent *)realloc(h->a, nc * sizeof(or_hent));
        if (!na) return -1;
        h->a = na; h->cap = nc;
    }
    size_t i = h->n++;
    while (i > 0) {
        size_t p = (i - 1) / 2;
        if (h->a[p].key <= key) break;
        h->a[i] = h->a[p];
        i = p;
    }
    h->a[i].key = key; h->a[i].v = v;
    return 0;
}

static or_hent heap_pop(or_heap *h) {
    or_hent top = h->a[0];
    or_hent last = h->a[--h->n];
    size_t i = 0;
    for (;;) {
        size_t c = 2 * i + 1;
        if (c >= h->n) break;
        if (c + 1 < h->n && h->a[c + 1].key < h->a[c].key) c++;
        if (h->a[c].key >= last.key) break;
        h->a[i] = h->a[c];
        i = c;
    }
    if (h->n) h->a[i] = last;
    return top;
}

/* ------------------------------------------------------------- Dijkstra */
/* Returns 0 on success, 1 if a path sum does not fit in 32 bits, -1 on OOM. */
int or_dijkstra_u32(uint32_t n, const uint64_t *row, const uint32_t *col,
                    const uint32_t *w, uint32_t src, uint32_t *dist) {
    uint64_t *d = (uint64_t *)malloc(sizeof(uint64_t) * (n ? n : 1));
    char *done = (char *)calloc(n ? n : 1, 1);
    or_heap h = {0};
    int rc = 0;
    if (!d || !done) { free(d); free(done); return -1; }
    for (uint32_t v = 0; v < n; v++) d[v] = UINT64_MAX;
    d[src] = 0;
    if (heap_push(&h, 0.0, src)) rc = -1;
    while (!rc && h.n) {
        or_hent t = heap_pop(&h);
        uint32_t u = t.v;
        if (done[u]) continue;
        done[u] = 1;
        for (uint64_t e = row[u]; e < row[u + 1]; e++) {
            uint64_t nd = d[u] + w[e];
            uint32_t v = col[e];
            if (nd < d[v]) {
                d[v] = nd;
                if (heap_push(&h, (double)nd, v)) { rc = -1; break; }
            }
        }
    }
    for (uint32_t v = 0; v < n && rc >= 0; v++) {
        if (d[v] == UINT64_MAX) dist[v] = OR_UNREACHED_U32;
        else if (d[v] >= OR_UNREACHED_U32) { rc = 1; dist[v] = OR_UNREACHED_U32; }
        else dist[v] = (uint32_t)d[v];
    }
    free(h.a); free(d); free(done);
    return rc;
}

int or_dijkstra_f32(uint32_t n, const uint64_t *row, const uint32_t *col,
                    const float *w, uint32_t src, float *dist) {
    char *done = (char *)calloc(n ? n : 1, 1);
    or_heap h = {0};
    int rc = 0;
    if (!done) return -1;
    for (uint32_t v = 0; v < n; v++) dist[v] = INFINITY;
    dist[src] = 0.0f;
    if (heap_push(&h, 0.0, src)) rc = -1;
    while (!rc && h.n) {
        or_hent t = heap_pop(&h);
        uint32_t u = t.v;
        if (done[u]) continue;
        done[u] = 1;
        float du = dist[u];
        for (uint64_t e = row[u]; e < row[u + 1]; e++) {
            volatile float nd = du + w[e]; /* one float32 rounding */
            uint32_t v = col[e];
            if (nd < dist[v]) {
                dist[v] = nd;
                if (heap_push(&h, (double)nd, v)) { rc = -1; break; }
            }
        }
    }
    free(h.a); free(done);
    return rc;
}

/* float64 weights: every relaxation rounds once in double, as the
 * reference's relax does (sssp/csr_sspath_array.c:419-421). */
int or_dijkstra_f64(uint32_t n, const uint64_t *row, const uint32_t *col,
                    const double *w, uint32_t src, double *dist) {
    char *done = (char *)calloc(n ? n : 1, 1);
    or_heap h = {0};
    int rc = 0;
    if (!done) return -1;
    for (uint32_t v = 0; v < n; v++) dist[v] = INFINITY;
    dist[src] = 0.0;
    if (heap_push(&h, 0.0, src)) rc = -1;
    while (!rc && h.n) {
        or_hent t = heap_pop(&h);
        uint32_t u = t.v;
        if (done[u]) continue;
        done[u] = 1;
        double du = dist[u];
        for (uint64_t e = row[u]; e < row[u + 1]; e++) {
            volatile double nd = du + w[e];
            uint32_t v = col[e];
            if (nd < dist[v]) {
                dist[v] = nd;
                if (heap_push(&h, nd, v)) { rc = -1; break; }
            }
        }
    }
    free(h.a); free(done);
    return rc;
}

/* --------------------------------------------------------- predecessors */
int or_min_tight_pred_u32(uint32_t n, const uint64_t *row, const uint32_t *col,
                          const uint32_t *w, uint32_t src, const uint32_t *dist,
                          int32_t *pred) {
    for (uint32_t v = 0; v < n; v++) pred[v] = -1;
    for (uint32_t u = 0; u < n; u++) {
        if (dist[u] == OR_UNREACHED_U32) continue;
        for (uint64_t e = row[u]; e < row[u + 1]; e++) {
            uint32_t v = col[e];
            if (v == src) continue;
            if ((uint64_t)dist[u] + w[e] == (uint64_t)dist[v]) {
                if (pred[v] < 0 || (uint32_t)pred[v] > u) pred[v] = (int32_t)u;
            }
        }
    }
    pred[src] = (int32_t)src;
    return 0;
}

int or_min_tight_pred_f32(uint32_t n, const uint64_t *row, const uint32_t *col,
                          const float *w, uint32_t src, const float *dist,
                          int32_t *pred) {
    for (uint32_t v = 0; v < n; v++) pred[v] = -1;
    for (uint32_t u = 0; u < n; u++) {
        if (isinf(dist[u])) continue;
        for (uint64_t e = row[u]; e < row[u + 1]; e++) {
            uint32_t v = col[e];
            if (v == src) continue;
            volatile float nd = dist[u] + w[e];
            if (nd == dist[v]) {
                if (pred[v] < 0 || (uint32_t)pred[v] > u) pred[v] = (int32_t)u;
            }
        }
    }
    pred[src] = (int32_t)src;
    return 0;
}

int or_min_tight_pred_f64(uint32_t n, const uint64_t *row, const uint32_t *col,
                          const double *w, uint32_t src, const double *dist,
                          int32_t *pred) {
    for (uint32_t v = 0; v < n; v++) pred[v] = -1;
    for (uint32_t u = 0; u < n; u++) {
        if (isinf(dist[u])) continue;
        for (uint64_t e = row[u]; e < row[u + 1]; e++) {
            uint32_t v = col[e];
            if (v == src) continue;
            volatile double nd = dist[u] + w[e];
            if (nd == dist[v]) {
                if (pred[v] < 0 || (uint32_t)pred[v] > u) pred[v] = (int32_t)u;
            }
        }
    }
    pred[src] = (int32_t)src;
    return 0;
}

/* Checks that every reached v != src has pred[v] = u with an edge (u, v) such
 * that dist[u] + w == dist[v] (computed in the weight type), that unreached
 * vertices have pred -1, and returns the number of violations. */
int64_t or_check_preds_u32(uint32_t n, const uint64_t *row, const uint32_t *col,
                           const uint32_t *w, uint32_t src, const uint32_t *dist,
                           const int32_t *pred) {
    int64_t bad = 0;
    for (uint32_t v = 0; v < n; v++) {
        if (v == src) continue;
        if (dist[v] == OR_UNREACHED_U32) { bad += (pred[v] != -1); continue; }
        int32_t p = pred[v];
        if (p < 0 || (uint32_t)p >= n || dist[p] == OR_UNREACHED_U32) { bad++; continue; }
        int ok = 0;
        for (uint64_t e = row[p]; e < row[p + 1]; e++)
            if (col[e] == v && (uint64_t)dist[p] + w[e] == dist[v]) { ok = 1; break; }
        bad += !ok;
    }
    return bad;
}

int64_t or_check_preds_f32(uint32_t n, const uint64_t *row, const uint32_t *col,
                           const float *w, uint32_t src, const float *dist,
                           const int32_t *pred) {
    int64_t bad = 0;
    for (uint32_t v = 0; v < n; v++) {
        if (v == src) continue;
        if (isinf(dist[v])) { bad += (pred[v] != -1); continue; }
        int32_t p = pred[v];
        if (p < 0 || (uint32_t)p >= n || isinf(dist[p])) { bad++; continue; }
        int ok = 0;
        for (uint64_t e = row[p]; e < row[p + 1]; e++) {
            volatile float nd = dist[p] + w[e];
            if (col[e] == v && nd == dist[v]) { ok = 1; break; }
        }
        bad += !ok;
    }
    return bad;
}

int64_t or_check_preds_f64(uint32_t n, const uint64_t *row, const uint32_t *col,
                           const double *w, uint32_t src, const double *dist,
                           const int32_t *pred) {
    int64_t bad = 0;
    for (uint32_t v = 0; v < n; v++) {
        if (v == src) continue;
        if (isinf(dist[v])) { bad += (pred[v] != -1); continue; }
        int32_t p = pred[v];
        if (p < 0 || (uint32_t)p >= n || isinf(dist[p])) { bad++; continue; }
        int ok = 0;
        for (uint64_t e = row[p]; e < row[p + 1]; e++) {
            volatile double nd = dist[p] + w[e];
            if (col[e] == v && nd == dist[v]) { ok = 1; break; }
        }
        bad += !ok;
    }
    return bad;
}

/* All tight predecessors (one entry per tight edge), grouped by target:
 * count pass fills cnt[v]; fill pass writes into out at off[v] (exclusive
 * prefix of cnt) in increasing source order. */
void or_count_tight_preds_f64(uint32_t n, const uint64_t *row, const uint32_t *col,
                              const double *w, uint32_t src, const double *dist,
                              uint64_t *cnt) {
    memset(cnt, 0, sizeof(uint64_t) * n);
    for (uint32_t u = 0; u < n; u++) {
        if (isinf(dist[u])) continue;
        for (uint64_t e = row[u]; e < row[u + 1]; e++) {
            uint32_t v = col[e];
            if (v != src && dist[u] + w[e] == dist[v]) cnt[v]++;
        }
    }
}

void or_fill_tight_preds_f64(uint32_t n, const uint64_t *row, const uint32_t *col,
                             const double *w, uint32_t src, const double *dist,
                             const uint64_t *off, uint64_t *cursor, uint32_t *out) {
    memcpy(cursor, off, sizeof(uint64_t) * n);
    for (uint32_t u = 0; u < n; u++) {
        if (isinf(dist[u])) continue;
        for (uint64_t e = row[u]; e < row[u + 1]; e++) {
            uint32_t v = col[e];
            if (v != src && dist[u] + w[e] == dist[v]) out[cursor[v]++] = u;
        }
    }
}

/* ------------------------------------------------- delta-stepping (serial) */
/* Bucket array: entries are vertex ids, -1 is a tombstone
 * (structs/array.c:91-96, remove_find_arr).  idx = next free slot,
 * num = live entries (include/array.h:12-48). */
typedef struct { int64_t *a; int64_t idx, num, cap; } or_arr;

static int arr_push(or_arr *b, int64_t v) {
    if (b->idx == b->cap) {
        int64_t nc = b->cap ? b->cap * 2 : 64;
        int64_t *na = (int64_t *)realloc(b->a, sizeof(int64_t) * nc);
        if (!na) return -1;
        b->a = na; b->cap = nc;
    }
    b->a[b->idx++] = v;
    b->num++;
    return 0;
}

typedef struct { int64_t src, dst; double w; } or_req;   /* (src, dst, w) triple */
typedef struct { or_req *a; int64_t n, cap; } or_reqs;

static int req_push(or_reqs *r, int64_t s, int64_t d, double w) {
    if (r->n == r->cap) {
        int64_t nc = r->cap ? r->cap * 2 : 1024;
        or_req *na = (or_req *)realloc(r->a, sizeof(or_req) * nc);
        if (!na) return -1;
        r->a = na; r->cap = nc;
    }
    r->a[r->n].src = s; r->a[r->n].dst = d; r->a[r->n].w = w;
    r->n++;
    return 0;
}

typedef struct {
    or_arr *B;
    int64_t nb;
} or_buckets;

static or_arr *bucket_at(or_buckets *bs, int64_t i) {
    if (i >= bs->nb) {
        int64_t nn = bs->nb ? bs->nb : 16;
        while (nn <= i) nn *= 2;
        or_arr *na = (or_arr *)realloc(bs->B, sizeof(or_arr) * nn);
        if (!na) return NULL;
        memset(na + bs->nb, 0, sizeof(or_arr) * (nn - bs->nb));
        bs->B = na; bs->nb = nn;
    }
    return &bs->B[i];
}

/* DIST_T is the accumulation type; ADD rounds once to DIST_T. */
#define OR_DS_BODY(DIST_T, WEIGHT_T)                                              \
    const double delta_recip = 1.0 / delta;                                       \
    or_buckets bs = {0};                                                          \
    or_arr S = {0};                                                               \
    or_reqs R = {0};                                                              \
    int64_t *vb = (int64_t *)malloc(sizeof(int64_t) * (n ? n : 1));               \
    int64_t *vp = (int64_t *)malloc(sizeof(int64_t) * (n ? n : 1));               \
    int rc = 0;                                                                   \
    if (!vb || !vp) { free(vb); free(vp); return -1; }                            \
    for (uint32_t v = 0; v < n; v++) { d[v] = (DIST_T)INFINITY; vb[v] = -1; vp[v] = -1; } \
    /* source goes to B[0] (csr_sspath_array.c:226-230) */                        \
    if (arr_push(bucket_at(&bs, 0), src)) rc = -1;                                \
    vb[src] = 0; vp[src] = 0;                                                     \
    d[src] = (DIST_T)0;                                                           \
    int64_t b_total = 1, iter = 0;                                                \
    while (!rc && b_total > 0) {                    /* :237 */                    \
        or_arr *Bi;                                                               \
        for (;;) {                                  /* :240 while(B[iter]->num>0) */\
            Bi = bucket_at(&bs, iter);                                            \
            if (!Bi) { rc = -1; break; }                                          \
            if (Bi->num <= 0) break;                                              \
            /* request_arr_single over the light graph (:941-961) */              \
            R.n = 0;                                                              \
            for (int64_t j = 0; j < Bi->idx && !rc; j++) {                        \
                int64_t q = Bi->a[j];                                             \
                if (q == -1) continue;                                            \
                for (uint64_t e = row[q]; e < row[q + 1]; e++)                    \
                    if ((double)w[e] <= delta)                                    \
                        if (req_push(&R, q, col[e], (double)w[e])) { rc = -1; break; } \
            }                                                                     \
            /* remember_arr_single (:1019-1042) */                                \
            for (int64_t j = 0; j < Bi->idx && !rc; j++) {                        \
                int64_t q = Bi->a[j];                                             \
                if (q == -1) continue;                                            \
                if (arr_push(&S, q)) { rc = -1; break; }                          \
                S.num--; /* S counts entries via idx only */                      \
                Bi->a[j] = -1;                                                    \
                vb[q] = -1; vp[q] = -1;                                           \
            }                                                                     \
            b_total -= Bi->num;                                                   \
            Bi->idx = 0; Bi->num = 0;                                             \
            OR_RELAX(DIST_T, WEIGHT_T)                                            \
        }                                                                         \
        if (rc) break;                                                            \
        /* heavy requests over S (:340-349) */                                    \
        R.n = 0;                                                                  \
        for (int64_t j = 0; j < S.idx && !rc; j++) {                              \
            int64_t q = S.a[j];                                                   \
            for (uint64_t e = row[q]; e < row[q + 1]; e++)                        \
                if ((double)w[e] > delta)                                         \
                    if (req_push(&R, q, col[e], (double)w[e])) { rc = -1; break; } \
        }                                                                         \
        if (rc) break;                                                            \
        OR_RELAX(DIST_T, WEIGHT_T)                                                \
        S.idx = 0; S.num = 0;                       /* empty_arr(S) :351 */       \
        iter++;                                                                   \
    }                                                                             \
    if (phases) *phases = iter;                                                   \
    for (int64_t i = 0; i < bs.nb; i++) free(bs.B[i].a);                          \
    free(bs.B); free(S.a); free(R.a); free(vb); free(vp);                         \
    return rc;

/* relax_arr_single (:403-449) with D1 and D2 fixed.  w is carried as double in
 * the request (as in the reference's t_arr_elem.double_val) and converted to
 * the accumulation type before the add. */
#define OR_RELAX(DIST_T, WEIGHT_T)                                                \
    for (int64_t i = 0; i < R.n && !rc; i++) {                                    \
        int64_t s = R.a[i].src, t = R.a[i].dst;                                   \
        DIST_T ori = d[t];                                                        \
        volatile DIST_T nv = d[s] + (DIST_T)R.a[i].w;                             \
        if (nv <= ori) {                                                          \
            d[t] = nv;                                                            \
            int64_t nbk = (int64_t)((double)nv * delta_recip);                    \
            if (!isinf((double)ori)) {                                            \
                int64_t ob = vb[t];                                               \
                if (ob != nbk) {                                                  \
                    if (vp[t] != -1) {                                            \
                        bs.B[ob].a[vp[t]] = -1;                                   \
                        bs.B[ob].num--;                                           \
                    } else {                                                      \
                        b_total++;              /* D2 fix */                      \
                    }                                                             \
                    or_arr *nb_ = bucket_at(&bs, nbk);                            \
                    if (!nb_ || arr_push(nb_, t)) { rc = -1; break; }             \
                    vb[t] = nbk; vp[t] = nb_->idx - 1;   /* D1 fix: only on move */ \
                }                                                                 \
            } else {                                                              \
                or_arr *nb_ = bucket_at(&bs, nbk);                                \
                if (!nb_ || arr_push(nb_, t)) { rc = -1; break; }                 \
                b_total++;                                                        \
                vb[t] = nbk; vp[t] = nb_->idx - 1;                                \
            }                                                                     \
        }                                                                         \
    }

/* Returns 0 on success, -1 on allocation failure.  *phases = buckets walked. */
int or_delta_stepping_u32(uint32_t n, const uint64_t *row, const uint32_t *col,
                          const uint32_t *w, uint32_t src, double delta,
                          double *d, int64_t *phases) {
    OR_DS_BODY(double, uint32_t)
}

int or_delta_stepping_f32(uint32_t n, const uint64_t *row, const uint32_t *col,
                          const float *w, uint32_t src, double delta,
                          float *d, int64_t *phases) {
    OR_DS_BODY(float, float)
}

/* Same algorithm over double weights (the reference's own edge type). */
int or_delta_stepping_f64(uint32_t n, const uint64_t *row, const uint32_t *col,
                          const double *w, uint32_t src, double delta,
                          double *d, int64_t *phases) {
    OR_DS_BODY(double, double)
}

/* ------------------------------------------------ betweenness centrality */
/* Brandes over shortest paths, after btwcentral/csr_bc.c:16-123: for every
 * source, vertices in increasing distance order (csr_bc.c:43-49, q_sort of
 * the distances; ties broken by vertex id here), path counts
 * sigma[w] = sum of sigma over the tight predecessors of w (comp_num_spath,
 * :69-91), then in decreasing order the dependencies
 * delta[v] = sum over tight out-edges (v, w) of (1 + delta[w]) * sigma[v] /
 * sigma[w] (comp_delta, :93-116, each term with its order of operations), and
 * bc[v] += delta[v] for v != source (:54-58).  The tight edges are counted
 * once each (the reference's list path can hold a predecessor twice).  Path
 * counts are 64-bit sums that wrap like the reference's lint.  Weights must be
 * positive so that a predecessor's distance is strictly smaller.
 *
 * Summation order of delta[v] (floating point, so it is fixed here): the row
 * of v sorted by (weight, column) keeps its CSR positions row[v] ..
 * row[v+1]-1, grouped in 32-position words (position / 32).  A word's sum is
 * the butterfly of its 32 slots (slot = position % 32; 0 for positions of
 * other rows and for edges that are not tight): for h = 16, 8, 4, 2, 1,
 * s[i] = s[i] + s[i + h] for i < h, giving s[0].  The row's words, numbered
 * from its first word, form blocks of 32; each block's word sums are combined
 * by the same butterfly, and the block sums are added in block order starting
 * from 0.  (The reference adds the terms into delta[v] one by one in the
 * order of its distance sort; sums in different orders differ in the last
 * bits.) */
typedef struct { double d; uint32_t v; } or_dv;
static int cmp_dv(const void *a, const void *b) {
    const or_dv *x = (const or_dv *)a, *y = (const or_dv *)b;
    if (x->d < y->d) return -1;
    if (x->d > y->d) return 1;
    return (x->v > y->v) - (x->v < y->v);
}
static double or_butterfly32(double *v) {
    for (int h = 16; h > 0; h >>= 1)
        for (int i = 0; i < h; i++) v[i] = v[i] + v[i + h];
    return v[0];
}
typedef struct { double w; uint32_t c; } or_wc;
static int cmp_wc(const void *a, const void *b) {
    const or_wc *x = (const or_wc *)a, *y = (const or_wc *)b;
    if (x->w < y->w) return -1;
    if (x->w > y->w) return 1;
    return (x->c > y->c) - (x->c < y->c);
}

#define OR_BC_BODY(DT, WT, DIJKSTRA, TIGHT, INF_TEST)                                     \
    const uint64_t m = row[n];                                                            \
    uint32_t *scol = (uint32_t *)malloc(sizeof(uint32_t) * (m ? m : 1));                  \
    WT *sw = (WT *)malloc(sizeof(WT) * (m ? m : 1));                                      \
    or_wc *tmp = (or_wc *)malloc(sizeof(or_wc) * (m ? m : 1));                            \
    DT *dist = (DT *)malloc(sizeof(DT) * n);                                              \
    uint64_t *sig = (uint64_t *)malloc(8 * (size_t)n);                                    \
    double *del = (double *)malloc(8 * (size_t)n);                                        \
    or_dv *ord = (or_dv *)malloc(sizeof(or_dv) * n);                                      \
    int rc = 0;                                                                           \
    if (!scol || !sw || !tmp || !dist || !sig || !del || !ord) rc = -1;                   \
    for (uint32_t v = 0; v < n && !rc; v++) bc[v] = 0.0;                                  \
    /* rows sorted by (weight, column) at their own positions */                          \
    for (uint32_t u = 0; u < n && !rc; u++) {                                             \
        const uint64_t b = row[u], d = row[u + 1] - row[u];                               \
        for (uint64_t i = 0; i < d; i++) {                                                \
            tmp[b + i].w = (double)w[b + i];                                              \
            tmp[b + i].c = col[b + i];                                                    \
        }                                                                                 \
        qsort(tmp + b, d, sizeof(or_wc), cmp_wc);                                         \
        for (uint64_t i = 0; i < d; i++) {                                                \
            scol[b + i] = tmp[b + i].c;                                                   \
            sw[b + i] = (WT)tmp[b + i].w;                                                 \
        }                                                                                 \
    }                                                                                     \
    for (uint32_t k = 0; k < nsrc && !rc; k++) {                                          \
        const uint32_t s = srcs ? srcs[k] : k;                                            \
        if (DIJKSTRA(n, row, col, w, s, dist)) { rc = -1; break; }                        \
        for (uint32_t v = 0; v < n; v++) {                                                \
            ord[v].d = INF_TEST(dist[v]) ? INFINITY : (double)dist[v];                    \
            ord[v].v = v;                                                                 \
            sig[v] = 0;                                                                   \
            del[v] = 0.0;                                                                 \
        }                                                                                 \
        qsort(ord, n, sizeof(or_dv), cmp_dv);                                             \
        sig[s] = 1;                                                                       \
        for (uint32_t i = 0; i < n; i++) {                                                \
            const uint32_t x = ord[i].v;                                                  \
            if (INF_TEST(dist[x])) continue;                                              \
            for (uint64_t e = row[x]; e < row[x + 1]; e++)                                \
                if (TIGHT(dist[x], sw[e], dist[scol[e]])) sig[scol[e]] += sig[x];         \
        }                                                                                 \
        for (uint32_t i = n; i-- > 0;) {                                                  \
            const uint32_t x = ord[i].v;                                                  \
            if (x == s || INF_TEST(dist[x]) || row[x] == row[x + 1]) continue;            \
            const double sx = (double)(int64_t)sig[x];                                    \
            const uint64_t wb = row[x] / 32, nw = (row[x + 1] - 1) / 32 + 1 - wb;         \
            double acc = 0.0;                                                             \
            for (uint64_t b = 0; b * 32 < nw; b++) {                                      \
                double q[32];                                                             \
                for (int j = 0; j < 32; j++) {                                            \
                    q[j] = 0.0;                                                           \
                    if (b * 32 + j >= nw) continue;                                       \
                    const uint64_t W = wb + b * 32 + j;                                   \
                    double t[32];                                                         \
                    for (int i = 0; i < 32; i++) {                                        \
                        const uint64_t e = W * 32 + i;                                    \
                        t[i] = 0.0;                                                       \
                        if (e < row[x] || e >= row[x + 1]) continue;                      \
                        const uint32_t y = scol[e];                                       \
                        if (TIGHT(dist[x], sw[e], dist[y]))                               \
                            t[i] = (1.0 + del[y]) * sx / (double)(int64_t)sig[y];         \
                    }                                                                     \
                    q[j] = or_butterfly32(t);                                             \
                }                                                                         \
                acc += or_butterfly32(q);                                                 \
            }                                                                             \
            del[x] = acc;                                                                 \
        }                                                                                 \
        for (uint32_t v = 0; v < n; v++)                                                  \
            if (v != s) bc[v] += del[v];                                                  \
    }                                                                                     \
    free(scol); free(sw); free(tmp); free(dist); free(sig); free(del); free(ord);         \
    return rc;

#define OR_TIGHT_U32(du, w, dv) ((dv) != OR_UNREACHED_U32 && (uint64_t)(du) + (w) == (uint64_t)(dv))
#define OR_INF_U32(d) ((d) == OR_UNREACHED_U32)
static int or_tight_f32(float du, float w, float dv) { volatile float s = du + w; return s == dv; }
static int or_tight_f64(double du, double w, double dv) { volatile double s = du + w; return s == dv; }
#define OR_INF_FP(d) (isinf(d))

int or_bc_u32(uint32_t n, const uint64_t *row, const uint32_t *col, const uint32_t *w, uint32_t nsrc,
              const uint32_t *srcs, double *bc) {
    OR_BC_BODY(uint32_t, uint32_t, or_dijkstra_u32, OR_TIGHT_U32, OR_INF_U32)
}
int or_bc_f32(uint32_t n, const uint64_t *row, const uint32_t *col, const float *w, uint32_t nsrc,
              const uint32_t *srcs, double *bc) {
    OR_BC_BODY(float, float, or_dijkstra_f32, or_tight_f32, OR_INF_FP)
}
int or_bc_f64(uint32_t n, const uint64_t *row, const uint32_t *col, const double *w, uint32_t nsrc,
              const uint32_t *srcs, double *bc) {
    OR_BC_BODY(double, double, or_dijkstra_f64, or_tight_f64, OR_INF_FP)
}

/* ------------------------------------------------------------ PageRank */
/* The reference's PageRank iteration (pagerank/pagerank_mpi.c:667-1043 on
 * one node; constants RDM_JMP 0.3 and THRESH 1e-6, include/graph.h:17-18):
 * weight[v] = 1 (init_weight, :64-68), recip[v] = 1 / out-degree(v) (the
 * partitioner's recip files, partition/csr_partition_bin_mpi.c:227),
 * wb[v] = rj, diff[v] = weight[v] * recip[v] (:752-754); every iteration
 *   wb[v] += (1 - rj) * diff[u] over the in-edges u of v       (:879-890)
 *   diff[v] = (wb[v] - weight[v]) * recip[v]                   (:995-997)
 *   done unless some |diff[v]| > thresh; weight[v] = wb[v]      (:998-1002)
 * row/col: the IN-edge CSR (row v lists the u with an edge u -> v).
 * Summation order of the per-iteration increment of wb[v] (fixed here; the
 * reference adds straight into wb[v] in row order): the row keeps its CSR
 * positions, grouped in 32-position words; a word's terms are added from the
 * lowest position up starting from 0; the row's words, numbered from its first
 * word, form blocks of 32 whose word sums are combined by the butterfly
 * (h = 16..1: s[i] += s[i + h]); the block sums are added in order from 0;
 * wb[v] += that sum.  Returns the iterations taken (< 0 on error). */
int or_pagerank(uint32_t n, const uint64_t *row, const uint32_t *col, double rj, double thresh,
                uint32_t max_iters, double *weight_out) {
    const double pj = 1.0 - rj;
    double *weight = weight_out, *wb = (double *)malloc(8 * (size_t)n);
    double *recip = (double *)malloc(8 * (size_t)n), *diff = (double *)malloc(8 * (size_t)n);
    double *nd = (double *)malloc(8 * (size_t)n);
    uint64_t *outdeg = (uint64_t *)calloc((size_t)n, 8);
    if (!wb || !recip || !diff || !nd || !outdeg) return -1;
    for (uint64_t e = 0; e < row[n]; e++) outdeg[col[e]]++;
    for (uint32_t v = 0; v < n; v++) {
        weight[v] = 1.0;
        recip[v] = 1.0 / (double)outdeg[v];
        wb[v] = rj;
        diff[v] = weight[v] * recip[v];
    }
    uint32_t it = 0;
    for (;;) {
        it++;
        int done = 1;
        for (uint32_t v = 0; v < n; v++) {
            double acc = 0.0;
            if (row[v + 1] > row[v]) {
                const uint64_t wb0 = row[v] / 32, nw = (row[v + 1] - 1) / 32 + 1 - wb0;
                for (uint64_t b = 0; b * 32 < nw; b++) {
                    double q[32];
                    for (int j = 0; j < 32; j++) {
                        q[j] = 0.0;
                        if (b * 32 + j >= nw) continue;
                        const uint64_t W = wb0 + b * 32 + j;
                        const uint64_t lo = W * 32 > row[v] ? W * 32 : row[v];
                        const uint64_t hi = W * 32 + 32 < row[v + 1] ? W * 32 + 32 : row[v + 1];
                        double p = 0.0;
                        for (uint64_t e = lo; e < hi; e++) p += pj * diff[col[e]];
                        q[j] = p;
                    }
                    acc += or_butterfly32(q);
                }
            }
            wb[v] += acc;
            nd[v] = (wb[v] - weight[v]) * recip[v];
        }
        for (uint32_t v = 0; v < n; v++) {
            if (fabs(nd[v]) > thresh) done = 0;
            weight[v] = wb[v];
            diff[v] = nd[v];
        }
        if (done || it >= max_iters) break;
    }
    free(wb); free(recip); free(diff); free(nd); free(outdeg);
    return (int)it;
}
