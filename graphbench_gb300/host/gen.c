/*
 * gen.c -- synthetic graph generators of libgbsssp (host C, pthreads).
 *
 * The reference reads Graph500 Kronecker edge lists (read_csr_bin,
 * graph/csr.c:211-299; README:18-21) and DIMACS-like text (scan_csr_idx /
 * read_graph_csr, graph/csr.c:4-202); no such file ships with it, so these
 * seeded generators stand in for them with the same R-MAT parameters.  The
 * generated CSR is deterministic for a given seed and independent of the
 * thread count:
 *
 *   mix64           splitmix64 finaliser
 *   key(s, t)       mix64(s * 0x100000001B3 + t)      (t: 1 R-MAT, 2 permutation,
 *                                                      3 weights, 4 sources)
 *   rnd(k, i)       mix64(k + i * 0xD1B54A32D192ED03)
 *   R-MAT level l of sample e: r = rnd(key1, e*scale + l) >> 32 picks quadrant
 *   (0,0) r < 2448131358, (0,1) r < 3264175144, (1,0) r < 4080218931, else
 *   (1,1), bits appended most-significant first; ids pass through
 *   x -> ((x*(p0|1) + p2) mod 2^s) ^ (.. >> (s/2+1)), then the same with
 *   p1, p3 (p_i = rnd(key2, i)); self loops dropped; both directions stored;
 *   duplicates removed; rows sorted by column.
 *   Weight of pair {a<b}: r = rnd(key3, a<<32 | b) >> 32; uint32: wmin + r %
 *   (wmax-wmin+1); float32: 1 + (r % 16367616) / 16384.
 */
#include "gbsssp.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static inline uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static inline uint64_t skey(uint64_t seed, uint64_t stream) {
    return mix64(seed * 0x100000001B3ull + stream);
}
static inline uint64_t rnd(uint64_t key, uint64_t i) {
    return mix64(key + i * 0xD1B54A32D192ED03ull);
}

/* ------------------------------------------------------------ threading */
typedef void (*range_fn)(void *ctx, uint64_t lo, uint64_t hi, int tid);
typedef struct { range_fn fn; void *ctx; uint64_t lo, hi; int tid; } par_job;

static void *par_trampoline(void *p) {
    par_job *j = (par_job *)p;
    j->fn(j->ctx, j->lo, j->hi, j->tid);
    return NULL;
}

static int gen_threads(void) {
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    if (c < 1) c = 1;
    if (c > 64) c = 64;
    return (int)c;
}

/* Splits [0, count) into nt contiguous ranges and runs fn on each. */
static void parallel_for(uint64_t count, int nt, range_fn fn, void *ctx) {
    if (nt <= 1 || count < 4096) { fn(ctx, 0, count, 0); return; }
    pthread_t th[64];
    par_job jobs[64];
    for (int t = 0; t < nt; t++) {
        jobs[t].fn = fn; jobs[t].ctx = ctx; jobs[t].tid = t;
        jobs[t].lo = count * (uint64_t)t / (uint64_t)nt;
        jobs[t].hi = count * (uint64_t)(t + 1) / (uint64_t)nt;
        if (pthread_create(&th[t], NULL, par_trampoline, &jobs[t]) != 0) {
            fn(ctx, jobs[t].lo, jobs[t].hi, t);
            th[t] = 0;
        }
    }
    for (int t = 0; t < nt; t++) if (th[t]) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------- pair -> CSR */
typedef struct {
    uint32_t n;
    const uint32_t *a, *b;   /* endpoint arrays, count entries, a[i]==b[i] skipped */
    uint64_t count;
    uint64_t *deg;           /* n+1, atomically counted */
    uint64_t *cursor;        /* n */
    uint32_t *adj;           /* scatter target */
    uint64_t *row;           /* offsets of the scattered (undeduped) rows */
    uint64_t *ndeg;          /* deduped degree */
    uint64_t *nrow;          /* deduped offsets */
    uint32_t *col;           /* final columns */
    void *w;
    gbs_weight_type wtype;
    uint32_t wmin, wmax;
    uint64_t wkey;
    uint32_t *tmp[64];       /* per-thread radix scratch */
    uint64_t tmp_len;
} csr_ctx;

static void count_fn(void *p, uint64_t lo, uint64_t hi, int tid) {
    csr_ctx *c = (csr_ctx *)p;
    (void)tid;
    for (uint64_t i = lo; i < hi; i++) {
        uint32_t a = c->a[i], b = c->b[i];
        if (a == b) continue;
        __atomic_fetch_add(&c->deg[a], 1, __ATOMIC_RELAXED);
        __atomic_fetch_add(&c->deg[b], 1, __ATOMIC_RELAXED);
    }
}

static void scatter_fn(void *p, uint64_t lo, uint64_t hi, int tid) {
    csr_ctx *c = (csr_ctx *)p;
    (void)tid;
    for (uint64_t i = lo; i < hi; i++) {
        uint32_t a = c->a[i], b = c->b[i];
        if (a == b) continue;
        uint64_t pa = __atomic_fetch_add(&c->cursor[a], 1, __ATOMIC_RELAXED);
        uint64_t pb = __atomic_fetch_add(&c->cursor[b], 1, __ATOMIC_RELAXED);
        c->adj[pa] = b;
        c->adj[pb] = a;
    }
}

static void sort_u32(uint32_t *x, uint64_t len, uint32_t *tmp, uint32_t nbits) {
    if (len <= 48) {
        for (uint64_t i = 1; i < len; i++) {
            uint32_t v = x[i];
            uint64_t j = i;
            while (j > 0 && x[j - 1] > v) { x[j] = x[j - 1]; j--; }
            x[j] = v;
        }
        return;
    }
    /* LSD radix sort, 8-bit digits over the bits that can be set */
    uint32_t *src = x, *dst = tmp;
    uint32_t passes = (nbits + 7) / 8;
    if (passes == 0) passes = 1;
    for (uint32_t p = 0; p < passes; p++) {
        uint64_t cnt[257];
        memset(cnt, 0, sizeof cnt);
        uint32_t sh = 8 * p;
        for (uint64_t i = 0; i < len; i++) cnt[((src[i] >> sh) & 255u) + 1]++;
        for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
        for (uint64_t i = 0; i < len; i++) dst[cnt[(src[i] >> sh) & 255u]++] = src[i];
        uint32_t *t = src; src = dst; dst = t;
    }
    if (src != x) memcpy(x, src, sizeof(uint32_t) * len);
}

static uint32_t bits_for(uint32_t n) {
    uint32_t b = 0;
    while (b < 32 && (1ull << b) < (uint64_t)n) b++;
    return b;
}

static void sort_unique_fn(void *p, uint64_t lo, uint64_t hi, int tid) {
    csr_ctx *c = (csr_ctx *)p;
    uint32_t nb = bits_for(c->n);
    for (uint64_t v = lo; v < hi; v++) {
        uint32_t *r = c->adj + c->row[v];
        uint64_t len = c->row[v + 1] - c->row[v];
        sort_u32(r, len, c->tmp[tid], nb);
        uint64_t k = 0;
        for (uint64_t i = 0; i < len; i++)
            if (k == 0 || r[k - 1] != r[i]) r[k++] = r[i];
        c->ndeg[v] = k;
    }
}

static void compact_fn(void *p, uint64_t lo, uint64_t hi, int tid) {
    csr_ctx *c = (csr_ctx *)p;
    (void)tid;
    for (uint64_t v = lo; v < hi; v++) {
        const uint32_t *r = c->adj + c->row[v];
        uint64_t o = c->nrow[v];
        uint64_t len = c->ndeg[v];
        for (uint64_t i = 0; i < len; i++) {
            uint32_t u = (uint32_t)v, x = r[i];
            uint32_t lo_ = u < x ? u : x, hi_ = u < x ? x : u;
            uint64_t h = rnd(c->wkey, ((uint64_t)lo_ << 32) | hi_) >> 32;
            c->col[o + i] = x;
            if (c->wtype == GBS_WEIGHT_U32)
                ((uint32_t *)c->w)[o + i] = c->wmin + (uint32_t)(h % ((uint64_t)c->wmax - c->wmin + 1));
            else
                ((float *)c->w)[o + i] = (float)(1.0 + (double)(h % 16367616ull) / 16384.0);
        }
    }
}

/* Symmetrise + dedup + sort rows + weights.  Takes ownership of nothing. */
static gbs_status pairs_to_csr(uint32_t n, const uint32_t *a, const uint32_t *b, uint64_t count,
                               uint64_t seed, gbs_weight_type wtype, uint32_t wmin, uint32_t wmax,
                               gbs_host_csr **out) {
    int nt = gen_threads();
    csr_ctx c;
    memset(&c, 0, sizeof c);
    c.n = n; c.a = a; c.b = b; c.count = count;
    c.wtype = wtype; c.wmin = wmin; c.wmax = wmax;
    c.wkey = skey(seed, 3);
    gbs_status st = GBS_OK;
    gbs_host_csr *g = (gbs_host_csr *)calloc(1, sizeof(gbs_host_csr));
    c.deg = (uint64_t *)calloc((size_t)n + 1, sizeof(uint64_t));
    c.row = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)n + 1));
    c.cursor = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)n + 1));
    c.ndeg = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)n + 1));
    if (!g || !c.deg || !c.row || !c.cursor || !c.ndeg) { st = GBS_ERR_NO_MEMORY; goto fail; }
    parallel_for(count, nt, count_fn, &c);
    c.row[0] = 0;
    for (uint32_t v = 0; v < n; v++) c.row[v + 1] = c.row[v] + c.deg[v];
    memcpy(c.cursor, c.row, sizeof(uint64_t) * n);
    c.adj = (uint32_t *)malloc(sizeof(uint32_t) * (c.row[n] ? c.row[n] : 1));
    if (!c.adj) { st = GBS_ERR_NO_MEMORY; goto fail; }
    parallel_for(count, nt, scatter_fn, &c);
    uint64_t maxdeg = 0;
    for (uint32_t v = 0; v < n; v++) if (c.deg[v] > maxdeg) maxdeg = c.deg[v];
    c.tmp_len = maxdeg ? maxdeg : 1;
    for (int t = 0; t < nt; t++) {
        c.tmp[t] = (uint32_t *)malloc(sizeof(uint32_t) * c.tmp_len);
        if (!c.tmp[t]) { st = GBS_ERR_NO_MEMORY; goto fail; }
    }
    parallel_for(n, nt, sort_unique_fn, &c);
    g->row_offsets = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)n + 1));
    if (!g->row_offsets) { st = GBS_ERR_NO_MEMORY; goto fail; }
    g->row_offsets[0] = 0;
    for (uint32_t v = 0; v < n; v++) g->row_offsets[v + 1] = g->row_offsets[v] + c.ndeg[v];
    g->n = n;
    g->m = g->row_offsets[n];
    g->wtype = wtype;
    g->cols = (uint32_t *)malloc(sizeof(uint32_t) * (g->m ? g->m : 1));
    g->weights = malloc(4 * (g->m ? g->m : 1));
    if (!g->cols || !g->weights) { st = GBS_ERR_NO_MEMORY; goto fail; }
    c.nrow = g->row_offsets; c.col = g->cols; c.w = g->weights;
    parallel_for(n, nt, compact_fn, &c);
    *out = g;
    g = NULL;
fail:
    for (int t = 0; t < 64; t++) free(c.tmp[t]);
    free(c.deg); free(c.row); free(c.cursor); free(c.ndeg); free(c.adj);
    if (g) gbs_host_csr_free(g);
    return st;
}

/* ------------------------------------------------------------- R-MAT */
typedef struct {
    uint32_t scale;
    uint64_t k1;
    uint64_t p[4];
    uint32_t *a, *b;
} rmat_ctx;

static inline uint32_t rmat_perm(const rmat_ctx *c, uint64_t x) {
    uint64_t mask = (c->scale >= 64) ? ~0ull : ((1ull << c->scale) - 1);
    uint32_t sh = c->scale / 2 + 1;
    x = (x * (c->p[0] | 1ull) + c->p[2]) & mask;
    x ^= x >> sh;
    x = (x * (c->p[1] | 1ull) + c->p[3]) & mask;
    x ^= x >> sh;
    return (uint32_t)x;
}

static void rmat_fn(void *p, uint64_t lo, uint64_t hi, int tid) {
    rmat_ctx *c = (rmat_ctx *)p;
    (void)tid;
    const uint32_t TA = 2448131358u, TB = 3264175144u, TC = 4080218931u;
    for (uint64_t e = lo; e < hi; e++) {
        uint64_t u = 0, v = 0;
        for (uint32_t l = 0; l < c->scale; l++) {
            uint32_t r = (uint32_t)(rnd(c->k1, e * c->scale + l) >> 32);
            uint32_t bu = r >= TB;
            uint32_t bv = (r >= TA && r < TB) || r >= TC;
            u = (u << 1) | bu;
            v = (v << 1) | bv;
        }
        c->a[e] = rmat_perm(c, u);
        c->b[e] = rmat_perm(c, v);
    }
}

gbs_status gbs_gen_rmat(uint32_t scale, uint32_t edgefactor, uint64_t seed,
                        gbs_weight_type wtype, uint32_t wmin, uint32_t wmax,
                        gbs_host_csr **out) {
    if (!out || scale < 1 || scale > 31 || edgefactor < 1 ||
        (wtype != GBS_WEIGHT_U32 && wtype != GBS_WEIGHT_F32) || wmin > wmax)
        return GBS_ERR_INVALID_ARG;
    uint64_t E = (uint64_t)edgefactor << scale;
    rmat_ctx c;
    c.scale = scale;
    c.k1 = skey(seed, 1);
    uint64_t k2 = skey(seed, 2);
    for (int i = 0; i < 4; i++) c.p[i] = rnd(k2, (uint64_t)i);
    c.a = (uint32_t *)malloc(sizeof(uint32_t) * E);
    c.b = (uint32_t *)malloc(sizeof(uint32_t) * E);
    if (!c.a || !c.b) { free(c.a); free(c.b); return GBS_ERR_NO_MEMORY; }
    parallel_for(E, gen_threads(), rmat_fn, &c);
    gbs_status st = pairs_to_csr(1u << scale, c.a, c.b, E, seed, wtype, wmin, wmax, out);
    free(c.a); free(c.b);
    return st;
}

gbs_status gbs_gen_grid(uint32_t rows, uint32_t cols, uint64_t seed,
                        gbs_weight_type wtype, uint32_t wmin, uint32_t wmax,
                        gbs_host_csr **out) {
    if (!out || rows < 1 || cols < 1 || (uint64_t)rows * cols > 0xFFFFFFFFull ||
        (wtype != GBS_WEIGHT_U32 && wtype != GBS_WEIGHT_F32) || wmin > wmax)
        return GBS_ERR_INVALID_ARG;
    uint64_t n = (uint64_t)rows * cols;
    uint64_t E = (uint64_t)rows * (cols - 1) + (uint64_t)(rows - 1) * cols;
    uint32_t *a = (uint32_t *)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint32_t *b = (uint32_t *)malloc(sizeof(uint32_t) * (E ? E : 1));
    if (!a || !b) { free(a); free(b); return GBS_ERR_NO_MEMORY; }
    uint64_t k = 0;
    for (uint64_t r = 0; r < rows; r++)
        for (uint64_t c = 0; c + 1 < cols; c++) { a[k] = (uint32_t)(r * cols + c); b[k] = a[k] + 1; k++; }
    for (uint64_t r = 0; r + 1 < rows; r++)
        for (uint64_t c = 0; c < cols; c++) { a[k] = (uint32_t)(r * cols + c); b[k] = a[k] + cols; k++; }
    gbs_status st = pairs_to_csr((uint32_t)n, a, b, E, seed, wtype, wmin, wmax, out);
    free(a); free(b);
    return st;
}

gbs_status gbs_sample_sources(const gbs_host_csr *g, uint32_t count, uint64_t seed,
                              uint32_t *out, uint32_t *got) {
    if (!g || !out || !got || g->n == 0) return GBS_ERR_INVALID_ARG;
    uint64_t key = skey(seed, 4);
    uint8_t *seen = (uint8_t *)calloc(g->n, 1);
    if (!seen) return GBS_ERR_NO_MEMORY;
    uint32_t k = 0;
    uint64_t limit = 64ull * count + 100000ull;
    for (uint64_t i = 0; k < count && i < limit; i++) {
        uint32_t v = (uint32_t)((rnd(key, i) >> 11) % g->n);
        if (g->row_offsets[v + 1] > g->row_offsets[v] && !seen[v]) {
            seen[v] = 1;
            out[k++] = v;
        }
    }
    free(seen);
    *got = k;
    return GBS_OK;
}

void gbs_host_csr_free(gbs_host_csr *g) {
    if (!g) return;
    free(g->row_offsets);
    free(g->cols);
    free(g->weights);
    free(g);
}
