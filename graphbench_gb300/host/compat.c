/*
 * compat.c -- run_sspath_arr / run_sspath over the reference's t_csr
 * (include/gbsssp_compat.h), built as libgbsssp_compat.so on top of
 * libgbsssp.so.  Host C only: the computation is gbs_sssp on a cached
 * device copy of the graph.
 *
 * t_csr (include/graph.h:113-127): vet_idx[v] is the inclusive end of row v
 * (row v starts at vet_idx[v-1], 0 for v = 0, as in
 * sssp/csr_sspath_array.c:891-892), edge_idx[e] the target, and
 * edge_info[e].edge_weight the double weight.  Distances go to
 * vet_info[v].weight (INFINITY when unreached, as the reference initialises
 * them, :205-206).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gbsssp_compat.h"

#define CACHE_SLOTS 4
#define SAMPLE_POINTS 257

typedef struct {
    const t_csr *gs;
    const lint *vet_idx;
    const lint *edge_idx;
    const t_e *edge_info;
    lint v_size, e_size;
    uint64_t sample;
    gbs_graph *g;
    gbs_weight_type wt;
    uint64_t used;
} slot_t;

static slot_t g_cache[CACHE_SLOTS];
static uint64_t g_clock;
static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;
static int g_exit_on_error = 1;
static int g_allow_f32 = 0;
static gbs_status g_status = GBS_OK;
static char g_msg[512];

static uint64_t mix(uint64_t h, uint64_t x) {
    h ^= x + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    return h ^ (h >> 29);
}

/* A few hundred entries of every array, spread evenly: catches a different
 * graph placed at the same addresses, not every in-place edit. */
static uint64_t sample_hash(const t_csr *gs) {
    uint64_t h = mix((uint64_t)gs->v_size, (uint64_t)gs->e_size);
    for (int i = 0; i < SAMPLE_POINTS; ++i) {
        if (gs->v_size > 0) {
            const lint v = (lint)((double)i / (SAMPLE_POINTS - 1) * (double)(gs->v_size - 1));
            h = mix(h, (uint64_t)gs->vet_idx[v]);
        }
        if (gs->e_size > 0) {
            const lint e = (lint)((double)i / (SAMPLE_POINTS - 1) * (double)(gs->e_size - 1));
            uint64_t wb;
            memcpy(&wb, &gs->edge_info[e].edge_weight, 8);
            h = mix(mix(h, (uint64_t)gs->edge_idx[e]), wb);
        }
    }
    return h;
}

static int set_status(gbs_status st, const char *fn, const char *why) {
    g_status = st;
    if (st == GBS_OK) return 0;
    snprintf(g_msg, sizeof g_msg, "%s: %s (%s)", fn, gbs_status_string(st), why ? why : "");
    if (g_exit_on_error) {
        fprintf(stderr, "Error: %s\n", g_msg);
        fflush(stderr);
        exit(123);
    }
    return -1;
}

/* The weight type to run in: uint32 when every weight is an integer (exact,
 * the same sums as the reference's doubles), float32 when allowed and every
 * weight is float32-exact, float64 otherwise (the reference's arithmetic);
 * -1 for a negative or non-finite weight.  Integer weights whose path sums
 * reach 2^32 - 1 make the uint32 run report GBS_ERR_OVERFLOW; run_common
 * then converts the graph again in float64 (exact for integer sums below
 * 2^53, like the reference's doubles) and runs it there. */
static int weight_type_of(const t_csr *gs) {
    int all_int = 1, all_f32 = 1;
    for (lint e = 0; e < gs->e_size; ++e) {
        const double w = gs->edge_info[e].edge_weight;
        if (!(w >= 0.0) || isinf(w)) return -1;
        if (all_int && !(w == floor(w) && w <= 4294967294.0)) all_int = 0;
        if (all_f32 && (double)(float)w != w) all_f32 = 0;
    }
    if (all_int) return GBS_WEIGHT_U32;
    if (all_f32 && g_allow_f32) return GBS_WEIGHT_F32;
    return GBS_WEIGHT_F64;
}

static gbs_status convert(const t_csr *gs, int force_f64, gbs_graph **out, gbs_weight_type *wt_out,
                          const char **why) {
    const lint n = gs->v_size, m = gs->e_size;
    *why = "";
    if (n <= 0 || n >= 0x7FFFFFFFll) { *why = "v_size must be in [1, 2^31)"; return GBS_ERR_INVALID_ARG; }
    if (m < 0 || m >= 0xFFFFFFFFll) { *why = "e_size must be in [0, 2^32)"; return GBS_ERR_UNSUPPORTED; }
    if (!gs->vet_idx || (m && (!gs->edge_idx || !gs->edge_info))) { *why = "NULL CSR array"; return GBS_ERR_INVALID_ARG; }
    if (gs->vet_idx[n - 1] != m) { *why = "vet_idx[v_size-1] != e_size"; return GBS_ERR_INVALID_ARG; }
    int wt = weight_type_of(gs);
    if (wt < 0) {
        *why = "edge weights must be finite and >= 0";
        return GBS_ERR_INVALID_ARG;
    }
    if (force_f64) wt = GBS_WEIGHT_F64;
    const size_t wsize = wt == GBS_WEIGHT_F64 ? 8 : 4;
    uint64_t *row = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n + 1));
    uint32_t *col = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(m ? m : 1));
    unsigned char *w = (unsigned char *)malloc(wsize * (size_t)(m ? m : 1));
    gbs_status st = GBS_OK;
    if (!row || !col || !w) {
        st = GBS_ERR_NO_MEMORY;
        *why = "host conversion buffers";
        goto done;
    }
    row[0] = 0;
    for (lint v = 0; v < n; ++v) {
        const lint end = gs->vet_idx[v];
        if (end < (lint)row[v] || end > m) {
            st = GBS_ERR_INVALID_ARG;
            *why = "vet_idx must be non-decreasing inclusive row ends";
            goto done;
        }
        row[v + 1] = (uint64_t)end;
    }
    for (lint e = 0; e < m; ++e) {
        const lint c = gs->edge_idx[e];
        if (c < 0 || c >= n) {
            st = GBS_ERR_INVALID_ARG;
            *why = "edge_idx out of range";
            goto done;
        }
        col[e] = (uint32_t)c;
        const double d = gs->edge_info[e].edge_weight;
        if (wt == GBS_WEIGHT_U32) {
            const uint32_t u = (uint32_t)d;
            memcpy(w + 4 * (size_t)e, &u, 4);
        } else if (wt == GBS_WEIGHT_F32) {
            const float f = (float)d;
            memcpy(w + 4 * (size_t)e, &f, 4);
        } else {
            memcpy(w + 8 * (size_t)e, &d, 8);
        }
    }
    st = gbs_graph_create((uint32_t)n, (uint64_t)m, row, col, w, (gbs_weight_type)wt, out);
    if (st != GBS_OK) *why = gbs_last_error();
    *wt_out = (gbs_weight_type)wt;
done:
    free(row);
    free(col);
    free(w);
    return st;
}

/* Cached device graph of gs (called with g_mu held).  force_f64 replaces a
 * cached uint32 copy by a float64 one (after a uint32 overflow). */
static gbs_status lookup(const t_csr *gs, int force_f64, slot_t **hit, const char **why) {
    const uint64_t h = sample_hash(gs);
    slot_t *lru = &g_cache[0];
    for (int i = 0; i < CACHE_SLOTS; ++i) {
        slot_t *s = &g_cache[i];
        if (s->g && s->gs == gs && s->vet_idx == gs->vet_idx && s->edge_idx == gs->edge_idx &&
            s->edge_info == gs->edge_info && s->v_size == gs->v_size && s->e_size == gs->e_size &&
            s->sample == h) {
            if (force_f64 && s->wt != GBS_WEIGHT_F64) {
                gbs_graph_destroy(s->g);
                memset(s, 0, sizeof *s);
                lru = s;
                break;
            }
            s->used = ++g_clock;
            *hit = s;
            return GBS_OK;
        }
        if (!s->g || s->used < lru->used) lru = s;
        if (!s->g) break;
    }
    if (lru->g) {
        gbs_graph_destroy(lru->g);
        lru->g = NULL;
    }
    gbs_weight_type wt = GBS_WEIGHT_U32;
    gbs_graph *g = NULL;
    const gbs_status st = convert(gs, force_f64, &g, &wt, why);
    if (st != GBS_OK) return st;
    lru->gs = gs;
    lru->vet_idx = gs->vet_idx;
    lru->edge_idx = gs->edge_idx;
    lru->edge_info = gs->edge_info;
    lru->v_size = gs->v_size;
    lru->e_size = gs->e_size;
    lru->sample = h;
    lru->g = g;
    lru->wt = wt;
    lru->used = ++g_clock;
    *hit = lru;
    return GBS_OK;
}

/* Frees every node after the head of a predecessor list. */
static void list_clear(p_list head) {
    p_list e = head->next;
    while (e) {
        p_list nx = e->next;
        free(e);
        e = nx;
    }
    head->next = NULL;
}

/* Inserts right after the head, as the reference's add_list_one does
 * (structs/list.c). */
static int list_push(p_list head, lint u) {
    p_list e = (p_list)malloc(sizeof(t_list));
    if (!e) return -1;
    e->int_val = u;
    e->int_val1 = -1;
    e->double_val = -1;
    e->next = head->next;
    head->next = e;
    return 0;
}

static void run_common(const char *fn, t_csr *gs, p_list *predecesor, lint source, double delta, int all_tight) {
    pthread_mutex_lock(&g_mu);
    const char *why = "";
    slot_t *s = NULL;
    void *dist = NULL;
    int32_t *pred = NULL;
    lint *last = NULL;
    gbs_status st = GBS_OK;
    if (!gs) {
        st = GBS_ERR_INVALID_ARG;
        why = "gs is NULL";
        goto out;
    }
    if (source < 0 || source >= gs->v_size) {
        st = GBS_ERR_INVALID_ARG;
        why = "source out of range";
        goto out;
    }
    st = lookup(gs, 0, &s, &why);
    if (st != GBS_OK) goto out;
    const lint n = gs->v_size;
    dist = malloc(8 * (size_t)n);
    pred = (int32_t *)malloc(4 * (size_t)n);
    if (!dist || !pred) {
        st = GBS_ERR_NO_MEMORY;
        why = "host result buffers";
        goto out;
    }
    gbs_params p;
    memset(&p, 0, sizeof p);
    p.delta = delta > 0 ? delta : 0.0;   /* the bucket width, and the light bound (w <= delta) */
    p.light = -1.0;
    st = gbs_sssp(s->g, (uint32_t)source, &p, dist, pred, NULL);
    if (st == GBS_ERR_OVERFLOW && s->wt == GBS_WEIGHT_U32) {
        /* integer weights whose path sums do not fit uint32: the same graph
         * in float64, cached in place of the uint32 copy */
        st = lookup(gs, 1, &s, &why);
        if (st != GBS_OK) goto out;
        st = gbs_sssp(s->g, (uint32_t)source, &p, dist, pred, NULL);
    }
    if (st != GBS_OK) {
        why = gbs_last_error();
        goto out;
    }
    const int f32 = s->wt == GBS_WEIGHT_F32, f64 = s->wt == GBS_WEIGHT_F64;
    const uint32_t *du = (const uint32_t *)dist;
    const float *df = (const float *)dist;
    const double *dd = (const double *)dist;
    for (lint v = 0; v < n; ++v) {
        if (pred[v] < 0) gs->vet_info[v].weight = INFINITY;
        else gs->vet_info[v].weight = f64 ? dd[v] : (f32 ? (double)df[v] : (double)du[v]);
    }
    if (!predecesor) goto out;
    if (!all_tight) {
        for (lint v = 0; v < n; ++v) {
            if (pred[v] < 0 || v == source || !predecesor[v]) continue;
            list_clear(predecesor[v]);
            if (list_push(predecesor[v], pred[v])) {
                st = GBS_ERR_NO_MEMORY;
                why = "predecessor list node";
                goto out;
            }
        }
        goto out;
    }
    /* every tight in-edge, each predecessor once: the edge (u, v) is tight
     * when dist[u] + w == dist[v] in the weight type */
    last = (lint *)malloc(sizeof(lint) * (size_t)n);
    if (!last) {
        st = GBS_ERR_NO_MEMORY;
        why = "host scratch";
        goto out;
    }
    for (lint v = 0; v < n; ++v) {
        last[v] = -1;
        if (pred[v] >= 0 && predecesor[v]) list_clear(predecesor[v]);
    }
    for (lint u = 0; u < n; ++u) {
        if (pred[u] < 0) continue;
        const lint b = u == 0 ? 0 : gs->vet_idx[u - 1];
        const lint e_end = gs->vet_idx[u];
        for (lint e = b; e < e_end; ++e) {
            const lint v = gs->edge_idx[e];
            if (pred[v] < 0 || last[v] == u || !predecesor[v]) continue;
            const double w = gs->edge_info[e].edge_weight;
            int tight;
            if (f64) {
                volatile double sum = dd[u] + w;
                tight = sum == dd[v];
            } else if (f32) {
                volatile float sum = df[u] + (float)w;
                tight = sum == df[v];
            } else {
                tight = (uint64_t)du[u] + (uint64_t)w == (uint64_t)du[v];
            }
            if (!tight) continue;
            last[v] = u;
            if (list_push(predecesor[v], u)) {
                st = GBS_ERR_NO_MEMORY;
                why = "predecessor list node";
                goto out;
            }
        }
    }
out:
    free(dist);
    free(pred);
    free(last);
    pthread_mutex_unlock(&g_mu);
    set_status(st, fn, why);
}

void run_sspath_arr(t_csr *gs, p_list *predecesor, lint source, double delta) {
    run_common("run_sspath_arr", gs, predecesor, source, delta, 0);
}

void run_sspath(t_csr *gs, p_list *predecesor, lint source, double delta) {
    run_common("run_sspath", gs, predecesor, source, delta, 1);
}

void gbs_compat_forget(const t_csr *gs) {
    pthread_mutex_lock(&g_mu);
    for (int i = 0; i < CACHE_SLOTS; ++i) {
        if (g_cache[i].g && g_cache[i].gs == gs) {
            gbs_graph_destroy(g_cache[i].g);
            memset(&g_cache[i], 0, sizeof g_cache[i]);
        }
    }
    pthread_mutex_unlock(&g_mu);
}

void gbs_compat_forget_all(void) {
    pthread_mutex_lock(&g_mu);
    for (int i = 0; i < CACHE_SLOTS; ++i) {
        if (g_cache[i].g) gbs_graph_destroy(g_cache[i].g);
        memset(&g_cache[i], 0, sizeof g_cache[i]);
    }
    pthread_mutex_unlock(&g_mu);
}

void gbs_compat_allow_float32(int allow) { g_allow_f32 = allow != 0; }

void gbs_compat_set_exit(int exit_on_error) { g_exit_on_error = exit_on_error != 0; }

gbs_status gbs_compat_status(void) { return g_status; }

/* ------------------------------------------------------------ readers
 * graph/csr.c's readers with the parsing and CSR build on the GPU
 * (gbs_read_text / gbs_read_bin); the t_csr is filled exactly as the
 * reference fills it.  scan_csr_idx reads the whole file and keeps the edge
 * arrays for the read_graph_csr call that follows on the same t_csr.       */

/* The reference's OFFSET for binary targets (include/graph.h:28-32). */
#ifndef GBS_COMPAT_BIN_OFFSET
#define GBS_COMPAT_BIN_OFFSET 1
#endif

typedef struct {
    const t_csr *gs;
    uint32_t *col;
    double *w;
    uint64_t m;
} pending_t;
static pending_t g_pending;

static void *alloc64(size_t bytes) {
    void *p = NULL;
    if (posix_memalign(&p, 64, bytes ? bytes : 64) != 0) return NULL;
    return p;
}

static void join_path(char *out, size_t cap, const char *dir, const char *file) {
    snprintf(out, cap, "%s%s", dir ? dir : "", file ? file : "");
}

static int export_csr(gbs_device_csr *c, uint64_t **row, uint32_t **col, double **w, uint32_t *n, uint64_t *m) {
    gbs_status st = gbs_device_csr_info(c, n, m);
    if (st != GBS_OK) return st;
    *row = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)*n + 1));
    *col = (uint32_t *)malloc(sizeof(uint32_t) * (*m ? *m : 1));
    *w = (double *)malloc(sizeof(double) * (*m ? *m : 1));
    if (!*row || !*col || !*w) return GBS_ERR_NO_MEMORY;
    return gbs_device_csr_export(c, *row, *col, *w);
}

static void fill_rows(t_csr *graph, const uint64_t *row, uint32_t n, int bin) {
    graph->vet_idx = (lint *)alloc64(sizeof(lint) * (n ? n : 1));
    graph->vet_info = (t_vi *)alloc64(sizeof(t_vi) * (n ? n : 1));
    for (uint32_t v = 0; v < n; ++v) {
        const lint deg = (lint)(row[v + 1] - row[v]);
        graph->vet_idx[v] = (lint)row[v + 1];            /* inclusive end */
        /* scan_csr_idx (:163-168, :195-196) / read_csr_bin (:238-243) */
        graph->vet_info[v].weight = bin ? INFINITY : 1.0;
        graph->vet_info[v].wb = 0;
        graph->vet_info[v].recip = bin ? 0.0 : 1.0 / (double)deg;
        graph->vet_info[v].vet_deg = bin ? 0 : deg;
    }
}

static void fill_edges(t_csr *graph, const uint32_t *col, const double *w, uint64_t m) {
    const size_t cap = (size_t)(graph->e_size > (lint)m ? graph->e_size : (lint)m);
    graph->edge_idx = (lint *)alloc64(sizeof(lint) * (cap ? cap : 1));
    graph->edge_info = (t_e *)alloc64(sizeof(t_e) * (cap ? cap : 1));
    memset(graph->edge_idx, 0, sizeof(lint) * (cap ? cap : 1));
    memset(graph->edge_info, 0, sizeof(t_e) * (cap ? cap : 1));
    for (uint64_t e = 0; e < m; ++e) {
        graph->edge_idx[e] = (lint)col[e];
        graph->edge_info[e].edge_weight = w[e];
    }
}

void scan_csr_idx(t_csr *graph, char *file, char *dir, sint type) {
    char path[4096];
    join_path(path, sizeof path, dir, file);
    gbs_device_csr *c = NULL;
    gbs_ingest_info info;
    uint64_t *row = NULL;
    uint32_t *col = NULL, n = 0;
    double *w = NULL;
    uint64_t m = 0;
    gbs_status st = gbs_read_text(path, type ? GBS_DIR_SEND : GBS_DIR_RECV, &c, &info);
    if (st == GBS_OK) st = export_csr(c, &row, &col, &w, &n, &m);
    if (c) gbs_device_csr_destroy(c);
    if (st == GBS_OK) {
        graph->offset = info.offset;
        graph->v_size = info.v_num;
        graph->e_size = info.e_num;
        graph->global_v_size = info.g_v_size;
        fill_rows(graph, row, n, 0);
        pthread_mutex_lock(&g_mu);
        free(g_pending.col);
        free(g_pending.w);
        g_pending.gs = graph;
        g_pending.col = col;
        g_pending.w = w;
        g_pending.m = m;
        col = NULL;
        w = NULL;
        pthread_mutex_unlock(&g_mu);
    }
    free(row);
    free(col);
    free(w);
    set_status(st, "scan_csr_idx", st == GBS_OK ? NULL : gbs_last_error());
}

void read_graph_csr(t_csr *graph, char *file, char *dir, sint type) {
    pthread_mutex_lock(&g_mu);
    int have = g_pending.gs == graph && g_pending.col;
    pending_t p = g_pending;
    if (have) memset(&g_pending, 0, sizeof g_pending);
    pthread_mutex_unlock(&g_mu);
    gbs_status st = GBS_OK;
    if (!have) {   /* not preceded by scan_csr_idx on this t_csr: read again */
        char path[4096];
        join_path(path, sizeof path, dir, file);
        gbs_device_csr *c = NULL;
        gbs_ingest_info info;
        uint64_t *row = NULL;
        uint32_t n = 0;
        st = gbs_read_text(path, type ? GBS_DIR_SEND : GBS_DIR_RECV, &c, &info);
        if (st == GBS_OK) st = export_csr(c, &row, &p.col, &p.w, &n, &p.m);
        if (c) gbs_device_csr_destroy(c);
        free(row);
    }
    if (st == GBS_OK) fill_edges(graph, p.col, p.w, p.m);
    free(p.col);
    free(p.w);
    set_status(st, "read_graph_csr", st == GBS_OK ? NULL : gbs_last_error());
}

void read_csr_bin(t_csr *graph, char *file, char *dir, sint type, int myrank) {
    (void)myrank;
    char path[4096];
    join_path(path, sizeof path, dir, file);
    gbs_device_csr *c = NULL;
    gbs_ingest_info info;
    uint64_t *row = NULL;
    uint32_t *col = NULL, n = 0;
    double *w = NULL;
    uint64_t m = 0;
    gbs_status st = gbs_read_bin(path, type ? GBS_DIR_SEND : GBS_DIR_RECV, GBS_COMPAT_BIN_OFFSET, 0, &c, &info);
    if (st == GBS_OK) st = export_csr(c, &row, &col, &w, &n, &m);
    if (c) gbs_device_csr_destroy(c);
    if (st == GBS_OK) {
        graph->offset = info.offset;
        graph->v_size = info.v_num;
        graph->e_size = info.e_num;
        graph->global_v_size = info.g_v_size;
        fill_rows(graph, row, n, 1);
        fill_edges(graph, col, w, m);
    }
    free(row);
    free(col);
    free(w);
    set_status(st, "read_csr_bin", st == GBS_OK ? NULL : gbs_last_error());
}

/* ------------------------------------------------------------ run_bc
 * btwcentral/csr_bc.c:16-64: read the graph (read_csr_bin when the
 * program's `bin` flag is set, else the text reader, type SEND), Brandes over
 * every vertex as source on the GPU (gbs_bc), and the reference's printout.
 * The graph goes to the device straight from the device CSR. */
extern int bin __attribute__((weak));

void run_bc(char *file, char *dir) {
    char path[4096];
    join_path(path, sizeof path, dir, file);
    gbs_device_csr *c = NULL;
    gbs_ingest_info info;
    gbs_graph *g = NULL;
    double *bc = NULL;
    uint32_t n = 0;
    gbs_status st = (&bin && bin) ? gbs_read_bin(path, GBS_DIR_SEND, GBS_COMPAT_BIN_OFFSET, 0, &c, &info)
                                  : gbs_read_text(path, GBS_DIR_SEND, &c, &info);
    if (st == GBS_OK) st = gbs_device_csr_info(c, &n, NULL);
    if (st == GBS_OK) st = gbs_graph_from_device_csr(c, GBS_WEIGHT_F64, &g);
    if (c) gbs_device_csr_destroy(c);
    if (st == GBS_OK) {
        bc = (double *)malloc(sizeof(double) * (n ? n : 1));
        if (!bc) st = GBS_ERR_NO_MEMORY;
    }
    if (st == GBS_OK) st = gbs_bc(g, NULL, n, NULL, bc, NULL);
    if (st == GBS_OK) {
        printf("the final result for betweeness centrality is:\n");
        for (uint32_t i = 0; i < n; i++) printf("%lld:%lf ", (long long)i + 1, bc[i]);
        printf("\n");
    }
    if (g) gbs_graph_destroy(g);
    free(bc);
    set_status(st, "run_bc", st == GBS_OK ? NULL : gbs_last_error());
}
