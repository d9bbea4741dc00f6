/*
 * ref_driver.c -- calls the reference's own SSSP entry points on an in-memory
 * CSR.  TEST INFRASTRUCTURE ONLY (linked into oracle/_ref/libref_*.so next to
 * the patched reference sources; see oracle/build_ref.py).
 *
 * It plays the role of main/main.c:205-225: it defines the CLI globals the
 * reference declares extern (include/graph.h:79-92, values as in
 * main/main.c:8-22), fills a t_csr (include/graph.h:113-127) with inclusive
 * end offsets, and calls run_sspath_arr (sssp/csr_sspath_array.c:149) or
 * run_sspath (sssp/csr_sspath.c:38).  The reference never frees what it
 * allocates and keeps file-scope state (`iter`, :15), so each call runs in a
 * forked child; distances come back through a shared mapping.  The child also
 * works in a scratch directory holding ./data/log, which the reference opens
 * unconditionally (:163-164, csr_sspath.c:43-44).
 */
#include "graph.h"
#include "list.h"
#include <stdint.h>
#include <unistd.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <sys/wait.h>
#include <time.h>

/* main/main.c:8-22 */
sint num_threads = 1;
sint num_nodes = 1;
int is_bin = 1;
lint g_v_num = 1;
int g_e_num = 1;
char *par_extend = "parex/";
char *data_extend = "datex/";
char *idx_extend = "idxex/";
char *base_dir = "./";
char *nodes_extension = "";
int bin = 0;
int buck_size = 10;
sint use_partition = FALSE;
int buff_size = 10000;
lint prefetch_dis = 10;

int gbref_log_buckets = 0;
double gbref_cap_mult = 2.0;

extern lint iter; /* sssp/csr_sspath_array.c:15, never reset by the reference */
void run_sspath_arr(t_csr *gs, p_list *predecesor, lint source, double delta);

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static t_csr *make_csr(int64_t n, int64_t m, const int64_t *row, const int64_t *col,
                       const double *w) {
    t_csr *gs = (t_csr *)calloc(1, sizeof(t_csr));
    gs->v_size = n;
    gs->e_size = m;
    gs->offset = 1;
    gs->csr_type = SEND;
    gs->global_v_size = n;
    gs->vet_idx = (lint *)_mm_malloc(sizeof(lint) * (n ? n : 1), 64);
    gs->vet_info = (t_vi *)_mm_malloc(sizeof(t_vi) * (n ? n : 1), 64);
    gs->edge_idx = (lint *)_mm_malloc(sizeof(lint) * (m ? m : 1), 64);
    gs->edge_info = (t_e *)_mm_malloc(sizeof(t_e) * (m ? m : 1), 64);
    for (int64_t v = 0; v < n; v++) {
        gs->vet_idx[v] = row[v + 1];           /* inclusive end offset */
        gs->vet_info[v].weight = INFINITY;
        gs->vet_info[v].vet_deg = row[v + 1] - row[v];
    }
    for (int64_t e = 0; e < m; e++) {
        gs->edge_idx[e] = col[e];
        gs->edge_info[e].node_id = 0;
        gs->edge_info[e].edge_weight = w[e];
    }
    return gs;
}

typedef struct {
    double seconds;
    int32_t status;
    int64_t pred_total;
} ref_result;

static int enter_scratch(char *dirbuf, size_t len) {
    snprintf(dirbuf, len, "/tmp/gbref_XXXXXX");
    if (!mkdtemp(dirbuf)) return -1;
    if (chdir(dirbuf) != 0) return -1;
    mkdir("data", 0755);
    mkdir("data/log", 0755);
    return 0;
}

static void quiet_stdout(void) {
    int fd = open("/dev/null", O_WRONLY);
    if (fd >= 0) { dup2(fd, 1); close(fd); }
}

/*
 * run_sspath_arr on (row, col, w) from `src` with bucket width `delta`.
 * threads: OpenMP team size (the OpenMP build honours it, the serial one
 * ignores it).  buckets: the reference's fixed bucket count (it has no bounds
 * check; the caller sizes it as floor(maxdist/delta)+2).  dist_out receives
 * gs->vet_info[v].weight.  Returns 0, or a negative code if the child failed.
 */
int gbref_sssp_arr(int64_t n, int64_t m, const int64_t *row, const int64_t *col,
                   const double *w, int64_t src, double delta, int threads,
                   int buckets, double cap_mult, double *dist_out, double *seconds) {
    size_t dist_bytes = sizeof(double) * (size_t)(n ? n : 1);
    size_t map_bytes = sizeof(ref_result) + dist_bytes;
    void *map = mmap(NULL, map_bytes, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
    if (map == MAP_FAILED) return -10;
    ref_result *res = (ref_result *)map;
    double *dist = (double *)((char *)map + sizeof(ref_result));
    res->status = -1;
    fflush(NULL);
    pid_t pid = fork();
    if (pid < 0) { munmap(map, map_bytes); return -11; }
    if (pid == 0) {
        char dir[64];
        if (enter_scratch(dir, sizeof dir) != 0) _exit(3);
        quiet_stdout();
        num_threads = threads > 0 ? threads : 1;
        buck_size = buckets;
        gbref_cap_mult = cap_mult;
        iter = 0;
        t_csr *gs = make_csr(n, m, row, col, w);
        p_list *pred = (p_list *)malloc(sizeof(p_list) * (n ? n : 1));
        for (int64_t v = 0; v < n; v++) {
            pred[v] = (p_list)malloc(sizeof(t_list));
            creat_list(pred[v]);
        }
        double t0 = now_s();
        run_sspath_arr(gs, pred, src, delta);
        double t1 = now_s();
        for (int64_t v = 0; v < n; v++) dist[v] = gs->vet_info[v].weight;
        res->seconds = t1 - t0;
        res->status = 0;
        unlink("data/log/plog");
        rmdir("data/log");
        rmdir("data");
        if (chdir("/tmp") == 0) rmdir(dir);
        _exit(0);
    }
    int st = 0;
    waitpid(pid, &st, 0);
    int rc = 0;
    if (!WIFEXITED(st) || WEXITSTATUS(st) != 0 || res->status != 0) {
        rc = WIFSIGNALED(st) ? -100 - WTERMSIG(st) : -12;
    } else {
        memcpy(dist_out, dist, sizeof(double) * (size_t)n);
        if (seconds) *seconds = res->seconds;
    }
    munmap(map, map_bytes);
    return rc;
}

/*
 * run_sspath (the list variant that BC calls, btwcentral/csr_bc.c:43) with
 * its predecessor lists.  It allocates 1000 buckets (sssp/csr_sspath.c:45-49),
 * so the caller must keep maxdist/delta below 1000.  pred_cnt[v] gets the
 * length of v's list; pred_out (capacity pred_cap) receives the lists
 * concatenated in vertex order, each in the reference's list order.
 */
int gbref_sssp_list(int64_t n, int64_t m, const int64_t *row, const int64_t *col,
                    const double *w, int64_t src, double delta, double *dist_out,
                    int64_t *pred_cnt, int64_t *pred_out, int64_t pred_cap,
                    double *seconds) {
    size_t map_bytes = sizeof(ref_result) + sizeof(double) * (size_t)(n ? n : 1) +
                       sizeof(int64_t) * (size_t)(n ? n : 1) +
                       sizeof(int64_t) * (size_t)(pred_cap ? pred_cap : 1);
    void *map = mmap(NULL, map_bytes, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
    if (map == MAP_FAILED) return -10;
    ref_result *res = (ref_result *)map;
    double *dist = (double *)((char *)map + sizeof(ref_result));
    int64_t *cnt = (int64_t *)(dist + (n ? n : 1));
    int64_t *lst = cnt + (n ? n : 1);
    res->status = -1;
    fflush(NULL);
    pid_t pid = fork();
    if (pid < 0) { munmap(map, map_bytes); return -11; }
    if (pid == 0) {
        char dir[64];
        if (enter_scratch(dir, sizeof dir) != 0) _exit(3);
        quiet_stdout();
        t_csr *gs = make_csr(n, m, row, col, w);
        p_list *pred = (p_list *)malloc(sizeof(p_list) * (n ? n : 1));
        for (int64_t v = 0; v < n; v++) {
            pred[v] = (p_list)malloc(sizeof(t_list));
            creat_list(pred[v]);
        }
        double t0 = now_s();
        run_sspath(gs, pred, src, delta);
        double t1 = now_s();
        int64_t k = 0;
        for (int64_t v = 0; v < n; v++) {
            dist[v] = gs->vet_info[v].weight;
            int64_t c = 0;
            for (p_list p = pred[v]->next; p; p = p->next) {
                if (k < pred_cap) lst[k] = p->int_val;
                k++; c++;
            }
            cnt[v] = c;
        }
        res->pred_total = k;
        res->seconds = t1 - t0;
        res->status = k <= pred_cap ? 0 : 2;
        unlink("data/log/ori");
        rmdir("data/log");
        rmdir("data");
        if (chdir("/tmp") == 0) rmdir(dir);
        _exit(0);
    }
    int st = 0;
    waitpid(pid, &st, 0);
    int rc = 0;
    if (!WIFEXITED(st) || WEXITSTATUS(st) != 0 || res->status != 0) {
        rc = WIFSIGNALED(st) ? -100 - WTERMSIG(st) : (res->status == 2 ? -13 : -12);
    } else {
        memcpy(dist_out, dist, sizeof(double) * (size_t)n);
        memcpy(pred_cnt, cnt, sizeof(int64_t) * (size_t)n);
        memcpy(pred_out, lst, sizeof(int64_t) * (size_t)res->pred_total);
        if (seconds) *seconds = res->seconds;
    }
    munmap(map, map_bytes);
    return rc;
}

/* btwcentral/csr_bc.c:16-64 (run_bc) without its file reading: for every
 * source in `srcs` (all vertices when srcs is NULL) run_sspath with bucket
 * width `delta` (run_bc passes 0.1), sort the distances with q_sort_double
 * (utils/utils.c:82), then the reference's comp_num_spath and comp_delta
 * (csr_bc.c:67-116), summing delta[j] over j != source into bc_out.  Runs in
 * one forked child; dup_out (may be NULL) receives how many predecessor list
 * entries repeated an earlier entry of the same list, summed over sources.
 * With `dedup` set, such repeats are unlinked before comp_num_spath runs
 * (run_sspath appends u again each time it re-relaxes an edge to an equal
 * distance, sssp/csr_sspath.c:100-118, and its S list is never emptied,
 * :51-72, so heavy edges are re-relaxed every bucket). */
void q_sort_double(double *a, lint *b, lint l, lint r);
void comp_num_spath(lint source, lint *num_spath, lint *dis_idx, p_list *predecesor, lint v_size);
void comp_delta(lint source, lint *num_spath, double *delta, lint *dis_idx, p_list *predecesor,
                lint v_size);
void empty_predecesor(p_list *predecesor, lint v_size);

int gbref_bc(int64_t n, int64_t m, const int64_t *row, const int64_t *col, const double *w,
             int64_t nsrc, const int64_t *srcs, double delta, int dedup, double *bc_out,
             int64_t *dup_out, double *seconds) {
    size_t map_bytes = sizeof(ref_result) + sizeof(double) * (size_t)(n ? n : 1);
    void *map = mmap(NULL, map_bytes, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
    if (map == MAP_FAILED) return -10;
    ref_result *res = (ref_result *)map;
    double *tot = (double *)((char *)map + sizeof(ref_result));
    res->status = -1;
    fflush(NULL);
    pid_t pid = fork();
    if (pid < 0) { munmap(map, map_bytes); return -11; }
    if (pid == 0) {
        char dir[64];
        if (enter_scratch(dir, sizeof dir) != 0) _exit(3);
        quiet_stdout();
        t_csr *gs = make_csr(n, m, row, col, w);
        p_list *pred = (p_list *)malloc(sizeof(p_list) * (n ? n : 1));
        double *dl = (double *)malloc(sizeof(double) * (n ? n : 1));
        double *distance = (double *)malloc(sizeof(double) * (n ? n : 1));
        lint *dis_idx = (lint *)malloc(sizeof(lint) * (n ? n : 1));
        lint *num_spath = (lint *)malloc(sizeof(lint) * (n ? n : 1));
        unsigned char *seen = (unsigned char *)calloc((size_t)(n ? n : 1), 1);
        for (int64_t v = 0; v < n; v++) {
            pred[v] = (p_list)malloc(sizeof(t_list));
            creat_list(pred[v]);
            tot[v] = 0.0;
        }
        int64_t dups = 0;
        double t0 = now_s();
        for (int64_t k = 0; k < nsrc; k++) {
            lint source = srcs ? srcs[k] : k;
            run_sspath(gs, pred, source, delta);
            for (int64_t j = 0; j < n; j++) {
                distance[j] = gs->vet_info[j].weight;
                dis_idx[j] = j;
            }
            q_sort_double(distance, dis_idx, 0, n - 1);
            for (int64_t v = 0; v < n; v++) {
                for (p_list q = pred[v], p = q->next; p; p = q->next) {
                    if (seen[p->int_val]) {
                        dups++;
                        if (dedup) { q->next = p->next; free(p); continue; }
                    }
                    seen[p->int_val] = 1;
                    q = p;
                }
                for (p_list p = pred[v]->next; p; p = p->next) seen[p->int_val] = 0;
            }
            comp_num_spath(source, num_spath, dis_idx, pred, n);
            comp_delta(source, num_spath, dl, dis_idx, pred, n);
            for (int64_t j = 0; j < n; j++)
                if (j != source) tot[j] += dl[j];
            empty_predecesor(pred, n);
        }
        double t1 = now_s();
        res->pred_total = dups;
        res->seconds = t1 - t0;
        res->status = 0;
        unlink("data/log/ori");
        rmdir("data/log");
        rmdir("data");
        if (chdir("/tmp") == 0) rmdir(dir);
        _exit(0);
    }
    int st = 0;
    waitpid(pid, &st, 0);
    int rc = 0;
    if (!WIFEXITED(st) || WEXITSTATUS(st) != 0 || res->status != 0) {
        rc = WIFSIGNALED(st) ? -100 - WTERMSIG(st) : -12;
    } else {
        memcpy(bc_out, tot, sizeof(double) * (size_t)n);
        if (dup_out) *dup_out = res->pred_total;
        if (seconds) *seconds = res->seconds;
    }
    munmap(map, map_bytes);
    return rc;
}

/* graph/csr.c readers on the file dir/file: scan_csr_idx + read_graph_csr
 * (text, :4-202) when bin == 0, read_csr_bin (:211-299) when bin == 1, with
 * type SEND (1) or RECV (0).  Copies out v_size, e_size, the inclusive row
 * ends vet_idx, edge_idx and edge_info[].edge_weight (at most cap_n / cap_m
 * entries).  Runs in a forked child: the readers allocate and never free, and
 * stop the process on a missing file. */
void scan_csr_idx(t_csr *graph, char *file, char *dir, sint type);
void read_graph_csr(t_csr *graph, char *file, char *dir, sint type);
void read_csr_bin(t_csr *graph, char *file, char *dir, sint type, int myrank);

int gbref_read_graph(const char *dir, const char *file, int bin, int type, int64_t cap_n, int64_t cap_m,
                     int64_t *nm_out, int64_t *row_end, int64_t *col, double *w) {
    size_t map_bytes = sizeof(ref_result) + 16 + 8 * (size_t)(cap_n + 2 * cap_m + 3);
    void *map = mmap(NULL, map_bytes, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
    if (map == MAP_FAILED) return -10;
    ref_result *res = (ref_result *)map;
    int64_t *nm = (int64_t *)((char *)map + sizeof(ref_result));
    int64_t *re = nm + 2;
    int64_t *cl = re + cap_n + 1;
    double *wt = (double *)(cl + cap_m + 1);
    res->status = -1;
    fflush(NULL);
    pid_t pid = fork();
    if (pid < 0) { munmap(map, map_bytes); return -11; }
    if (pid == 0) {
        quiet_stdout();
        t_csr *gs = (t_csr *)calloc(1, sizeof(t_csr));
        char d[4096], f[4096];
        snprintf(d, sizeof d, "%s", dir);
        snprintf(f, sizeof f, "%s", file);
        if (bin) {
            read_csr_bin(gs, f, d, (sint)type, 0);
        } else {
            scan_csr_idx(gs, f, d, (sint)type);
            read_graph_csr(gs, f, d, (sint)type);
        }
        nm[0] = gs->v_size;
        nm[1] = gs->e_size;
        if (gs->v_size > cap_n || gs->e_size > cap_m) { res->status = 2; _exit(0); }
        for (int64_t v = 0; v < gs->v_size; v++) re[v] = gs->vet_idx[v];
        for (int64_t e = 0; e < gs->e_size; e++) {
            cl[e] = gs->edge_idx[e];
            wt[e] = gs->edge_info[e].edge_weight;
        }
        res->status = 0;
        _exit(0);
    }
    int st = 0;
    waitpid(pid, &st, 0);
    int rc = 0;
    nm_out[0] = nm[0];
    nm_out[1] = nm[1];
    if (!WIFEXITED(st) || WEXITSTATUS(st) != 0 || res->status != 0) {
        rc = WIFSIGNALED(st) ? -100 - WTERMSIG(st) : (res->status == 2 ? -13 : -12);
    } else {
        memcpy(row_end, re, 8 * (size_t)nm[0]);
        memcpy(col, cl, 8 * (size_t)nm[1]);
        memcpy(w, wt, 8 * (size_t)nm[1]);
    }
    munmap(map, map_bytes);
    return rc;
}
