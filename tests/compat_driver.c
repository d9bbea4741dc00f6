/*
 * compat_driver.c -- test program for libgbsssp_compat.so, written the way a
 * GRAPHBENCH caller uses the SSSP entry points (main/main.c:207-223): it
 * builds a t_csr, one predecessor list head per vertex, and calls
 * run_sspath_arr or run_sspath.
 *
 *   compat_driver IN OUT arr|list REPS [f32] [noexit]
 *
 * IN:  int64 n, int64 m, int64 source, double delta, int64 vet_idx[n]
 *      (inclusive row ends), int64 edge_idx[m], double weight[m]
 * OUT: double dist[n]; then per vertex int64 count and the list entries in
 *      list order.  The call is made REPS times on the same t_csr (the
 *      device copy is cached after the first).
 * With "noexit", errors return instead of exiting; the status is written to
 * stdout as "status N".
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gbsssp_compat.h"

static void *read_exact(FILE *f, size_t bytes) {
    void *p = malloc(bytes ? bytes : 1);
    if (!p || fread(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "short read\n");
        exit(2);
    }
    return p;
}

int main(int argc, char **argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s IN OUT arr|list REPS [f32] [noexit]\n", argv[0]);
        return 2;
    }
    int list_mode = strcmp(argv[3], "list") == 0;
    int reps = atoi(argv[4]);
    for (int i = 5; i < argc; ++i) {
        if (!strcmp(argv[i], "f32")) gbs_compat_allow_float32(1);
        if (!strcmp(argv[i], "noexit")) gbs_compat_set_exit(0);
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    long long hdr[3];
    double delta;
    if (fread(hdr, 8, 3, f) != 3 || fread(&delta, 8, 1, f) != 1) return 2;
    const lint n = hdr[0], m = hdr[1], source = hdr[2];
    t_csr *gs = (t_csr *)calloc(1, sizeof(t_csr));
    gs->v_size = n;
    gs->e_size = m;
    gs->vet_idx = (lint *)read_exact(f, 8 * (size_t)n);
    gs->edge_idx = (lint *)read_exact(f, 8 * (size_t)m);
    double *w = (double *)read_exact(f, 8 * (size_t)m);
    fclose(f);
    gs->edge_info = (t_e *)calloc((size_t)(m ? m : 1), sizeof(t_e));
    for (lint e = 0; e < m; ++e) gs->edge_info[e].edge_weight = w[e];
    gs->vet_info = (t_vi *)calloc((size_t)n, sizeof(t_vi));
    p_list *pred = (p_list *)malloc(sizeof(p_list) * (size_t)n);
    for (lint v = 0; v < n; ++v) {
        pred[v] = (p_list)malloc(sizeof(t_list));
        pred[v]->int_val = -1;
        pred[v]->int_val1 = -1;
        pred[v]->double_val = -1;
        pred[v]->next = NULL;
    }
    for (int r = 0; r < reps; ++r) {
        if (list_mode) run_sspath(gs, pred, source, delta);
        else run_sspath_arr(gs, pred, source, delta);
        if (gbs_compat_status() != GBS_OK) {
            printf("status %d\n", (int)gbs_compat_status());
            return 0;
        }
    }
    printf("status 0\n");
    FILE *o = fopen(argv[2], "wb");
    if (!o) return 2;
    for (lint v = 0; v < n; ++v) fwrite(&gs->vet_info[v].weight, 8, 1, o);
    for (lint v = 0; v < n; ++v) {
        long long c = 0;
        for (p_list e = pred[v]->next; e; e = e->next) ++c;
        fwrite(&c, 8, 1, o);
        for (p_list e = pred[v]->next; e; e = e->next) fwrite(&e->int_val, 8, 1, o);
    }
    fclose(o);
    gbs_compat_forget(gs);
    return 0;
}
