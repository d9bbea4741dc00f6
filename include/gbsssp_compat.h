/*
 * gbsssp_compat.h -- link-compatible replacements for GRAPHBENCH's SSSP entry
 * points, implemented in libgbsssp_compat.so on top of libgbsssp (gbsssp.h).
 *
 * A program built against the reference keeps its own CSR readers
 * (scan_csr_idx / read_graph_csr / read_csr_bin, graph/csr.c) and its
 * predecessor lists, drops the reference's SSSP objects
 * (sssp/csr_sspath_array.c, sssp/csr_sspath.c) and links this library
 * instead: the two functions below have the reference's names, signatures and
 * argument meaning, and read and write the same structures.
 *
 *   run_sspath_arr  sssp/csr_sspath_array.c:149-151 (called from
 *                   main/main.c:223; declared in no header there)
 *   run_sspath      include/list.h:32-33, sssp/csr_sspath.c:38-80
 *
 * Behaviour:
 *   - distances are written to gs->vet_info[v].weight as doubles (INFINITY
 *     for unreached vertices), as the reference does;
 *   - the graph is converted once to a device CSR and cached (key: the t_csr
 *     address, its array addresses and sizes, and a sample of its contents);
 *     after changing a t_csr in place call gbs_compat_forget(gs);
 *   - edge weights must be finite and >= 0.  Integer weights in [0, 2^32-2]
 *     run in uint32 (exact, equal to the reference's double sums); any other
 *     weights run in float64, the reference's own arithmetic (one rounding
 *     per relaxation), so the distances equal its doubles bit for bit.
 *     gbs_compat_allow_float32(1) runs float32-exact weights in float32
 *     instead (faster, but float32 sums, not the reference's doubles);
 *   - errors print one line to stderr and exit(123), the reference's
 *     ERROR_PRINT behaviour (include/graph.h:74); gbs_compat_set_exit(0) makes
 *     them return instead, with gbs_compat_status() holding the status;
 *   - predecessors: run_sspath_arr leaves one entry per reached vertex
 *     (other than the source) in predecesor[v], the smallest-id tight
 *     predecessor (the reference's array path writes none); run_sspath
 *     leaves every tight predecessor u (dist[u] + w(u,v) == dist[v]), each
 *     once, which is what the reference's list path accumulates for
 *     betweenness centrality (sssp/csr_sspath.c:116-118).  Lists of reached
 *     vertices are emptied first (their nodes freed); lists of unreached
 *     vertices are left as they are.  predecesor may be NULL.
 */
#ifndef GBSSSP_COMPAT_H
#define GBSSSP_COMPAT_H

#include "gbsssp.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Same layout as the reference's types (include/graph.h:93-127,
 * include/list.h:3-11); skipped when the reference's headers are included. */
#ifndef _H_GRAPH
typedef long long int lint;
typedef int sint;

struct vet_info {
    double weight;   /* distance output */
    double wb;
    double recip;
    lint vet_deg;
};
typedef struct vet_info t_vi;

struct edge_info {
    lint node_id;
    double edge_weight;
};
typedef struct edge_info t_e;

struct CSR {
    lint *vet_idx;     /* INCLUSIVE end offset of each row */
    lint *edge_idx;    /* edge targets */
    t_vi *vet_info;
    t_e *edge_info;
    lint v_size;
    lint e_size;
    lint offset;
    sint csr_type;
    lint global_v_size;
};
typedef struct CSR t_csr;

struct list_elem {
    lint int_val;
    lint int_val1;
    double double_val;
    struct list_elem *next;
};
typedef struct list_elem t_list;
typedef struct list_elem *p_list;
#endif

void run_sspath_arr(t_csr *gs, p_list *predecesor, lint source, double delta);
void run_sspath(t_csr *gs, p_list *predecesor, lint source, double delta);

/* Library-specific controls (no counterpart in the reference). */
void gbs_compat_forget(const t_csr *gs);        /* drop the cached device copy of gs */
void gbs_compat_forget_all(void);
void gbs_compat_allow_float32(int allow);        /* float32 arithmetic for float32-exact weights */
void gbs_compat_set_exit(int exit_on_error);     /* 1 (default): exit(123) on error */
gbs_status gbs_compat_status(void);              /* status of the last call */

#ifdef __cplusplus
}
#endif
#endif /* GBSSSP_COMPAT_H */
