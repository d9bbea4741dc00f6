/*
 * gbsssp_compat.h -- link-compatible replacements for GRAPHBENCH's SSSP entry
 * points, implemented in libgbsssp_compat.so on top of libgbsssp (gbsssp.h).
 *
 * A program built against the reference drops the reference's SSSP objects
 * (sssp/csr_sspath_array.c, sssp/csr_sspath.c) -- and, if it wants them on
 * the GPU, its CSR readers (graph/csr.c) and betweenness
 * (btwcentral/csr_bc.c) -- and links this library instead: the functions
 * below have the reference's names, signatures and argument meaning, and read
 * and write the same structures.
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
 *     run in uint32 (exact, equal to the reference's double sums); when a
 *     path sum would reach 2^32-1 the call converts the graph again and
 *     reruns it in float64 (integer sums below 2^53 stay exact), and the
 *     float64 copy stays cached for later calls on that graph; any other
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

/*
 * The readers of graph/csr.c with parsing and CSR build on the GPU
 * (gbs_read_text / gbs_read_bin); the t_csr is filled as the reference fills
 * it: v_size, e_size, offset and global_v_size from the header, vet_idx the
 * inclusive row ends, rows in file order, edge_info[].edge_weight where the
 * reference stores it, vet_info as scan_csr_idx (weight 1, recip 1/degree,
 * vet_deg the degree) or read_csr_bin (weight INFINITY, recip 0, vet_deg 0)
 * leaves it.  Arrays are 64-byte aligned (posix_memalign); the reference never
 * frees them either.  A program that keeps graph/csr.c linked keeps its own
 * readers (its definitions take precedence).
 *
 *   scan_csr_idx    graph/csr.c:133-202 (reads the whole file; the edges are
 *                   kept for the read_graph_csr call that follows)
 *   read_graph_csr  graph/csr.c:4-60
 *   read_csr_bin    graph/csr.c:211-299 (targets shifted by
 *                   GBS_COMPAT_BIN_OFFSET, the reference's OFFSET, 1 unless
 *                   the library is built with -DGBS_COMPAT_BIN_OFFSET=0)
 *   run_bc          btwcentral/csr_bc.c:16-64: reads the graph (read_csr_bin
 *                   when the program's global `bin` is set, else the text
 *                   reader, SEND), betweenness over every vertex on the GPU
 *                   (gbs_bc, float64 weights), and the reference's printout
 *                   ("the final result for betweeness centrality is:" then
 *                   "i:value " for i = 1..n).  Each tight edge counts once.
 */
void scan_csr_idx(t_csr *graph, char *file, char *dir, sint type);
void read_graph_csr(t_csr *graph, char *file, char *dir, sint type);
void read_csr_bin(t_csr *graph, char *file, char *dir, sint type, int myrank);
void run_bc(char *file, char *dir);

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
