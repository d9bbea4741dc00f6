/*
 * gbsssp.h -- native C ABI of the GB300 delta-stepping SSSP library
 * (libgbsssp.so).  Plain C types only; every call returns a gbs_status.
 *
 * It replaces the single-source shortest path of GRAPHBENCH:
 *   run_sspath_arr(t_csr *gs, p_list *predecesor, lint source, double delta)
 *       sssp/csr_sspath_array.c:149-151 (declared in no header; called from
 *       main/main.c:223)
 *   run_sspath(t_csr *gs, p_list *predecesor, lint source, double delta)
 *       include/list.h:32-33, sssp/csr_sspath.c:38
 * over the CSR that graph/csr.c builds (scan_csr_idx/read_graph_csr
 * include/csr.h:4-5, read_csr_bin include/csr.h:15-16, separate_csr
 * graph/csr.c:74).  The reference-shaped entry points over t_csr live in
 * gbsssp_compat.h; this header is the handle-based API underneath them.
 *
 * Differences from the reference interface, by design:
 *   - the graph is uploaded once (gbs_graph_create) and stays resident on the
 *     GPU; the reference re-splits it into light/heavy copies on every call
 *     (separate_csr inside run_sspath_arr, :173);
 *   - errors are status codes, never exit() (the reference's ERROR_PRINT,
 *     include/graph.h:74);
 *   - no global state: calls on different graphs are independent; calls on
 *     the same graph must not overlap (one workspace per graph);
 *   - distances are computed in the weight type (uint32 or float32) and are
 *     bit-identical to the least fixpoint (Dijkstra) for any bucket width;
 *     the predecessor of v is the smallest-id u with dist[u] + w(u,v) ==
 *     dist[v] (one tight predecessor per vertex, see gbs_sssp).
 */
#ifndef GBSSSP_H
#define GBSSSP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBS_ABI_VERSION 1

typedef enum gbs_status {
    GBS_OK = 0,
    GBS_ERR_INVALID_ARG = 1,  /* null pointer, malformed CSR, source out of range */
    GBS_ERR_CUDA = 2,         /* a CUDA runtime call failed (see gbs_last_error) */
    GBS_ERR_NO_MEMORY = 3,    /* device or pinned host allocation failed */
    GBS_ERR_CAPACITY = 4,     /* a device work list would overflow its bound */
    GBS_ERR_TIMEOUT = 5,      /* a device-side wait ran past its limit */
    GBS_ERR_OVERFLOW = 6,     /* a uint32 path sum reached 2^32 - 1 */
    GBS_ERR_UNSUPPORTED = 7,  /* no usable GPU, or a size the build does not handle */
    GBS_ERR_INTERNAL = 8
} gbs_status;

typedef enum gbs_weight_type {
    GBS_WEIGHT_U32 = 0,       /* uint32 weights, uint32 distances (UINT32_MAX = unreached) */
    GBS_WEIGHT_F32 = 1,       /* float32 weights >= 0, float32 distances (+inf = unreached) */
    GBS_WEIGHT_F64 = 2        /* float64 weights >= 0, float64 distances (+inf = unreached): the
                                 reference's own arithmetic (doubles, one rounding per
                                 relaxation); single-source calls only (not packs or plans) */
} gbs_weight_type;

typedef struct gbs_graph gbs_graph;

/* Per-call knobs.  Zero-initialise and set what you need. */
typedef struct gbs_params {
    double delta;            /* bucket width; <= 0 selects max_w / average out-degree
                                (the published configs' rule).  uint32 graphs use
                                floor(delta), at least 1. */
    double light;            /* light/heavy split: an edge is light iff w <= light.
                                < 0 selects light = delta (the reference's rule,
                                graph/csr.c:84). */
    uint32_t flags;          /* GBS_F_* */
    uint32_t wait_limit_ms;  /* device-side wait limit; 0 = 4000 ms (a whole run
                                is limited to 16 times this) */
    uint32_t solo_entries;   /* a scan of at most this many frontier entries runs on
                                one CTA without a grid barrier; 0 = 1024 */
    uint32_t solo_descs;     /* likewise for a relaxation of at most this many
                                128-edge descriptors; 0 = 64 */
    uint32_t inline_edges;   /* rows of at most this many edges are relaxed by the
                                scanning warp, longer rows are cut into 128-edge
                                descriptors relaxed one warp each; 0 = 32 */
    uint32_t full_items;     /* a bucket whose lists hold at most this many entries
                                when it starts relaxes whole rows (light and heavy
                                edges together, no heavy phase); 0 = every bucket,
                                so the light bound only shapes runs that set this
                                (max(1024, vertices / 16) keeps the split for the
                                large buckets; batched plans always use that) */
    uint32_t fuse_rounds;    /* bucket fusion: a whole-row scan relaxes the vertices
                                it improves into the current bucket itself, for up
                                to this many rounds per warp, before the next ones
                                wait for the next frontier scan; 0 = 2 (uint32 and
                                float32 weights; GBS_F_NO_FUSE turns it off) */
} gbs_params;

#define GBS_F_NO_STATS 0x1u  /* skip the reached-vertex/edge reduction */
#define GBS_F_TRACE 0x2u     /* record one gbs_phase_rec per grid phase (gbs_trace) */
#define GBS_F_NO_SOLO 0x4u   /* run every phase on the whole grid */
#define GBS_F_FEATURES 0x8u  /* record the controller inputs at every bucket start (gbs_features) */
#define GBS_F_LEARNED 0x10u  /* bucket widths from the graph's learned controller
                                (gbs_graph_set_controller) */
#define GBS_F_BC_SINGLE 0x20u /* gbs_bc: one single-source launch per source instead of
                                batched launches of up to 64 sources */
#define GBS_F_NO_FUSE 0x40u  /* no bucket fusion (gbs_params.fuse_rounds): a vertex
                                improved into the current bucket always waits for
                                the next frontier scan */
/* Failure-path test: one CTA never arrives at the first grid barrier, so every
 * other CTA's bounded wait runs out; the call returns GBS_ERR_TIMEOUT after
 * wait_limit_ms and the device stays usable.  Never set in normal use. */
#define GBS_F_TEST_STALL 0x80000000u

typedef struct gbs_stats {
    double device_ms;        /* CUDA-event time of the whole run: reset + kernel + outputs */
    double kernel_ms;        /* CUDA-event time of the persistent relaxation kernel */
    uint64_t reached;        /* vertices with a finite distance */
    uint64_t edges_reached;  /* sum of out-degrees of reached vertices (the GTEPS numerator) */
    uint64_t improvements;   /* successful distance decreases */
    uint32_t buckets;        /* buckets processed */
    uint32_t phases;         /* grid-wide synchronised phases */
    uint32_t pending_scans;  /* times the far list was re-bucketed */
    uint32_t blocks;         /* CTAs of the persistent launch */
    double delta_used;       /* bucket width actually used */
    double light_used;       /* light/heavy split actually used */
    uint32_t solo_phases;    /* phases run by one CTA without a grid barrier */
    uint32_t learned;        /* GBS_F_LEARNED calls: 1 the learned controller chose
                                the widths; 3 it ran past its guard and the plain
                                schedule was run instead; 2 it had lost on this
                                graph before, so the plain schedule ran directly.
                                Times include every run the call made. */
} gbs_stats;

/* Library / device */
const char *gbs_status_string(gbs_status s);
/* Last error message of the calling thread ("" if none). */
const char *gbs_last_error(void);
int gbs_abi_version(void);
/* 1 if a CUDA device of compute capability 10.x or newer is usable, else 0. */
int gbs_device_available(void);

/*
 * Graph.  row_offsets has n+1 entries (row v is [row_offsets[v],
 * row_offsets[v+1])), cols and weights have m entries.  The arrays are host
 * memory and are copied; the caller keeps ownership.  uint32 weights may be
 * any value; float32 weights must be finite and >= 0 (-0.0 is read as +0.0).
 * Parallel edges and self loops are allowed.  Replaces the CSR produced by
 * scan_csr_idx + read_graph_csr (graph/csr.c:4-202) or read_csr_bin
 * (graph/csr.c:211-299), which use inclusive int64 end offsets instead.
 */
gbs_status gbs_graph_create(uint32_t n, uint64_t m, const uint64_t *row_offsets,
                            const uint32_t *cols, const void *weights,
                            gbs_weight_type wtype, gbs_graph **out);
gbs_status gbs_graph_destroy(gbs_graph *g);
gbs_status gbs_graph_info(const gbs_graph *g, uint32_t *n, uint64_t *m,
                          gbs_weight_type *wtype, double *max_weight,
                          double *default_delta);

/*
 * One single-source shortest path, outputs in HOST memory.  Page-locked
 * outputs (gbs_host_alloc, cudaMallocHost, cudaHostRegister) are written by
 * the device directly, with no copy after the run; any other host memory
 * receives a copy of a device buffer.  dist_out: n uint32 or float32 values in
 * the graph's weight type; pred_out: n int32 values (pred[source] = source,
 * -1 for unreached vertices).  Either output may be NULL.  params and stats
 * may be NULL.  Replaces run_sspath_arr (sssp/csr_sspath_array.c:149), whose
 * distances land in gs->vet_info[v].weight as doubles and whose predecessor
 * argument is never written.
 */
gbs_status gbs_sssp(gbs_graph *g, uint32_t source, const gbs_params *params,
                    void *dist_out, int32_t *pred_out, gbs_stats *stats);

/*
 * Same computation with outputs in DEVICE memory allocated by the caller
 * (cudaMalloc; n elements each; NULL skips that output).  Results stay on the
 * GPU; the call returns after the run finished.
 */
gbs_status gbs_sssp_device(gbs_graph *g, uint32_t source, const gbs_params *params,
                           void *dist_dev, int32_t *pred_dev, gbs_stats *stats);

/*
 * Many sources over one graph (the source loop of btwcentral/csr_bc.c:40-43).
 * dist_out / pred_out are host arrays of k*n elements, row i belonging to
 * sources[i] (either may be NULL).  Each row is identical to what gbs_sssp
 * returns for that source.
 */
gbs_status gbs_sssp_multi(gbs_graph *g, const uint32_t *sources, uint32_t k,
                          const gbs_params *params, void *dist_out, int32_t *pred_out,
                          gbs_stats *stats);

/*
 * Graph ingest on the GPU: the reference's readers (graph/csr.c) with the
 * parsing and the CSR build done on the device.  A gbs_device_csr holds the
 * graph exactly as the reference's t_csr would: n = v_num rows, each row's
 * edges in file order, and the weights where the reference puts them.
 *
 * gbs_read_text / gbs_parse_text: scan_csr_idx + read_graph_csr
 *   (graph/csr.c:4-202).  Lines "p <name> v_num e_num offset g_v_size" and
 *   "a v_id v_to weight"; other lines are skipped; the first e_num "a" lines
 *   are read.  GBS_DIR_SEND: row = v_id - offset, column = v_to - 1;
 *   GBS_DIR_RECV: row = v_to - offset, column = v_id - 1.  Weights: the k-th
 *   "a" line's v_to / v_num, stored at CSR position k (the reference's
 *   edge_info[e_num_read]; the same as the edge's own weight only for files
 *   sorted by row); the line's third number is ignored, as there.
 * gbs_read_bin / gbs_parse_bin: read_csr_bin (graph/csr.c:211-299).  int64
 *   v_num, e_num, offset, g_v_size, then e_num int64 (from, to) pairs.
 *   SEND: row = from - offset, column = to - target_offset; RECV: row = to -
 *   offset, column = from - target_offset (target_offset: the reference's
 *   OFFSET, 1 in its default build, 0 in its Graph500 build).  Weight of CSR
 *   position p: 0.1 (p even) or 0.2 (p odd).  dedup != 0 first drops every
 *   (from, to) pair that appeared earlier in the file (remove_duplicate,
 *   partition/csr_partition_bin_mpi.c:47-105).
 * Rows and columns outside [0, v_num) are rejected (GBS_ERR_INVALID_ARG,
 * gbs_last_error names the edge).
 */
#define GBS_DIR_RECV 0
#define GBS_DIR_SEND 1
typedef struct gbs_device_csr gbs_device_csr;
typedef struct gbs_ingest_info {
    int64_t v_num, e_num, offset, g_v_size;   /* the file's header */
    uint64_t records;        /* "a" lines (text) or pairs (binary) in the file */
    uint64_t edges;          /* edges in the CSR */
    uint64_t duplicates;     /* pairs dropped by dedup */
    double read_ms;          /* host file read (gbs_read_*) */
    double parse_ms;         /* device: copy in, parse / split, duplicate removal */
    double build_ms;         /* device: CSR build */
} gbs_ingest_info;

gbs_status gbs_read_text(const char *path, int direction, gbs_device_csr **out, gbs_ingest_info *info);
gbs_status gbs_parse_text(const char *bytes, size_t len, int direction, gbs_device_csr **out,
                          gbs_ingest_info *info);
gbs_status gbs_read_bin(const char *path, int direction, int64_t target_offset, int dedup,
                        gbs_device_csr **out, gbs_ingest_info *info);
gbs_status gbs_parse_bin(const void *bytes, size_t len, int direction, int64_t target_offset, int dedup,
                         gbs_device_csr **out, gbs_ingest_info *info);
gbs_status gbs_device_csr_info(const gbs_device_csr *c, uint32_t *n, uint64_t *m);
/* Host copies: row_offsets n+1 exclusive offsets, cols m, weights m (any may be NULL). */
gbs_status gbs_device_csr_export(const gbs_device_csr *c, uint64_t *row_offsets, uint32_t *cols,
                                 double *weights);
/* A resident graph built on the device from the CSR (rows sorted by (weight,
 * column) as gbs_graph_create sorts them).  GBS_WEIGHT_F64 keeps the weights
 * exactly; F32 rounds them; U32 needs integer weights.  The CSR may be
 * destroyed afterwards. */
gbs_status gbs_graph_from_device_csr(const gbs_device_csr *c, gbs_weight_type wtype, gbs_graph **out);
gbs_status gbs_device_csr_destroy(gbs_device_csr *c);

/*
 * PageRank, the reference's iteration (pagerank/pagerank_mpi.c:667-1043 on
 * one node) as a pull over an IN-edge CSR (row v lists the u with an edge
 * u -> v: gbs_read_text(path, GBS_DIR_RECV, ...) as the reference reads it,
 * or gbs_device_csr_transpose of an out-edge CSR).  weight = 1, recip =
 * 1 / out-degree (the count of each vertex among the columns), wb =
 * random_jump, diff = weight * recip; each iteration wb[v] += (1 -
 * random_jump) * sum of diff[u] over the in-edges, diff[v] = (wb[v] -
 * weight[v]) * recip[v], weight = wb, until no |diff| exceeds threshold.
 * rank_out: n doubles (host), the final weight.  params may be NULL:
 * random_jump 0.3 and threshold 1e-6 (RDM_JMP, THRESH, include/graph.h:17-18).
 */
typedef struct gbs_pagerank_params {
    double random_jump;      /* <= 0: 0.3 */
    double threshold;        /* <= 0: 1e-6 */
    uint32_t max_iters;      /* 0: 10000 */
    uint32_t reserved;
} gbs_pagerank_params;

typedef struct gbs_pagerank_stats {
    uint32_t iterations;
    uint32_t converged;      /* 1: stopped on the threshold, 0: on max_iters */
    double device_ms;        /* CUDA events around the iterations */
    uint64_t edges;
} gbs_pagerank_stats;

gbs_status gbs_pagerank(const gbs_device_csr *in_edges, const gbs_pagerank_params *params, double *rank_out,
                        gbs_pagerank_stats *stats);
/* The transposed CSR (row v lists the rows that list v, in row order),
 * weights carried along. */
gbs_status gbs_device_csr_transpose(const gbs_device_csr *c, gbs_device_csr **out);

/*
 * Betweenness centrality (Brandes over shortest paths), the computation of
 * run_bc (btwcentral/csr_bc.c:16-64) on a resident graph instead of a file:
 * for every source s (sources[0..k), or every vertex when sources is NULL)
 * bc[v] += delta_s(v) for v != s, where delta_s(v) = sum over the tight
 * out-edges (v, w) -- dist(v) + w == dist(w) in the weight type -- of
 * (1 + delta_s(w)) * sigma_s(v) / sigma_s(w), and sigma_s counts the tight
 * paths from s (comp_num_spath / comp_delta, csr_bc.c:67-116; sigma in
 * 64-bit integers like the reference's lint, the rest in double).  Each
 * tight edge is counted once (the reference's predecessor lists can hold an
 * entry more than once, sssp/csr_sspath.c:100-118, which changes its result
 * when a vertex has several shortest-path predecessors).  Weights must be
 * positive (GBS_ERR_INVALID_ARG otherwise).  bc_out: n doubles in host
 * memory.  params: the schedule of the shortest-path runs (NULL: the
 * default); the result does not depend on it.  uint32 / float32 graphs solve
 * the shortest paths of up to 64 sources in one batched launch (as
 * gbs_plan_sources) unless GBS_F_BC_SINGLE or GBS_F_LEARNED is set; float64
 * graphs run one source at a time.
 */
typedef struct gbs_bc_stats {
    double device_ms;        /* CUDA-event time of all shortest-path runs and DAG passes */
    double sssp_ms;          /* the shortest-path runs alone */
    double dag_ms;           /* the path-count / dependency passes alone */
    uint64_t edges_reached;  /* sum over sources of the edges out of reached vertices */
    uint64_t tight_edges;    /* sum over sources of the shortest-path DAG's edges */
    uint64_t dag_vertices;   /* sum over sources of the reached vertices */
    uint32_t max_levels;     /* deepest DAG in hop levels (the source's is level 0) */
    uint32_t sources;
    uint32_t blocks;         /* CTAs of the DAG kernel */
    uint32_t reserved;
} gbs_bc_stats;

gbs_status gbs_bc(gbs_graph *g, const uint32_t *sources, uint32_t k, const gbs_params *params,
                  double *bc_out, gbs_bc_stats *stats);

/* Same with the result in DEVICE memory (n doubles, cudaMalloc). */
gbs_status gbs_bc_device(gbs_graph *g, const uint32_t *sources, uint32_t k, const gbs_params *params,
                         double *bc_dev, gbs_bc_stats *stats);

/*
 * Per-phase record of the last run made with GBS_F_TRACE (the GPU analogue
 * of the reference's per-phase rdtsc slots and bucket dumps,
 * sssp/csr_sspath_array.c:1121-1170).  kind (low 4 bits; +16 if the phase ran
 * on one CTA without a grid barrier): 0 scan of a new bucket, 1 scan
 * of a repeated light frontier, 2 scan of the settled list for heavy edges,
 * 3 edge relaxation, 4 pending re-bucketing (its edges field counts entries
 * that had already left the pending list).  items: frontier entries
 * (scans), edge descriptors (relaxation) or pending entries; edges: edges
 * the scan handed to the relaxation; end_ns: device time since kernel start.
 * After gbs_bc with GBS_F_TRACE the records are those of the last source's
 * path-count / dependency launch: kind 8 the tight-edge count, 9 a forward
 * level, 10 a backward level, 11 the first part of a backward level whose
 * long rows are then finished; bucket = the level, items = its vertices,
 * edges = the mask words of its rows longer than 32 edges.
 * *count receives the number of records (may exceed cap).
 */
typedef struct gbs_phase_rec {
    uint32_t kind;
    uint32_t bucket;
    uint32_t items;
    uint32_t edges;
    uint32_t pending;        /* entries of the live pending list after the phase */
    uint32_t window;         /* ring window base during the phase */
    uint64_t end_ns;
} gbs_phase_rec;

gbs_status gbs_trace(gbs_graph *g, gbs_phase_rec *out, uint32_t cap, uint32_t *count);

/*
 * Learned bucket-width controller (no counterpart in the reference).  An FP32
 * MLP, 16 inputs -> 64 -> 64 (ReLU) -> 2 outputs, evaluated by the deciding
 * warp at every bucket start of a GBS_F_LEARNED run: output 0 predicts
 * log2(delta / default delta), output 1 is the logit of "split light/heavy at
 * the predicted delta" (else every edge is light).  The run's base width is
 * half the width predicted for the first bucket (that prediction clamped to
 * 2^-2 .. 2^14 times the default); each bucket spans 2^k base widths (k in
 * 0..3) as output 0 says.  Inputs: log2(1 + entries) of the
 * first 1, 2, 4, .., 32 base buckets from the bucket start and of the whole
 * window (7 inputs), log2(1 + pending), log2(1 + distance reached in default
 * widths), log2(1 + buckets done), log2(1 + phases done), the log2 share of
 * the window's entries in the next base bucket, log2(average degree),
 * log2(max weight), mean / max weight, log2(base width / default delta).
 * None of them grows with the vertex count by itself.
 * params: 5410 floats: input means[16], input scales[16], W1[16][64], b1[64],
 * W2[64][64], b2[64], W3[64][2], b3[2] (row-major, inputs first).  margin
 * (<= 0: 0.25): a learned run that runs longer than (1 + margin) times the
 * plain schedule on this graph stops and the plain schedule runs instead.  If
 * that plain run finished within the limit (5% timing noise allowed), the
 * controller lost: from then on GBS_F_LEARNED calls on the graph run the plain
 * schedule (until the controller is set again); otherwise the plain time the
 * limit is based on rises to that run's.  The first learned run on a graph
 * times the plain schedule first.  The
 * distances and predecessors never depend on the schedule.  params NULL
 * removes the controller.  The trace records of a run carry each bucket's
 * span (bits 8-15 of kind) and whether it relaxed whole rows (bit 16).
 */
gbs_status gbs_graph_set_controller(gbs_graph *g, const float *params, uint32_t count, double margin);

/* Controller inputs recorded by the last GBS_F_FEATURES run: 16 floats per
 * bucket start, in order; *count receives how many were recorded. */
gbs_status gbs_features(gbs_graph *g, float *out, uint32_t cap, uint32_t *count);

/*
 * Controller training on the GPU (hand-written forward, backward and Adam
 * kernels; no counterpart in the reference).  A gbs_mlp holds one parameter
 * block (layout of gbs_graph_set_controller), its gradient, Adam moments and
 * a data set: x (n x 16 raw inputs), t (n x 2 targets: log2 of the best
 * width scale, 1/0 for split/no split) and optional sample weights w.  Loss:
 * sum_i w_i [(y0 - t0)^2 + BCE(sigmoid(y1), t1)] / sum_i w_i.  The input
 * means and scales in the block are not trained.
 */
typedef struct gbs_mlp gbs_mlp;
gbs_status gbs_mlp_create(gbs_mlp **out);
gbs_status gbs_mlp_destroy(gbs_mlp *m);
gbs_status gbs_mlp_set_params(gbs_mlp *m, const float *params);   /* 5410 floats; resets Adam */
gbs_status gbs_mlp_get_params(gbs_mlp *m, float *params);
gbs_status gbs_mlp_set_data(gbs_mlp *m, const float *x, const float *t, const float *w, uint32_t n);
/* Loss and gradient over samples [first, first + count) in stored order;
 * grad (5378 floats: W1, b1, W2, b2, W3, b3) may be NULL. */
gbs_status gbs_mlp_loss_grad(gbs_mlp *m, uint32_t first, uint32_t count, double *loss, float *grad);
/* One Adam step with the last gradient. */
gbs_status gbs_mlp_adam(gbs_mlp *m, float lr, float beta1, float beta2, float eps);
/* Minibatch Adam (beta 0.9 / 0.999, eps 1e-8), samples reshuffled every
 * epoch; epoch_loss (epochs entries, may be NULL) gets the mean batch loss. */
gbs_status gbs_mlp_train(gbs_mlp *m, uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                         double *epoch_loss);
/* Outputs for n raw input rows (n x 2). */
gbs_status gbs_mlp_predict(gbs_mlp *m, const float *x, uint32_t n, float *y);

/*
 * Batched SSSP: many independent instances in one persistent launch.
 *
 * The reference solves several sources one after the other, as the source
 * loop of its betweenness centrality (btwcentral/csr_bc.c:16-123 calls
 * run_sspath per source); it has no batched call.  Here a plan fixes a set of
 * instances -- K sources on one resident graph (gbs_plan_sources) or one
 * source on each graph of a pack of independent graphs (gbs_plan_pack) --
 * with their bucket schedules and device outputs.  The launch cuts the grid
 * into groups of group_ctas CTAs; each group owns its own bucket queues and
 * takes instances from a shared queue until none is left.  The launch
 * sequence is captured in a CUDA graph once and replayed by gbs_plan_launch.
 * Results equal gbs_sssp's bit for bit, instance by instance.
 */
typedef struct gbs_pack gbs_pack;
typedef struct gbs_plan gbs_plan;

/* One host CSR of a pack (same layout as gbs_graph_create's arguments). */
typedef struct gbs_csr_view {
    uint32_t n;
    uint64_t m;
    const uint64_t *row_offsets;   /* n+1, exclusive */
    const uint32_t *cols;          /* m */
    const void *weights;           /* m uint32 or float32 */
} gbs_csr_view;

typedef struct gbs_batch_params {
    double delta;          /* > 0: bucket width of every instance; <= 0: the
                              graph's default (max weight / average out-degree)
                              times delta_scale */
    double delta_scale;    /* multiplier of the default width (<= 0: 1) */
    double light;          /* >= 0: light bound of every instance; < 0: the
                              instance's delta; +INFINITY: no split (every edge
                              light) */
    uint32_t group_ctas;   /* CTAs per group (0: one group per instance while the
                              groups' distance words, 8 bytes per vertex each,
                              fit in L2; fewer and wider groups beyond) */
    uint32_t flags;        /* GBS_F_NO_SOLO, GBS_F_NO_FUSE */
    uint32_t wait_limit_ms;
    uint32_t solo_entries;
    uint32_t solo_descs;
    uint32_t inline_edges;   /* as gbs_params.inline_edges */
    uint32_t fuse_rounds;    /* as gbs_params.fuse_rounds */
} gbs_batch_params;

/* Per-instance result record (device times from %globaltimer). */
typedef struct gbs_inst_stats {
    uint32_t done;           /* 1 when the instance completed */
    uint32_t error;          /* device error code of its group (0 = none) */
    uint32_t group;
    uint32_t phases;
    uint32_t buckets;
    uint32_t pending_scans;
    uint32_t solo_phases;
    uint32_t pad;
    uint64_t reached;
    uint64_t edges_reached;
    uint64_t improvements;
    uint64_t start_ns;
    uint64_t end_ns;
} gbs_inst_stats;

typedef struct gbs_batch_stats {
    double device_ms;        /* the whole graph launch (CUDA events) */
    uint32_t instances;
    uint32_t completed;
    uint32_t groups;
    uint32_t group_ctas;
    uint32_t blocks;
    uint32_t max_phases;
    uint64_t phases;
    uint64_t reached;
    uint64_t edges_reached;  /* GTEPS numerator summed over instances */
} gbs_batch_stats;

/* Uploads count host CSRs into one device allocation (rows sorted as in
 * gbs_graph_create).  Same validation; every graph has the same wtype. */
gbs_status gbs_pack_create(uint32_t count, const gbs_csr_view *graphs, gbs_weight_type wtype,
                           gbs_pack **out);
gbs_status gbs_pack_destroy(gbs_pack *p);
/* vertex_offsets (count+1, may be NULL) receives where each graph's vertices
 * start in a pack-wide vertex array: the layout of gbs_plan_pack's outputs. */
gbs_status gbs_pack_info(const gbs_pack *p, uint32_t *count, uint64_t *total_n, uint64_t *total_m,
                         uint64_t *vertex_offsets);

/* K sources on g.  dist_dev: k*n uint32/float32 (instance i at i*n), pred_dev:
 * k*n int32 or NULL.  g must outlive the plan. */
gbs_status gbs_plan_sources(gbs_graph *g, const uint32_t *sources, uint32_t k,
                            const gbs_batch_params *params, void *dist_dev, int32_t *pred_dev,
                            gbs_plan **out);
/* sources[i] on graph i of the pack.  dist_dev / pred_dev: total_n entries
 * in the gbs_pack_info vertex layout.  The pack must outlive the plan. */
gbs_status gbs_plan_pack(gbs_pack *p, const uint32_t *sources, const gbs_batch_params *params,
                         void *dist_dev, int32_t *pred_dev, gbs_plan **out);
/* Replays the captured launch on the plan's stream and returns at once. */
gbs_status gbs_plan_launch(gbs_plan *plan);
/* Waits for the last launch; per_instance (instances entries) may be NULL.
 * Returns the first device error, or GBS_ERR_TIMEOUT if instances were left
 * unsolved. */
gbs_status gbs_plan_wait(gbs_plan *plan, gbs_batch_stats *stats, gbs_inst_stats *per_instance);
gbs_status gbs_plan_destroy(gbs_plan *plan);

/*
 * Autotuner (no counterpart in the reference, which fixes the bucket width:
 * 0.4 in main/main.c:223, 0.1 in btwcentral/csr_bc.c:43).  Times candidate
 * schedules on the given sources and returns the fastest.  Every schedule
 * gives bit-identical distances and predecessors; only time changes.
 *
 * gbs_autotune (single source): bucket width as a multiple of the default
 * (max weight / average out-degree), light/heavy split at delta or none,
 * inline-row threshold, solo thresholds.  Coordinate search: the width for
 * each split, then the other knobs one at a time around the best.
 * gbs_autotune_plan_* (batched): CTAs per group, then the schedule.
 * budget_ms bounds the device time spent (0 = 4000 ms); at least the default
 * and one candidate are always timed.
 */
typedef struct gbs_tune_report {
    gbs_params best;         /* fastest schedule (delta and light explicit) */
    double best_ms;          /* its mean kernel time per source */
    double default_ms;       /* the plain schedule: default delta, light = delta */
    double delta_scale;      /* best delta / default delta */
    uint32_t candidates;     /* schedules timed */
    uint32_t runs;           /* SSSP runs made */
    int32_t no_split;        /* 1: the best schedule has no light/heavy split */
    uint32_t reserved;
} gbs_tune_report;

gbs_status gbs_autotune(gbs_graph *g, const uint32_t *sources, uint32_t count, double budget_ms,
                        gbs_tune_report *out);

typedef struct gbs_batch_tune_report {
    gbs_batch_params best;
    double best_ms;          /* device time of one launch with the best parameters */
    double default_ms;       /* the same with group_ctas chosen by the library, default schedule */
    uint32_t candidates;
    uint32_t reserved;
} gbs_batch_tune_report;

gbs_status gbs_autotune_plan_sources(gbs_graph *g, const uint32_t *sources, uint32_t k, double budget_ms,
                                     gbs_batch_tune_report *out);
gbs_status gbs_autotune_plan_pack(gbs_pack *p, const uint32_t *sources, double budget_ms,
                                  gbs_batch_tune_report *out);

/*
 * SSSP that allocates no memory (no counterpart in the reference).  For
 * callers that cannot call cudaMalloc/cudaFree while serving a query: a host
 * application that owns all device memory through its own pool, or a
 * latency-bound service for which an allocation (which may synchronise the
 * device or fail with out-of-memory mid-request) is not acceptable.  The
 * caller passes device buffers it owns:
 *   row_dev  n+1 uint32 exclusive row offsets (row_dev[0] = 0, row_dev[n] = m)
 *   adj_dev  2*m uint32: per edge {target, weight bits}, rows in any order;
 *            read 8 bytes at a time, so adj_dev must be 8-byte aligned
 *   dist_dev n uint32/float32 distances (required), pred_dev n int32 (may be NULL)
 * row_dev, dist_dev and pred_dev must be 4-byte aligned; a misaligned pointer
 * returns GBS_ERR_INVALID_ARG before any device work.
 * Weights are uint32 or float32 (>= 0) per wtype; delta <= 0 selects max
 * weight / average out-degree.  Results equal gbs_sssp's bit for bit.
 * Everything else lives in one static device array of about 21 MB that the
 * library holds on every GPU that loads it: n must be at most 65,536 and m at
 * most 2,097,152 (larger inputs return GBS_ERR_INVALID_ARG).  The input CSR is
 * validated on the device first (GBS_ERR_INVALID_ARG if malformed).  Runs on
 * `stream` (a cudaStream_t, NULL = default stream) and waits for that stream
 * before returning (it reads the input check and the error word back).
 * The first call on a device (with that device current) looks up the static
 * array's address and caches it; make that first call before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race and
 * must be serialised by the caller.
 */
gbs_status gbs_sssp_noalloc(uint32_t n, uint64_t m, const uint32_t *row_dev,
                            const uint32_t *adj_dev, gbs_weight_type wtype, uint32_t source,
                            double delta, void *dist_dev, int32_t *pred_dev, void *stream);

/* Pinned host memory for fast transfers. */
gbs_status gbs_host_alloc(size_t bytes, void **out);
gbs_status gbs_host_free(void *p);
/* Device memory for gbs_sssp_device outputs (plain cudaMalloc / cudaFree). */
gbs_status gbs_device_alloc(size_t bytes, void **out);
gbs_status gbs_device_free(void *p);
/* Blocks until all work the library queued on the device has finished. */
gbs_status gbs_device_synchronize(void);
/* Synchronous copy between any host and device buffers (cudaMemcpyDefault). */
gbs_status gbs_memcpy(void *dst, const void *src, size_t bytes);

/*
 * Synthetic inputs (host-side C generators; deterministic for a given seed).
 * R-MAT: edgefactor * 2^scale samples with a,b,c,d = .57,.19,.19,.05, vertex
 * ids permuted, self loops dropped, symmetrised, duplicates removed.  Grid:
 * rows x cols vertices, 4-neighbour, symmetric.  Weights belong to the
 * undirected pair: uint32 uniform in [wmin, wmax], or float32 uniform in
 * [1, 1000) on a 2^-14 lattice.  Rows are sorted by column.
 */
typedef struct gbs_host_csr {
    uint32_t n;
    uint64_t m;
    uint64_t *row_offsets;   /* n+1 */
    uint32_t *cols;          /* m */
    void *weights;           /* m uint32 or float32 */
    gbs_weight_type wtype;
} gbs_host_csr;

gbs_status gbs_gen_rmat(uint32_t scale, uint32_t edgefactor, uint64_t seed,
                        gbs_weight_type wtype, uint32_t wmin, uint32_t wmax,
                        gbs_host_csr **out);
gbs_status gbs_gen_grid(uint32_t rows, uint32_t cols, uint64_t seed,
                        gbs_weight_type wtype, uint32_t wmin, uint32_t wmax,
                        gbs_host_csr **out);
/* count distinct vertices of out-degree > 0, drawn with the given seed */
gbs_status gbs_sample_sources(const gbs_host_csr *g, uint32_t count, uint64_t seed,
                              uint32_t *out, uint32_t *got);
void gbs_host_csr_free(gbs_host_csr *g);

#ifdef __cplusplus
}
#endif
#endif /* GBSSSP_H */
