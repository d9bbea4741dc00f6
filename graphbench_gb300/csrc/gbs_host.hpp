// gbs_host.hpp -- host-side pieces shared by the translation units of
// libgbsssp: the resident graph handle, error reporting, the bucket schedule
// resolution and the workspace allocation.
#pragma once

#include <string>
#include <vector>

#include "gbs_sssp_persistent.cuh"

namespace gbs {

// Sets the thread's last-error message and returns the status.
inline gbs_status fail(gbs_status s, const std::string &msg) {
    set_last_error(msg.c_str());
    return s;
}

#define GBS_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return ::gbs::fail(e_ == cudaErrorMemoryAllocation ? GBS_ERR_NO_MEMORY : GBS_ERR_CUDA, \
                               std::string(#call) + ": " + cudaGetErrorString(e_));          \
    } while (0)

}  // namespace gbs

// A graph resident on one device: CSR with rows sorted by (weight, col), the
// per-run workspace of the single-source kernel and the cached light split.
struct gbs_graph {
    uint32_t n = 0;
    uint64_t m = 0;
    gbs_weight_type wtype = GBS_WEIGHT_U32;
    double max_w = 0.0;
    bool zero_w = false;                    // some edge weighs 0
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    uint32_t *d_row = nullptr;
    uint2 *d_adj = nullptr;
    unsigned long long *d_w64 = nullptr;    // float64 graphs: weights in adj order
    // workspace
    bool ws_ready = false;
    gbs::Workspace ws{};
    uint32_t *d_dist = nullptr;
    int32_t *d_pred = nullptr;
    unsigned long long mid_light_key = 0;   // light bound the cached split index was built for
    bool mid_valid = false;
    uint32_t epoch = 1, hround = 1;
    uint32_t trace_n = 0;
    int blocks = 0;
    gbs::Ctl host_ctl{};
    double mean_w = 0.0;
    // learned bucket-width controller (gbs_graph_set_controller)
    float *d_mlp = nullptr;
    std::vector<float> mlp_host;
    double ctrl_margin = 0.25;
    double plain_ms = 0.0;        // kernel time of the plain schedule on this graph (the guard)
    bool ctrl_lost = false;       // a learned run lost to plain here: run plain from now on
    // recorded controller inputs (GBS_F_FEATURES)
    float *d_feat = nullptr;
    uint32_t feat_cap = 0, feat_n = 0;
    // betweenness state (gbs_bc), allocated on first use
    void *bc = nullptr;
};

// A CSR on the device as the reference's readers lay it out (gbs_ingest.cu):
// rows in file order, weights where the reference stores them.
struct gbs_device_csr {
    uint32_t n = 0;
    uint64_t m = 0;
    unsigned long long *d_row = nullptr;   // exclusive offsets, n + 1
    uint32_t *d_col = nullptr;
    double *d_w = nullptr;
};

namespace gbs {

// Bucket width and light bound of one run, as the kernel uses them.
struct Resolved {
    double delta, light;
    uint32_t delta_u, light_bits;
    float inv_delta_f;
    double inv_delta_d;                 // float64 graphs
    unsigned long long light_key;       // bits of the light bound in the weight type
};

// Bytes of one distance in the weight type (4, or 8 for float64).
size_t dist_bytes(gbs_weight_type wt);

// max weight / average out-degree (1 for an empty graph).
double default_delta(double max_w, uint32_t n, uint64_t m);
// delta <= 0 selects default_delta; light < 0 selects light = delta.
Resolved resolve_schedule(gbs_weight_type wt, double max_w, uint32_t n, uint64_t m, double delta, double light);
// Bit pattern of the largest weight (uint32 value or float32 bits).
uint32_t max_weight_bits(gbs_weight_type wt, double max_w);

// Sorts each row by (weight bits, col) into adj (host, all cores).
void sort_rows(const uint64_t *row, const uint32_t *cols, const uint32_t *wbits, uint32_t n,
               std::vector<uint2> &adj);

// Validates a host CSR (offsets, targets, weights: finite and >= 0 for
// float32, -0 stored as +0) and returns its uint32 offsets, its rows sorted
// by (weight, col) as {col, weight bits} and its largest weight.
// float64 weights (w64 given) keep adj = {col, 0} and the weights in w64.
gbs_status prepare_csr(uint32_t n, uint64_t m, const uint64_t *row_offsets, const uint32_t *cols,
                       const void *weights, gbs_weight_type wtype, std::vector<uint32_t> &row32,
                       std::vector<uint2> &adj, double &max_w, std::vector<unsigned long long> *w64 = nullptr);

// Launches the first-heavy-edge search: mid[v] = first edge of row v whose
// weight bits exceed light_bits.
gbs_status launch_mid(const uint32_t *row, const uint2 *adj, uint32_t n, uint32_t light_bits, uint32_t *mid,
                      int sms, cudaStream_t s);

// Allocates the lists of a workspace for graphs of at most n_cap vertices
// and m_cap edges (dp, tag, fst, hst, ring, fq, S, pend, desc, ctl; fst, hst
// and ctl zeroed).  mid and trace are left to the caller.
gbs_status alloc_workspace(Workspace &w, uint32_t n_cap, uint64_t m_cap, cudaStream_t s);
void free_workspace(Workspace &w);

// Resident CTAs of the persistent kernels on one SM (0 if they cannot run).
int persistent_ctas_per_sm(gbs_weight_type wt, bool batch);

// A graph handle without device arrays (stream, events, device attributes);
// the caller fills d_row / d_adj / d_w64 (free_graph releases them).
gbs_status graph_shell(uint32_t n, uint64_t m, gbs_weight_type wtype, double max_w, double mean_w, bool zero_w,
                       gbs_graph **out);
void free_graph(gbs_graph *g);

// Allocates the single-source workspace of a graph on first use.
gbs_status ensure_workspace(gbs_graph *g);
// One single-source run (learned controller and its guard included) with the
// outputs in device memory (either may be null); the distances stay in the
// workspace's state words until the next run.
gbs_status run_sssp(gbs_graph *g, uint32_t src, const gbs_params *p, void *dist_dev, int32_t *pred_dev,
                    gbs_stats *stats);
// Releases the betweenness state of a graph.
void free_bc(gbs_graph *g);

}  // namespace gbs
