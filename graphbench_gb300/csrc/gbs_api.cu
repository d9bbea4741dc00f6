// gbs_api.cu -- the C ABI of libgbsssp (include/gbsssp.h): graph upload,
// workspace, launch sequence of one SSSP run, error reporting.
//
// One run on the graph's stream:
//   [mid]   first-heavy-edge index per row, only when the light split changes
//   reset   dp = unreached, tag = none, control block, source in ring bucket 0
//   persistent cooperative kernel (gbs_sssp_persistent.cuh)
//   unpack  dp -> dist / pred in the caller's layout
//   [stats] reached vertices and edges (the GTEPS numerator)
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gbs_host.hpp"

using namespace gbs;

namespace {

thread_local std::string g_last_error;

}  // namespace

void gbs::set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }

namespace {

// ------------------------------------------------------------------ kernels
__global__ void k_mid(const uint32_t *__restrict__ row, const uint2 *__restrict__ adj, uint32_t n,
                      uint32_t light_bits, uint32_t *__restrict__ mid) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        uint32_t lo = row[v], hi = row[v + 1];
        while (lo < hi) {  // first edge with weight > light
            const uint32_t m = lo + ((hi - lo) >> 1);
            if (adj[m].y <= light_bits) lo = m + 1;
            else hi = m;
        }
        mid[v] = lo;
    }
}

// src_word: the source's state word (uint32 / float32: dist 0, pred = src;
// float64: the distance 0.0 alone)
__global__ void k_reset(unsigned long long *__restrict__ dp, uint32_t *__restrict__ tag, uint32_t n,
                        uint32_t src, unsigned long long src_word, uint32_t *__restrict__ ring0, Ctl *ctl,
                        uint32_t span0, uint32_t full0) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        dp[v] = (v == src) ? src_word : kUnreached;
        tag[v] = (v == src) ? 0u : kTagInit;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ring0[0] = src;
        ctl->ring_cnt[0].v = 1;
        ctl->pend_min[0].v = kTagInit;
        ctl->pend_min[1].v = kTagInit;
        ctl->pub_phase = kPhLightFirst;
        ctl->pub_b = 0;
        ctl->pub_span = span0;   // bucket 0 spans span0 base widths
        ctl->pub_full = full0;
    }
}

template <bool F32>
__global__ void k_unpack(const unsigned long long *__restrict__ dp, uint32_t n, uint32_t src,
                         uint32_t *__restrict__ dist, int32_t *__restrict__ pred) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const unsigned long long x = dp[v];
        const bool reached = x != kUnreached;
        if (dist) dist[v] = reached ? (uint32_t)(x >> 32) : (F32 ? 0x7F800000u : 0xFFFFFFFFu);
        if (pred) pred[v] = reached ? (v == src ? (int32_t)src : (int32_t)(uint32_t)x) : -1;
    }
}

// float64 runs: dp holds the distance alone.  dist gets the double (+inf
// unreached); pred starts at the source / "not found yet" / -1 for k_pred64.
constexpr unsigned long long kInfBits64 = 0x7FF0000000000000ull;
__global__ void k_unpack64(const unsigned long long *__restrict__ dp, uint32_t n, uint32_t src,
                           unsigned long long *__restrict__ dist, int32_t *__restrict__ pred) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const unsigned long long x = dp[v];
        const bool reached = x != kUnreached;
        if (dist) dist[v] = reached ? x : kInfBits64;
        if (pred) pred[v] = reached ? (v == src ? (int32_t)src : INT32_MAX) : -1;
    }
}

// float64 predecessors: the smallest u with an edge (u, v) and dist[u] + w ==
// dist[v] in double (the same rounded add as the relaxation).  One warp per
// row; every reached vertex other than the source has such an edge.
__global__ void k_pred64(const uint32_t *__restrict__ row, const uint2 *__restrict__ adj,
                         const unsigned long long *__restrict__ w64, const unsigned long long *__restrict__ dp,
                         uint32_t n, uint32_t src, int32_t *__restrict__ pred) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += warps) {
        const unsigned long long du = dp[u];
        if (du == kUnreached) continue;
        const double d = __longlong_as_double((long long)du);
        for (uint32_t e = row[u] + lane; e < row[u + 1]; e += 32u) {
            const uint32_t v = adj[e].x;
            if (v == src) continue;
            const unsigned long long dv = __ldg(dp + v);
            if (dv == kUnreached) continue;
            const double s = __dadd_rn(d, __longlong_as_double((long long)w64[e]));
            if ((unsigned long long)__double_as_longlong(s) == dv) atomicMin(pred + v, (int32_t)u);
        }
    }
}

__global__ void k_mid64(const uint32_t *__restrict__ row, const unsigned long long *__restrict__ w64, uint32_t n,
                        unsigned long long light_bits, uint32_t *__restrict__ mid) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        uint32_t lo = row[v], hi = row[v + 1];
        while (lo < hi) {  // first edge with weight > light
            const uint32_t m = lo + ((hi - lo) >> 1);
            if (w64[m] <= light_bits) lo = m + 1;
            else hi = m;
        }
        mid[v] = lo;
    }
}

__global__ void k_stats(const unsigned long long *__restrict__ dp, const uint32_t *__restrict__ row,
                        uint32_t n, Ctl *ctl) {
    unsigned long long r = 0, e = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        if (dp[v] != kUnreached) {
            ++r;
            e += row[v + 1] - row[v];
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_down_sync(0xffffffffu, r, o);
        e += __shfl_down_sync(0xffffffffu, e, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (r) atomicAdd(&ctl->st_reached, r);
        if (e) atomicAdd(&ctl->st_edges_reached, e);
    }
}

}  // namespace

namespace gbs {

void sort_rows(const uint64_t *row, const uint32_t *cols, const uint32_t *wbits, uint32_t n,
               std::vector<uint2> &adj) {
    unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::atomic<uint32_t> next{0};
    const uint32_t grain = 4096;
    auto worker = [&]() {
        std::vector<uint64_t> keys;
        for (;;) {
            const uint32_t v0 = next.fetch_add(grain);
            if (v0 >= n) break;
            const uint32_t v1 = std::min<uint64_t>((uint64_t)v0 + grain, n);
            for (uint32_t v = v0; v < v1; ++v) {
                const uint64_t b = row[v], e = row[v + 1];
                keys.resize(e - b);
                for (uint64_t i = b; i < e; ++i) keys[i - b] = ((uint64_t)wbits[i] << 32) | cols[i];
                std::sort(keys.begin(), keys.end());
                for (uint64_t i = b; i < e; ++i)
                    adj[i] = make_uint2((uint32_t)keys[i - b], (uint32_t)(keys[i - b] >> 32));
            }
        }
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; ++t) th.emplace_back(worker);
    worker();
    for (auto &t : th) t.join();
}

// float64 rows: sorted by (weight bits, col); adj gets {col, 0}, w64 the
// weights in the same order.
void sort_rows64(const uint64_t *row, const uint32_t *cols, const uint64_t *wbits, uint32_t n,
                 std::vector<uint2> &adj, std::vector<unsigned long long> &w64) {
    unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::atomic<uint32_t> next{0};
    const uint32_t grain = 4096;
    auto worker = [&]() {
        std::vector<std::pair<uint64_t, uint32_t>> keys;
        for (;;) {
            const uint32_t v0 = next.fetch_add(grain);
            if (v0 >= n) break;
            const uint32_t v1 = std::min<uint64_t>((uint64_t)v0 + grain, n);
            for (uint32_t v = v0; v < v1; ++v) {
                const uint64_t b = row[v], e = row[v + 1];
                keys.resize(e - b);
                for (uint64_t i = b; i < e; ++i) keys[i - b] = {wbits[i], cols[i]};
                std::sort(keys.begin(), keys.end());
                for (uint64_t i = b; i < e; ++i) {
                    adj[i] = make_uint2(keys[i - b].second, 0u);
                    w64[i] = keys[i - b].first;
                }
            }
        }
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; ++t) th.emplace_back(worker);
    worker();
    for (auto &t : th) t.join();
}

gbs_status prepare_csr(uint32_t n, uint64_t m, const uint64_t *row_offsets, const uint32_t *cols,
                       const void *weights, gbs_weight_type wtype, std::vector<uint32_t> &row32,
                       std::vector<uint2> &adj, double &max_w, std::vector<unsigned long long> *w64) {
    if (!row_offsets || (m && (!cols || !weights)))
        return fail(GBS_ERR_INVALID_ARG, "NULL CSR array");
    if (wtype != GBS_WEIGHT_U32 && wtype != GBS_WEIGHT_F32 && !(wtype == GBS_WEIGHT_F64 && w64))
        return fail(GBS_ERR_INVALID_ARG, "unknown or unsupported weight type");
    if (n == 0 || n > 0x7FFFFFFFu) return fail(GBS_ERR_INVALID_ARG, "vertex count must be in [1, 2^31)");
    if (m >= 0xFFFFFFFFull) return fail(GBS_ERR_UNSUPPORTED, "edge count must be < 2^32");
    if (row_offsets[0] != 0 || row_offsets[n] != m)
        return fail(GBS_ERR_INVALID_ARG, "row_offsets must start at 0 and end at m");
    for (uint32_t v = 0; v < n; ++v)
        if (row_offsets[v + 1] < row_offsets[v]) return fail(GBS_ERR_INVALID_ARG, "row_offsets decrease");
    max_w = 0.0;
    if (wtype == GBS_WEIGHT_F64) {
        std::vector<uint64_t> wb(m);
        for (uint64_t e = 0; e < m; ++e) {
            if (cols[e] >= n) return fail(GBS_ERR_INVALID_ARG, "column index out of range");
            double w = ((const double *)weights)[e];
            if (!(w >= 0.0) || std::isinf(w))
                return fail(GBS_ERR_INVALID_ARG, "float64 weights must be finite and >= 0");
            if (w == 0.0) w = 0.0;  // -0.0 -> +0.0
            std::memcpy(&wb[e], &w, 8);
            if (w > max_w) max_w = w;
        }
        adj.resize(m);
        w64->resize(m);
        sort_rows64(row_offsets, cols, wb.data(), n, adj, *w64);
        row32.resize((size_t)n + 1);
        for (uint32_t v = 0; v <= n; ++v) row32[v] = (uint32_t)row_offsets[v];
        return GBS_OK;
    }
    std::vector<uint32_t> wbits(m);
    for (uint64_t e = 0; e < m; ++e) {
        if (cols[e] >= n) return fail(GBS_ERR_INVALID_ARG, "column index out of range");
        if (wtype == GBS_WEIGHT_U32) {
            const uint32_t w = ((const uint32_t *)weights)[e];
            wbits[e] = w;
            if (w > max_w) max_w = w;
        } else {
            float w = ((const float *)weights)[e];
            if (!(w >= 0.0f) || std::isinf(w))
                return fail(GBS_ERR_INVALID_ARG, "float32 weights must be finite and >= 0");
            if (w == 0.0f) w = 0.0f;  // -0.0 -> +0.0
            std::memcpy(&wbits[e], &w, 4);
            if (w > max_w) max_w = w;
        }
    }
    adj.resize(m);
    sort_rows(row_offsets, cols, wbits.data(), n, adj);
    row32.resize((size_t)n + 1);
    for (uint32_t v = 0; v <= n; ++v) row32[v] = (uint32_t)row_offsets[v];
    return GBS_OK;
}

gbs_status alloc_workspace(Workspace &w, uint32_t n_cap, uint64_t m_cap, cudaStream_t s) {
    const size_t n = n_cap ? n_cap : 1;
    GBS_CUDA(cudaMalloc(&w.dp, sizeof(unsigned long long) * n));
    GBS_CUDA(cudaMalloc(&w.tag, sizeof(uint32_t) * n));
    GBS_CUDA(cudaMalloc(&w.fst, sizeof(uint32_t) * n));
    GBS_CUDA(cudaMalloc(&w.hst, sizeof(uint32_t) * n));
    GBS_CUDA(cudaMalloc(&w.ring, sizeof(uint32_t) * n * kNB));
    GBS_CUDA(cudaMalloc(&w.fq, sizeof(uint32_t) * n * 3));
    GBS_CUDA(cudaMalloc(&w.pend, sizeof(uint32_t) * n * 2));
    // a SCAN reads at most n entries and cuts each row into ceil(len/kDescEdges)
    // descriptors, so it emits at most n + m/kDescEdges of them
    const uint64_t cap = (uint64_t)n_cap + m_cap / kDescEdges + 64;
    w.desc_cap = (uint32_t)std::min<uint64_t>(cap, 0xFFFFFFF0ull);
    GBS_CUDA(cudaMalloc(&w.desc, sizeof(uint4) * (size_t)w.desc_cap));
    GBS_CUDA(cudaMalloc(&w.hdesc, sizeof(uint4) * (size_t)w.desc_cap));
    GBS_CUDA(cudaMalloc(&w.ctl, sizeof(Ctl)));
    GBS_CUDA(cudaMemsetAsync(w.fst, 0, sizeof(uint32_t) * n, s));
    GBS_CUDA(cudaMemsetAsync(w.hst, 0, sizeof(uint32_t) * n, s));
    GBS_CUDA(cudaMemsetAsync(w.ctl, 0, sizeof(Ctl), s));
    w.n_cap = n_cap;
    return GBS_OK;
}

void free_workspace(Workspace &w) {
    cudaFree(w.dp); cudaFree(w.tag); cudaFree(w.fst); cudaFree(w.hst);
    cudaFree(w.ring); cudaFree(w.fq); cudaFree(w.pend); cudaFree(w.desc); cudaFree(w.hdesc); cudaFree(w.ctl);
    w = Workspace{};
}

int persistent_ctas_per_sm(gbs_weight_type wt, bool batch) {
    const void *kfn;
    if (batch) {
        if (wt == GBS_WEIGHT_F64) return 0;   // batched launches take uint32 / float32 graphs
        kfn = wt == GBS_WEIGHT_F32 ? (const void *)sssp_batch<kWF32> : (const void *)sssp_batch<kWU32>;
    } else {
        kfn = wt == GBS_WEIGHT_F64   ? (const void *)sssp_persistent<kWF64>
              : wt == GBS_WEIGHT_F32 ? (const void *)sssp_persistent<kWF32>
                                     : (const void *)sssp_persistent<kWU32>;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, kTPB, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm;
}

gbs_status launch_mid(const uint32_t *row, const uint2 *adj, uint32_t n, uint32_t light_bits, uint32_t *mid,
                      int sms, cudaStream_t s) {
    const int tb = 256;
    const int eb = std::max(1, std::min<int>((n + tb - 1) / tb, sms * 8));
    k_mid<<<eb, tb, 0, s>>>(row, adj, n, light_bits, mid);
    GBS_CUDA(cudaGetLastError());
    return GBS_OK;
}

gbs_status ensure_workspace(gbs_graph *g) {
    if (g->ws_ready) return GBS_OK;
    const size_t n = g->n ? g->n : 1;
    gbs_status st = alloc_workspace(g->ws, g->n, g->m, g->stream);
    if (st != GBS_OK) return st;
    GBS_CUDA(cudaMalloc(&g->ws.mid, sizeof(uint32_t) * n));
    g->ws.trace = nullptr;
    g->ws.trace_cap = 0;
    GBS_CUDA(cudaMalloc(&g->d_dist, dist_bytes(g->wtype) * n));
    GBS_CUDA(cudaMalloc(&g->d_pred, sizeof(int32_t) * n));
    g->epoch = 1;
    g->hround = 1;
    const int per_sm = persistent_ctas_per_sm(g->wtype, false);
    if (per_sm < 1) return fail(GBS_ERR_UNSUPPORTED, "persistent kernel cannot be resident");
    g->blocks = per_sm * g->sms;
    g->ws_ready = true;
    return GBS_OK;
}

void free_graph(gbs_graph *g) {
    if (!g) return;
    cudaFree(g->d_row);
    cudaFree(g->d_adj);
    cudaFree(g->d_w64);
    cudaFree(g->ws.mid);
    cudaFree(g->ws.trace);
    free_workspace(g->ws);
    cudaFree(g->d_dist);
    cudaFree(g->d_pred);
    cudaFree(g->d_mlp);
    cudaFree(g->d_feat);
    free_bc(g);
    for (auto &e : g->ev) if (e) cudaEventDestroy(e);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

double default_delta(double max_w, uint32_t n, uint64_t m) {
    if (m == 0 || n == 0) return 1.0;
    const double avg = (double)m / (double)n;
    const double d = max_w / avg;
    return d > 0 ? d : 1.0;
}

size_t dist_bytes(gbs_weight_type wt) { return wt == GBS_WEIGHT_F64 ? 8 : 4; }

uint32_t max_weight_bits(gbs_weight_type wt, double max_w) {
    if (wt == GBS_WEIGHT_U32) return (uint32_t)max_w;
    const float mf = (float)max_w;
    uint32_t bits;
    std::memcpy(&bits, &mf, 4);
    return bits;
}

Resolved resolve_schedule(gbs_weight_type wt, double max_w, uint32_t n, uint64_t m, double delta, double light) {
    Resolved r{};
    if (!(delta > 0)) delta = default_delta(max_w, n, m);
    if (!(light >= 0)) light = -1.0;
    if (wt == GBS_WEIGHT_U32) {
        double fd = std::floor(delta);
        r.delta_u = (uint32_t)std::min(std::max(fd, 1.0), 4294967295.0);
        r.delta = r.delta_u;
        if (light < 0) light = r.delta;
        const double fl = std::floor(light);
        r.light_bits = (uint32_t)std::min(std::max(fl, 0.0), 4294967295.0);
        r.light = r.light_bits;
        r.inv_delta_f = 0.f;
        r.light_key = r.light_bits;
    } else if (wt == GBS_WEIGHT_F64) {
        r.delta = delta;
        r.inv_delta_d = 1.0 / delta;
        r.inv_delta_f = (float)r.inv_delta_d;
        if (light < 0) light = delta;
        if (std::isinf(light)) light = 1.7976931348623157e308;
        r.light = light;
        std::memcpy(&r.light_key, &light, 8);
        r.light_bits = 0;
        r.delta_u = 1;
    } else {
        r.delta = delta;
        r.inv_delta_f = (float)(1.0 / delta);
        if (light < 0) light = delta;
        float lf = (float)light;
        if ((double)lf > light) lf = std::nextafter(lf, -INFINITY);
        if (lf < 0) lf = 0;
        if (std::isinf(lf)) lf = 3.4028234663852886e38f;
        uint32_t bits;
        std::memcpy(&bits, &lf, 4);
        r.light_bits = bits;
        r.light = lf;
        r.delta_u = 1;
        r.light_key = bits;
    }
    return r;
}

// The controller network on the host (first prediction of a learned run).
float mlp_host(const float *P, const float (&x)[kFeat], float &y1) {
    float xn[kFeat], h1[kHid], h2[kHid];
    for (int i = 0; i < kFeat; ++i) xn[i] = (x[i] - P[i]) / P[kFeat + i];
    for (int o = 0; o < kHid; ++o) {
        float acc = P[kMlpB1 + o];
        for (int i = 0; i < kFeat; ++i) acc = std::fma(xn[i], P[kMlpW1 + i * kHid + o], acc);
        h1[o] = std::max(acc, 0.f);
    }
    for (int o = 0; o < kHid; ++o) {
        float acc = P[kMlpB2 + o];
        for (int i = 0; i < kHid; ++i) acc = std::fma(h1[i], P[kMlpW2 + i * kHid + o], acc);
        h2[o] = std::max(acc, 0.f);
    }
    float y0 = P[kMlpB3], y = P[kMlpB3 + 1];
    for (int o = 0; o < kHid; ++o) {
        y0 += h2[o] * P[kMlpW3 + 2 * o];
        y += h2[o] * P[kMlpW3 + 2 * o + 1];
    }
    y1 = y;
    return y0;
}

// Graph inputs of the controller: f[1..3] are inputs 12..14 (average
// degree, largest weight, mean / largest weight), f[4] (input 15, the base
// width over the plain one) is set per run.  f[0] (log2 of the vertex count)
// is kept for reports only: the network sees no input that grows with the
// graph by itself, so it does not extrapolate along the graph size.
void graph_features(const gbs_graph *g, float *f) {
    const double avg = g->n ? (double)g->m / (double)g->n : 0.0;
    f[0] = (float)std::log2((double)std::max<uint32_t>(g->n, 1));
    f[1] = (float)std::log2(std::max(avg, 1e-3));
    f[2] = (float)std::log2(std::max(g->max_w, 1e-30));
    f[3] = g->max_w > 0 ? (float)(g->mean_w / g->max_w) : 0.f;
}

gbs_status launch_run(gbs_graph *g, uint32_t src, const gbs_params *p, void *dist_dev,
                      int32_t *pred_dev, gbs_stats *stats, bool learned, bool *guard_hit) {
    if (src >= g->n) return fail(GBS_ERR_INVALID_ARG, "source out of range");
    if (guard_hit) *guard_hit = false;
    gbs_status st = ensure_workspace(g);
    if (st != GBS_OK) return st;
    const double d_def = default_delta(g->max_w, g->n, g->m);
    Resolved r;
    float gfeat[5];
    graph_features(g, gfeat);
    float span_bias = 0.f;
    uint32_t span0 = 1, full0 = 0;
    if (learned) {
        // the controller's first prediction (bucket 0 holds only the source),
        // clamped to the range the training labels cover, fixes the base
        // width: half the predicted delta, so spans of 1..8 base widths reach
        // 2x below and 4x above it; the split is at the predicted delta.
        // (Measured with the same trained block: spans of up to 64 base
        // widths of an eighth of the prediction let the per-bucket outputs
        // run 4-16x wide on R-MAT 22 / 24, 0.49x / 0.29x of plain; up to 8
        // of a half, 0.92x / 0.83x, and the grids and smaller R-MATs gain.)
        // input: the source alone in the window, whose entries input (6)
        // carries log2(1 + n), the vertices the run will settle (the
        // controller's training pipeline encodes the initial state the same
        // way), and the graph inputs
        float x[kFeat];
        for (int i = 0; i < 6; ++i) x[i] = 1.f;
        x[6] = (float)std::log2(1.0 + (double)g->n);
        for (int i = 7; i < 12; ++i) x[i] = 0.f;
        for (int i = 1; i < 4; ++i) x[11 + i] = gfeat[i];
        x[15] = 0.f;
        float y1 = 0.f;
        const float y0 = mlp_host(g->mlp_host.data(), x, y1);
        const double p0 = std::rint(std::min(std::max((double)y0, -2.0), 14.0));
        r = resolve_schedule(g->wtype, g->max_w, g->n, g->m, d_def * std::exp2(p0 - 1.0), d_def * std::exp2(p0));
        span_bias = (float)std::log2(d_def / r.delta);
        int e0 = (int)std::rint(y0 + span_bias);
        e0 = std::min(std::max(e0, 0), (int)kLearnedSpanLog);
        span0 = 1u << e0;
        full0 = y1 <= 0.f ? 1u : 0u;
    } else {
        r = resolve_schedule(g->wtype, g->max_w, g->n, g->m, p ? p->delta : 0.0, p ? p->light : -1.0);
    }
    gfeat[4] = (float)std::log2(r.delta / d_def);
    cudaStream_t s = g->stream;
    const int tb = 256;
    const int eb = std::max(1, std::min<int>((g->n + tb - 1) / tb, g->sms * 8));
    if (!g->mid_valid || g->mid_light_key != r.light_key) {
        if (g->wtype == GBS_WEIGHT_F64) {
            k_mid64<<<eb, tb, 0, s>>>(g->d_row, g->d_w64, g->n, r.light_key, g->ws.mid);
            GBS_CUDA(cudaGetLastError());
        } else {
            st = launch_mid(g->d_row, g->d_adj, g->n, r.light_bits, g->ws.mid, g->sms, s);
            if (st != GBS_OK) return st;
        }
        g->mid_light_key = r.light_key;
        g->mid_valid = true;
    }
    if (g->epoch > 0xF0000000u || g->hround > 0xF0000000u) {
        GBS_CUDA(cudaMemsetAsync(g->ws.fst, 0, sizeof(uint32_t) * g->n, s));
        GBS_CUDA(cudaMemsetAsync(g->ws.hst, 0, sizeof(uint32_t) * g->n, s));
        g->epoch = 1;
        g->hround = 1;
    }
    SsspArgs a{};
    a.g.n = g->n;
    a.g.m = g->m;
    a.g.wtype = g->wtype;
    a.g.row = g->d_row;
    a.g.adj = g->d_adj;
    a.ws = g->ws;
    a.source = src;
    a.epoch0 = g->epoch;
    a.hround0 = g->hround;
    a.delta_u = r.delta_u;
    a.inv_delta_f = r.inv_delta_f;
    a.inv_delta_d = r.inv_delta_d;
    a.g.w64 = g->d_w64;
    a.wait_ns = (unsigned long long)((p && p->wait_limit_ms) ? p->wait_limit_ms : 4000u) * 1000000ull;
    a.flags = p ? p->flags : 0u;
    const bool no_solo = (a.flags & GBS_F_NO_SOLO) != 0;
    a.solo_items = no_solo ? 0u : ((p && p->solo_entries) ? p->solo_entries : 1024u);
    a.solo_desc = no_solo ? 0u : ((p && p->solo_descs) ? p->solo_descs : 64u);
    a.no_heavy = (g->wtype == GBS_WEIGHT_F64 ? r.light >= g->max_w
                                             : r.light_bits >= max_weight_bits(g->wtype, g->max_w)) ? 1u : 0u;
    a.inline_max = (p && p->inline_edges) ? p->inline_edges : kInlineEdges;
    a.full_items = (p && p->full_items) ? p->full_items : std::max(g->n, kFullItems);
    a.fuse_rounds = (a.flags & GBS_F_NO_FUSE) ? 0u : ((p && p->fuse_rounds) ? p->fuse_rounds : kFuseRounds);
    a.run_ns = a.wait_ns * 16ull;
    a.ctrl = learned ? kCtrlLearned : kCtrlFixed;
    a.span_fixed = 1;
    a.span_bias = span_bias;
    a.mlp = learned ? g->d_mlp : nullptr;
    for (int i = 0; i < 5; ++i) a.gfeat[i] = gfeat[i];
    a.guard_ns = (learned && g->plain_ms > 0)
                     ? (unsigned long long)(g->plain_ms * (1.0 + g->ctrl_margin) * 1e6)
                     : 0ull;
    // the source's bucket holds one entry: whole rows under the fixed
    // schedule's rule (full_items >= 1), as every later bucket of that size
    if (!learned || a.no_heavy) full0 = (a.no_heavy || (!learned && a.full_items >= 1u)) ? 1u : 0u;
    if (a.flags & GBS_F_FEATURES) {
        if (!g->d_feat) {
            g->feat_cap = 1u << 18;
            GBS_CUDA(cudaMalloc(&g->d_feat, sizeof(float) * kFeat * g->feat_cap));
        }
        a.feat = g->d_feat;
        a.feat_cap = g->feat_cap;
    }
    a.group = 0;
    a.group_ctas = (uint32_t)g->blocks;
    a.ws.n_cap = g->n;
    if (a.flags & GBS_F_TRACE) {
        if (!g->ws.trace) {
            g->ws.trace_cap = 1u << 20;
            GBS_CUDA(cudaMalloc(&g->ws.trace, sizeof(TraceRec) * g->ws.trace_cap));
        }
        a.ws = g->ws;
    }

    GBS_CUDA(cudaEventRecord(g->ev[0], s));
    GBS_CUDA(cudaMemsetAsync(g->ws.ctl, 0, sizeof(Ctl), s));
    const unsigned long long src_word = g->wtype == GBS_WEIGHT_F64 ? 0ull : (unsigned long long)src;
    k_reset<<<eb, tb, 0, s>>>(g->ws.dp, g->ws.tag, g->n, src, src_word, g->ws.ring, g->ws.ctl, span0, full0);
    GBS_CUDA(cudaGetLastError());
    GBS_CUDA(cudaEventRecord(g->ev[1], s));
    void *args[] = {&a};
    const void *kfn = g->wtype == GBS_WEIGHT_F64   ? (const void *)sssp_persistent<kWF64>
                      : g->wtype == GBS_WEIGHT_F32 ? (const void *)sssp_persistent<kWF32>
                                                   : (const void *)sssp_persistent<kWU32>;
    GBS_CUDA(cudaLaunchCooperativeKernel(kfn, dim3(g->blocks), dim3(kTPB), args, 0, s));
    GBS_CUDA(cudaEventRecord(g->ev[2], s));
    if (dist_dev || pred_dev) {
        if (g->wtype == GBS_WEIGHT_F64) {
            k_unpack64<<<eb, tb, 0, s>>>(g->ws.dp, g->n, src, static_cast<unsigned long long *>(dist_dev), pred_dev);
            GBS_CUDA(cudaGetLastError());
            if (pred_dev) {
                k_pred64<<<g->sms * 8, 256, 0, s>>>(g->d_row, g->d_adj, g->d_w64, g->ws.dp, g->n, src, pred_dev);
                GBS_CUDA(cudaGetLastError());
            }
        } else if (g->wtype == GBS_WEIGHT_F32) {
            k_unpack<true><<<eb, tb, 0, s>>>(g->ws.dp, g->n, src, static_cast<uint32_t *>(dist_dev), pred_dev);
        } else {
            k_unpack<false><<<eb, tb, 0, s>>>(g->ws.dp, g->n, src, static_cast<uint32_t *>(dist_dev), pred_dev);
        }
        GBS_CUDA(cudaGetLastError());
    }
    GBS_CUDA(cudaEventRecord(g->ev[3], s));
    const bool want_stats = !(p && (p->flags & GBS_F_NO_STATS));
    if (want_stats) {
        k_stats<<<eb, tb, 0, s>>>(g->ws.dp, g->d_row, g->n, g->ws.ctl);
        GBS_CUDA(cudaGetLastError());
    }
    GBS_CUDA(cudaMemcpyAsync(&g->host_ctl, g->ws.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    GBS_CUDA(cudaStreamSynchronize(s));
    const Ctl &c = g->host_ctl;
    g->epoch = c.next_epoch + 1;
    g->hround = c.next_hround + 1;
    g->trace_n = (a.flags & GBS_F_TRACE) ? std::min(c.trace_n, g->ws.trace_cap) : 0u;
    g->feat_n = (a.flags & GBS_F_FEATURES) ? std::min(c.feat_n, g->feat_cap) : 0u;
    if (c.error != kErrNone) {
        // stamps of an aborted run are unknown: start over next time
        g->epoch = 0xF0000001u;
        if (c.error == kErrGuard && guard_hit) {
            // the time of the abandoned run is charged to the call
            *guard_hit = true;
            if (stats) {
                float ms = 0.f;
                std::memset(stats, 0, sizeof(*stats));
                GBS_CUDA(cudaEventElapsedTime(&ms, g->ev[0], g->ev[3]));
                stats->device_ms = ms;
                GBS_CUDA(cudaEventElapsedTime(&ms, g->ev[1], g->ev[2]));
                stats->kernel_ms = ms;
            }
            return GBS_OK;
        }
        switch (c.error) {
            case kErrTimeout: return fail(GBS_ERR_TIMEOUT, "device-side wait limit exceeded");
            case kErrCapacity: return fail(GBS_ERR_CAPACITY, "device work list overflow");
            case kErrOverflow: return fail(GBS_ERR_OVERFLOW, "uint32 path sum overflow");
            default: return fail(GBS_ERR_INTERNAL, "device error");
        }
    }
    if (stats) {
        float ms = 0.f;
        std::memset(stats, 0, sizeof(*stats));
        GBS_CUDA(cudaEventElapsedTime(&ms, g->ev[0], g->ev[3]));
        stats->device_ms = ms;
        GBS_CUDA(cudaEventElapsedTime(&ms, g->ev[1], g->ev[2]));
        stats->kernel_ms = ms;
        stats->reached = want_stats ? c.st_reached : 0;
        stats->edges_reached = want_stats ? c.st_edges_reached : 0;
        stats->improvements = c.st_improvements;
        stats->buckets = c.st_buckets;
        stats->phases = c.st_phases;
        stats->pending_scans = c.st_pending_scans;
        stats->blocks = (uint32_t)g->blocks;
        stats->solo_phases = c.st_solo_phases;
        stats->delta_used = r.delta;
        stats->light_used = r.light;
        stats->learned = learned ? 1u : 0u;
    }
    return GBS_OK;
}

// One SSSP with the schedule the flags ask for.  GBS_F_LEARNED: the first
// learned run on a graph is preceded by a plain run that times the plain
// schedule; a learned run that passes (1 + margin) x that time stops and the
// plain schedule runs instead.  When that plain run finished within the limit
// the controller lost, and later learned calls on the graph run the plain
// schedule directly; otherwise the source is just longer than the one timed
// and the plain time is raised to it.  Reported times include every run the
// call made.
gbs_status run_sssp(gbs_graph *g, uint32_t src, const gbs_params *p, void *dist_dev, int32_t *pred_dev,
                    gbs_stats *stats) {
    const bool learned = p && (p->flags & GBS_F_LEARNED);
    if (!learned) return launch_run(g, src, p, dist_dev, pred_dev, stats, false, nullptr);
    if (!g->d_mlp) return fail(GBS_ERR_INVALID_ARG, "GBS_F_LEARNED: no controller set (gbs_graph_set_controller)");
    gbs_params plain = *p;
    plain.flags &= ~GBS_F_LEARNED;
    plain.delta = 0.0;    // the plain heuristic: max weight / average out-degree
    plain.light = -1.0;   // light = delta
    gbs_stats ps{}, ls{}, rs{};
    gbs_status st;
    if (g->ctrl_lost) {   // the controller lost to plain on this graph before
        st = launch_run(g, src, &plain, dist_dev, pred_dev, &rs, false, nullptr);
        if (st != GBS_OK) return st;
        rs.learned = 2u;
        if (stats) *stats = rs;
        return GBS_OK;
    }
    if (!(g->plain_ms > 0)) {
        st = launch_run(g, src, &plain, nullptr, nullptr, &ps, false, nullptr);
        if (st != GBS_OK) return st;
        g->plain_ms = ps.kernel_ms;
    }
    bool guard = false;
    st = launch_run(g, src, p, dist_dev, pred_dev, &ls, true, &guard);
    if (st != GBS_OK) return st;
    if (!guard) {
        ls.kernel_ms += ps.kernel_ms;
        ls.device_ms += ps.device_ms;
        if (stats) *stats = ls;
        return GBS_OK;
    }
    st = launch_run(g, src, &plain, dist_dev, pred_dev, &rs, false, nullptr);
    if (st != GBS_OK) return st;
    // the learned run was stopped at the limit; it lost if the plain schedule
    // finished this source within that limit (5% timing noise allowed).  A
    // source whose plain run itself takes longer says nothing about the
    // controller: the limit grows to it instead.
    const double limit_ms = g->plain_ms * (1.0 + g->ctrl_margin);
    if (rs.kernel_ms <= limit_ms * 1.05) g->ctrl_lost = true;
    g->plain_ms = std::max(g->plain_ms, rs.kernel_ms);
    rs.kernel_ms += ps.kernel_ms + ls.kernel_ms;
    rs.device_ms += ps.device_ms + ls.device_ms;
    rs.learned = 3u;
    if (stats) *stats = rs;
    return GBS_OK;
}

gbs_status graph_shell(uint32_t n, uint64_t m, gbs_weight_type wtype, double max_w, double mean_w,
                       bool zero_w, gbs_graph **out) {
    int dev = 0;
    GBS_CUDA(cudaGetDevice(&dev));
    gbs_graph *g = new gbs_graph();
    g->n = n;
    g->m = m;
    g->wtype = wtype;
    g->max_w = max_w;
    g->mean_w = mean_w;
    g->zero_w = zero_w;
    g->device = dev;
    cudaError_t e;
    if ((e = cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        free_graph(g);
        return fail(GBS_ERR_CUDA, cudaGetErrorString(e));
    }
    for (auto &ev : g->ev) {
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) {
            free_graph(g);
            return fail(GBS_ERR_CUDA, cudaGetErrorString(e));
        }
    }
    *out = g;
    return GBS_OK;
}

}  // namespace gbs

// ===================================================================== C ABI
extern "C" {

const char *gbs_status_string(gbs_status s) {
    switch (s) {
        case GBS_OK: return "ok";
        case GBS_ERR_INVALID_ARG: return "invalid argument";
        case GBS_ERR_CUDA: return "CUDA error";
        case GBS_ERR_NO_MEMORY: return "out of memory";
        case GBS_ERR_CAPACITY: return "device work list capacity exceeded";
        case GBS_ERR_TIMEOUT: return "device wait limit exceeded";
        case GBS_ERR_OVERFLOW: return "uint32 distance overflow";
        case GBS_ERR_UNSUPPORTED: return "unsupported";
        case GBS_ERR_INTERNAL: return "internal error";
    }
    return "unknown status";
}

const char *gbs_last_error(void) { return g_last_error.c_str(); }

int gbs_abi_version(void) { return GBS_ABI_VERSION; }

int gbs_device_available(void) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) {
        cudaGetLastError();
        return 0;
    }
    int dev = 0, major = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) return 0;
    return major >= 10 ? 1 : 0;
}

gbs_status gbs_graph_create(uint32_t n, uint64_t m, const uint64_t *row_offsets, const uint32_t *cols,
                            const void *weights, gbs_weight_type wtype, gbs_graph **out) {
    if (!out) return fail(GBS_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    std::vector<uint32_t> row32;
    std::vector<uint2> adj;
    double max_w = 0.0;
    std::vector<unsigned long long> w64;
    gbs_status st = prepare_csr(n, m, row_offsets, cols, weights, wtype, row32, adj, max_w, &w64);
    if (st != GBS_OK) return st;
    double wsum = 0.0;
    for (uint64_t e = 0; e < m; ++e)
        wsum += wtype == GBS_WEIGHT_U32   ? (double)((const uint32_t *)weights)[e]
                : wtype == GBS_WEIGHT_F32 ? (double)((const float *)weights)[e]
                                          : ((const double *)weights)[e];
    bool zero_w = false;
    // rows are sorted by weight: a zero weight is the first of its row
    for (uint32_t v = 0; v < n && !zero_w; ++v)
        if (row32[v] < row32[v + 1])
            zero_w = wtype == GBS_WEIGHT_F64 ? w64[row32[v]] == 0ull : adj[row32[v]].y == 0u;
    gbs_graph *g = nullptr;
    st = graph_shell(n, m, wtype, max_w, m ? wsum / (double)m : 0.0, zero_w, &g);
    if (st != GBS_OK) return st;
    cudaError_t e;
    if ((e = cudaMalloc(&g->d_row, sizeof(uint32_t) * (n + 1))) != cudaSuccess ||
        (e = cudaMalloc(&g->d_adj, sizeof(uint2) * (m ? m : 1))) != cudaSuccess ||
        (e = cudaMemcpy(g->d_row, row32.data(), sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (m && (e = cudaMemcpy(g->d_adj, adj.data(), sizeof(uint2) * m, cudaMemcpyHostToDevice)) !=
                  cudaSuccess) ||
        (wtype == GBS_WEIGHT_F64 &&
         ((e = cudaMalloc(&g->d_w64, sizeof(unsigned long long) * (m ? m : 1))) != cudaSuccess ||
          (m && (e = cudaMemcpy(g->d_w64, w64.data(), sizeof(unsigned long long) * m, cudaMemcpyHostToDevice)) !=
                    cudaSuccess)))) {
        free_graph(g);
        return fail(e == cudaErrorMemoryAllocation ? GBS_ERR_NO_MEMORY : GBS_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = g;
    return GBS_OK;
}

gbs_status gbs_graph_destroy(gbs_graph *g) {
    if (!g) return fail(GBS_ERR_INVALID_ARG, "graph is NULL");
    cudaStreamSynchronize(g->stream);
    free_graph(g);
    return GBS_OK;
}

gbs_status gbs_graph_info(const gbs_graph *g, uint32_t *n, uint64_t *m, gbs_weight_type *wtype,
                          double *max_weight, double *def_delta) {
    if (!g) return fail(GBS_ERR_INVALID_ARG, "graph is NULL");
    if (n) *n = g->n;
    if (m) *m = g->m;
    if (wtype) *wtype = g->wtype;
    if (max_weight) *max_weight = g->max_w;
    if (def_delta) *def_delta = default_delta(g->max_w, g->n, g->m);
    return GBS_OK;
}

gbs_status gbs_sssp_device(gbs_graph *g, uint32_t source, const gbs_params *params, void *dist_dev,
                           int32_t *pred_dev, gbs_stats *stats) {
    if (!g) return fail(GBS_ERR_INVALID_ARG, "graph is NULL");
    return run_sssp(g, source, params, dist_dev, pred_dev, stats);
}

// The device address of page-locked host memory (gbs_host_alloc,
// cudaMallocHost, cudaHostRegister), or null for any other pointer.
static void *device_view(void *host) {
    if (!host) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError();   // a pointer the runtime does not know: not an error of the call
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

gbs_status gbs_sssp(gbs_graph *g, uint32_t source, const gbs_params *params, void *dist_out,
                    int32_t *pred_out, gbs_stats *stats) {
    if (!g) return fail(GBS_ERR_INVALID_ARG, "graph is NULL");
    // page-locked outputs: the unpack kernel writes dist / pred straight into
    // them over the host link (the run synchronises its stream before it
    // returns), with no device staging buffer and no copy afterwards
    void *dist_view = device_view(dist_out);
    void *pred_view = device_view(pred_out);
    if ((!dist_out || dist_view) && (!pred_out || pred_view) && (dist_out || pred_out))
        return run_sssp(g, source, params, dist_view, static_cast<int32_t *>(pred_view), stats);
    gbs_status st = ensure_workspace(g);
    if (st != GBS_OK) return st;
    st = run_sssp(g, source, params, dist_out ? g->d_dist : nullptr, pred_out ? g->d_pred : nullptr,
                    stats);
    if (st != GBS_OK) return st;
    if (dist_out)
        GBS_CUDA(cudaMemcpyAsync(dist_out, g->d_dist, dist_bytes(g->wtype) * g->n, cudaMemcpyDeviceToHost,
                                 g->stream));
    if (pred_out)
        GBS_CUDA(cudaMemcpyAsync(pred_out, g->d_pred, sizeof(int32_t) * g->n, cudaMemcpyDeviceToHost,
                                 g->stream));
    GBS_CUDA(cudaStreamSynchronize(g->stream));
    return GBS_OK;
}

gbs_status gbs_sssp_multi(gbs_graph *g, const uint32_t *sources, uint32_t k, const gbs_params *params,
                          void *dist_out, int32_t *pred_out, gbs_stats *stats) {
    if (!g || (k && !sources)) return fail(GBS_ERR_INVALID_ARG, "NULL argument");
    gbs_stats total{};
    for (uint32_t i = 0; i < k; ++i) {
        gbs_stats one{};
        void *d = dist_out ? (void *)((char *)dist_out + dist_bytes(g->wtype) * (size_t)i * g->n) : nullptr;
        int32_t *pr = pred_out ? pred_out + (size_t)i * g->n : nullptr;
        gbs_status st = gbs_sssp(g, sources[i], params, d, pr, &one);
        if (st != GBS_OK) return st;
        total.device_ms += one.device_ms;
        total.kernel_ms += one.kernel_ms;
        total.reached += one.reached;
        total.edges_reached += one.edges_reached;
        total.improvements += one.improvements;
        total.buckets += one.buckets;
        total.phases += one.phases;
        total.pending_scans += one.pending_scans;
        total.blocks = one.blocks;
        total.delta_used = one.delta_used;
        total.light_used = one.light_used;
    }
    if (stats) *stats = total;
    return GBS_OK;
}

gbs_status gbs_graph_set_controller(gbs_graph *g, const float *params, uint32_t count, double margin) {
    if (!g) return fail(GBS_ERR_INVALID_ARG, "graph is NULL");
    if (!params) {   // back to no controller
        cudaFree(g->d_mlp);
        g->d_mlp = nullptr;
        g->mlp_host.clear();
        return GBS_OK;
    }
    if (count != (uint32_t)kMlpFloats) return fail(GBS_ERR_INVALID_ARG, "controller block must hold 5410 floats");
    for (int i = 0; i < kFeat; ++i)
        if (!(params[kFeat + i] > 0.f)) return fail(GBS_ERR_INVALID_ARG, "controller: input scales must be > 0");
    if (!g->d_mlp) GBS_CUDA(cudaMalloc(&g->d_mlp, sizeof(float) * kMlpFloats));
    GBS_CUDA(cudaMemcpy(g->d_mlp, params, sizeof(float) * kMlpFloats, cudaMemcpyHostToDevice));
    g->mlp_host.assign(params, params + kMlpFloats);
    // default 0.25: on R-MAT 22 the learned / plain time of single sources
    // ranges from 0.71 to 1.27 (16 sources, geometric mean 0.96), so a
    // tighter limit reverts on one unlucky source of a graph the controller
    // wins on; R-MAT 24 (geometric mean 1.50) trips it within a few sources
    g->ctrl_margin = margin > 0 ? margin : 0.25;
    g->plain_ms = 0.0;
    g->ctrl_lost = false;
    return GBS_OK;
}

gbs_status gbs_features(gbs_graph *g, float *out, uint32_t cap, uint32_t *count) {
    if (!g || !count) return fail(GBS_ERR_INVALID_ARG, "NULL argument");
    *count = g->feat_n;
    const uint32_t k = std::min(cap, g->feat_n);
    if (k && out) GBS_CUDA(cudaMemcpy(out, g->d_feat, sizeof(float) * kFeat * k, cudaMemcpyDeviceToHost));
    return GBS_OK;
}

gbs_status gbs_trace(gbs_graph *g, gbs_phase_rec *out, uint32_t cap, uint32_t *count) {
    if (!g || !count) return fail(GBS_ERR_INVALID_ARG, "NULL argument");
    static_assert(sizeof(gbs_phase_rec) == sizeof(TraceRec), "trace record layout");
    *count = g->trace_n;
    const uint32_t k = std::min(cap, g->trace_n);
    if (k && out)
        GBS_CUDA(cudaMemcpy(out, g->ws.trace, sizeof(TraceRec) * k, cudaMemcpyDeviceToHost));
    return GBS_OK;
}

gbs_status gbs_host_alloc(size_t bytes, void **out) {
    if (!out) return fail(GBS_ERR_INVALID_ARG, "out is NULL");
    GBS_CUDA(cudaMallocHost(out, bytes ? bytes : 1));
    return GBS_OK;
}

gbs_status gbs_host_free(void *p) {
    GBS_CUDA(cudaFreeHost(p));
    return GBS_OK;
}

gbs_status gbs_device_alloc(size_t bytes, void **out) {
    if (!out) return fail(GBS_ERR_INVALID_ARG, "out is NULL");
    GBS_CUDA(cudaMalloc(out, bytes ? bytes : 1));
    return GBS_OK;
}

gbs_status gbs_device_free(void *p) {
    GBS_CUDA(cudaFree(p));
    return GBS_OK;
}

gbs_status gbs_device_synchronize(void) {
    GBS_CUDA(cudaDeviceSynchronize());
    return GBS_OK;
}

gbs_status gbs_memcpy(void *dst, const void *src, size_t bytes) {
    if (bytes && (!dst || !src)) return fail(GBS_ERR_INVALID_ARG, "NULL buffer");
    if (bytes) GBS_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault));
    return GBS_OK;
}

}  // extern "C"
