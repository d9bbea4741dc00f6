// gbs_bc.cu -- betweenness centrality on the GPU (sm_103a): Brandes over the
// shortest paths of every source, after btwcentral/csr_bc.c:16-123.
//
// Per source, the persistent delta-stepping kernel leaves the distances in
// the graph's workspace; one cooperative launch of bc_dag then works on the
// shortest-path DAG, the edges (u, v) with dist(u) + w == dist(v) computed in
// the weight type (the reference keeps these as predecessor lists,
// sssp/csr_sspath.c:116-118; here they are derived from the distances):
//
//   COUNT     every reached vertex: sigma := [v == source]; for each tight
//             out-edge (u, v) indeg[v] += 1 (atomics).
//   FORWARD   Kahn levels from the source: level L+1 holds the vertices whose
//             last tight in-edge came from level L.  A level's vertices push
//             sigma[v] += sigma[u] (64-bit integer atomics: exact, and wrapping
//             like the reference's lint sums, comp_num_spath, csr_bc.c:67-91).
//             The levels are appended to one order list; a grid barrier
//             separates levels and the CTA that arrives last publishes the
//             next level's bounds.
//   BACKWARD  levels in reverse: every vertex pulls
//             delta[u] = sum over tight out-edges (u, v) of
//                        (1 + delta[v]) * sigma[u] / sigma[v]
//             (comp_delta, csr_bc.c:93-116) in reverse row order, and adds it
//             to bc[u].  No atomics: each vertex is written once per source.
//
// Rows are sorted by (weight, column), so reverse row order visits the
// targets by decreasing (distance, id) whenever equal distances come from
// equal weights -- always for uint32 weights -- which is the order the
// reference's reverse sweep over the distance-sorted vertices adds them in;
// every product and quotient is the same IEEE double operation, so uint32
// results are bit-identical to a serial Brandes over the same DAG.
//
// HBM per source: COUNT, FORWARD and BACKWARD each stream the rows of the
// vertices they touch (8 B per edge) and gather the targets' state words; the
// per-vertex arrays (dist 8 B, sigma 8 B, delta 8 B, indeg 4 B, order 4 B)
// stay in L2 for graphs of a few million vertices.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gbs_host.hpp"
#include "gbs_internal.cuh"

namespace gbs {
namespace {

constexpr uint32_t kShortRow = 32;   // rows up to this long are walked by one lane

// Control block of one bc_dag launch (zeroed before every launch).
struct __align__(128) BcCtl {
    uint32_t bar_count;
    uint32_t pad0[31];
    uint32_t bar_gen;
    uint32_t pad1[31];
    uint32_t error;
    uint32_t pub_lo;       // order[pub_lo, pub_hi) is the level to process next
    uint32_t pub_hi;
    uint32_t levels;       // forward levels (the source's is level 0)
    uint32_t pad2[28];
    Line ord_cnt;          // vertices appended to the order list
};
static_assert(sizeof(BcCtl) % 128 == 0, "BcCtl lines");

// Sums over all sources of one gbs_bc call (zeroed once per call).
struct BcTotals {
    unsigned long long tight;   // tight edges found
    unsigned long long reached; // vertices in the DAGs
    uint32_t max_levels;
    uint32_t error;
};

struct BcArgs {
    const uint32_t *row;
    const uint2 *adj;
    const unsigned long long *w64;
    const unsigned long long *dp;    // the SSSP's state words: distance (| pred)
    uint32_t n;
    uint32_t source;
    unsigned long long *sigma;
    double *delta;
    uint32_t *indeg;
    uint32_t *order;
    uint32_t *lvl;                   // order index where each level starts (n + 1)
    double *bc;
    BcCtl *ctl;
    BcTotals *tot;
    unsigned long long wait_ns;
    uint32_t nblocks;
};

// dist(u) + w(e) == dist(v) in the weight type (both state words reached).
template <int WT>
__device__ __forceinline__ bool tight(unsigned long long pu, unsigned long long pv, uint2 ew,
                                      const unsigned long long *w64, uint32_t e) {
    if constexpr (WT == 2) {
        const double s = __dadd_rn(__longlong_as_double((long long)pu), __longlong_as_double((long long)__ldg(w64 + e)));
        return (unsigned long long)__double_as_longlong(s) == pv;
    } else if constexpr (WT == 1) {
        const float s = __fadd_rn(__uint_as_float((uint32_t)(pu >> 32)), __uint_as_float(ew.y));
        return __float_as_uint(s) == (uint32_t)(pv >> 32);
    } else {
        return (unsigned long long)(uint32_t)(pu >> 32) + ew.y == (pv >> 32);
    }
}

__device__ __forceinline__ void set_error(const BcArgs &a, uint32_t code) {
    atomicCAS(&a.ctl->error, 0u, code);
    atomicCAS(&a.tot->error, 0u, code);
}

// Grid barrier; the CTA that arrives last runs `decide` (thread 0 alone, all
// other CTAs at rest) before releasing the rest.  Waits are bounded by
// a.wait_ns; on expiry the error word is set.  s_pub receives pub_lo/pub_hi.
// Returns false when the launch must stop.
template <typename Decide>
__device__ __forceinline__ bool grid_step(const BcArgs &a, uint32_t &gen, uint32_t *s_pub, Decide decide) {
    __syncthreads();
    if (threadIdx.x == 0) {
        BcCtl *c = a.ctl;
        __threadfence();
        const bool last = atomicAdd(&c->bar_count, 1u) == a.nblocks - 1u;
        if (last) {
            __threadfence();
            decide();
            c->bar_count = 0;
            __threadfence();
            st_release(&c->bar_gen, gen + 1u);
        } else {
            const unsigned long long t0 = globaltimer();
            uint32_t spins = 0;
            while (ld_acquire(&c->bar_gen) != gen + 1u) {
                if ((++spins & 255u) == 0) {
                    if (ld_relaxed(&c->error) != 0) break;
                    if (globaltimer() - t0 > a.wait_ns) {
                        set_error(a, kErrTimeout);
                        break;
                    }
                }
            }
        }
        s_pub[0] = ld_relaxed(&c->pub_lo);
        s_pub[1] = ld_relaxed(&c->pub_hi);
        s_pub[2] = ld_relaxed(&c->error);
    }
    __syncthreads();
    ++gen;
    return s_pub[2] == 0;
}

// Appends the lanes whose `take` is set to the order list: one counter atomic
// per warp.  All 32 lanes call it together.
__device__ __forceinline__ void append_order(const BcArgs &a, bool take, uint32_t v) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned b = __ballot_sync(0xffffffffu, take);
    if (!b) return;
    uint32_t base = 0;
    if (lane == (unsigned)(__ffs(b) - 1)) base = atomicAdd(&a.ctl->ord_cnt.v, (uint32_t)__popc(b));
    base = __shfl_sync(0xffffffffu, base, __ffs(b) - 1);
    if (take) a.order[base + __popc(b & ((1u << lane) - 1u))] = v;
}

// COUNT for rows [base, base + 32): sigma reset and tight in-degrees.
template <int WT>
__device__ __forceinline__ void count_rows(const BcArgs &a, uint32_t base, unsigned long long &tight_n) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t u = base + lane;
    unsigned long long pu = kUnreached;
    uint32_t beg = 0, end = 0;
    if (u < a.n) {
        pu = __ldg(a.dp + u);
        if (pu != kUnreached) {
            beg = __ldg(a.row + u);
            end = __ldg(a.row + u + 1);
            a.sigma[u] = u == a.source ? 1ull : 0ull;
        }
    }
    const uint32_t deg = end - beg;
    const bool is_long = deg > kShortRow;
    // short rows: one lane each
    if (!is_long) {
        for (uint32_t e = beg; e < end; ++e) {
            const uint2 ew = __ldg(a.adj + e);
            const unsigned long long pv = __ldg(a.dp + ew.x);
            if (pv != kUnreached && tight<WT>(pu, pv, ew, a.w64, e)) {
                atomicAdd(a.indeg + ew.x, 1u);
                ++tight_n;
            }
        }
    }
    // long rows: the whole warp, one after another
    unsigned lm = __ballot_sync(0xffffffffu, is_long);
    while (lm) {
        const int src_lane = __ffs(lm) - 1;
        lm &= lm - 1;
        const unsigned long long qu = __shfl_sync(0xffffffffu, pu, src_lane);
        const uint32_t qb = __shfl_sync(0xffffffffu, beg, src_lane);
        const uint32_t qe = __shfl_sync(0xffffffffu, end, src_lane);
        for (uint32_t e = qb + lane; e < qe; e += 32u) {
            const uint2 ew = __ldg(a.adj + e);
            const unsigned long long pv = __ldg(a.dp + ew.x);
            if (pv != kUnreached && tight<WT>(qu, pv, ew, a.w64, e)) {
                atomicAdd(a.indeg + ew.x, 1u);
                ++tight_n;
            }
        }
    }
}

// FORWARD for order[i0 + lane], i0 + lane < hi.
template <int WT>
__device__ __forceinline__ void forward_rows(const BcArgs &a, uint32_t i0, uint32_t hi) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t i = i0 + lane;
    uint32_t u = 0, beg = 0, end = 0;
    unsigned long long pu = 0, su = 0;
    if (i < hi) {
        u = __ldcg(a.order + i);
        pu = __ldg(a.dp + u);
        su = __ldcg(a.sigma + u);
        beg = __ldg(a.row + u);
        end = __ldg(a.row + u + 1);
    }
    const uint32_t deg = end - beg;
    const bool is_long = deg > kShortRow;
    // short rows in lockstep, so that appends aggregate per warp
    const uint32_t steps = __reduce_max_sync(0xffffffffu, is_long ? 0u : deg);
    for (uint32_t k = 0; k < steps; ++k) {
        bool take = false;
        uint32_t v = 0;
        if (!is_long && k < deg) {
            const uint32_t e = beg + k;
            const uint2 ew = __ldg(a.adj + e);
            v = ew.x;
            const unsigned long long pv = __ldg(a.dp + v);
            if (pv != kUnreached && tight<WT>(pu, pv, ew, a.w64, e)) {
                atomicAdd(a.sigma + v, su);
                take = atomicSub(a.indeg + v, 1u) == 1u;
            }
        }
        append_order(a, take, v);
    }
    unsigned lm = __ballot_sync(0xffffffffu, is_long);
    while (lm) {
        const int src_lane = __ffs(lm) - 1;
        lm &= lm - 1;
        const unsigned long long qu = __shfl_sync(0xffffffffu, pu, src_lane);
        const unsigned long long qs = __shfl_sync(0xffffffffu, su, src_lane);
        const uint32_t qb = __shfl_sync(0xffffffffu, beg, src_lane);
        const uint32_t qe = __shfl_sync(0xffffffffu, end, src_lane);
        for (uint32_t e0 = qb; e0 < qe; e0 += 32u) {
            const uint32_t e = e0 + lane;
            bool take = false;
            uint32_t v = 0;
            if (e < qe) {
                const uint2 ew = __ldg(a.adj + e);
                v = ew.x;
                const unsigned long long pv = __ldg(a.dp + v);
                if (pv != kUnreached && tight<WT>(qu, pv, ew, a.w64, e)) {
                    atomicAdd(a.sigma + v, qs);
                    take = atomicSub(a.indeg + v, 1u) == 1u;
                }
            }
            append_order(a, take, v);
        }
    }
}

// One dependency term (1 + delta[v]) * sigma[u] / sigma[v], in the order of
// operations of comp_delta (csr_bc.c:110).
__device__ __forceinline__ double dep_term(double su, double dv, unsigned long long sv) {
    return __ddiv_rn(__dmul_rn(__dadd_rn(1.0, dv), su), __ll2double_rn((long long)sv));
}

// BACKWARD for order[i0 + lane], i0 + lane < hi.
template <int WT>
__device__ __forceinline__ void backward_rows(const BcArgs &a, uint32_t i0, uint32_t hi) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t i = i0 + lane;
    uint32_t u = 0, beg = 0, end = 0;
    unsigned long long pu = 0;
    double su = 0.0;
    if (i < hi) {
        u = __ldcg(a.order + i);
        pu = __ldg(a.dp + u);
        su = __ll2double_rn((long long)__ldcg(a.sigma + u));
        beg = __ldg(a.row + u);
        end = __ldg(a.row + u + 1);
    }
    const uint32_t deg = end - beg;
    const bool is_long = deg > kShortRow;
    double acc = 0.0;
    if (!is_long) {
        for (uint32_t e = end; e-- > beg;) {
            const uint2 ew = __ldg(a.adj + e);
            const unsigned long long pv = __ldg(a.dp + ew.x);
            if (pv != kUnreached && tight<WT>(pu, pv, ew, a.w64, e))
                acc = __dadd_rn(acc, dep_term(su, __ldcg(a.delta + ew.x), __ldcg(a.sigma + ew.x)));
        }
    }
    unsigned lm = __ballot_sync(0xffffffffu, is_long);
    while (lm) {
        const int src_lane = __ffs(lm) - 1;
        lm &= lm - 1;
        const unsigned long long qu = __shfl_sync(0xffffffffu, pu, src_lane);
        const double qs = __shfl_sync(0xffffffffu, su, src_lane);
        const uint32_t qb = __shfl_sync(0xffffffffu, beg, src_lane);
        const uint32_t qe = __shfl_sync(0xffffffffu, end, src_lane);
        double qacc = 0.0;
        // 32 edges per round from the end of the row: lane l takes the l-th
        // edge from the top, and the terms are added from lane 0 up, i.e. in
        // reverse row order
        for (uint32_t top = qe; top > qb;) {
            const uint32_t cnt = min(32u, top - qb);
            double t = 0.0;
            bool is_t = false;
            if (lane < cnt) {
                const uint32_t e = top - 1u - lane;
                const uint2 ew = __ldg(a.adj + e);
                const unsigned long long pv = __ldg(a.dp + ew.x);
                if (pv != kUnreached && tight<WT>(qu, pv, ew, a.w64, e)) {
                    t = dep_term(qs, __ldcg(a.delta + ew.x), __ldcg(a.sigma + ew.x));
                    is_t = true;
                }
            }
            unsigned tm = __ballot_sync(0xffffffffu, is_t);
            while (tm) {
                const int l = __ffs(tm) - 1;
                tm &= tm - 1;
                qacc = __dadd_rn(qacc, __shfl_sync(0xffffffffu, t, l));
            }
            top -= cnt;
        }
        if (lane == (unsigned)src_lane) acc = qacc;
    }
    if (i < hi) {
        a.delta[u] = acc;
        a.bc[u] = __dadd_rn(a.bc[u], acc);
    }
}

template <int WT>
__global__ void __launch_bounds__(kTPB, 1) bc_dag(BcArgs a) {
    __shared__ uint32_t s_pub[3];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (a.nblocks * blockDim.x) >> 5;
    uint32_t gen = 0;
    // ---- COUNT
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.order[0] = a.source;
        a.ctl->ord_cnt.v = 1u;
        a.lvl[0] = 0u;
    }
    unsigned long long tight_n = 0;
    for (uint32_t base = gwarp * 32u; base < a.n; base += nwarps * 32u) count_rows<WT>(a, base, tight_n);
    for (int o = 16; o > 0; o >>= 1) tight_n += __shfl_down_sync(0xffffffffu, tight_n, o);
    if (lane == 0 && tight_n) atomicAdd(&a.tot->tight, tight_n);
    BcCtl *c = a.ctl;
    uint32_t L = 0;
    auto first = [&]() {
        c->pub_lo = 0u;
        c->pub_hi = 1u;
    };
    if (!grid_step(a, gen, s_pub, first)) return;
    // ---- FORWARD: level L is order[lo, hi)
    for (;;) {
        const uint32_t lo = s_pub[0], hi = s_pub[1];
        if (lo >= hi) break;
        for (uint32_t i0 = lo + gwarp * 32u; i0 < hi; i0 += nwarps * 32u) forward_rows<WT>(a, i0, hi);
        auto next = [&]() {
            a.lvl[L + 1] = hi;
            c->pub_lo = hi;
            c->pub_hi = ld_relaxed(&c->ord_cnt.v);
            c->levels = L + 1;
        };
        if (!grid_step(a, gen, s_pub, next)) return;
        ++L;
    }
    // L = number of levels; level k is order[lvl[k], lvl[k + 1])
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicMax(&a.tot->max_levels, L);
        atomicAdd(&a.tot->reached, (unsigned long long)s_pub[1]);
    }
    // ---- BACKWARD: levels L-1 .. 1 (level 0 is the source alone)
    for (uint32_t k = L; k-- > 1;) {
        const uint32_t lo = __ldcg(a.lvl + k), hi = __ldcg(a.lvl + k + 1);
        for (uint32_t i0 = lo + gwarp * 32u; i0 < hi; i0 += nwarps * 32u) backward_rows<WT>(a, i0, hi);
        if (k > 1 && !grid_step(a, gen, s_pub, [] {})) return;
    }
}

struct BcState {
    unsigned long long *sigma = nullptr;
    double *delta = nullptr;
    uint32_t *indeg = nullptr;
    uint32_t *order = nullptr;
    uint32_t *lvl = nullptr;
    double *bc = nullptr;
    BcCtl *ctl = nullptr;
    BcTotals *tot = nullptr;
    int blocks = 0;
};

const void *bc_kernel(gbs_weight_type wt) {
    return wt == GBS_WEIGHT_F64   ? (const void *)bc_dag<2>
           : wt == GBS_WEIGHT_F32 ? (const void *)bc_dag<1>
                                  : (const void *)bc_dag<0>;
}

gbs_status alloc_bc(gbs_graph *g) {
    BcState *b = new BcState();
    g->bc = b;
    const size_t n = g->n;
    GBS_CUDA(cudaMalloc(&b->sigma, sizeof(unsigned long long) * n));
    GBS_CUDA(cudaMalloc(&b->delta, sizeof(double) * n));
    GBS_CUDA(cudaMalloc(&b->indeg, sizeof(uint32_t) * n));
    GBS_CUDA(cudaMalloc(&b->order, sizeof(uint32_t) * n));
    GBS_CUDA(cudaMalloc(&b->lvl, sizeof(uint32_t) * (n + 1)));
    GBS_CUDA(cudaMalloc(&b->bc, sizeof(double) * n));
    GBS_CUDA(cudaMalloc(&b->ctl, sizeof(BcCtl)));
    GBS_CUDA(cudaMalloc(&b->tot, sizeof(BcTotals)));
    // in-degrees return to zero at the end of every FORWARD pass
    GBS_CUDA(cudaMemsetAsync(b->indeg, 0, sizeof(uint32_t) * n, g->stream));
    int per_sm = 0;
    GBS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bc_kernel(g->wtype), kTPB, 0));
    if (per_sm < 1) return fail(GBS_ERR_UNSUPPORTED, "betweenness kernel cannot be resident");
    b->blocks = std::min(per_sm, 1) * g->sms;
    return GBS_OK;
}

}  // namespace

void free_bc(gbs_graph *g) {
    BcState *b = static_cast<BcState *>(g->bc);
    if (!b) return;
    cudaFree(b->sigma);
    cudaFree(b->delta);
    cudaFree(b->indeg);
    cudaFree(b->order);
    cudaFree(b->lvl);
    cudaFree(b->bc);
    cudaFree(b->ctl);
    cudaFree(b->tot);
    delete b;
    g->bc = nullptr;
}

gbs_status ensure_bc(gbs_graph *g) {
    if (g->bc) return GBS_OK;
    const gbs_status st = alloc_bc(g);
    if (st != GBS_OK) free_bc(g);
    return st;
}


// Sums the dependencies of `k` sources into the device array bc_dev (n
// doubles, zeroed first).
gbs_status run_bc(gbs_graph *g, const uint32_t *sources, uint32_t k, const gbs_params *params, double *bc_dev,
                  gbs_bc_stats *stats) {
    if (g->zero_w) return fail(GBS_ERR_INVALID_ARG, "betweenness needs positive edge weights");
    gbs_status st = ensure_workspace(g);
    if (st != GBS_OK) return st;
    st = ensure_bc(g);
    if (st != GBS_OK) return st;
    for (uint32_t i = 0; i < k; ++i)
        if ((sources ? sources[i] : i) >= g->n) return fail(GBS_ERR_INVALID_ARG, "source out of range");
    BcState *b = static_cast<BcState *>(g->bc);
    cudaStream_t s = g->stream;
    cudaEvent_t e0, e1;
    GBS_CUDA(cudaEventCreate(&e0));
    GBS_CUDA(cudaEventCreate(&e1));
    GBS_CUDA(cudaMemsetAsync(bc_dev, 0, sizeof(double) * g->n, s));
    GBS_CUDA(cudaMemsetAsync(b->tot, 0, sizeof(BcTotals), s));
    gbs_params p = params ? *params : gbs_params{};
    p.flags &= ~(uint32_t)(GBS_F_TRACE | GBS_F_FEATURES);
    BcArgs a{};
    a.row = g->d_row;
    a.adj = g->d_adj;
    a.w64 = g->d_w64;
    a.dp = g->ws.dp;
    a.n = g->n;
    a.sigma = b->sigma;
    a.delta = b->delta;
    a.indeg = b->indeg;
    a.order = b->order;
    a.lvl = b->lvl;
    a.bc = bc_dev;
    a.ctl = b->ctl;
    a.tot = b->tot;
    a.wait_ns = (unsigned long long)(p.wait_limit_ms ? p.wait_limit_ms : 4000u) * 1000000ull;
    a.nblocks = (uint32_t)b->blocks;
    const void *kfn = bc_kernel(g->wtype);
    gbs_bc_stats tot{};
    double dag_ms = 0.0;
    for (uint32_t i = 0; i < k; ++i) {
        const uint32_t src = sources ? sources[i] : i;
        gbs_stats one{};
        st = run_sssp(g, src, &p, nullptr, nullptr, &one);
        if (st != GBS_OK) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return st;
        }
        tot.sssp_ms += one.device_ms;
        tot.edges_reached += one.edges_reached;
        a.source = src;
        void *args[] = {&a};
        GBS_CUDA(cudaEventRecord(e0, s));
        GBS_CUDA(cudaMemsetAsync(b->ctl, 0, sizeof(BcCtl), s));
        GBS_CUDA(cudaLaunchCooperativeKernel(kfn, dim3(b->blocks), dim3(kTPB), args, 0, s));
        GBS_CUDA(cudaEventRecord(e1, s));
        // the next source's SSSP synchronises the stream; time this one now
        GBS_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        GBS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        dag_ms += ms;
    }
    BcTotals t{};
    GBS_CUDA(cudaMemcpyAsync(&t, b->tot, sizeof(t), cudaMemcpyDeviceToHost, s));
    GBS_CUDA(cudaStreamSynchronize(s));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (t.error != kErrNone)
        return fail(t.error == kErrTimeout ? GBS_ERR_TIMEOUT : GBS_ERR_INTERNAL, "betweenness: device-side wait limit exceeded");
    if (stats) {
        tot.dag_ms = dag_ms;
        tot.device_ms = tot.sssp_ms + dag_ms;
        tot.sources = k;
        tot.tight_edges = t.tight;
        tot.dag_vertices = t.reached;
        tot.max_levels = t.max_levels;
        tot.blocks = (uint32_t)b->blocks;
        *stats = tot;
    }
    return GBS_OK;
}

}  // namespace gbs

extern "C" {

gbs_status gbs_bc_device(gbs_graph *g, const uint32_t *sources, uint32_t k, const gbs_params *params,
                         double *bc_dev, gbs_bc_stats *stats) {
    if (!g || !bc_dev) return gbs::fail(GBS_ERR_INVALID_ARG, "NULL argument");
    if (!sources) k = g->n;
    return gbs::run_bc(g, sources, k, params, bc_dev, stats);
}

gbs_status gbs_bc(gbs_graph *g, const uint32_t *sources, uint32_t k, const gbs_params *params, double *bc_out,
                  gbs_bc_stats *stats) {
    if (!g || !bc_out) return gbs::fail(GBS_ERR_INVALID_ARG, "NULL argument");
    if (!sources) k = g->n;
    gbs_status st = gbs::ensure_workspace(g);
    if (st != GBS_OK) return st;
    st = gbs::ensure_bc(g);
    if (st != GBS_OK) return st;
    double *acc = static_cast<gbs::BcState *>(g->bc)->bc;
    st = gbs::run_bc(g, sources, k, params, acc, stats);
    if (st != GBS_OK) return st;
    GBS_CUDA(cudaMemcpyAsync(bc_out, acc, sizeof(double) * g->n, cudaMemcpyDeviceToHost, g->stream));
    GBS_CUDA(cudaStreamSynchronize(g->stream));
    return GBS_OK;
}

}  // extern "C"
