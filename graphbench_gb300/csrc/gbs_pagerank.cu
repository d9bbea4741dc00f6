// gbs_pagerank.cu -- PageRank on the GPU (sm_103a): the reference's iteration
// (pagerank/pagerank_mpi.c:667-1043, one node, constants RDM_JMP and THRESH
// of include/graph.h:17-18) as a pull over the in-edge CSR, replacing the MPI
// message exchange.
//
//   weight = 1, recip = 1 / out-degree, wb = rj, diff = weight * recip
//   per iteration:  wb[v] += sum over in-edges u of (1 - rj) * diff[u]
//                   diff'[v] = (wb[v] - weight[v]) * recip[v]
//                   weight[v] = wb[v]; stop when no |diff'| exceeds thresh
//
// diff is double-buffered (iteration t reads t-1's).  The per-iteration sum of
// a row has a fixed order shared with the oracle: the row's CSR positions in
// 32-position words, each word summed from its lowest position up, the word
// sums of each block of 32 words combined by a butterfly, the block sums added
// in order.  Rows of at most 32 edges (two words) are summed by one thread
// (their butterfly is the plain sum of the two word sums); the words of longer
// rows are summed one per thread into a buffer, and a second kernel combines
// them (a thread per row of up to 8 words, a warp per longer row).  Two
// launches and one 4-byte read-back (the convergence flag) per iteration.
//
// HBM per iteration: the in-edge columns (4 B per edge) and the gathered
// diff[u] (8 B per edge, L2-resident for a few million vertices), plus ~40 B
// of per-vertex state.
#include <algorithm>
#include <cmath>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "gbs_host.hpp"

namespace gbs {
namespace {

constexpr uint32_t kShort = 32;   // rows up to this many edges are summed by one thread

struct PrArgs {
    const unsigned long long *row;
    const uint32_t *col;
    uint32_t n;
    double pj;          // 1 - random jump
    double thresh;
    const double *recip;
    double *weight, *wb;
    const double *diff;     // this iteration's input, times (1 - rj)
    double *diff_next;      // its output, times (1 - rj)
    const uint32_t *srow;    // the rows of at most kShort edges, grouped by degree
    uint32_t n_short;
    const uint32_t *lw_row;  // words of the long rows: row, mask word
    const uint32_t *lw_w;
    uint32_t n_lw;
    double *part;            // one sum per long-row word
    const uint32_t *lr_row;  // long rows: row, first word, number of words
    const uint32_t *lr_first;
    const uint32_t *lr_nw;
    uint32_t n_lr;
    uint32_t *flag;          // set when some |diff'| > thresh
};

__global__ void k_outdeg(const uint32_t *__restrict__ col, unsigned long long m, uint32_t *__restrict__ deg) {
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < m;
         e += (unsigned long long)gridDim.x * blockDim.x)
        atomicAdd(deg + col[e], 1u);
}

// diff is kept multiplied by (1 - rj): every edge term (1 - rj) * diff[u] is
// then a load, the same product computed once per vertex instead of per edge.
__global__ void k_pr_init(const uint32_t *__restrict__ deg, uint32_t n, double rj, double *__restrict__ recip,
                          double *__restrict__ weight, double *__restrict__ wb, double *__restrict__ diff) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const double r = __ddiv_rn(1.0, (double)deg[v]);   // 1/0 = +inf, as the reference's 1.0 / 0
        recip[v] = r;
        weight[v] = 1.0;
        wb[v] = rj;
        diff[v] = __dmul_rn(1.0 - rj, __dmul_rn(1.0, r));
    }
}

__device__ __forceinline__ void pr_update(const PrArgs &a, uint32_t v, double s) {
    const double w = __dadd_rn(a.wb[v], s);
    const double d = __dmul_rn(__dadd_rn(w, -a.weight[v]), a.recip[v]);
    a.wb[v] = w;
    a.weight[v] = w;
    a.diff_next[v] = __dmul_rn(a.pj, d);
    if (fabs(d) > a.thresh) *a.flag = 1u;   // NaN compares false, as in the reference
}

// Positions [lo, hi) of one row added in order into p (acc takes p at each
// change of 32-position word); 8 gathers in flight before their adds.
constexpr int kPull = 8;
__device__ __forceinline__ void pull_range(const PrArgs &a, unsigned long long lo, unsigned long long hi, double &acc,
                                           double &p, unsigned long long &cur) {
    for (unsigned long long e0 = lo; e0 < hi; e0 += kPull) {
        uint32_t u[kPull];
        double t[kPull];
#pragma unroll
        for (int k = 0; k < kPull; ++k) u[k] = e0 + k < hi ? __ldg(a.col + e0 + k) : 0u;
#pragma unroll
        for (int k = 0; k < kPull; ++k) t[k] = e0 + k < hi ? __ldg(a.diff + u[k]) : 0.0;
#pragma unroll
        for (int k = 0; k < kPull; ++k) {
            const unsigned long long e = e0 + k;
            if (e < hi) {
                if ((e >> 5) != cur) {
                    acc = __dadd_rn(acc, p);
                    p = 0.0;
                    cur = e >> 5;
                }
                p = __dadd_rn(p, t[k]);
            }
        }
    }
}

// Short rows summed by their thread; word sums of the long rows.
__global__ void __launch_bounds__(256) k_pr_pull(PrArgs a) {
    const uint32_t stride = gridDim.x * blockDim.x;
    // a warp's rows have equal degrees, so its FP64 adds run with every lane busy
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_short; i += stride) {
        const uint32_t v = a.srow[i];
        const unsigned long long beg = a.row[v], end = a.row[v + 1];
        double acc = 0.0, p = 0.0;
        unsigned long long cur = beg >> 5;
        pull_range(a, beg, end, acc, p, cur);
        acc = __dadd_rn(acc, p);
        pr_update(a, v, acc);
    }
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < a.n_lw; x += stride) {
        const uint32_t v = a.lw_row[x];
        const unsigned long long W = a.lw_w[x];
        const unsigned long long beg = a.row[v], end = a.row[v + 1];
        const unsigned long long lo = max(beg, W << 5), hi = min(end, (W << 5) + 32ull);
        double acc = 0.0, p = 0.0;
        unsigned long long cur = W;
        pull_range(a, lo, hi, acc, p, cur);
        a.part[x] = p;
    }
}

__device__ __forceinline__ double butterfly32(double t) {
    for (int h = 16; h > 0; h >>= 1) t = __dadd_rn(t, __shfl_down_sync(0xffffffffu, t, h));
    return t;
}

// Long rows: blocks of 32 word sums by the butterfly, block sums in order.
// Rows of at most 8 words by their lane, longer ones by the warp.
__global__ void __launch_bounds__(256) k_pr_long(PrArgs a) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t s0 = gwarp * 32u; s0 < a.n_lr; s0 += nwarps * 32u) {
        const uint32_t sl = s0 + lane;
        uint32_t v = 0, first = 0, nw = 0;
        if (sl < a.n_lr) {
            v = a.lr_row[sl];
            first = a.lr_first[sl];
            nw = a.lr_nw[sl];
        }
        if (nw && nw <= 8u) {
            double q[8];
#pragma unroll
            for (uint32_t k = 0; k < 8u; ++k) q[k] = k < nw ? a.part[first + k] : 0.0;
#pragma unroll
            for (uint32_t h = 4; h > 0; h >>= 1)
#pragma unroll
                for (uint32_t k = 0; k < h; ++k) q[k] = __dadd_rn(q[k], q[k + h]);
            pr_update(a, v, q[0]);
        }
        unsigned big = __ballot_sync(0xffffffffu, nw > 8u);
        while (big) {
            const int q = __ffs(big) - 1;
            big &= big - 1;
            const uint32_t bv = __shfl_sync(0xffffffffu, v, q), bf = __shfl_sync(0xffffffffu, first, q);
            const uint32_t bn = __shfl_sync(0xffffffffu, nw, q);
            double r = 0.0;
            double cur = lane < bn ? a.part[bf + lane] : 0.0;
            for (uint32_t t0 = 0; t0 < bn; t0 += 32u) {
                const uint32_t nx = t0 + 32u + lane;
                const double next = nx < bn ? a.part[bf + nx] : 0.0;
                r = __dadd_rn(r, __shfl_sync(0xffffffffu, butterfly32(cur), 0));
                cur = next;
            }
            if (lane == 0) pr_update(a, bv, r);
        }
    }
}

__global__ void k_src_of(const unsigned long long *__restrict__ row, uint32_t n, uint32_t *__restrict__ src) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps)
        for (unsigned long long e = row[v] + lane; e < row[v + 1]; e += 32ull) src[e] = v;
}

__global__ void k_iota32(uint32_t *__restrict__ id, unsigned long long m) {
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < m;
         k += (unsigned long long)gridDim.x * blockDim.x)
        id[k] = (uint32_t)k;
}

__global__ void k_transpose_place(const uint32_t *__restrict__ idx, const uint32_t *__restrict__ src,
                                  const double *__restrict__ w, unsigned long long m, uint32_t *__restrict__ col,
                                  double *__restrict__ wout) {
    for (unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; p < m;
         p += (unsigned long long)gridDim.x * blockDim.x) {
        col[p] = src[idx[p]];
        wout[p] = w[idx[p]];
    }
}

__global__ void k_hist64(const uint32_t *__restrict__ col, unsigned long long m, unsigned long long *__restrict__ cnt) {
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < m;
         e += (unsigned long long)gridDim.x * blockDim.x)
        atomicAdd(cnt + col[e], 1ull);
}

int grid_of(unsigned long long items, int sms) {
    return (int)std::max<unsigned long long>(1, std::min<unsigned long long>((items + 255) / 256, (unsigned long long)sms * 16));
}

// Device buffers of one call.
struct Pool {
    std::vector<void *> p;
    ~Pool() {
        for (void *q : p) cudaFree(q);
    }
    template <typename T> cudaError_t get(T **out, size_t count) {
        void *q = nullptr;
        const cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
        if (e == cudaSuccess) p.push_back(q);
        *out = static_cast<T *>(q);
        return e;
    }
};

}  // namespace

gbs_status run_pagerank(const gbs_device_csr *c, const gbs_pagerank_params *params, double *rank_out,
                        gbs_pagerank_stats *stats) {
    const uint32_t n = c->n;
    const unsigned long long m = c->m;
    const double rj = (params && params->random_jump > 0) ? params->random_jump : 0.3;
    const double thresh = (params && params->threshold > 0) ? params->threshold : 1e-6;
    const uint32_t max_iters = (params && params->max_iters) ? params->max_iters : 10000u;
    if (!(rj < 1.0)) return fail(GBS_ERR_INVALID_ARG, "random_jump must be in (0, 1)");
    int dev = 0, sms = 0;
    GBS_CUDA(cudaGetDevice(&dev));
    GBS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // the long rows' words and the rows themselves (host side, once per call)
    std::vector<unsigned long long> row(n + 1ull);
    GBS_CUDA(cudaMemcpy(row.data(), c->d_row, sizeof(unsigned long long) * (n + 1ull), cudaMemcpyDeviceToHost));
    std::vector<uint32_t> lw_row, lw_w, lr_row, lr_first, lr_nw;
    std::vector<uint32_t> short_cnt(kShort + 2, 0), srow;
    for (uint32_t v = 0; v < n; ++v)
        if (row[v + 1] - row[v] <= kShort) ++short_cnt[row[v + 1] - row[v] + 1];
    for (uint32_t d = 1; d < kShort + 2; ++d) short_cnt[d] += short_cnt[d - 1];
    srow.resize(short_cnt[kShort + 1]);
    for (uint32_t v = 0; v < n; ++v) {
        const unsigned long long beg = row[v], end = row[v + 1];
        if (end - beg <= kShort) {
            srow[short_cnt[end - beg]++] = v;
            continue;
        }
        const unsigned long long wb = beg >> 5, we = (end >> 5) + ((end & 31ull) != 0ull);
        lr_row.push_back(v);
        lr_first.push_back((uint32_t)lw_row.size());
        lr_nw.push_back((uint32_t)(we - wb));
        for (unsigned long long W = wb; W < we; ++W) {
            lw_row.push_back(v);
            lw_w.push_back((uint32_t)W);
        }
    }
    cudaStream_t s;
    GBS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamFree {
        cudaStream_t s;
        ~StreamFree() { cudaStreamDestroy(s); }
    } sf{s};
    cudaEvent_t e0, e1;
    GBS_CUDA(cudaEventCreate(&e0));
    GBS_CUDA(cudaEventCreate(&e1));
    struct EvFree {
        cudaEvent_t a, b;
        ~EvFree() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } ef{e0, e1};
    Pool pool;
    uint32_t *deg = nullptr, *flag = nullptr, *lwr = nullptr, *lww = nullptr, *lrr = nullptr, *lrf = nullptr, *lrn = nullptr;
    uint32_t *srw = nullptr;
    double *recip = nullptr, *weight = nullptr, *wb = nullptr, *diff[2] = {nullptr, nullptr}, *part = nullptr;
    GBS_CUDA(pool.get(&deg, n));
    GBS_CUDA(pool.get(&flag, 1));
    GBS_CUDA(pool.get(&recip, n));
    GBS_CUDA(pool.get(&weight, n));
    GBS_CUDA(pool.get(&wb, n));
    GBS_CUDA(pool.get(&diff[0], n));
    GBS_CUDA(pool.get(&diff[1], n));
    GBS_CUDA(pool.get(&part, lw_row.size()));
    GBS_CUDA(pool.get(&lwr, lw_row.size()));
    GBS_CUDA(pool.get(&lww, lw_w.size()));
    GBS_CUDA(pool.get(&lrr, lr_row.size()));
    GBS_CUDA(pool.get(&lrf, lr_first.size()));
    GBS_CUDA(pool.get(&lrn, lr_nw.size()));
    GBS_CUDA(pool.get(&srw, srow.size()));
    if (!srow.empty()) GBS_CUDA(cudaMemcpyAsync(srw, srow.data(), 4 * srow.size(), cudaMemcpyHostToDevice, s));
    if (!lw_row.empty()) {
        GBS_CUDA(cudaMemcpyAsync(lwr, lw_row.data(), 4 * lw_row.size(), cudaMemcpyHostToDevice, s));
        GBS_CUDA(cudaMemcpyAsync(lww, lw_w.data(), 4 * lw_w.size(), cudaMemcpyHostToDevice, s));
        GBS_CUDA(cudaMemcpyAsync(lrr, lr_row.data(), 4 * lr_row.size(), cudaMemcpyHostToDevice, s));
        GBS_CUDA(cudaMemcpyAsync(lrf, lr_first.data(), 4 * lr_first.size(), cudaMemcpyHostToDevice, s));
        GBS_CUDA(cudaMemcpyAsync(lrn, lr_nw.data(), 4 * lr_nw.size(), cudaMemcpyHostToDevice, s));
    }
    GBS_CUDA(cudaEventRecord(e0, s));
    GBS_CUDA(cudaMemsetAsync(deg, 0, 4ull * (n ? n : 1), s));
    k_outdeg<<<grid_of(m, sms), 256, 0, s>>>(c->d_col, m, deg);
    k_pr_init<<<grid_of(n, sms), 256, 0, s>>>(deg, n, rj, recip, weight, wb, diff[0]);
    GBS_CUDA(cudaGetLastError());
    PrArgs a{};
    a.row = c->d_row;
    a.col = c->d_col;
    a.n = n;
    a.pj = 1.0 - rj;
    a.thresh = thresh;
    a.recip = recip;
    a.weight = weight;
    a.wb = wb;
    a.srow = srw;
    a.n_short = (uint32_t)srow.size();
    a.lw_row = lwr;
    a.lw_w = lww;
    a.n_lw = (uint32_t)lw_row.size();
    a.part = part;
    a.lr_row = lrr;
    a.lr_first = lrf;
    a.lr_nw = lrn;
    a.n_lr = (uint32_t)lr_row.size();
    a.flag = flag;
    const int g1 = grid_of(std::max<unsigned long long>(srow.size(), lw_row.size()), sms);
    const int g2 = std::max(1, std::min<int>((int)((lr_row.size() + 255) / 256), sms * 16));
    uint32_t it = 0, more = 1;
    while (more && it < max_iters) {
        a.diff = diff[it & 1u];
        a.diff_next = diff[(it + 1u) & 1u];
        GBS_CUDA(cudaMemsetAsync(flag, 0, 4, s));
        k_pr_pull<<<g1, 256, 0, s>>>(a);
        if (a.n_lr) k_pr_long<<<g2, 256, 0, s>>>(a);
        GBS_CUDA(cudaGetLastError());
        GBS_CUDA(cudaMemcpyAsync(&more, flag, 4, cudaMemcpyDeviceToHost, s));
        GBS_CUDA(cudaStreamSynchronize(s));
        ++it;
    }
    GBS_CUDA(cudaEventRecord(e1, s));
    if (rank_out) GBS_CUDA(cudaMemcpyAsync(rank_out, weight, 8ull * n, cudaMemcpyDeviceToHost, s));
    GBS_CUDA(cudaStreamSynchronize(s));
    if (stats) {
        float ms = 0.f;
        GBS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        stats->iterations = it;
        stats->converged = more ? 0u : 1u;
        stats->device_ms = ms;
        stats->edges = m;
    }
    return GBS_OK;
}

gbs_status transpose_csr(const gbs_device_csr *c, gbs_device_csr *t) {
    const uint32_t n = c->n;
    const unsigned long long m = c->m;
    int dev = 0, sms = 0;
    GBS_CUDA(cudaGetDevice(&dev));
    GBS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    Pool pool;
    uint32_t *src = nullptr, *id = nullptr, *id_s = nullptr, *key_s = nullptr;
    unsigned long long *cnt = nullptr;
    GBS_CUDA(pool.get(&src, m));
    GBS_CUDA(pool.get(&id, m));
    GBS_CUDA(pool.get(&id_s, m));
    GBS_CUDA(pool.get(&key_s, m));
    GBS_CUDA(pool.get(&cnt, (size_t)n + 1));
    k_src_of<<<std::max(1, std::min<int>((n + 7) / 8, sms * 16)), 256>>>(c->d_row, n, src);
    k_iota32<<<grid_of(m, sms), 256>>>(id, m);
    GBS_CUDA(cudaGetLastError());
    size_t tmp = 0;
    GBS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, c->d_col, key_s, id, id_s, (int64_t)m));
    char *t_mem = nullptr;
    GBS_CUDA(pool.get(&t_mem, tmp));
    GBS_CUDA(cub::DeviceRadixSort::SortPairs(t_mem, tmp, c->d_col, key_s, id, id_s, (int64_t)m));
    GBS_CUDA(cudaMemset(cnt, 0, 8ull * (n + 1ull)));
    k_hist64<<<grid_of(m, sms), 256>>>(c->d_col, m, cnt);
    GBS_CUDA(cudaGetLastError());
    GBS_CUDA(cudaMalloc(&t->d_row, 8ull * (n + 1ull)));
    size_t tmp2 = 0;
    GBS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp2, cnt, t->d_row, (int64_t)n + 1));
    char *t2 = nullptr;
    GBS_CUDA(pool.get(&t2, tmp2));
    GBS_CUDA(cub::DeviceScan::ExclusiveSum(t2, tmp2, cnt, t->d_row, (int64_t)n + 1));
    GBS_CUDA(cudaMalloc(&t->d_col, 4ull * (m ? m : 1)));
    GBS_CUDA(cudaMalloc(&t->d_w, 8ull * (m ? m : 1)));
    k_transpose_place<<<grid_of(m, sms), 256>>>(id_s, src, c->d_w, m, t->d_col, t->d_w);
    GBS_CUDA(cudaGetLastError());
    GBS_CUDA(cudaDeviceSynchronize());
    t->n = n;
    t->m = m;
    return GBS_OK;
}

}  // namespace gbs

extern "C" {

gbs_status gbs_pagerank(const gbs_device_csr *in_edges, const gbs_pagerank_params *params, double *rank_out,
                        gbs_pagerank_stats *stats) {
    if (!in_edges) return gbs::fail(GBS_ERR_INVALID_ARG, "csr is NULL");
    return gbs::run_pagerank(in_edges, params, rank_out, stats);
}

gbs_status gbs_device_csr_transpose(const gbs_device_csr *c, gbs_device_csr **out) {
    if (!c || !out) return gbs::fail(GBS_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    gbs_device_csr *t = new gbs_device_csr();
    const gbs_status st = gbs::transpose_csr(c, t);
    if (st != GBS_OK) {
        gbs_device_csr_destroy(t);
        return st;
    }
    *out = t;
    return GBS_OK;
}

}  // extern "C"
