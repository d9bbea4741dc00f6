// gbs_bc.cu -- betweenness centrality on the GPU (sm_103a): Brandes over the
// shortest paths of every source, after btwcentral/csr_bc.c:16-123.
//
// Per source, the persistent delta-stepping kernel leaves the distances in
// the graph's workspace; one cooperative launch of bc_dag then works on the
// shortest-path DAG, the edges (u, v) with dist(u) + w == dist(v) computed in
// the weight type (the reference keeps these as predecessor lists,
// sssp/csr_sspath.c:116-118; here they are derived from the distances):
//
//   COUNT     every reached vertex: sigma := [v == source]; every tight
//             out-edge (u, v) sets its bit in the tight-edge mask (one bit per
//             CSR position, 32 to a word) and adds 1 to indeg[v].  The grid
//             walks the CSR one 32-position word per warp step, whatever the
//             row lengths (a per-word index gives each position's row).
//   FORWARD   Kahn levels from the source: level L+1 holds the vertices whose
//             last tight in-edge came from level L.  Along the tight edges of
//             a level, sigma[v] += sigma[u] (64-bit integer atomics: exact,
//             and wrapping like the reference's lint sums, comp_num_spath,
//             csr_bc.c:67-91).
//   BACKWARD  levels in reverse: every vertex pulls
//             delta[u] = sum over tight out-edges (u, v) of
//                        (1 + delta[v]) * sigma[u] / sigma[v]
//             (comp_delta, csr_bc.c:93-116) and adds it to bc[u].
//
// Work layout.  A level is the slice order[lo, hi) of one order list.  Rows
// of at most kLaneRow edges (two mask words) are walked by one lane.  A longer
// row, when its vertex is appended, reserves its mask words in the level's
// "word space", so the next pass shares the words of all long rows of a level
// evenly over the grid, one word per lane, however skewed the degrees.  A grid
// barrier separates levels; the CTA that arrives last publishes the next
// level's bounds.
//
// Summation order.  delta[u] is fixed independently of the launch shape.  A
// 32-position mask word's sum is the butterfly of its 32 slots (for h = 16,
// 8, 4, 2, 1: s[i] += s[i + h]; slots of other rows or of edges that are not
// tight hold 0); the row's words, numbered from its first word, form blocks
// of 32 whose word sums are combined by the same butterfly, and the block sums
// are added in order.  The trees keep the chains of dependent FP64 adds short
// (55 cycles each on this part); the oracle follows the same order, so
// results are bit-identical for every weight type.
//
// HBM per source: COUNT streams every row of a reached vertex (8 B per edge)
// and gathers the targets' state words; FORWARD and BACKWARD read 1 bit per
// edge plus the tight edges' entries.  The per-vertex arrays (dist 8 B,
// sigma 8 B, delta 8 B, indeg 4 B, order 4 B) stay in L2 for graphs of a few
// million vertices.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gbs_host.hpp"
#include "gbs_internal.cuh"

namespace gbs {
namespace {

constexpr int kBcTPB = 1024;          // threads per CTA of the DAG kernel (one CTA per SM)
constexpr uint32_t kLaneRow = 32;     // FORWARD / BACKWARD: rows up to this long are walked by one lane
constexpr unsigned kFull = 0xffffffffu;

struct __align__(128) LineU64 {
    unsigned long long v;
    uint32_t pad[30];
};

// Control block of one bc_dag launch (zeroed before every launch).
struct __align__(128) BcCtl {
    uint32_t bar_count;
    uint32_t pad0[31];
    uint32_t bar_gen;
    uint32_t pad1[31];
    uint32_t error;
    uint32_t pub_lo;       // order[pub_lo, pub_hi) is the level to process next,
    uint32_t pub_hi;
    uint32_t pub_wlo;      // [pub_wlo, pub_whi) the words of its long rows
    uint32_t pub_whi;
    uint32_t pub_slo;      // [pub_slo, pub_shi) its long rows
    uint32_t pub_shi;
    uint32_t levels;       // forward levels (the source's is level 0)
    uint32_t trace_n;      // phase records written (GBS_F_TRACE)
    uint32_t pad2[21];
    unsigned long long t0; // globaltimer when CTA 0 started
    Line ord_cnt;          // vertices appended to the order list
    LineU64 long_cnt;      // (long rows << 32) | words reserved
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
    uint32_t *wlv;                   // word-space index where each level starts (n + 1)
    uint32_t *slv;                   // long-row index where each level starts (n + 1)
    uint32_t *mask;                  // tight-edge bits: position e is bit e % 32 of word e / 32
    uint32_t *lr_u;                  // long rows: vertex,
    uint32_t *lr_b;                  //   first word in the word space,
    uint32_t *lr_n;                  //   number of words
    uint32_t *vw_u;                  // word space: the vertex of each word,
    uint32_t *vw_w;                  //   its mask word,
    uint32_t *vw_rm;                 //   the slots of that word inside the row,
    double *vw_part;                 //   and its BACKWARD partial sum
    const uint32_t *ne_rows;         // the rows with at least one edge, in order
    const uint2 *wown;               // per mask word: {index in ne_rows of the row owning its
                                     //   first position, bit p set if a row starts at position p > 0}
    uint32_t n_words;                // mask words holding positions (m / 32 rounded up)
    uint32_t m;
    double *bc;
    BcCtl *ctl;
    BcTotals *tot;
    TraceRec *trace;                 // GBS_F_TRACE: one record per phase (kinds kTrCount..kTrBackward)
    uint32_t trace_cap;
    unsigned long long wait_ns;
    uint32_t nblocks;
};

// Trace record kinds of the betweenness phases (bucket = level, items =
// vertices of the level, edges = mask words of its long rows).
constexpr uint32_t kTrCount = 8, kTrForward = 9, kTrBackward = 10, kTrBackwardWords = 11;

// Called by the deciding thread: one record for the phase that just ended.
__device__ __forceinline__ void trace_phase(const BcArgs &a, uint32_t kind, uint32_t level, uint32_t items,
                                            uint32_t words) {
    if (!a.trace) return;
    BcCtl *c = a.ctl;
    const uint32_t i = c->trace_n;
    if (i < a.trace_cap) {
        TraceRec r;
        r.kind = kind;
        r.bucket = level;
        r.items = items;
        r.edges = words;
        r.pending = 0;
        r.window = 0;
        r.end_ns = globaltimer() - c->t0;
        a.trace[i] = r;
    }
    c->trace_n = i + 1;
}

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

// One past the last mask word of a row ending at position `end` (no overflow near 2^32).
__device__ __forceinline__ uint32_t words_end(uint32_t end) { return (end >> 5) + ((end & 31u) != 0u); }

// Mask word W restricted to the positions of row [beg, end).
__device__ __forceinline__ uint32_t row_bits(uint32_t word, uint32_t W, uint32_t beg, uint32_t end) {
    const unsigned long long base = (unsigned long long)W << 5;
    if (beg > base) word &= kFull << (uint32_t)(beg - base);
    if ((unsigned long long)end < base + 32ull) word &= (1u << (uint32_t)(end - base)) - 1u;
    return word;
}

// The mask bits of a row of at most 32 edges, bit i = position beg + i.
__device__ __forceinline__ unsigned long long short_row_bits(const BcArgs &a, uint32_t beg, uint32_t end) {
    if (end <= beg) return 0ull;
    const uint32_t w0 = beg >> 5;
    unsigned long long x = __ldcg(a.mask + w0);
    if (((end - 1u) >> 5) != w0) x |= (unsigned long long)__ldcg(a.mask + w0 + 1) << 32;
    x >>= (beg & 31u);
    return x & ((1ull << (end - beg)) - 1ull);
}

__device__ __forceinline__ void set_error(const BcArgs &a, uint32_t code) {
    atomicCAS(&a.ctl->error, 0u, code);
    atomicCAS(&a.tot->error, 0u, code);
}

// Grid barrier; the CTA that arrives last runs `decide` (thread 0 alone, all
// other CTAs at rest) before releasing the rest.  Waits are bounded by
// a.wait_ns; on expiry the error word is set.  s_pub receives the published
// level bounds.  Returns false when the launch must stop.
template <typename Decide>
__device__ __forceinline__ bool grid_step(const BcArgs &a, uint32_t &gen, uint32_t *s_pub, Decide decide) {
    __syncthreads();
    if (threadIdx.x == 0) {
        BcCtl *c = a.ctl;
        const bool last = atom_add_acq_rel(&c->bar_count, 1u) == a.nblocks - 1u;
        if (last) {
            decide();
            c->bar_count = 0;
            st_release(&c->bar_gen, gen + 1u);   // releases the decision and the reset
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
        s_pub[2] = ld_relaxed(&c->pub_wlo);
        s_pub[3] = ld_relaxed(&c->pub_whi);
        s_pub[4] = ld_relaxed(&c->pub_slo);
        s_pub[5] = ld_relaxed(&c->pub_shi);
        s_pub[6] = ld_relaxed(&c->error);
    }
    __syncthreads();
    ++gen;
    return s_pub[6] == 0;
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x) {
    const unsigned lane = threadIdx.x & 31u;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    return x;
}

// Records a long row reserved at slot `slot`, words [wb, wb + nw) of the word
// space.  All 32 lanes call it with the same arguments.
__device__ __forceinline__ void fill_row(const BcArgs &a, uint32_t slot, uint32_t v, uint32_t wb, uint32_t nw) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t beg = __ldg(a.row + v), end = __ldg(a.row + v + 1);
    if (lane == 0) {
        a.lr_u[slot] = v;
        a.lr_b[slot] = wb;
        a.lr_n[slot] = nw;
    }
    for (uint32_t i = lane; i < nw; i += 32u) {
        const uint32_t W = (beg >> 5) + i;
        a.vw_u[wb + i] = v;
        a.vw_w[wb + i] = W;
        a.vw_rm[wb + i] = row_bits(kFull, W, beg, end);
    }
}

// Appends the lanes whose `take` is set to the order list (one counter
// atomic per warp); rows longer than kLaneRow also reserve their mask words
// in the word space (one more atomic per warp), and the warp writes the
// reserved words' owner.  All 32 lanes call it.
__device__ __forceinline__ void append_order(const BcArgs &a, bool take, uint32_t v) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned b = __ballot_sync(kFull, take);
    if (!b) return;
    const int l0 = __ffs(b) - 1;
    uint32_t base = 0;
    if ((int)lane == l0) base = atomicAdd(&a.ctl->ord_cnt.v, (uint32_t)__popc(b));
    base = __shfl_sync(kFull, base, l0);
    const unsigned below = (1u << lane) - 1u;
    uint32_t nw = 0, wb = 0, slot = 0;
    if (take) {
        a.order[base + __popc(b & below)] = v;
        const uint32_t beg = __ldg(a.row + v), end = __ldg(a.row + v + 1);
        if (end - beg > kLaneRow) nw = words_end(end) - (beg >> 5);
    }
    unsigned lb = __ballot_sync(kFull, nw != 0);
    if (!lb) return;
    const uint32_t incl = warp_incl_scan(nw);
    const uint32_t tot = __shfl_sync(kFull, incl, 31);
    const int l1 = __ffs(lb) - 1;
    unsigned long long old = 0;
    if ((int)lane == l1) old = atomicAdd(&a.ctl->long_cnt.v, ((unsigned long long)__popc(lb) << 32) | tot);
    old = __shfl_sync(kFull, old, l1);
    if (nw) {
        slot = (uint32_t)(old >> 32) + __popc(lb & below);
        wb = (uint32_t)old + incl - nw;
    }
    while (lb) {
        const int q = __ffs(lb) - 1;
        lb &= lb - 1;
        fill_row(a, __shfl_sync(kFull, slot, q), __shfl_sync(kFull, v, q), __shfl_sync(kFull, wb, q),
                 __shfl_sync(kFull, nw, q));
    }
}

// L2 policies for COUNT: the edge stream is read once (evict first), the
// state words it gathers are reused across the whole pass (evict last).
__device__ __forceinline__ unsigned long long l2_policy_first() {
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ unsigned long long l2_policy_last() {
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint2 ld_edge_once(const uint2 *ptr, unsigned long long pol) {
    uint2 v;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
                 : "=r"(v.x), "=r"(v.y) : "l"(ptr), "l"(pol));
    return v;
}
__device__ __forceinline__ unsigned long long ld_state_keep(const unsigned long long *ptr,
                                                            unsigned long long pol) {
    unsigned long long v;
    asm volatile("ld.global.nc.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(ptr), "l"(pol));
    return v;
}

// COUNT over mask words: the warp takes kCountUnroll words per round, one
// position per lane, all loads of the round in flight before any is used.
// The row owning position W * 32 + l is ne_rows[k0 + popc(starts & bits 1..l)].
constexpr uint32_t kCountUnroll = 4;
template <int WT>
__device__ __forceinline__ void count_words(const BcArgs &a, uint32_t W0, uint32_t stride,
                                            unsigned long long &tight_n) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t below = (2u << lane) - 1u;
    const unsigned long long pol_first = l2_policy_first(), pol_last = l2_policy_last();
    for (uint32_t Wb = W0; Wb < a.n_words; Wb += stride * kCountUnroll) {
        uint32_t e[kCountUnroll], u[kCountUnroll];
        uint2 ew[kCountUnroll];
        unsigned long long pu[kCountUnroll], pv[kCountUnroll];
        bool ok[kCountUnroll];
#pragma unroll
        for (uint32_t j = 0; j < kCountUnroll; ++j) {
            const uint32_t W = Wb + j * stride;
            const unsigned long long e64 = ((unsigned long long)W << 5) + lane;
            ok[j] = W < a.n_words && e64 < a.m;
            e[j] = (uint32_t)e64;
            u[j] = 0;
            if (ok[j]) {
                const uint2 o = __ldg(a.wown + W);
                u[j] = o.x + (uint32_t)__popc(o.y & below);
            }
            ew[j] = ok[j] ? ld_edge_once(a.adj + e[j], pol_first) : make_uint2(0u, 0u);
        }
#pragma unroll
        for (uint32_t j = 0; j < kCountUnroll; ++j) u[j] = ok[j] ? __ldg(a.ne_rows + u[j]) : 0u;
#pragma unroll
        for (uint32_t j = 0; j < kCountUnroll; ++j) {
            pu[j] = ok[j] ? ld_state_keep(a.dp + u[j], pol_last) : kUnreached;
            pv[j] = ok[j] ? ld_state_keep(a.dp + ew[j].x, pol_last) : kUnreached;
        }
#pragma unroll
        for (uint32_t j = 0; j < kCountUnroll; ++j)
            if (pu[j] != kUnreached && pv[j] != kUnreached && tight<WT>(pu[j], pv[j], ew[j], a.w64, e[j])) {
                atomicAdd(a.indeg + ew[j].x, 1u);
                atomicOr(a.mask + (e[j] >> 5), 1u << (e[j] & 31u));
                ++tight_n;
            }
    }
}

// ---------------------------------------------------------------- appends
// Vertices whose last tight in-edge was just consumed are staged in shared
// memory (one shared atomic per warp) and written to the order list by
// flush_appends at the end of the level, with one global atomic per CTA for
// the order slots and one for the word space.  Past kStage entries a warp
// appends straight to global memory.
constexpr uint32_t kStage = 6144;
struct Stage {
    uint32_t v[kStage];
    uint32_t n;
    uint32_t base;
    unsigned long long wbase;
    unsigned long long scan[33];
};

__device__ __forceinline__ void stage_append(const BcArgs &a, Stage &st, bool take, uint32_t v) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned b = __ballot_sync(kFull, take);
    if (!b) return;
    const int l0 = __ffs(b) - 1;
    uint32_t base = 0;
    if ((int)lane == l0) base = atomicAdd(&st.n, (uint32_t)__popc(b));
    base = __shfl_sync(kFull, base, l0);
    const uint32_t pos = base + __popc(b & ((1u << lane) - 1u));
    if (take && pos < kStage) st.v[pos] = v;
    if (base + __popc(b) > kStage) append_order(a, take && pos >= kStage, v);
}

__device__ __forceinline__ unsigned long long warp_incl_scan64(unsigned long long x) {
    const unsigned lane = threadIdx.x & 31u;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(kFull, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    return x;
}

// Block-wide exclusive scan of x; *total gets the sum.  Every thread calls it.
__device__ __forceinline__ unsigned long long block_excl_scan64(unsigned long long x, Stage &st,
                                                                unsigned long long &total) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned long long incl = warp_incl_scan64(x);
    if (lane == 31) st.scan[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const unsigned long long w = lane < (blockDim.x >> 5) ? st.scan[lane] : 0ull;
        const unsigned long long wi = warp_incl_scan64(w);
        st.scan[lane] = wi - w;
        if (lane == 31) st.scan[32] = wi;
    }
    __syncthreads();
    const unsigned long long r = st.scan[warp] + incl - x;
    total = st.scan[32];
    __syncthreads();
    return r;
}

// Writes the staged vertices to the order list; rows longer than kLaneRow
// reserve their mask words in the word space.  Every thread calls it.
__device__ __forceinline__ void flush_appends(const BcArgs &a, Stage &st) {
    __syncthreads();
    const uint32_t n = min(st.n, kStage);
    if (n) {
        if (threadIdx.x == 0) st.base = atomicAdd(&a.ctl->ord_cnt.v, n);
        __syncthreads();
        for (uint32_t i0 = 0; i0 < n; i0 += blockDim.x) {
            const uint32_t i = i0 + threadIdx.x;
            uint32_t v = 0, nw = 0;
            if (i < n) {
                v = st.v[i];
                a.order[st.base + i] = v;
                const uint32_t beg = __ldg(a.row + v), end = __ldg(a.row + v + 1);
                if (end - beg > kLaneRow) nw = words_end(end) - (beg >> 5);
            }
            // (long rows << 32) | words, scanned over the block
            unsigned long long tot = 0;
            const unsigned long long ex = block_excl_scan64(nw ? (1ull << 32) | nw : 0ull, st, tot);
            if (tot) {
                if (threadIdx.x == 0) st.wbase = atomicAdd(&a.ctl->long_cnt.v, tot);
                __syncthreads();
                const unsigned long long at = st.wbase + ex;
                const uint32_t slot = (uint32_t)(at >> 32), wb = (uint32_t)at;
                unsigned lb = __ballot_sync(kFull, nw != 0);
                while (lb) {
                    const int q = __ffs(lb) - 1;
                    lb &= lb - 1;
                    fill_row(a, __shfl_sync(kFull, slot, q), __shfl_sync(kFull, v, q), __shfl_sync(kFull, wb, q),
                             __shfl_sync(kFull, nw, q));
                }
                __syncthreads();
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) st.n = 0;
    __syncthreads();
}

// ------------------------------------------------------- flattened walks
// The lanes of a warp hold tight-edge bits (bit i = position e0 + i).  The
// walks number all of the warp's tight edges -- lane 0's first, each lane's
// from the lowest (FORWARD) or highest (BACKWARD) position -- and hand out
// 32 per round, so every lane has work whatever the split of the bits.

// The lane whose bits hold edge number k: the smallest j with incl_j > k.
__device__ __forceinline__ uint32_t flat_owner(uint32_t incl, uint32_t k) {
    uint32_t j = 0;
    for (uint32_t s = 16; s; s >>= 1) {
        const uint32_t c = __shfl_sync(kFull, incl, j + s - 1u);
        if (k >= c) j += s;
    }
    return min(j, 31u);
}
__device__ __forceinline__ uint32_t nth_low_bit(unsigned long long x, uint32_t n) {
    for (uint32_t r = 0; r < n; ++r) x &= x - 1ull;
    return (uint32_t)(__ffsll((long long)x) - 1);
}

// One dependency term (1 + delta[v]) * sigma[u] / sigma[v], in the order of
// operations of comp_delta (csr_bc.c:110).
// Multiplying or dividing by a path count of 1 is exact, so those operations
// (the division costs ~570 cycles here) are skipped.
__device__ __forceinline__ double dep_term(const BcArgs &a, unsigned long long su, uint32_t e) {
    const uint32_t v = __ldg(a.adj + e).x;
    const unsigned long long sv = __ldcg(a.sigma + v);
    double t = __dadd_rn(1.0, __ldcg(a.delta + v));
    if (su != 1ull) t = __dmul_rn(t, __ll2double_rn((long long)su));
    if (sv != 1ull) t = __ddiv_rn(t, __ll2double_rn((long long)sv));
    return t;
}

// Butterfly of one double per lane: lane 0 gets the tree sum.  All 32 lanes call it.
__device__ __forceinline__ double butterfly32(double t) {
    for (int h = 16; h > 0; h >>= 1) t = __dadd_rn(t, __shfl_down_sync(kFull, t, h));
    return t;
}

// Word sums of the lanes' words (W, bits restricted to the row; su the row's
// path count): a word with at most two tight slots is summed by its lane (the
// butterfly of at most two non-zero slots is their sum); heavier words are
// summed by the whole warp, one slot per lane.  All 32 lanes call it.
__device__ __forceinline__ double word_sums(const BcArgs &a, uint32_t W, uint32_t bits, unsigned long long su) {
    const unsigned lane = threadIdx.x & 31u;
    double p = 0.0;
    const uint32_t cnt = __popc(bits);
    if (cnt && cnt <= 2u) {
        const uint32_t b0 = (uint32_t)(__ffs(bits) - 1);
        p = dep_term(a, su, (W << 5) + b0);
        const uint32_t rest = bits & (bits - 1u);
        if (rest) p = __dadd_rn(p, dep_term(a, su, (W << 5) + (uint32_t)(__ffs(rest) - 1)));
    }
    unsigned heavy = __ballot_sync(kFull, cnt > 2u);
    while (heavy) {
        const int q = __ffs(heavy) - 1;
        heavy &= heavy - 1;
        const uint32_t qW = __shfl_sync(kFull, W, q);
        const uint32_t qb = __shfl_sync(kFull, bits, q);
        const unsigned long long qs = __shfl_sync(kFull, su, q);
        const double t = ((qb >> lane) & 1u) ? dep_term(a, qs, (qW << 5) + lane) : 0.0;
        const double r = __shfl_sync(kFull, butterfly32(t), 0);
        if ((int)lane == q) p = r;
    }
    return p;
}

// FORWARD: sigma[v] += sigma[u] and the in-degree count-down along every
// tight edge of the warp; vertices reaching zero are staged.  When no lane
// holds more than one edge the lanes go straight to their own.
__device__ __forceinline__ void push_flat(const BcArgs &a, Stage &st, unsigned long long bits, uint32_t e0,
                                          unsigned long long su) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t cnt = __popcll((long long)bits);
    if (__reduce_max_sync(kFull, cnt) <= 1u) {
        bool take = false;
        uint32_t v = 0;
        if (cnt) {
            v = __ldg(a.adj + e0 + (uint32_t)(__ffsll((long long)bits) - 1)).x;
            atomicAdd(a.sigma + v, su);
            take = atomicSub(a.indeg + v, 1u) == 1u;
        }
        stage_append(a, st, take, v);
        return;
    }
    const uint32_t incl = warp_incl_scan(cnt);
    const uint32_t total = __shfl_sync(kFull, incl, 31);
    for (uint32_t base = 0; base < total; base += 32u) {
        const uint32_t k = base + lane;
        const uint32_t j = flat_owner(incl, k);
        const unsigned long long bj = __shfl_sync(kFull, bits, j);
        const unsigned long long sj = __shfl_sync(kFull, su, j);
        const uint32_t ej = __shfl_sync(kFull, e0, j);
        const uint32_t xj = __shfl_sync(kFull, incl - cnt, j);
        bool take = false;
        uint32_t v = 0;
        if (k < total) {
            v = __ldg(a.adj + ej + nth_low_bit(bj, k - xj)).x;
            atomicAdd(a.sigma + v, sj);
            take = atomicSub(a.indeg + v, 1u) == 1u;
        }
        stage_append(a, st, take, v);
    }
}

// A word of the word space: its row's vertex, mask word and tight slots.
struct SpaceWord {
    uint32_t u, W, bits;
};
__device__ __forceinline__ SpaceWord space_word(const BcArgs &a, uint32_t x) {
    SpaceWord r;
    r.u = __ldcg(a.vw_u + x);
    r.W = __ldcg(a.vw_w + x);
    r.bits = __ldcg(a.mask + r.W) & __ldcg(a.vw_rm + x);
    return r;
}

// FORWARD for order[i0 + lane], i0 + lane < hi: rows of at most kLaneRow edges.
__device__ __forceinline__ void forward_rows(const BcArgs &a, Stage &st, uint32_t i0, uint32_t hi) {
    const uint32_t i = i0 + (threadIdx.x & 31u);
    unsigned long long bits = 0, su = 0;
    uint32_t beg = 0;
    if (i < hi) {
        const uint32_t u = __ldcg(a.order + i);
        beg = __ldg(a.row + u);
        const uint32_t end = __ldg(a.row + u + 1);
        if (end - beg <= kLaneRow) {
            bits = short_row_bits(a, beg, end);
            if (bits) su = __ldcg(a.sigma + u);
        }
    }
    push_flat(a, st, bits, beg, su);
}

// Words of the word space one warp takes at a time: 32 consecutive ones on
// a big level, fewer on a level of few (hub) words so that every warp gets
// some (a hub word holds up to 32 tight edges, and one warp working through
// 32 of them while the others wait at the barrier was the cost of such
// levels).  The mapping changes no result: every word's sum is formed alone.
__device__ __forceinline__ uint32_t words_per_warp(uint32_t words, uint32_t nwarps) {
    const uint32_t c = (words + nwarps - 1u) / nwarps;
    return c < 1u ? 1u : (c > 32u ? 32u : c);
}

// FORWARD for the words x0 + lane < xe of the level's long rows.
__device__ __forceinline__ void forward_words(const BcArgs &a, Stage &st, uint32_t x0, uint32_t xe) {
    const uint32_t x = x0 + (threadIdx.x & 31u);
    unsigned long long su = 0;
    uint32_t bits = 0, W = 0;
    if (x < xe) {
        const SpaceWord sw = space_word(a, x);
        bits = sw.bits;
        W = sw.W;
        if (bits) su = __ldcg(a.sigma + sw.u);
    }
    push_flat(a, st, bits, W << 5, su);
}

// BACKWARD for order[i0 + lane], i0 + lane < hi: rows of at most kLaneRow
// edges, i.e. at most two mask words (word slots 0 and 1 of the row's block,
// whose butterfly is their sum).
__device__ __forceinline__ void backward_rows(const BcArgs &a, uint32_t i0, uint32_t hi) {
    const uint32_t i = i0 + (threadIdx.x & 31u);
    uint32_t u = 0, beg = 0, end = 0, w0 = 0, b0 = 0, b1 = 0;
    unsigned long long su = 0;
    bool mine = false;
    if (i < hi) {
        u = __ldcg(a.order + i);
        beg = __ldg(a.row + u);
        end = __ldg(a.row + u + 1);
        mine = end - beg <= kLaneRow;
        if (mine && end > beg) {
            w0 = beg >> 5;
            b0 = row_bits(__ldcg(a.mask + w0), w0, beg, end);
            if (((end - 1u) >> 5) != w0) b1 = row_bits(__ldcg(a.mask + w0 + 1), w0 + 1, beg, end);
            if (b0 | b1) su = __ldcg(a.sigma + u);
        }
    }
    const double p0 = word_sums(a, w0, b0, su);
    const double p1 = word_sums(a, w0 + 1, b1, su);
    if (mine) {
        const double d = __dadd_rn(p0, p1);
        a.delta[u] = d;
        a.bc[u] = __dadd_rn(a.bc[u], d);
    }
}

// BACKWARD for the words x0 + lane < xe of the level's long rows: each
// word's sum goes to vw_part.
__device__ __forceinline__ void backward_words(const BcArgs &a, uint32_t x0, uint32_t xe) {
    const uint32_t x = x0 + (threadIdx.x & 31u);
    SpaceWord sw{};
    unsigned long long su = 0;
    if (x < xe) {
        sw = space_word(a, x);
        if (sw.bits) su = __ldcg(a.sigma + sw.u);
    }
    const double p = word_sums(a, sw.W, sw.bits, su);
    if (x < xe) a.vw_part[x] = p;
}

// BACKWARD, after backward_words: delta of long rows.  Each block of 32 word
// sums is combined by the butterfly and the block sums are added in order.
// finish_rows: slots s0 + lane < shi; a row of at most 8 words is finished by
// its lane (the butterfly of slots 0..7, the other slots being 0), longer
// rows by the whole warp.  finish_row: one row, the whole warp, a block per
// step (the next block loads while one is added).  All 32 lanes call them.
__device__ __forceinline__ void finish_row(const BcArgs &a, uint32_t bu, uint32_t bf, uint32_t bn) {
    const unsigned lane = threadIdx.x & 31u;
    double r = 0.0;
    double cur = lane < bn ? __ldcg(a.vw_part + bf + lane) : 0.0;
    for (uint32_t t0 = 0; t0 < bn; t0 += 32u) {
        const uint32_t nx = t0 + 32u + lane;
        const double next = nx < bn ? __ldcg(a.vw_part + bf + nx) : 0.0;
        r = __dadd_rn(r, __shfl_sync(kFull, butterfly32(cur), 0));
        cur = next;
    }
    if (lane == 0) {
        a.delta[bu] = r;
        a.bc[bu] = __dadd_rn(a.bc[bu], r);
    }
}

__device__ __forceinline__ void finish_rows(const BcArgs &a, uint32_t s0, uint32_t shi) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t sl = s0 + lane;
    uint32_t u = 0, first = 0, nw = 0;
    if (sl < shi) {
        u = __ldcg(a.lr_u + sl);
        first = __ldcg(a.lr_b + sl);
        nw = __ldcg(a.lr_n + sl);
    }
    if (nw && nw <= 8u) {
        double q[8];
#pragma unroll
        for (uint32_t k = 0; k < 8u; ++k) q[k] = k < nw ? __ldcg(a.vw_part + first + k) : 0.0;
#pragma unroll
        for (uint32_t h = 4; h > 0; h >>= 1)
#pragma unroll
            for (uint32_t k = 0; k < h; ++k) q[k] = __dadd_rn(q[k], q[k + h]);
        a.delta[u] = q[0];
        a.bc[u] = __dadd_rn(a.bc[u], q[0]);
    }
    unsigned big = __ballot_sync(kFull, nw > 8u);
    while (big) {
        const int qn = __ffs(big) - 1;
        big &= big - 1;
        finish_row(a, __shfl_sync(kFull, u, qn), __shfl_sync(kFull, first, qn), __shfl_sync(kFull, nw, qn));
    }
}

template <int WT>
__global__ void __launch_bounds__(kBcTPB, 1) bc_dag(BcArgs a) {
    __shared__ uint32_t s_pub[7];
    __shared__ uint32_t s_nw;
    __shared__ Stage st;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (a.nblocks * blockDim.x) >> 5;
    uint32_t gen = 0;
    BcCtl *c = a.ctl;
    // ---- COUNT (CTA 0 also puts the source on level 0)
    if (threadIdx.x == 0) st.n = 0;
    if (blockIdx.x == 0) {
        if (threadIdx.x == 0) {
            c->t0 = globaltimer();
            a.order[0] = a.source;
            c->ord_cnt.v = 1u;
            a.lvl[0] = 0u;
            a.wlv[0] = 0u;
            a.slv[0] = 0u;
            const uint32_t beg = __ldg(a.row + a.source), end = __ldg(a.row + a.source + 1);
            s_nw = end - beg > kLaneRow ? words_end(end) - (beg >> 5) : 0u;
            if (s_nw) c->long_cnt.v = (1ull << 32) | s_nw;
        }
        __syncthreads();
        if (threadIdx.x < 32 && s_nw) fill_row(a, 0u, a.source, 0u, s_nw);
    }
    unsigned long long tight_n = 0;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < a.n; u += a.nblocks * blockDim.x)
        if (__ldg(a.dp + u) != kUnreached) a.sigma[u] = u == a.source ? 1ull : 0ull;
    count_words<WT>(a, gwarp, nwarps, tight_n);
    for (int o = 16; o > 0; o >>= 1) tight_n += __shfl_down_sync(kFull, tight_n, o);
    if (lane == 0 && tight_n) atomicAdd(&a.tot->tight, tight_n);
    uint32_t L = 0;
    auto first = [&]() {
        trace_phase(a, kTrCount, 0, a.n, a.n_words);
        c->pub_lo = 0u;
        c->pub_hi = 1u;
        c->pub_wlo = 0u;
        c->pub_whi = (uint32_t)c->long_cnt.v;
        c->pub_slo = 0u;
        c->pub_shi = (uint32_t)(c->long_cnt.v >> 32);
    };
    if (!grid_step(a, gen, s_pub, first)) return;
    // ---- FORWARD: level L is order[lo, hi), its long rows' words [wlo, whi)
    for (;;) {
        const uint32_t lo = s_pub[0], hi = s_pub[1], wlo = s_pub[2], whi = s_pub[3], shi = s_pub[5];
        if (lo >= hi) break;
        for (uint32_t i0 = lo + gwarp * 32u; i0 < hi; i0 += nwarps * 32u) forward_rows(a, st, i0, hi);
        const uint32_t cw = words_per_warp(whi - wlo, nwarps);
        for (uint32_t x0 = wlo + gwarp * cw; x0 < whi; x0 += nwarps * cw) forward_words(a, st, x0, min(x0 + cw, whi));
        flush_appends(a, st);
        auto next = [&]() {
            trace_phase(a, kTrForward, L, hi - lo, whi - wlo);
            a.lvl[L + 1] = hi;
            a.wlv[L + 1] = whi;
            a.slv[L + 1] = shi;
            const unsigned long long lc = c->long_cnt.v;
            c->pub_lo = hi;
            c->pub_hi = ld_relaxed(&c->ord_cnt.v);
            c->pub_wlo = whi;
            c->pub_whi = (uint32_t)lc;
            c->pub_slo = shi;
            c->pub_shi = (uint32_t)(lc >> 32);
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
        const uint32_t wlo = __ldcg(a.wlv + k), whi = __ldcg(a.wlv + k + 1);
        for (uint32_t i0 = lo + gwarp * 32u; i0 < hi; i0 += nwarps * 32u) backward_rows(a, i0, hi);
        const uint32_t cw = words_per_warp(whi - wlo, nwarps);
        for (uint32_t x0 = wlo + gwarp * cw; x0 < whi; x0 += nwarps * cw) backward_words(a, x0, min(x0 + cw, whi));
        if (whi > wlo) {   // the level's long rows: add up their word sums
            auto words_done = [&]() { trace_phase(a, kTrBackwardWords, k, hi - lo, whi - wlo); };
            if (!grid_step(a, gen, s_pub, words_done)) return;
            const uint32_t slo = __ldcg(a.slv + k), shi = __ldcg(a.slv + k + 1);
            if (shi - slo <= 4u * nwarps) {   // few rows: a warp each
                for (uint32_t sl = slo + gwarp; sl < shi; sl += nwarps)
                    finish_row(a, __ldcg(a.lr_u + sl), __ldcg(a.lr_b + sl), __ldcg(a.lr_n + sl));
            } else {
                for (uint32_t s0 = slo + gwarp * 32u; s0 < shi; s0 += nwarps * 32u) finish_rows(a, s0, shi);
            }
        }
        if (a.trace || k > 1) {
            auto done = [&]() { trace_phase(a, kTrBackward, k, hi - lo, whi - wlo); };
            if (!grid_step(a, gen, s_pub, done)) return;
        }
    }
}

// Batched shortest paths hand back plain distances (uint32 / float32 bits,
// UINT32_MAX / +inf unreached); the DAG passes read state words.
template <bool F32>
__global__ void k_pack_dist(const uint32_t *__restrict__ dist, uint32_t n, unsigned long long *__restrict__ dp) {
    const uint32_t unreached = F32 ? 0x7F800000u : 0xFFFFFFFFu;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t d = dist[v];
        dp[v] = d == unreached ? kUnreached : (unsigned long long)d << 32;
    }
}

constexpr uint32_t kBcBatch = 64;   // sources per batched shortest-path launch

struct BcState {
    unsigned long long *sigma = nullptr;
    double *delta = nullptr;
    uint32_t *indeg = nullptr;
    uint32_t *order = nullptr;
    uint32_t *lvl = nullptr;
    uint32_t *wlv = nullptr;
    uint32_t *lr_u = nullptr;
    uint32_t *lr_b = nullptr;
    uint32_t *slv = nullptr;
    uint32_t *lr_n = nullptr;
    uint32_t *vw_u = nullptr;
    uint32_t *vw_w = nullptr;
    uint32_t *vw_rm = nullptr;
    double *vw_part = nullptr;
    uint32_t *mask = nullptr;
    uint32_t *ne_rows = nullptr;
    uint2 *wown = nullptr;
    uint32_t n_words = 0;
    size_t mask_words = 0;
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
    // the rows COUNT shares out word by word, and the hub count
    std::vector<uint32_t> row(n + 1);
    GBS_CUDA(cudaMemcpy(row.data(), g->d_row, sizeof(uint32_t) * (n + 1), cudaMemcpyDeviceToHost));
    size_t n_long = 0, long_words = 0;   // rows longer than kLaneRow and their mask words
    std::vector<uint32_t> ne_rows;
    for (uint32_t v = 0; v < g->n; ++v) {
        const uint32_t beg = row[v], end = row[v + 1];
        if (end == beg) continue;
        ne_rows.push_back(v);
        if (end - beg > kLaneRow) {
            ++n_long;
            long_words += ((end >> 5) + ((end & 31u) != 0u)) - (beg >> 5);
        }
    }
    // per mask word: the non-empty row owning its first position and the
    // positions where later rows start
    const uint32_t n_words = (uint32_t)((g->m >> 5) + ((g->m & 31u) != 0u));
    std::vector<uint2> wown(std::max<uint32_t>(n_words, 1u), make_uint2(0u, 0u));
    for (size_t k = 0; k < ne_rows.size(); ++k) {
        const uint32_t beg = row[ne_rows[k]], end = row[ne_rows[k] + 1];
        if (beg & 31u) wown[beg >> 5].y |= 1u << (beg & 31u);
        const uint32_t w_first = (beg + 31u) >> 5, w_end = (end >> 5) + ((end & 31u) != 0u);
        for (uint32_t W = w_first; W < w_end; ++W) wown[W].x = (uint32_t)k;   // rows covering position W * 32
    }
    b->n_words = n_words;
    b->mask_words = (size_t)(g->m >> 5) + 1;
    GBS_CUDA(cudaMalloc(&b->sigma, sizeof(unsigned long long) * n));
    GBS_CUDA(cudaMalloc(&b->delta, sizeof(double) * n));
    GBS_CUDA(cudaMalloc(&b->indeg, sizeof(uint32_t) * n));
    GBS_CUDA(cudaMalloc(&b->order, sizeof(uint32_t) * n));
    GBS_CUDA(cudaMalloc(&b->lvl, sizeof(uint32_t) * (n + 1)));
    GBS_CUDA(cudaMalloc(&b->wlv, sizeof(uint32_t) * (n + 1)));
    GBS_CUDA(cudaMalloc(&b->lr_u, sizeof(uint32_t) * std::max<size_t>(n_long, 1)));
    GBS_CUDA(cudaMalloc(&b->lr_b, sizeof(uint32_t) * std::max<size_t>(n_long, 1)));
    GBS_CUDA(cudaMalloc(&b->slv, sizeof(uint32_t) * (n + 1)));
    GBS_CUDA(cudaMalloc(&b->lr_n, sizeof(uint32_t) * std::max<size_t>(n_long, 1)));
    GBS_CUDA(cudaMalloc(&b->vw_u, sizeof(uint32_t) * std::max<size_t>(long_words, 1)));
    GBS_CUDA(cudaMalloc(&b->vw_w, sizeof(uint32_t) * std::max<size_t>(long_words, 1)));
    GBS_CUDA(cudaMalloc(&b->vw_rm, sizeof(uint32_t) * std::max<size_t>(long_words, 1)));
    GBS_CUDA(cudaMalloc(&b->vw_part, sizeof(double) * std::max<size_t>(long_words, 1)));
    GBS_CUDA(cudaMalloc(&b->mask, sizeof(uint32_t) * b->mask_words));
    GBS_CUDA(cudaMalloc(&b->ne_rows, sizeof(uint32_t) * std::max<size_t>(ne_rows.size(), 1)));
    GBS_CUDA(cudaMalloc(&b->wown, sizeof(uint2) * wown.size()));
    if (!ne_rows.empty())
        GBS_CUDA(cudaMemcpy(b->ne_rows, ne_rows.data(), sizeof(uint32_t) * ne_rows.size(), cudaMemcpyHostToDevice));
    GBS_CUDA(cudaMemcpy(b->wown, wown.data(), sizeof(uint2) * wown.size(), cudaMemcpyHostToDevice));
    GBS_CUDA(cudaMalloc(&b->bc, sizeof(double) * n));
    GBS_CUDA(cudaMalloc(&b->ctl, sizeof(BcCtl)));
    GBS_CUDA(cudaMalloc(&b->tot, sizeof(BcTotals)));
    // in-degrees return to zero at the end of every FORWARD pass
    GBS_CUDA(cudaMemsetAsync(b->indeg, 0, sizeof(uint32_t) * n, g->stream));
    int per_sm = 0;
    GBS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bc_kernel(g->wtype), kBcTPB, 0));
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
    cudaFree(b->wlv);
    cudaFree(b->lr_u);
    cudaFree(b->lr_b);
    cudaFree(b->slv);
    cudaFree(b->lr_n);
    cudaFree(b->vw_u);
    cudaFree(b->vw_w);
    cudaFree(b->vw_rm);
    cudaFree(b->vw_part);
    cudaFree(b->mask);
    cudaFree(b->ne_rows);
    cudaFree(b->wown);
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
    a.wlv = b->wlv;
    a.lr_u = b->lr_u;
    a.lr_b = b->lr_b;
    a.slv = b->slv;
    a.lr_n = b->lr_n;
    a.vw_u = b->vw_u;
    a.vw_w = b->vw_w;
    a.vw_rm = b->vw_rm;
    a.vw_part = b->vw_part;
    a.mask = b->mask;
    a.ne_rows = b->ne_rows;
    a.wown = b->wown;
    a.n_words = b->n_words;
    a.m = (uint32_t)g->m;
    a.bc = bc_dev;
    a.ctl = b->ctl;
    a.tot = b->tot;
    a.wait_ns = (unsigned long long)(p.wait_limit_ms ? p.wait_limit_ms : 4000u) * 1000000ull;
    a.nblocks = (uint32_t)b->blocks;
    const bool want_trace = params && (params->flags & GBS_F_TRACE);
    if (want_trace) {
        if (!g->ws.trace) {
            g->ws.trace_cap = 1u << 20;
            GBS_CUDA(cudaMalloc(&g->ws.trace, sizeof(TraceRec) * g->ws.trace_cap));
        }
        a.trace = g->ws.trace;
        a.trace_cap = g->ws.trace_cap;
    }
    const void *kfn = bc_kernel(g->wtype);
    gbs_bc_stats tot{};
    double dag_ms = 0.0;
    // one DAG launch on the distances now in the workspace's state words
    auto dag = [&](uint32_t src) -> gbs_status {
        a.source = src;
        void *args[] = {&a};
        GBS_CUDA(cudaEventRecord(e0, s));
        GBS_CUDA(cudaMemsetAsync(b->ctl, 0, sizeof(BcCtl), s));
        GBS_CUDA(cudaMemsetAsync(b->mask, 0, sizeof(uint32_t) * b->mask_words, s));
        GBS_CUDA(cudaLaunchCooperativeKernel(kfn, dim3(b->blocks), dim3(kBcTPB), args, 0, s));
        GBS_CUDA(cudaEventRecord(e1, s));
        GBS_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        GBS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        dag_ms += ms;
        return GBS_OK;
    };
    const bool batched = g->wtype != GBS_WEIGHT_F64 && k > 1 &&
                         !(p.flags & (GBS_F_BC_SINGLE | GBS_F_LEARNED));
    if (!batched) {
        for (uint32_t i = 0; i < k && st == GBS_OK; ++i) {
            const uint32_t src = sources ? sources[i] : i;
            gbs_stats one{};
            st = run_sssp(g, src, &p, nullptr, nullptr, &one);
            if (st != GBS_OK) break;
            tot.sssp_ms += one.device_ms;
            tot.edges_reached += one.edges_reached;
            st = dag(src);
        }
    } else {
        // up to kBcBatch sources per batched launch, distances kept on the
        // device; each source's DAG passes then run on its distances
        gbs_batch_params bp{};
        bp.delta = p.delta;
        bp.light = p.light;
        bp.flags = p.flags & (GBS_F_NO_SOLO | GBS_F_NO_FUSE);
        bp.wait_limit_ms = p.wait_limit_ms;
        bp.solo_entries = p.solo_entries;
        bp.solo_descs = p.solo_descs;
        bp.inline_edges = p.inline_edges;
        const uint32_t chunk = std::min(k, kBcBatch);
        uint32_t *bdist = nullptr;
        if (cudaMalloc(&bdist, sizeof(uint32_t) * (size_t)chunk * g->n) != cudaSuccess) {
            cudaGetLastError();
            st = fail(GBS_ERR_NO_MEMORY, "betweenness: no room for the batched distances");
        }
        std::vector<uint32_t> cs(chunk);
        for (uint32_t i0 = 0; i0 < k && st == GBS_OK; i0 += chunk) {
            const uint32_t cnt = std::min(chunk, k - i0);
            for (uint32_t j = 0; j < cnt; ++j) cs[j] = sources ? sources[i0 + j] : i0 + j;
            gbs_plan *plan = nullptr;
            st = gbs_plan_sources(g, cs.data(), cnt, &bp, bdist, nullptr, &plan);
            if (st != GBS_OK) break;
            gbs_batch_stats bs{};
            st = gbs_plan_launch(plan);
            if (st == GBS_OK) st = gbs_plan_wait(plan, &bs, nullptr);
            gbs_plan_destroy(plan);
            if (st != GBS_OK) break;
            tot.sssp_ms += bs.device_ms;
            tot.edges_reached += bs.edges_reached;
            const int tb = 256, eb = std::max(1, std::min<int>((g->n + tb - 1) / tb, g->sms * 8));
            for (uint32_t j = 0; j < cnt && st == GBS_OK; ++j) {
                if (g->wtype == GBS_WEIGHT_F32)
                    k_pack_dist<true><<<eb, tb, 0, s>>>(bdist + (size_t)j * g->n, g->n, g->ws.dp);
                else
                    k_pack_dist<false><<<eb, tb, 0, s>>>(bdist + (size_t)j * g->n, g->n, g->ws.dp);
                if (cudaGetLastError() != cudaSuccess) st = fail(GBS_ERR_CUDA, "betweenness: launch failed");
                else st = dag(cs[j]);
            }
        }
        cudaFree(bdist);
    }
    if (st != GBS_OK) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return st;
    }
    BcTotals t{};
    BcCtl last{};
    GBS_CUDA(cudaMemcpyAsync(&t, b->tot, sizeof(t), cudaMemcpyDeviceToHost, s));
    GBS_CUDA(cudaMemcpyAsync(&last, b->ctl, sizeof(last), cudaMemcpyDeviceToHost, s));
    GBS_CUDA(cudaStreamSynchronize(s));
    g->trace_n = want_trace && k ? std::min(last.trace_n, g->ws.trace_cap) : 0u;
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
