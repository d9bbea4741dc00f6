// gbs_sssp_kernel.cuh -- the persistent delta-stepping kernel (sm_103a).
//
// One cooperative launch runs a whole single-source shortest path: every CTA
// is resident, phases are separated by a grid barrier, and the CTA that
// arrives last at a barrier decides what the next phase is (it alone sees all
// counters at rest) and publishes the decision before releasing the others.
//
// Algorithm (delta-stepping, after sssp/csr_sspath_array.c:149-363):
//   bucket b holds vertices with bucket(dist) == b, bucket(d) = d / delta
//   (uint32) or floor(d * (1/delta)) (float32, the reference's multiply by
//   delta_recip, :408,425).  For the lowest non-empty bucket:
//     LIGHT   relax the light edges (w <= L, a row prefix) of the frontier; a
//             target that lands in the same bucket joins the next frontier
//             (request_arr + relax_arr, :246-274), every processed vertex
//             joins S (remember_arr, :263)
//     ...repeat LIGHT until the frontier is empty (:240)
//     HEAVY   relax the heavy edges of S once (:310-331); if that puts a
//             vertex back into the bucket, LIGHT runs again
//   Vertices pushed further than the ring window wait in a pending list that
//   is re-bucketed when the window reaches them.  Any relaxation order reaches
//   the same least fixpoint because fl(d + w) is monotone in d, so the
//   distances are bit-identical to Dijkstra's for every delta and split.
//
// Each LIGHT/HEAVY step is one or two grid phases:
//   SCAN   one thread per frontier entry: validate and read the row range.
//          Rows of at most inline_max edges are relaxed right away by the
//          scanning warp; longer rows become edge descriptors {u, dist(u),
//          first, end} of at most kDescEdges edges (the reference's request
//          list R, without one triple per edge).
//   EDGES  only if descriptors exist: one warp per descriptor.
// Relaxation is warp-collective, kUnroll x 32 edges per round (short rows of
// a SCAN are flattened by a warp prefix sum): every load and every atomic of
// a round is issued before any result is used, and the targets that improved
// are appended with one counter atomic per target list per round.
#pragma once

#include "gbs_internal.cuh"

namespace gbs {

enum Phase : uint32_t {
    kPhLightFirst = 0,    // SCAN of the ring list of a new bucket
    kPhLight = 1,         // SCAN of the next frontier of the same bucket
    kPhHeavy = 2,         // SCAN of S for heavy edges
    kPhEdges = 3,         // relax the descriptors of the preceding SCAN
    kPhPending = 4,       // re-bucket the pending list
    kPhDone = 5,
    // batched launches only
    kPhInit = 6,          // reset the state of a new instance
    kPhFinish = 7,        // write dist / pred, count reached vertices and edges
    kPhTake = 8,          // nothing to run: take the first instance
};

constexpr int kUnroll = 4;
constexpr uint32_t kDescEdges = 32u * kUnroll;   // edges per descriptor (one warp round)
constexpr uint32_t kInlineEdges = 32u;           // default inline_max: rows up to this long are relaxed in SCAN
constexpr uint32_t kFullItems = 1024u;           // least split threshold
// A bucket whose lists hold at most full_items entries when it starts relaxes
// whole rows: its heavy edges go through its light scans instead of a heavy
// phase of their own (a grid step fewer per bucket; a vertex scanned again
// in the bucket relaxes them again).  split_full_items is the threshold that
// keeps the light/heavy split for the large buckets, max(1024, n / 16); the
// single-source default is every bucket (n).  Measured with the plain width
// (kernel ms), before bucket fusion: R-MAT 20 1.40 at 1024 -> 1.21 at n / 16,
// R-MAT 22 2.56 -> 2.29; with fusion and 896 threads, n / 16 -> every bucket:
// R-MAT 20 1.059 -> 1.080, R-MAT 22 2.142 -> 2.002, R-MAT 24 7.57 -> 6.88,
// 4096^2 grid 209.6 -> 209.7.
inline uint32_t split_full_items(uint32_t n) { return n / 16u > kFullItems ? n / 16u : kFullItems; }

// Values identical in every CTA (the kernel's uniform state).
struct Uniform {
    uint32_t phase;       // phase being executed
    uint32_t logical;     // kPhLight or kPhHeavy: the SCAN an EDGES phase belongs to
    uint32_t b;           // current bucket
    uint32_t W;           // ring window base
    uint32_t epoch;       // frontier stamp of the current frontier
    uint32_t hround;      // heavy-round stamp (selects the S list)
    uint32_t pend_sel;
    uint32_t inst;        // batched: instance being solved
    uint32_t span;        // base widths the current bucket spans (1..kNB)
    uint32_t full;        // 1: light scans relax whole rows and no heavy scan runs
    uint32_t items;       // entries of the phase's input list (kNoItems: read the counters)
    uint32_t gen;         // barrier generation
    unsigned long long t0;  // globaltimer at kernel entry (per CTA)
};

// Arithmetic of a run: uint32 weights (exact sums, overflow reported),
// float32 (one rounding per relaxation) or float64 (one rounding in double,
// the reference's own arithmetic).  uint32 and float32 distances share one
// 64-bit word with the predecessor ((dist << 32) | pred); float64 distances
// fill the word (non-negative doubles order like their bit patterns) and the
// predecessor is found after the run.
enum : int { kWU32 = 0, kWF32 = 1, kWF64 = 2 };
template <int WT> struct Arith {
    using D = uint32_t;            // distance bits
    using Wt = uint32_t;           // weight bits
};
template <> struct Arith<kWF64> {
    using D = unsigned long long;
    using Wt = unsigned long long;
};

template <int WT>
__device__ __forceinline__ typename Arith<WT>::D dist_of(unsigned long long p) {
    if constexpr (WT == kWF64) return p;
    else return (uint32_t)(p >> 32);
}

template <int WT>
__device__ __forceinline__ unsigned long long pack_dist(typename Arith<WT>::D d, uint32_t u) {
    if constexpr (WT == kWF64) return d;
    else return ((unsigned long long)d << 32) | u;
}

// Weight of edge e whose {col, weight bits} word is ew.
template <int WT>
__device__ __forceinline__ typename Arith<WT>::Wt weight_at(const SsspArgs &a, uint32_t e, uint2 ew) {
    if constexpr (WT == kWF64) return __ldg(a.g.w64 + e);
    else return ew.y;
}

template <int WT>
__device__ __forceinline__ uint32_t bucket_of(typename Arith<WT>::D d, const SsspArgs &a) {
    if constexpr (WT == kWF64) {
        const double q = floor(__dmul_rn(__longlong_as_double((long long)d), a.inv_delta_d));
        return q >= 4294967040.0 ? kBucketMax : (uint32_t)q;
    } else if constexpr (WT == kWF32) {
        float q = floorf(__fmul_rn(__uint_as_float(d), a.inv_delta_f));
        return q >= 4294967040.0f ? kBucketMax : (uint32_t)q;
    } else {
        uint32_t q = d / a.delta_u;
        return q > kBucketMax ? kBucketMax : q;
    }
}

constexpr int kQueues = kNB + 2;   // next frontier, kNB ring lists, pending
constexpr int kFlush = 64;         // candidates per atomic round (two per lane)
constexpr int kCand = kFlush + 32; // candidate buffer: < kFlush kept + <= 32 per append

// Per-warp shared-memory scratch.
struct WarpScratch {
    uint32_t cnt[kQueues];         // enqueue histogram
    uint32_t cv[kCand];            // candidate target
    uint32_t cnd[kCand];           // candidate tentative distance bits (low word)
    uint32_t cu[kCand];            // candidate source; float64 runs: distance high word
                                   // (their predecessors are found after the run)
};

// Targets of one phase's appends.
struct Targets {
    uint32_t cur_hi;      // buckets < cur_hi belong to the current bucket
    uint32_t W;
    uint32_t stamp_next;
    uint32_t fq_next;     // index of the next-frontier list
    uint32_t pend_sel;    // pending list to append to
    WarpScratch *scr;     // this warp's shared-memory scratch
    Ctrs c;               // the list counters (global, or the deciding CTA's shared copy)
    uint32_t fuse;        // bucket fusion rounds of this phase (0: none)
};

// Bucket fusion.  During a scan that relaxes whole rows, a target that
// improves into the current bucket is kept by the lane whose atomicMin
// improved it (one slot per lane) and relaxed by that warp later in the same
// phase, instead of joining the next frontier and costing a phase of its
// own: chains of light hops inside a bucket (high-diameter graphs) run
// without a barrier per hop.  A kept target is relaxed with the distance its
// own improvement wrote, so each improvement is relaxed at least once
// (possibly twice, if the frontier holds the vertex as well) and the least
// fixpoint is the same; a lane whose slot is taken sends the target to the
// next frontier as before.
constexpr uint32_t kNoLocal = 0xFFFFFFFFu;   // empty slot
constexpr uint32_t kNoKeep = 0xFFFFFFFEu;    // closed slot: the warp's last fusion round
struct Local {
    uint32_t v;   // the kept vertex, or kNoLocal / kNoKeep
    uint32_t d;   // distance bits written by the improvement
};

// Queue ids: -1 none, 0 next frontier, 1..kNB ring slots, kNB+1 pending.
__device__ __forceinline__ uint32_t *queue_counter(const Targets &t, int q) {
    if (q == 0) return t.c.at(kCFq + t.fq_next);
    if (q <= kNB) return t.c.at(kCRing + (uint32_t)(q - 1));
    return t.c.at(kCPend + t.pend_sel);
}
__device__ __forceinline__ uint32_t *queue_list(const SsspArgs &a, const Targets &t, int q) {
    const size_t n = a.g.n;
    if (q == 0) return a.ws.fq + (size_t)t.fq_next * n;
    if (q <= kNB) return a.ws.ring + (size_t)(q - 1) * n;
    return a.ws.pend + (size_t)t.pend_sel * n;
}

// Appends every (q[j], v[j]) with q[j] >= 0 of the whole warp.  A
// shared-memory histogram over the kQueues target lists gives each item its
// rank; then lanes reserve space for all non-empty lists at once (one global
// atomic per list, all in flight together; lane l reserves lists l, l + 32
// and l + 64) and every item is written at the base its list's lane hands
// over by shuffle.
template <int U>
__device__ __forceinline__ void warp_enqueue(const SsspArgs &a, const Targets &t, const int (&q)[U],
                                             const uint32_t (&v)[U]) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    unsigned has = 0;
#pragma unroll
    for (int j = 0; j < U; ++j) has |= (q[j] >= 0 ? 1u : 0u) << j;
    if (__ballot_sync(FULL, has != 0) == 0) return;
    uint32_t *cnt = t.scr->cnt;
    for (int i = (int)lane; i < kQueues; i += 32) cnt[i] = 0;
    __syncwarp();
    uint32_t rank[U];
#pragma unroll
    for (int j = 0; j < U; ++j) rank[j] = ((has >> j) & 1u) ? atomicAdd(&cnt[q[j]], 1u) : 0u;
    __syncwarp();
    const int i0 = (int)lane, i1 = (int)lane + 32, i2 = (int)lane + 64;
    const uint32_t c0 = cnt[i0], c1 = cnt[i1], c2 = i2 < kQueues ? cnt[i2] : 0u;
    const uint32_t b0 = c0 ? atomicAdd(queue_counter(t, i0), c0) : 0u;
    const uint32_t b1 = c1 ? atomicAdd(queue_counter(t, i1), c1) : 0u;
    const uint32_t b2 = c2 ? atomicAdd(queue_counter(t, i2), c2) : 0u;
    const uint32_t n = a.g.n;
#pragma unroll
    for (int j = 0; j < U; ++j) {
        const bool mine = (has >> j) & 1u;
        const int src = mine ? (q[j] & 31) : 0;
        const uint32_t x0 = __shfl_sync(FULL, b0, src), x1 = __shfl_sync(FULL, b1, src);
        const uint32_t x2 = __shfl_sync(FULL, b2, src);
        if (mine) {
            const uint32_t pos = (q[j] < 32 ? x0 : q[j] < 64 ? x1 : x2) + rank[j];
            if (pos < n) queue_list(a, t, q[j])[pos] = v[j];
            else atomicExch(&a.ws.ctl->error, (uint32_t)kErrCapacity);
            // a pending entry may be re-bucketed by the very next phase, on
            // this CTA alone, which reads the list from L2 after nothing but
            // __syncthreads: the store must have reached L2 first
            if (q[j] == kNB + 1) __threadfence();
        }
    }
    __syncwarp();
}

// Appends v to one list for every lane with flag set (warp-aggregated).
__device__ __forceinline__ void warp_append(uint32_t *buf, uint32_t *cnt, uint32_t cap, bool flag,
                                            uint32_t v, Ctl *ctl) {
    const unsigned FULL = 0xffffffffu;
    const unsigned m = __ballot_sync(FULL, flag);
    if (!m) return;
    const unsigned lane = lane_id();
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(cnt, (uint32_t)__popc(m));
    base = __shfl_sync(FULL, base, leader);
    if (flag) {
        uint32_t pos = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
        if (pos < cap) buf[pos] = v;
        else atomicExch(&ctl->error, (uint32_t)kErrCapacity);
    }
}

// Tentative distance of an edge (u32: overflow check; f32 / f64: one rounding).
template <int WT>
__device__ __forceinline__ bool edge_sum(typename Arith<WT>::D du, typename Arith<WT>::Wt wbits,
                                         typename Arith<WT>::D &nd) {
    if constexpr (WT == kWF64) {
        nd = (unsigned long long)__double_as_longlong(
            __dadd_rn(__longlong_as_double((long long)du), __longlong_as_double((long long)wbits)));
        return true;
    } else if constexpr (WT == kWF32) {
        nd = __float_as_uint(__fadd_rn(__uint_as_float(du), __uint_as_float(wbits)));
        return true;
    } else {
        const unsigned long long s = (unsigned long long)du + wbits;
        nd = (uint32_t)s;
        return s < 0xFFFFFFFFull;
    }
}

// Relaxes U candidate edges (u[j] -> v[j], tentative distance nd[j],
// cand[j] = passed the read-only filter) and returns in q[j] the list each
// improved target joins.  Every step issues its U atomics before using any
// result, so they are in flight together:
//   1. packed (dist << 32 | pred) atomicMin: did the distance drop?
//   2. dedup: same bucket -> frontier stamp; window -> smallest queued
//      bucket (tag); beyond the window -> pending (tag = kTagPending)
template <int WT, int U>
__device__ __forceinline__ void improve_batch(const SsspArgs &a, const Targets &t, const bool (&cand)[U],
                                              const uint32_t (&v)[U], const uint32_t (&uo)[U],
                                              const typename Arith<WT>::D (&nd)[U], int (&q)[U], uint32_t &imp,
                                              Local &loc) {
    unsigned long long old[U];
#pragma unroll
    for (int j = 0; j < U; ++j) old[j] = cand[j] ? atomicMin(a.ws.dp + v[j], pack_dist<WT>(nd[j], uo[j])) : 0ull;
    uint32_t nb[U], kind[U], r[U];
#pragma unroll
    for (int j = 0; j < U; ++j) {
        const unsigned long long packed = pack_dist<WT>(nd[j], uo[j]);
        const bool dec = cand[j] && packed < old[j] && nd[j] < dist_of<WT>(old[j]);
        imp += dec ? 1u : 0u;
        nb[j] = dec ? bucket_of<WT>(nd[j], a) : 0u;
        kind[j] = !dec ? 0u
                : nb[j] < t.cur_hi ? 1u
                : (unsigned long long)nb[j] < (unsigned long long)t.W + kNB ? 2u : 3u;
    }
#pragma unroll
    for (int j = 0; j < U; ++j) {
        r[j] = 0;
        if (kind[j] == 1u) {
            atomicMin(a.ws.tag + v[j], nb[j]);
            bool kept = false;
            if constexpr (WT != kWF64) {
                if (t.fuse && loc.v == kNoLocal) {
                    loc.v = v[j];
                    loc.d = nd[j];
                    kept = true;
                }
            }
            if (kept) {
                kind[j] = 4u;   // relaxed by this warp later in the phase
                prefetch_l1(a.g.row + v[j]);
            } else {
                r[j] = atomicExch(a.ws.fst + v[j], t.stamp_next);
            }
        } else if (kind[j] == 2u) {
            r[j] = atomicMin(a.ws.tag + v[j], nb[j]);
        } else if (kind[j] == 3u) {
            atomicMin(t.c.at(kCPmin + t.pend_sel), nb[j]);
            r[j] = atomicMin(a.ws.tag + v[j], kTagPending);
            // the pending minimum and tag steer the next decision and the
            // next re-bucketing, which a phase run by one CTA reaches through
            // __syncthreads alone: it does not wait for a global reduction
            // whose result is unused (a shared-memory minimum it does order)
            __threadfence();
        }
    }
#pragma unroll
    for (int j = 0; j < U; ++j) {
        q[j] = -1;
        if (kind[j] == 1u && r[j] != t.stamp_next) {
            q[j] = 0;
            prefetch_l2(a.g.row + v[j]);   // the next frontier scan reads it
        }
        else if (kind[j] == 2u && r[j] > nb[j]) q[j] = 1 + (int)(nb[j] % kNB);
        else if (kind[j] == 3u && r[j] == kTagInit) q[j] = kNB + 1;
    }
}

// Runs the atomic part (improve_batch + enqueue) on the top `take`
// (<= 32 U) candidates of the warp's buffer, U per lane: one chain of
// dependent atomics (distance, tag, list) per U x 32 candidates.
template <int WT, int U>
__device__ __forceinline__ void cand_flush(const SsspArgs &a, const Targets &t, uint32_t &nc, uint32_t take,
                                           uint32_t &imp, Local &loc) {
    const unsigned lane = lane_id();
    WarpScratch *s = t.scr;
    uint32_t v1[U], u1[U];
    typename Arith<WT>::D n1[U];
    bool c1[U];
#pragma unroll
    for (int j = 0; j < U; ++j) {
        const uint32_t k = lane + 32u * (uint32_t)j;
        const bool has = k < take;
        const uint32_t i = nc - take + k;
        c1[j] = has;
        v1[j] = has ? s->cv[i] : 0u;
        u1[j] = has ? s->cu[i] : 0u;
        if constexpr (WT == kWF64) {
            n1[j] = has ? (((unsigned long long)s->cu[i] << 32) | s->cnd[i]) : 0ull;
            u1[j] = 0u;
        } else {
            n1[j] = has ? s->cnd[i] : 0u;
        }
    }
    __syncwarp();
    nc -= take;
    int q[U];
    improve_batch<WT, U>(a, t, c1, v1, u1, n1, q, imp, loc);
    warp_enqueue<U>(a, t, q, v1);
}

// Warp-collective tail of one relaxation round: U edges per lane whose
// targets and weights are loaded (val[j] = the lane has an edge in slot j).
// Only edges that pass the read-only filter (packed tentative value below
// the current dp) become candidates; they collect in the warp's shared-memory
// buffer and the atomic chain runs once per kFlush of them, not once per round.
template <int WT, int U>
__device__ __forceinline__ void relax_candidates(const SsspArgs &a, const Targets &t, const bool (&val)[U],
                                                 const uint32_t (&v)[U], const typename Arith<WT>::Wt (&w)[U],
                                                 const uint32_t (&uo)[U], const typename Arith<WT>::D (&duo)[U],
                                                 uint32_t &nc, uint32_t &imp, Local &loc) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    unsigned long long cur[U];
#pragma unroll
    for (int j = 0; j < U; ++j) cur[j] = val[j] ? __ldcg(a.ws.dp + v[j]) : 0ull;
    WarpScratch *s = t.scr;
#pragma unroll
    for (int j = 0; j < U; ++j) {
        bool cand = false;
        typename Arith<WT>::D nd = 0;
        if (val[j]) {
            if (!edge_sum<WT>(duo[j], w[j], nd)) atomicExch(&a.ws.ctl->error, (uint32_t)kErrOverflow);
            else cand = pack_dist<WT>(nd, uo[j]) < cur[j];
        }
        const unsigned m = __ballot_sync(FULL, cand);
        if (m) {
            if (cand) {
                const uint32_t p = nc + (uint32_t)__popc(m & ((1u << lane) - 1u));
                s->cv[p] = v[j];
                s->cnd[p] = (uint32_t)nd;
                if constexpr (WT == kWF64) s->cu[p] = (uint32_t)(nd >> 32);
                else s->cu[p] = uo[j];
            }
            nc += (uint32_t)__popc(m);
            __syncwarp();
            if (nc >= (uint32_t)kFlush) cand_flush<WT, kFlush / 32>(a, t, nc, kFlush, imp, loc);
        }
    }
}

// Drains the warp's candidate buffer (end of a phase's relaxation work).
template <int WT>
__device__ __forceinline__ void cand_drain(const SsspArgs &a, const Targets &t, uint32_t &nc, uint32_t &imp,
                                           Local &loc) {
    if (nc > 32u) cand_flush<WT, kFlush / 32>(a, t, nc, nc, imp, loc);
    else if (nc) cand_flush<WT, 1>(a, t, nc, nc, imp, loc);
}

// Warp-collective: relaxes edges [s, s+len) of source u (distance bits du)
// given by every lane (len may be 0), kUnroll x 32 edges per round.
template <int WT>
__device__ __forceinline__ void relax_group(const SsspArgs &a, const Targets &t, uint32_t u,
                                            typename Arith<WT>::D du, uint32_t s, uint32_t len, uint32_t &nc,
                                            uint32_t &imp, Local &loc) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    uint32_t incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, o);
        if ((int)lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    const uint32_t excl = incl - len;
    for (uint32_t k0 = 0; k0 < total; k0 += 32u * kUnroll) {
        uint32_t v[kUnroll], uo[kUnroll];
        typename Arith<WT>::Wt w[kUnroll];
        typename Arith<WT>::D duo[kUnroll];
        bool val[kUnroll];
#pragma unroll
        for (int j = 0; j < kUnroll; ++j) {
            const uint32_t k = k0 + 32u * j + lane;
            int owner = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const int cand = owner + step;
                const uint32_t ex = __shfl_sync(FULL, excl, cand);
                if (ex <= k) owner = cand;
            }
            const uint32_t so = __shfl_sync(FULL, s, owner);
            const uint32_t exo = __shfl_sync(FULL, excl, owner);
            uo[j] = __shfl_sync(FULL, u, owner);
            duo[j] = __shfl_sync(FULL, du, owner);
            val[j] = k < total;
            v[j] = 0;
            w[j] = 0;
            if (val[j]) {
                const uint32_t e = so + (k - exo);
                const uint2 ew = ld_stream(a.g.adj + e);
                v[j] = ew.x;
                w[j] = weight_at<WT>(a, e, ew);
            }
        }
        relax_candidates<WT>(a, t, val, v, w, uo, duo, nc, imp, loc);
    }
}


}  // namespace gbs
