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
//          Rows of at most kInlineEdges edges are relaxed right away by the
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
};

constexpr int kUnroll = 4;
constexpr uint32_t kDescEdges = 32u * kUnroll;   // edges per descriptor (one warp round)
constexpr uint32_t kInlineEdges = 32u;           // rows up to this long are relaxed in SCAN

// Values identical in every CTA (the kernel's uniform state).
struct Uniform {
    uint32_t phase;       // phase being executed
    uint32_t logical;     // kPhLight or kPhHeavy: the SCAN an EDGES phase belongs to
    uint32_t b;           // current bucket
    uint32_t W;           // ring window base
    uint32_t epoch;       // frontier stamp of the current frontier
    uint32_t hround;      // heavy-round stamp (selects the S list)
    uint32_t pend_sel;
    uint32_t gen;         // barrier generation
    unsigned long long t0;  // globaltimer at kernel entry (per CTA)
};

template <bool F32>
__device__ __forceinline__ uint32_t bucket_of(uint32_t dbits, const SsspArgs &a) {
    if (F32) {
        float q = floorf(__fmul_rn(__uint_as_float(dbits), a.inv_delta_f));
        return q >= 4294967040.0f ? kBucketMax : (uint32_t)q;
    } else {
        uint32_t q = dbits / a.delta_u;
        return q > kBucketMax ? kBucketMax : q;
    }
}

constexpr int kQueues = kNB + 2;   // next frontier, kNB ring lists, pending
constexpr int kCand = 64;          // candidate buffer: < 32 kept + <= 32 per append

// Per-warp shared-memory scratch.
struct WarpScratch {
    uint32_t bins[2 * kQueues];    // enqueue histogram and list bases
    uint32_t cv[kCand];            // candidate target
    uint32_t cnd[kCand];           // candidate tentative distance bits
    uint32_t cu[kCand];            // candidate source
};

// Targets of one phase's appends.
struct Targets {
    uint32_t cur_hi;      // buckets < cur_hi belong to the current bucket
    uint32_t W;
    uint32_t stamp_next;
    uint32_t fq_next;     // index of the next-frontier list
    uint32_t pend_sel;    // pending list to append to
    WarpScratch *scr;     // this warp's shared-memory scratch
};

// Queue ids: -1 none, 0 next frontier, 1..kNB ring slots, kNB+1 pending.
__device__ __forceinline__ uint32_t *queue_counter(const SsspArgs &a, const Targets &t, int q) {
    Ctl *ctl = a.ws.ctl;
    if (q == 0) return &ctl->fq_cnt[t.fq_next].v;
    if (q <= kNB) return &ctl->ring_cnt[q - 1].v;
    return &ctl->pend_cnt[t.pend_sel].v;
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
// atomic per list, all in flight together) and every item is written.
template <int U>
__device__ __forceinline__ void warp_enqueue(const SsspArgs &a, const Targets &t, const int (&q)[U],
                                             const uint32_t (&v)[U]) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    unsigned has = 0;
#pragma unroll
    for (int j = 0; j < U; ++j) has |= (q[j] >= 0 ? 1u : 0u) << j;
    if (__ballot_sync(FULL, has != 0) == 0) return;
    uint32_t *cnt = t.scr->bins, *base = t.scr->bins + kQueues;
    for (int i = (int)lane; i < kQueues; i += 32) cnt[i] = 0;
    __syncwarp();
    uint32_t rank[U];
#pragma unroll
    for (int j = 0; j < U; ++j) rank[j] = ((has >> j) & 1u) ? atomicAdd(&cnt[q[j]], 1u) : 0u;
    __syncwarp();
    const int i0 = (int)lane, i1 = (int)lane + 32, i2 = (int)lane + 64;
    const uint32_t c0 = cnt[i0], c1 = cnt[i1], c2 = i2 < kQueues ? cnt[i2] : 0u;
    const uint32_t b0 = c0 ? atomicAdd(queue_counter(a, t, i0), c0) : 0u;
    const uint32_t b1 = c1 ? atomicAdd(queue_counter(a, t, i1), c1) : 0u;
    const uint32_t b2 = c2 ? atomicAdd(queue_counter(a, t, i2), c2) : 0u;
    if (c0) base[i0] = b0;
    if (c1) base[i1] = b1;
    if (c2) base[i2] = b2;
    __syncwarp();
    const uint32_t n = a.g.n;
#pragma unroll
    for (int j = 0; j < U; ++j) {
        if ((has >> j) & 1u) {
            const uint32_t pos = base[q[j]] + rank[j];
            if (pos < n) queue_list(a, t, q[j])[pos] = v[j];
            else atomicExch(&a.ws.ctl->error, (uint32_t)kErrCapacity);
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

// Tentative distance of an edge (u32: overflow check; f32: one rounding).
template <bool F32>
__device__ __forceinline__ bool edge_sum(uint32_t du, uint32_t wbits, uint32_t &nd) {
    if (F32) {
        nd = __float_as_uint(__fadd_rn(__uint_as_float(du), __uint_as_float(wbits)));
        return true;
    }
    const unsigned long long s = (unsigned long long)du + wbits;
    nd = (uint32_t)s;
    return s < 0xFFFFFFFFull;
}

// Relaxes U candidate edges (u[j] -> v[j], tentative distance nd[j],
// cand[j] = passed the read-only filter) and returns in q[j] the list each
// improved target joins.  Every step issues its U atomics before using any
// result, so they are in flight together:
//   1. packed (dist << 32 | pred) atomicMin: did the distance drop?
//   2. dedup: same bucket -> frontier stamp; window -> smallest queued
//      bucket (tag); beyond the window -> pending (tag = kTagPending)
template <bool F32, int U>
__device__ __forceinline__ void improve_batch(const SsspArgs &a, const Targets &t, const bool (&cand)[U],
                                              const uint32_t (&v)[U], const uint32_t (&uo)[U],
                                              const uint32_t (&nd)[U], int (&q)[U], uint32_t &imp) {
    unsigned long long old[U];
#pragma unroll
    for (int j = 0; j < U; ++j)
        old[j] = cand[j] ? atomicMin(a.ws.dp + v[j], ((unsigned long long)nd[j] << 32) | uo[j]) : 0ull;
    uint32_t nb[U], kind[U], r[U];
#pragma unroll
    for (int j = 0; j < U; ++j) {
        const unsigned long long packed = ((unsigned long long)nd[j] << 32) | uo[j];
        const bool dec = cand[j] && packed < old[j] && nd[j] < (uint32_t)(old[j] >> 32);
        imp += dec ? 1u : 0u;
        nb[j] = dec ? bucket_of<F32>(nd[j], a) : 0u;
        kind[j] = !dec ? 0u
                : nb[j] < t.cur_hi ? 1u
                : (unsigned long long)nb[j] < (unsigned long long)t.W + kNB ? 2u : 3u;
    }
#pragma unroll
    for (int j = 0; j < U; ++j) {
        r[j] = 0;
        if (kind[j] == 1u) {
            atomicMin(a.ws.tag + v[j], nb[j]);
            r[j] = atomicExch(a.ws.fst + v[j], t.stamp_next);
        } else if (kind[j] == 2u) {
            r[j] = atomicMin(a.ws.tag + v[j], nb[j]);
        } else if (kind[j] == 3u) {
            atomicMin(&a.ws.ctl->pend_min[t.pend_sel].v, nb[j]);
            r[j] = atomicMin(a.ws.tag + v[j], kTagPending);
        }
    }
#pragma unroll
    for (int j = 0; j < U; ++j) {
        q[j] = -1;
        if (kind[j] == 1u && r[j] != t.stamp_next) q[j] = 0;
        else if (kind[j] == 2u && r[j] > nb[j]) q[j] = 1 + (int)(nb[j] % kNB);
        else if (kind[j] == 3u && r[j] == kTagInit) q[j] = kNB + 1;
    }
}

// Warp-collective tail of one relaxation round: U edges per lane whose
// targets and weights are loaded (val[j] = the lane has an edge in slot j).
// Runs the atomic part (improve_batch + enqueue) on the top `take` (<= 32)
// candidates of the warp's buffer, one per lane.
template <bool F32>
__device__ __forceinline__ void cand_flush(const SsspArgs &a, const Targets &t, uint32_t &nc, uint32_t take,
                                           uint32_t &imp) {
    const unsigned lane = lane_id();
    WarpScratch *s = t.scr;
    const bool has = lane < take;
    const uint32_t i = nc - take + lane;
    uint32_t v1[1] = {has ? s->cv[i] : 0u};
    uint32_t u1[1] = {has ? s->cu[i] : 0u};
    uint32_t n1[1] = {has ? s->cnd[i] : 0u};
    const bool c1[1] = {has};
    __syncwarp();
    nc -= take;
    int q[1];
    improve_batch<F32, 1>(a, t, c1, v1, u1, n1, q, imp);
    warp_enqueue<1>(a, t, q, v1);
}

// Warp-collective tail of one relaxation round: U edges per lane whose
// targets and weights are loaded (val[j] = the lane has an edge in slot j).
// Only edges that pass the read-only filter (packed tentative value below
// the current dp) become candidates; they collect in the warp's shared-memory
// buffer and the atomic chain runs once per 32 of them, not once per round.
template <bool F32, int U>
__device__ __forceinline__ void relax_candidates(const SsspArgs &a, const Targets &t, const bool (&val)[U],
                                                 const uint32_t (&v)[U], const uint32_t (&w)[U],
                                                 const uint32_t (&uo)[U], const uint32_t (&duo)[U],
                                                 uint32_t &nc, uint32_t &imp) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    unsigned long long cur[U];
#pragma unroll
    for (int j = 0; j < U; ++j) cur[j] = val[j] ? __ldcg(a.ws.dp + v[j]) : 0ull;
    WarpScratch *s = t.scr;
#pragma unroll
    for (int j = 0; j < U; ++j) {
        bool cand = false;
        uint32_t nd = 0;
        if (val[j]) {
            if (!edge_sum<F32>(duo[j], w[j], nd)) atomicExch(&a.ws.ctl->error, (uint32_t)kErrOverflow);
            else cand = (((unsigned long long)nd << 32) | uo[j]) < cur[j];
        }
        const unsigned m = __ballot_sync(FULL, cand);
        if (m) {
            if (cand) {
                const uint32_t p = nc + (uint32_t)__popc(m & ((1u << lane) - 1u));
                s->cv[p] = v[j];
                s->cnd[p] = nd;
                s->cu[p] = uo[j];
            }
            nc += (uint32_t)__popc(m);
            __syncwarp();
            if (nc >= 32u) cand_flush<F32>(a, t, nc, 32u, imp);
        }
    }
}

// Drains the warp's candidate buffer (end of a phase's relaxation work).
template <bool F32>
__device__ __forceinline__ void cand_drain(const SsspArgs &a, const Targets &t, uint32_t &nc, uint32_t &imp) {
    if (nc) cand_flush<F32>(a, t, nc, nc, imp);
}

// Warp-collective: relaxes edges [s, s+len) of source u (distance bits du)
// given by every lane (len may be 0), kUnroll x 32 edges per round.
template <bool F32>
__device__ __forceinline__ void relax_group(const SsspArgs &a, const Targets &t, uint32_t u, uint32_t du,
                                            uint32_t s, uint32_t len, uint32_t &nc, uint32_t &imp) {
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
        uint32_t v[kUnroll], w[kUnroll], uo[kUnroll], duo[kUnroll];
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
                const uint2 ew = ld_stream(a.g.adj + so + (k - exo));
                v[j] = ew.x;
                w[j] = ew.y;
            }
        }
        relax_candidates<F32>(a, t, val, v, w, uo, duo, nc, imp);
    }
}

// ------------------------------------------------------------------- SCAN
// One thread per frontier entry.  vtag != kTagInit keeps only entries whose
// tag equals it (ring lists may hold entries that moved to a lower bucket).
template <bool F32>
__device__ void scan_frontier(const SsspArgs &a, const Targets &t, const uint32_t *F, uint32_t count,
                              uint32_t vtag, bool light, bool add_s, uint32_t hround, uint32_t &imp) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    const uint32_t n = a.g.n;
    Ctl *ctl = a.ws.ctl;
    uint32_t my_edges = 0;
    uint32_t nc = 0;   // candidates buffered by this warp
    for (uint32_t base = tid - lane; base < count; base += nthreads) {
        const uint32_t i = base + lane;
        uint32_t u = 0, du = 0, s = 0, e = 0;
        bool ok = false;
        if (i < count) {
            u = __ldcg(F + i);
            // the tag check and the row reads are independent: issue together
            const uint32_t tg = (vtag == kTagInit) ? vtag : __ldcg(a.ws.tag + u);
            du = (uint32_t)(__ldcg(a.ws.dp + u) >> 32);
            const uint32_t md = __ldg(a.ws.mid + u);
            const uint32_t r = light ? __ldg(a.g.row + u) : __ldg(a.g.row + u + 1);
            ok = tg == vtag;
            s = ok ? (light ? r : md) : 0u;
            e = ok ? (light ? md : r) : 0u;
        }
        // S membership is decided now; the append waits until after the
        // relaxation below so its latency overlaps that work
        uint32_t hold = hround;
        if (ok && add_s) hold = atomicExch(a.ws.hst + u, hround);
        const uint32_t len = e - s;
        // long rows -> descriptors, reserved with one atomic per warp
        const uint32_t nd = len > kInlineEdges ? (len + kDescEdges - 1) / kDescEdges : 0u;
        uint32_t incl = nd;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if ((int)lane >= o) incl += y;
        }
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        if (total) {
            uint32_t dbase = 0;
            if (lane == 31) dbase = atomicAdd(&ctl->desc_cnt.v, total);
            dbase = __shfl_sync(FULL, dbase, 31);
            const uint32_t pos = dbase + incl - nd;
            if (pos + nd <= a.ws.desc_cap) {
                for (uint32_t c = 0; c < nd; ++c) {
                    const uint32_t cs = s + c * kDescEdges;
                    a.ws.desc[pos + c] = make_uint4(u, du, cs, min(e, cs + kDescEdges));
                }
            } else if (nd) {
                atomicExch(&ctl->error, (uint32_t)kErrCapacity);
            }
            my_edges += nd ? len : 0u;
        }
        // short rows: relaxed by this warp now
        relax_group<F32>(a, t, u, du, s, nd ? 0u : len, nc, imp);
        warp_append(a.ws.S + (size_t)(hround & 1u) * n, &ctl->s_cnt[hround & 1u].v, n,
                    ok && add_s && hold != hround, u, ctl);
    }
    cand_drain<F32>(a, t, nc, imp);
    // edges handed to EDGES (statistics / trace)
    for (int o = 16; o > 0; o >>= 1) my_edges += __shfl_down_sync(FULL, my_edges, o);
    if (lane == 0 && my_edges) atomicAdd(&ctl->edge_cnt.v, my_edges);
}

// ------------------------------------------------------------------ EDGES
// One warp per descriptor (<= kDescEdges edges of one row = one round).
template <bool F32>
__device__ void relax_descriptors(const SsspArgs &a, const Targets &t, uint32_t count, uint32_t &imp) {
    const unsigned lane = lane_id();
    const uint32_t warp_g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    uint32_t nc = 0;   // candidates buffered by this warp
    for (uint32_t c = warp_g; c < count; c += nwarps) {
        const uint4 d = __ldcg(a.ws.desc + c);
        uint32_t v[kUnroll], w[kUnroll], uo[kUnroll], duo[kUnroll];
        bool val[kUnroll];
#pragma unroll
        for (int j = 0; j < kUnroll; ++j) {
            const uint32_t e = d.z + 32u * j + lane;
            val[j] = e < d.w;
            uo[j] = d.x;
            duo[j] = d.y;
            v[j] = 0;
            w[j] = 0;
            if (val[j]) {
                const uint2 ew = ld_stream(a.g.adj + e);
                v[j] = ew.x;
                w[j] = ew.y;
            }
        }
        relax_candidates<F32>(a, t, val, v, w, uo, duo, nc, imp);
    }
    cand_drain<F32>(a, t, nc, imp);
}

// Moves pending vertices whose bucket entered the window [W, W+kNB) into the
// ring; the rest go to the other pending list.
template <bool F32>
__device__ void rebucket_pending(const SsspArgs &a, const Uniform &U, WarpScratch *scr) {
    const uint32_t n = a.g.n;
    Ctl *ctl = a.ws.ctl;
    const uint32_t count = min(__ldcg(&ctl->pend_cnt[U.pend_sel].v), n);
    const uint32_t *list = a.ws.pend + (size_t)U.pend_sel * n;
    Targets t;
    t.cur_hi = 0;
    t.W = U.W;
    t.stamp_next = 0;
    t.fq_next = 0;
    t.pend_sel = U.pend_sel ^ 1u;
    t.scr = scr;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    for (uint32_t base = tid - lane_id(); base < count; base += nthreads) {
        const uint32_t i = base + lane_id();
        int q[1] = {-1};
        uint32_t v[1] = {0};
        if (i < count) {
            v[0] = __ldcg(list + i);
            if (__ldcg(a.ws.tag + v[0]) == kTagPending) {
                const uint32_t nb = bucket_of<F32>((uint32_t)(__ldcg(a.ws.dp + v[0]) >> 32), a);
                if ((unsigned long long)nb < (unsigned long long)U.W + kNB) {
                    a.ws.tag[v[0]] = nb;
                    q[0] = 1 + (int)(nb % kNB);
                } else {
                    atomicMin(&ctl->pend_min[t.pend_sel].v, nb);
                    q[0] = kNB + 1;
                }
            }
        }
        warp_enqueue<1>(a, t, q, v);
    }
}

__device__ __forceinline__ uint32_t scan_kind(uint32_t phase) {
    return phase == kPhHeavy ? (uint32_t)kPhHeavy : (uint32_t)kPhLight;
}

// Run by warp 0 of the CTA that arrives last at a barrier: every other CTA
// has finished the phase, so all counters are at rest.  Decides the next
// phase, resets the lists that phase will append to, and publishes.
__device__ inline void control_step(const SsspArgs &a, const Uniform &U) {
    Ctl *ctl = a.ws.ctl;
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    // one round trip: every counter the decision needs is loaded at once
    const uint32_t ring_lo = ld_relaxed(&ctl->ring_cnt[lane].v);
    const uint32_t ring_hi = ld_relaxed(&ctl->ring_cnt[lane + 32].v);
    const uint32_t desc_cnt = ld_relaxed(&ctl->desc_cnt.v);
    const uint32_t fq_next = ld_relaxed(&ctl->fq_cnt[(U.epoch + 1u) % 3u].v);
    const uint32_t pc0 = ld_relaxed(&ctl->pend_cnt[0].v), pc1 = ld_relaxed(&ctl->pend_cnt[1].v);
    const uint32_t pm0 = ld_relaxed(&ctl->pend_min[0].v), pm1 = ld_relaxed(&ctl->pend_min[1].v);
    const uint32_t err = ld_relaxed(&ctl->error);

    uint32_t next = kPhDone, nb = 0;
    uint32_t e2 = U.epoch, h2 = U.hround, ps2 = U.pend_sel;
    bool need_ring_scan = false;
    uint32_t scan_from = 0;
    if (U.phase == kPhPending) {
        ps2 ^= 1u;
        need_ring_scan = true;
        scan_from = U.W;
        if (lane == 0) { ctl->pend_cnt[U.pend_sel].v = 0; ctl->pend_min[U.pend_sel].v = kTagInit; }
    } else if (U.phase != kPhEdges && desc_cnt > 0) {
        next = kPhEdges;
    } else {
        const uint32_t logical = (U.phase == kPhEdges) ? U.logical : scan_kind(U.phase);
        e2 = U.epoch + 1;
        if (logical == kPhHeavy) h2 = U.hround + 1;
        if (fq_next > 0) {
            next = kPhLight;
        } else if (logical == kPhLight) {
            next = kPhHeavy;
        } else {
            if (lane == 0) ctl->ring_cnt[U.b % kNB].v = 0;
            need_ring_scan = true;
            scan_from = U.b + 1;
        }
    }
    if (need_ring_scan) {
        // first non-empty ring bucket in [scan_from, W + kNB); at a bucket end
        // scan_from = b + 1 = W + 1, so the slot just cleared is not read.
        const uint32_t lim = U.W + kNB;   // exclusive
        uint32_t found = 0xFFFFFFFFu;
#pragma unroll
        for (uint32_t off = 0; off < (uint32_t)kNB; off += 32u) {
            const uint32_t bk = scan_from + off + lane;
            const uint32_t slot = bk % kNB;
            const uint32_t c_lo = __shfl_sync(FULL, ring_lo, slot & 31u);
            const uint32_t c_hi = __shfl_sync(FULL, ring_hi, slot & 31u);
            const uint32_t c = slot < 32 ? c_lo : c_hi;
            const unsigned m = __ballot_sync(FULL, bk < lim && c > 0);
            if (m && found == 0xFFFFFFFFu) found = scan_from + off + (uint32_t)(__ffs(m) - 1);
        }
        const uint32_t pcnt = ps2 ? pc1 : pc0;
        const uint32_t pm = ps2 ? pm1 : pm0;
        if (pcnt > 0 && pm <= found) {
            next = kPhPending;
            nb = pm;
        } else if (found != 0xFFFFFFFFu) {
            next = kPhLightFirst;
            nb = found;
        } else {
            next = kPhDone;
        }
    }
    // whole-run limit: a run that has not finished within run_ns is stopped
    if (globaltimer() - U.t0 > a.run_ns) {
        next = kPhDone;
        if (lane == 0) atomicCAS(&ctl->error, 0u, (uint32_t)kErrTimeout);
    }
    if (err) next = kPhDone;
    if (lane == 0) {
        if ((a.flags & GBS_F_TRACE) && a.ws.trace) {
            const uint32_t ti = ctl->trace_n;
            if (ti < a.ws.trace_cap) {
                uint32_t items;
                switch (U.phase) {
                    case kPhLightFirst: items = ld_relaxed(&ctl->ring_cnt[U.b % kNB].v); break;
                    case kPhLight: items = ld_relaxed(&ctl->fq_cnt[U.epoch % 3u].v); break;
                    case kPhHeavy: items = ld_relaxed(&ctl->s_cnt[U.hround & 1u].v); break;
                    case kPhEdges: items = desc_cnt; break;
                    default: items = ld_relaxed(&ctl->pend_cnt[U.pend_sel].v); break;
                }
                TraceRec r;
                r.kind = U.phase;
                r.bucket = U.b;
                r.items = items;
                r.edges = ld_relaxed(&ctl->edge_cnt.v);
                r.end_ns = globaltimer() - U.t0;
                a.ws.trace[ti] = r;
            }
            ctl->trace_n = ti + 1;
        }
        if (next == kPhLight || next == kPhHeavy || next == kPhLightFirst) {
            ctl->fq_cnt[(e2 + 1u) % 3u].v = 0;
            ctl->desc_cnt.v = 0;
            ctl->edge_cnt.v = 0;
            if (h2 != U.hround || next == kPhLightFirst) ctl->s_cnt[h2 & 1u].v = 0;
        }
        ctl->mode = next;
        ctl->next_bucket = nb;
    }
    __syncwarp();
}

// Applies the published decision to the uniform state (identical in all CTAs).
__device__ __forceinline__ void advance_uniform(Uniform &U, uint32_t next, uint32_t nb) {
    if (U.phase == kPhPending) {
        U.pend_sel ^= 1u;
    } else if (next == kPhEdges) {
        U.logical = scan_kind(U.phase);
    } else {
        const uint32_t logical = (U.phase == kPhEdges) ? U.logical : scan_kind(U.phase);
        U.epoch += 1;
        if (logical == kPhHeavy) U.hround += 1;
    }
    if (next == kPhLightFirst) { U.b = nb; U.W = nb; }
    if (next == kPhPending) U.W = nb;
    U.phase = next;
}

// Grid barrier; the last CTA to arrive runs control_step before releasing.
// Waits are bounded by a.wait_ns (globaltimer); on expiry the error flag is
// set and every CTA leaves at its next check.
__device__ __forceinline__ void grid_barrier(const SsspArgs &a, Uniform &U) {
    Ctl *ctl = a.ws.ctl;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t last = 0;
        // GBS_F_TEST_STALL: CTA 0 skips its first arrival (failure-path test)
        const bool stall = (a.flags & GBS_F_TEST_STALL) && U.gen == 0 && blockIdx.x == 0;
        if (threadIdx.x == 0 && !stall) {
            __threadfence();
            const uint32_t arrived = atomicAdd(&ctl->bar_count, 1u);
            last = (arrived == gridDim.x - 1u);
        }
        last = __shfl_sync(0xffffffffu, last, 0);
        if (last) {
            __threadfence();
            control_step(a, U);
            if (threadIdx.x == 0) {
                ctl->bar_count = 0;
                __threadfence();
                st_release(&ctl->bar_gen, U.gen + 1u);
            }
        } else if (threadIdx.x == 0) {
            const unsigned long long t0 = globaltimer();
            uint32_t spins = 0;
            while (ld_acquire(&ctl->bar_gen) != U.gen + 1u) {
                if ((++spins & 255u) == 0) {
                    if (ld_relaxed(&ctl->error) != 0) break;
                    if (globaltimer() - t0 > a.wait_ns) {
                        atomicCAS(&ctl->error, 0u, (uint32_t)kErrTimeout);
                        break;
                    }
                }
            }
        }
        __syncwarp();
        if (threadIdx.x == 0) __threadfence();
    }
    __syncthreads();
    U.gen += 1;
}

template <bool F32>
__global__ void __launch_bounds__(kTPB, 1) sssp_persistent(SsspArgs a) {
    Ctl *ctl = a.ws.ctl;
    Uniform U;
    U.phase = ld_relaxed(&ctl->mode);
    U.logical = kPhLight;
    U.b = ld_relaxed(&ctl->next_bucket);
    U.W = U.b;
    U.epoch = a.epoch0;
    U.hround = a.hround0;
    U.pend_sel = 0;
    U.gen = 0;
    U.t0 = globaltimer();
    uint32_t imp = 0, nphases = 0, nbuckets = 0, nscans = 0;
    const uint32_t ncap = a.g.n;   // every vertex list holds at most n entries
    __shared__ uint32_t s_next[2];
    __shared__ WarpScratch s_scr[kTPB / 32];
    WarpScratch *scr = &s_scr[threadIdx.x >> 5];

    while (U.phase != kPhDone) {
        Targets t;
        t.cur_hi = U.b + 1;
        t.W = U.W;
        t.stamp_next = U.epoch + 1;
        t.fq_next = (U.epoch + 1) % 3u;
        t.pend_sel = U.pend_sel;
        t.scr = scr;
        const uint32_t n = a.g.n;
        switch (U.phase) {
            case kPhLightFirst:
                ++nbuckets;
                scan_frontier<F32>(a, t, a.ws.ring + (size_t)(U.b % kNB) * n,
                                   min(__ldcg(&ctl->ring_cnt[U.b % kNB].v), ncap), U.b, true, true,
                                   U.hround, imp);
                break;
            case kPhLight:
                scan_frontier<F32>(a, t, a.ws.fq + (size_t)(U.epoch % 3u) * n,
                                   min(__ldcg(&ctl->fq_cnt[U.epoch % 3u].v), ncap), kTagInit, true, true,
                                   U.hround, imp);
                break;
            case kPhHeavy:
                scan_frontier<F32>(a, t, a.ws.S + (size_t)(U.hround & 1u) * n,
                                   min(__ldcg(&ctl->s_cnt[U.hround & 1u].v), ncap), kTagInit, false, false,
                                   U.hround, imp);
                break;
            case kPhEdges:
                relax_descriptors<F32>(a, t, min(__ldcg(&ctl->desc_cnt.v), a.ws.desc_cap), imp);
                break;
            case kPhPending:
                ++nscans;
                rebucket_pending<F32>(a, U, scr);
                break;
            default:
                break;
        }
        grid_barrier(a, U);
        ++nphases;
        if (threadIdx.x == 0) {
            s_next[0] = ld_relaxed(&ctl->error) ? (uint32_t)kPhDone : ld_relaxed(&ctl->mode);
            s_next[1] = ld_relaxed(&ctl->next_bucket);
        }
        __syncthreads();
        const uint32_t next = s_next[0], nb = s_next[1];
        __syncthreads();
        advance_uniform(U, next, nb);
    }
    // statistics
    for (int o = 16; o > 0; o >>= 1) imp += __shfl_down_sync(0xffffffffu, imp, o);
    if (lane_id() == 0 && imp) atomicAdd(&ctl->st_improvements, (unsigned long long)imp);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->st_buckets = nbuckets;
        ctl->st_phases = nphases;
        ctl->st_pending_scans = nscans;
        ctl->next_epoch = U.epoch;        // next free stamps for the following run
        ctl->next_hround = U.hround;
    }
}

}  // namespace gbs
