// gbs_sssp_persistent.cuh -- phases, decisions and the persistent kernel.
//
// The relaxation machinery (candidate filter, packed atomicMin, list appends)
// is in gbs_sssp_kernel.cuh.  This file holds the phase bodies, the decision
// taken at every barrier, the grid barrier itself and the kernel.
//
// Phases run either on the whole grid or, when the input of the next phase is
// small, on the one CTA that took the decision ("solo"): it runs that phase
// and the following small ones with block-level syncs, and releases the other
// CTAs (which wait at the grid barrier) only when a phase is large again or
// the run ends.  High-diameter graphs and the long tail of small buckets of
// R-MAT are thousands of phases of a few hundred vertices; a block-level sync
// costs far less than a grid barrier plus the dependent round trips of a
// grid-wide decision.
#pragma once

#include "gbs_sssp_kernel.cuh"

namespace gbs {

// Who executes a phase: the CTA group (the whole grid for a single-source
// launch) or one CTA.  Lists are dealt to warps in chunks of 32 entries (one
// per lane), and the warps of a group are numbered CTA-minor: chunk c goes to
// CTA c % group_ctas, so a phase of a few thousand entries runs one warp on
// each of many SMs instead of 32 warps on each of a few (one SM issues every
// load and atomic of its warps; on the 4096^2 grid, whose buckets start with
// 1-8 K entries, a bucket took 2 of 152 SMs).
struct Exec {
    uint32_t tid, nthreads;   // thread index and count over the executors (vertex loops)
    uint32_t warp, nwarps;    // warp index (CTA-minor in a group) and count over the executors
};

__device__ __forceinline__ uint32_t group_rank(const SsspArgs &a) {
    return blockIdx.x - a.group * a.group_ctas;
}

__device__ __forceinline__ Exec group_exec(const SsspArgs &a) {
    Exec x;
    x.tid = group_rank(a) * blockDim.x + threadIdx.x;
    x.nthreads = a.group_ctas * blockDim.x;
    x.warp = (threadIdx.x >> 5) * a.group_ctas + group_rank(a);
    x.nwarps = x.nthreads >> 5;
    return x;
}

__device__ __forceinline__ Exec cta_exec() {
    Exec x;
    x.tid = threadIdx.x;
    x.nthreads = blockDim.x;
    x.warp = x.tid >> 5;
    x.nwarps = x.nthreads >> 5;
    return x;
}

// The list counters in global memory, and the global home of word i of the
// deciding CTA's shared copy (counters, then the statistics words).
__device__ __forceinline__ Ctrs global_ctrs(Ctl *ctl) { return Ctrs{&ctl->ring_cnt[0].v, 32u}; }
__device__ __forceinline__ uint32_t *counter_home(Ctl *ctl, uint32_t i) {
    switch (i) {
        case kSPhases: return &ctl->st_phases;
        case kSBuckets: return &ctl->st_buckets;
        case kSPending: return &ctl->st_pending_scans;
        case kSSolo: return &ctl->st_solo_phases;
        default: return global_ctrs(ctl).at(i);
    }
}

// The decision of a barrier as published (Ctl::pubw): kPubWords fields, each
// in the low half of a 64-bit word whose high half is the barrier generation.
enum PubField : uint32_t { kPubState = 0, kPubB, kPubW, kPubEpoch, kPubHround, kPubInst, kPubItems, kPubWords };
constexpr uint32_t kNoItems = 0xFFFFFFFFu;   // Uniform.items: not published, read the counters

// phase | logical << 8 | pend_sel << 16 | full << 17 | span << 24 (span <= kNB)
__device__ __forceinline__ uint32_t pack_state(const Uniform &N) {
    return (N.phase & 0xFFu) | ((N.logical & 0xFFu) << 8) | ((N.pend_sel & 1u) << 16) | ((N.full & 1u) << 17) |
           ((N.span & 0xFFu) << 24);
}

// Writes a warp's descriptors.  Lane l owns descriptors [excl_l, excl_l + n_l)
// of the warp's `total` (exclusive prefix excl); its descriptor c covers edges
// [s_l + c kDescEdges, min(e_l, s_l + (c + 1) kDescEdges)) of row u_l and
// carries y_l.  The 32 lanes write them together, 32 per round (each finds the
// owning lane by a binary search over excl), so the hundreds of descriptors
// of a hub row do not queue on its lane.
__device__ __forceinline__ void write_descs(uint4 *out, uint32_t base, uint32_t total, uint32_t excl, uint32_t u,
                                            uint32_t y, uint32_t s, uint32_t e) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    for (uint32_t k0 = 0; k0 < total; k0 += 32u) {
        const uint32_t k = k0 + lane;
        uint32_t own = 0;   // the largest lane whose excl <= k
#pragma unroll
        for (uint32_t b = 16; b > 0; b >>= 1) {
            const uint32_t x = __shfl_sync(FULL, excl, own + b);
            if (x <= k) own += b;
        }
        const uint32_t ou = __shfl_sync(FULL, u, own), oy = __shfl_sync(FULL, y, own);
        const uint32_t os = __shfl_sync(FULL, s, own), oe = __shfl_sync(FULL, e, own);
        const uint32_t ox = __shfl_sync(FULL, excl, own);
        if (k < total) {
            const uint32_t cs = os + (k - ox) * kDescEdges;
            out[base + k] = make_uint4(ou, oy, cs, min(oe, cs + kDescEdges));
        }
    }
}

// ------------------------------------------------------------------- SCAN
// Warp-collective: every lane's row range [s, e) of source u (distance bits
// du; an empty range for a lane without one).  Rows longer than inline_max
// become descriptors, reserved with one atomic per warp; the others are
// relaxed by this warp now.  Edges handed to EDGES add to my_edges.
template <int WT>
__device__ __forceinline__ void scan_rows(const SsspArgs &a, const Targets &t, uint32_t u,
                                          typename Arith<WT>::D du, uint32_t s, uint32_t e, uint32_t &my_edges,
                                          uint32_t &nc, uint32_t &imp, Local &loc) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    const uint32_t len = e - s;
    const uint32_t nd = len > a.inline_max ? (len + kDescEdges - 1) / kDescEdges : 0u;
    uint32_t incl = nd;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, o);
        if ((int)lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    if (total) {
        uint32_t dbase = 0;
        if (lane == 31) dbase = atomicAdd(t.c.at(kCDesc), total);
        dbase = __shfl_sync(FULL, dbase, 31);
        if (dbase + total <= a.ws.desc_cap) {
            // float64 distances do not fit the descriptor: the relaxation
            // reads dp[u] again (a fresher value is as valid)
            write_descs(a.ws.desc, dbase, total, incl - nd, u, WT == kWF64 ? 0u : (uint32_t)du, s, e);
        } else if (lane == 31) {
            atomicExch(&a.ws.ctl->error, (uint32_t)kErrCapacity);
        }
        my_edges += nd ? len : 0u;
    }
    relax_group<WT>(a, t, u, du, s, nd ? 0u : len, nc, imp, loc);
}

// Bucket fusion: the targets the warp's lanes kept, relaxed in rounds of one
// per lane (whole rows, long ones as descriptors), at most fuse_rounds of
// them: the last round keeps nothing, so a long chain goes back to the
// frontier instead of running hop after hop on one warp while the rest of
// the grid waits (and relaxing vertices whose distances later drop again).
// Warp-collective; ends with the candidate buffer drained.
template <int WT>
__device__ __forceinline__ void fuse_drain(const SsspArgs &a, const Targets &t, uint32_t &my_edges, uint32_t &nc,
                                           uint32_t &imp, Local &loc) {
    const unsigned FULL = 0xffffffffu;
    cand_drain<WT>(a, t, nc, imp, loc);
    if (!t.fuse) return;
    for (uint32_t round = 1; __ballot_sync(FULL, loc.v < kNoKeep); ++round) {
        const bool has = loc.v < kNoKeep;
        const uint32_t u = has ? loc.v : 0u;
        const uint32_t s = has ? __ldg(a.g.row + u) : 0u;
        const uint32_t e = has ? __ldg(a.g.row + u + 1) : 0u;
        const typename Arith<WT>::D du = loc.d;
        loc.v = round < t.fuse ? kNoLocal : kNoKeep;
        scan_rows<WT>(a, t, u, du, s, e, my_edges, nc, imp, loc);
        cand_drain<WT>(a, t, nc, imp, loc);
    }
}

// One thread per frontier entry.  vtag != kTagInit keeps only entries whose
// tag equals it (ring lists may hold entries that moved to a lower bucket).
// The scan relaxes the light prefix [row, mid) of each row, or the whole row
// when full.  With a split, a vertex scanned for the first time in the
// current heavy round also emits descriptors for its heavy edges [mid, end):
// the HEAVY phase relaxes them once the bucket's light loop has settled.
template <int WT>
__device__ void scan_frontier(const SsspArgs &a, const Targets &t, const Exec &x, const uint32_t *F,
                              uint32_t count, uint32_t vtag, bool full, uint32_t hround, uint32_t &imp) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    Ctl *ctl = a.ws.ctl;
    uint32_t my_edges = 0;
    uint32_t nc = 0;   // candidates buffered by this warp
    Local loc{kNoLocal, 0u};
    for (uint32_t base = x.warp * 32u; base < count; base += x.nthreads) {
        const uint32_t i = base + lane;
        uint32_t u = 0, s = 0, e = 0, he = 0;
        typename Arith<WT>::D du = 0;
        bool ok = false;
        if (i < count) {
            u = __ldcg(F + i);
            // the tag check and the row reads are independent: issue together
            const uint32_t tg = (vtag == kTagInit) ? vtag : __ldcg(a.ws.tag + u);
            du = dist_of<WT>(__ldcg(a.ws.dp + u));
            const uint32_t r = __ldg(a.g.row + u);
            const uint32_t re = __ldg(a.g.row + u + 1);
            const uint32_t md = full ? re : __ldg(a.ws.mid + u);
            ok = tg == vtag;
            s = ok ? r : 0u;
            e = ok ? md : 0u;
            he = ok ? re : 0u;
        }
        // heavy-round membership is decided now; the heavy descriptors are
        // written after the relaxation below so this latency overlaps it
        uint32_t hold = hround;
        if (ok && !full) hold = atomicExch(a.ws.hst + u, hround);
        scan_rows<WT>(a, t, u, du, s, e, my_edges, nc, imp, loc);
        if (!full) {
            const uint32_t hlen = (ok && hold != hround) ? he - e : 0u;
            const uint32_t hn = (hlen + kDescEdges - 1) / kDescEdges;
            uint32_t hincl = hn;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, hincl, o);
                if ((int)lane >= o) hincl += y;
            }
            const uint32_t htotal = __shfl_sync(FULL, hincl, 31);
            if (htotal) {
                uint32_t hbase = 0;
                if (lane == 31) hbase = atomicAdd(t.c.at(kCHdesc), htotal);
                hbase = __shfl_sync(FULL, hbase, 31);
                if (hbase + htotal <= a.ws.desc_cap) {
                    write_descs(a.ws.hdesc, hbase, htotal, hincl - hn, u, 0u, e, he);
                } else if (lane == 31) {
                    atomicExch(&ctl->error, (uint32_t)kErrCapacity);
                }
            }
        }
    }
    fuse_drain<WT>(a, t, my_edges, nc, imp, loc);
    // edges handed to EDGES (statistics / trace)
    for (int o = 16; o > 0; o >>= 1) my_edges += __shfl_down_sync(FULL, my_edges, o);
    if (lane == 0 && my_edges) atomicAdd(t.c.at(kCEdge), my_edges);
}

// Warp-collective: relaxes one chunk [first, end) (<= kDescEdges edges) of
// source u with all 32 lanes.
template <int WT>
__device__ __forceinline__ void relax_chunk(const SsspArgs &a, const Targets &t, uint32_t u,
                                            typename Arith<WT>::D du, uint32_t first, uint32_t end, uint32_t &nc,
                                            uint32_t &imp, Local &loc) {
    const unsigned lane = lane_id();
    uint32_t v[kUnroll], uo[kUnroll];
    typename Arith<WT>::Wt w[kUnroll];
    typename Arith<WT>::D duo[kUnroll];
    bool val[kUnroll];
#pragma unroll
    for (int j = 0; j < kUnroll; ++j) {
        const uint32_t e = first + 32u * j + lane;
        val[j] = e < end;
        uo[j] = u;
        duo[j] = du;
        v[j] = 0;
        w[j] = 0;
        if (val[j]) {
            const uint2 ew = ld_stream(a.g.adj + e);
            v[j] = ew.x;
            w[j] = weight_at<WT>(a, e, ew);
        }
    }
    relax_candidates<WT>(a, t, val, v, w, uo, duo, nc, imp, loc);
}

// ------------------------------------------------------------------ HEAVY
// One thread per heavy descriptor, with dist(u) read from dp: u's distance
// after the bucket's light loop.  Chunks longer than kInlineEdges are relaxed
// one after another by the whole warp; the shorter ones (most heavy ranges of
// a sparse graph) together, packed across the warp by a prefix sum.  Lane l
// of warp w takes descriptors w + nwarps * (32 k + l): the consecutive
// descriptors of one long row (a hub's heavy range is hundreds of them) go
// to different warps instead of queueing up in one.
template <int WT>
__device__ void relax_heavy(const SsspArgs &a, const Targets &t, const Exec &x, uint32_t count, uint32_t &imp) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    uint32_t nc = 0;   // candidates buffered by this warp
    uint32_t my_edges = 0;
    Local loc{kNoLocal, 0u};   // heavy phases never fuse
    for (unsigned long long j0 = 0; x.warp + (unsigned long long)x.nwarps * j0 < count; j0 += 32u) {
        const unsigned long long i = x.warp + (unsigned long long)x.nwarps * (j0 + lane);
        uint32_t u = 0, s = 0, len = 0;
        typename Arith<WT>::D du = 0;
        if (i < count) {
            const uint4 d = __ldcg(a.ws.hdesc + i);
            u = d.x;
            s = d.z;
            len = d.w - d.z;
            du = dist_of<WT>(__ldcg(a.ws.dp + u));
        }
        my_edges += len;
        const bool lng = len > kInlineEdges;
        unsigned lm = __ballot_sync(FULL, lng);
        while (lm) {
            const int src = __ffs(lm) - 1;
            lm &= lm - 1u;
            const uint32_t su = __shfl_sync(FULL, u, src);
            const uint32_t ss = __shfl_sync(FULL, s, src);
            const uint32_t sl = __shfl_sync(FULL, len, src);
            const typename Arith<WT>::D sd = __shfl_sync(FULL, du, src);
            relax_chunk<WT>(a, t, su, sd, ss, ss + sl, nc, imp, loc);
        }
        relax_group<WT>(a, t, u, du, s, lng ? 0u : len, nc, imp, loc);
    }
    cand_drain<WT>(a, t, nc, imp, loc);
    for (int o = 16; o > 0; o >>= 1) my_edges += __shfl_down_sync(FULL, my_edges, o);
    if (lane == 0 && my_edges) atomicAdd(t.c.at(kCEdge), my_edges);
}

// ------------------------------------------------------------------ EDGES
// One warp per descriptor (<= kDescEdges edges of one row = one round).
template <int WT>
__device__ void relax_descriptors(const SsspArgs &a, const Targets &t, const Exec &x, uint32_t count,
                                  uint32_t &imp) {
    const unsigned lane = lane_id();
    uint32_t nc = 0;   // candidates buffered by this warp
    Local loc{kNoLocal, 0u};   // EDGES phases never fuse: a descriptor they emitted would be lost
    for (uint32_t c = x.warp; c < count; c += x.nwarps) {
        const uint4 d = __ldcg(a.ws.desc + c);
        // float64 distances do not fit the descriptor: read dp[u] again
        typename Arith<WT>::D du;
        if constexpr (WT == kWF64) du = dist_of<WT>(__ldcg(a.ws.dp + d.x));
        else du = d.y;
        relax_chunk<WT>(a, t, d.x, du, d.z, d.w, nc, imp, loc);
    }
    cand_drain<WT>(a, t, nc, imp, loc);
}

// Moves pending vertices whose bucket entered the window [W, W+kNB) into the
// ring; the rest go to the other pending list.
template <int WT>
__device__ void rebucket_pending(const SsspArgs &a, const Uniform &U, const Exec &x, WarpScratch *scr,
                                 uint32_t count, const Ctrs &c) {
    const uint32_t n = a.g.n;
    const uint32_t *list = a.ws.pend + (size_t)U.pend_sel * n;
    Targets t;
    t.cur_hi = 0;
    t.W = U.W;
    t.stamp_next = 0;
    t.fq_next = 0;
    t.pend_sel = U.pend_sel ^ 1u;
    t.scr = scr;
    t.c = c;
    t.fuse = 0;
    uint32_t stale = 0;
    for (uint32_t base = x.warp * 32u; base < count; base += x.nthreads) {
        const uint32_t i = base + lane_id();
        int q[1] = {-1};
        uint32_t v[1] = {0};
        if (i < count) {
            v[0] = __ldcg(list + i);
            const uint32_t tg = __ldcg(a.ws.tag + v[0]);
            stale += tg != kTagPending ? 1u : 0u;
            if (tg == kTagPending) {
                const uint32_t nb = bucket_of<WT>(dist_of<WT>(__ldcg(a.ws.dp + v[0])), a);
                if ((unsigned long long)nb < (unsigned long long)U.W + kNB) {
                    a.ws.tag[v[0]] = nb;
                    q[0] = 1 + (int)(nb % kNB);
                } else {
                    atomicMin(c.at(kCPmin + t.pend_sel), nb);
                    q[0] = kNB + 1;
                }
            }
        }
        warp_enqueue<1>(a, t, q, v);
    }
    // the tags just stored and the pending minimum feed the next decision and
    // the next scan; on one CTA only __syncthreads separates them from this
    // phase, and it waits neither for the plain stores to reach L2 (where the
    // scan's L2-only loads read) nor for the reduction
    __threadfence();
    // entries that had already left the pending list (statistics / trace)
    for (int o = 16; o > 0; o >>= 1) stale += __shfl_down_sync(0xffffffffu, stale, o);
    if (lane_id() == 0 && stale) atomicAdd(c.at(kCEdge), stale);
}

// ------------------------------------------------------ batched instances
// INIT: every vertex of the new instance unreached and unqueued, the source
// at distance 0 (its own predecessor).  The decision that started the
// instance queued the source in ring bucket 0.  Epoch 1 means the stamps
// restarted (first use of the workspace, or wrap-around): clear them over the
// whole workspace, since later instances may be larger.
__device__ inline void init_instance(const SsspArgs &a, const Uniform &U, const Exec &x) {
    const uint32_t n = a.g.n;
    for (uint32_t v = x.tid; v < n; v += x.nthreads) {
        a.ws.dp[v] = (v == a.source) ? (unsigned long long)a.source : kUnreached;
        a.ws.tag[v] = (v == a.source) ? 0u : kTagInit;
    }
    if (U.epoch == 1u) {
        for (uint32_t v = x.tid; v < a.ws.n_cap; v += x.nthreads) {
            a.ws.fst[v] = 0u;
            a.ws.hst[v] = 0u;
        }
    }
}

// FINISH: packed state -> the caller's dist / pred, and the reached vertices
// and their out-edges (the GTEPS numerator) summed into the control block.
template <int WT>
__device__ void finish_instance(const SsspArgs &a, const Exec &x, uint32_t &imp) {
    const unsigned FULL = 0xffffffffu;
    const uint32_t n = a.g.n;
    Ctl *ctl = a.ws.ctl;
    unsigned long long r = 0, e = 0;
    for (uint32_t v = x.tid; v < n; v += x.nthreads) {
        const unsigned long long p = __ldcg(a.ws.dp + v);
        const bool reached = p != kUnreached;
        if (a.dist_out) a.dist_out[v] = reached ? (uint32_t)(p >> 32) : (WT == kWF32 ? 0x7F800000u : 0xFFFFFFFFu);
        if (a.pred_out) a.pred_out[v] = reached ? (v == a.source ? (int32_t)v : (int32_t)(uint32_t)p) : -1;
        if (reached) {
            ++r;
            e += __ldg(a.g.row + v + 1) - __ldg(a.g.row + v);
        }
    }
    unsigned long long im = imp;
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_down_sync(FULL, r, o);
        e += __shfl_down_sync(FULL, e, o);
        im += __shfl_down_sync(FULL, im, o);
    }
    if (lane_id() == 0) {
        if (r) atomicAdd(&ctl->st_reached, r);
        if (e) atomicAdd(&ctl->st_edges_reached, e);
        if (im) atomicAdd(&ctl->st_improvements, im);
    }
    imp = 0;
}

// Runs the phase U.phase with executor x (grid or one CTA).
template <int WT>
__device__ void run_phase(const SsspArgs &a, const Uniform &U, const Exec &x, WarpScratch *scr,
                          uint32_t &imp, const Ctrs &c) {
    const uint32_t n = a.g.n;
    Targets t;
    t.cur_hi = U.b + U.span;   // the bucket covers base buckets [b, b + span)
    t.W = U.W;
    t.stamp_next = U.epoch + 1;
    t.fq_next = (U.epoch + 1) % 3u;
    t.pend_sel = U.pend_sel;
    t.scr = scr;
    t.c = c;
    const bool full = U.full != 0;
    // bucket fusion in whole-row scans (EDGES could not keep the descriptors
    // a kept long row emits: the next scan resets their list)
    t.fuse = (full && WT != kWF64 && (U.phase == kPhLightFirst || U.phase == kPhLight)) ? a.fuse_rounds : 0u;
    // the input size comes with the decision (U.items); the counters are
    // read only where it was not published
    const bool pub = U.items != kNoItems;
    switch (U.phase) {
        case kPhLightFirst:
            // the ring lists of every base bucket the bucket spans, one after
            // the other (independent: no barrier between them)
            for (uint32_t j = 0; j < U.span; ++j) {
                const uint32_t bk = U.b + j;
                const uint32_t cnt = (pub && U.span == 1u) ? U.items : ld_relaxed_any(c.at(kCRing + bk % kNB));
                scan_frontier<WT>(a, t, x, a.ws.ring + (size_t)(bk % kNB) * n, min(cnt, n), bk, full, U.hround,
                                  imp);
            }
            break;
        case kPhLight:
            scan_frontier<WT>(a, t, x, a.ws.fq + (size_t)(U.epoch % 3u) * n,
                              min(pub ? U.items : ld_relaxed_any(c.at(kCFq + U.epoch % 3u)), n), kTagInit, full,
                              U.hround, imp);
            break;
        case kPhHeavy:
            relax_heavy<WT>(a, t, x, min(pub ? U.items : ld_relaxed_any(c.at(kCHdesc)), a.ws.desc_cap), imp);
            break;
        case kPhEdges:
            relax_descriptors<WT>(a, t, x, min(pub ? U.items : ld_relaxed_any(c.at(kCDesc)), a.ws.desc_cap), imp);
            break;
        case kPhPending:
            rebucket_pending<WT>(a, U, x, scr, min(pub ? U.items : ld_relaxed_any(c.at(kCPend + U.pend_sel)), n), c);
            break;
        case kPhInit:
            init_instance(a, U, x);
            break;
        case kPhFinish:
            finish_instance<WT>(a, x, imp);
            break;
        default:
            break;
    }
}

__device__ __forceinline__ uint32_t scan_kind(uint32_t phase) {
    return phase == kPhHeavy ? (uint32_t)kPhHeavy : (uint32_t)kPhLight;
}

// ------------------------------------------------------------ controller
// FP32 MLP kFeat -> kHid -> kHid -> 2 (ReLU), parameter block laid out as
// kMlp* says; inputs are standardised with the block's mu / sd.  Warp-
// collective: x is identical in every lane, y0 / y1 come back in every lane.
// Lane l owns hidden units l and l + 32 of each layer.
__device__ __forceinline__ void mlp_eval(const float *__restrict__ P, const float (&x)[kFeat], float &y0,
                                         float &y1) {
    const unsigned FULL = 0xffffffffu;
    const unsigned l = lane_id();
    float xn[kFeat];
#pragma unroll
    for (int i = 0; i < kFeat; ++i) xn[i] = (x[i] - __ldg(P + i)) / __ldg(P + kFeat + i);
    float ha = __ldg(P + kMlpB1 + l), hb = __ldg(P + kMlpB1 + 32 + l);
#pragma unroll
    for (int i = 0; i < kFeat; ++i) {
        ha = fmaf(xn[i], __ldg(P + kMlpW1 + i * kHid + l), ha);
        hb = fmaf(xn[i], __ldg(P + kMlpW1 + i * kHid + 32 + l), hb);
    }
    ha = fmaxf(ha, 0.f);
    hb = fmaxf(hb, 0.f);
    float ga = __ldg(P + kMlpB2 + l), gb = __ldg(P + kMlpB2 + 32 + l);
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
        const float hi = __shfl_sync(FULL, ha, i);
        ga = fmaf(hi, __ldg(P + kMlpW2 + i * kHid + l), ga);
        gb = fmaf(hi, __ldg(P + kMlpW2 + i * kHid + 32 + l), gb);
    }
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
        const float hi = __shfl_sync(FULL, hb, i);
        ga = fmaf(hi, __ldg(P + kMlpW2 + (32 + i) * kHid + l), ga);
        gb = fmaf(hi, __ldg(P + kMlpW2 + (32 + i) * kHid + 32 + l), gb);
    }
    ga = fmaxf(ga, 0.f);
    gb = fmaxf(gb, 0.f);
    float p0 = ga * __ldg(P + kMlpW3 + 2 * l) + gb * __ldg(P + kMlpW3 + 2 * (32 + l));
    float p1 = ga * __ldg(P + kMlpW3 + 2 * l + 1) + gb * __ldg(P + kMlpW3 + 2 * (32 + l) + 1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        p0 += __shfl_xor_sync(FULL, p0, o);
        p1 += __shfl_xor_sync(FULL, p1, o);
    }
    y0 = p0 + __ldg(P + kMlpB3);
    y1 = p1 + __ldg(P + kMlpB3 + 1);
}

// Span and split of the bucket that starts at base bucket nb, and the entries
// of the lists it spans (warp-collective: warp 0 of the deciding CTA).  The
// fixed schedule keeps span_fixed base widths; the learned one evaluates the
// controller on the occupancy of the next base buckets, the run so far and
// the graph.  GBS_F_FEATURES records the controller input.
__device__ __forceinline__ void decide_bucket(const SsspArgs &a, Ctl *ctl, const uint32_t *sc, uint32_t nb, uint32_t lim,
                                              uint32_t ring_lo, uint32_t ring_hi, uint32_t pend, uint32_t pm,
                                              uint32_t &span_out, uint32_t &full_out, uint32_t &first_items) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    auto ring_count = [&](uint32_t bucket) {
        const uint32_t slot = bucket % kNB;
        const uint32_t lo = __shfl_sync(FULL, ring_lo, slot & 31u);
        const uint32_t hi = __shfl_sync(FULL, ring_hi, slot & 31u);
        return slot < 32 ? lo : hi;
    };
    // occupancy of the base buckets from nb on (inside the window only)
    uint32_t c_lo = ring_count(nb + lane), c_hi = ring_count(nb + 32u + lane);
    c_lo = (nb + lane < lim) ? c_lo : 0u;
    c_hi = (nb + 32u + lane < lim) ? c_hi : 0u;
    uint32_t span = a.span_fixed ? a.span_fixed : 1u;
    uint32_t full = a.no_heavy;
    const bool want_feat = (a.flags & GBS_F_FEATURES) && a.feat;
    if (a.ctrl == kCtrlLearned || want_feat) {
        uint32_t incl = c_lo;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if ((int)lane >= o) incl += y;
        }
        uint32_t hi_sum = c_hi;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) hi_sum += __shfl_xor_sync(FULL, hi_sum, o);
        auto first = [&](uint32_t k) {   // entries of base buckets [nb, nb + k), k <= 32
            return (float)__shfl_sync(FULL, incl, k - 1u);
        };
        const uint32_t st_b = sc[kSBuckets], st_p = sc[kSPhases];
        float f[kFeat];
        f[0] = __log2f(1.f + first(1));
        f[1] = __log2f(1.f + first(2));
        f[2] = __log2f(1.f + first(4));
        f[3] = __log2f(1.f + first(8));
        f[4] = __log2f(1.f + first(16));
        f[5] = __log2f(1.f + first(32));
        f[6] = __log2f(1.f + first(32) + (float)hi_sum);
        f[7] = __log2f(1.f + (float)pend);
        // the distance reached, in plain widths (the base width is
        // 2^gfeat[4] plain widths)
        f[8] = __log2f(1.f + (float)nb * exp2f(a.gfeat[4]));
        f[9] = __log2f(1.f + (float)st_b);
        f[10] = __log2f(1.f + (float)st_p);
        // share of the window's entries in the next base bucket (<= 0): none
        // of the inputs grows with the vertex count by itself
        f[11] = f[0] - f[6];
#pragma unroll
        for (int i = 1; i < 5; ++i) f[11 + i] = a.gfeat[i];
        if (want_feat && lane == 0) {
            const uint32_t fi = ctl->feat_n;
            if (fi < a.feat_cap) {
#pragma unroll
                for (int i = 0; i < kFeat; ++i) a.feat[(size_t)fi * kFeat + i] = f[i];
            }
            ctl->feat_n = fi + 1u;
        }
        if (a.ctrl == kCtrlLearned) {
            float y0, y1;
            mlp_eval(a.mlp, f, y0, y1);
            int e = (int)rintf(y0 + a.span_bias);
            e = e < 0 ? 0 : (e > (int)kLearnedSpanLog ? (int)kLearnedSpanLog : e);
            span = 1u << e;
            full = (a.no_heavy || y1 <= 0.f) ? 1u : 0u;   // y1: logit of "split at the light bound"
        }
    }
    // a bucket never reaches past the smallest pending bucket
    while (span > 1u && pend > 0u && nb + span > pm) span >>= 1;
    span_out = span;
    full_out = full;
    // entries of the span's lists (for the solo decision)
    uint32_t cnt = (lane < span ? c_lo : 0u) + (lane + 32u < span ? c_hi : 0u);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(FULL, cnt, o);
    first_items = cnt;
    // a bucket that starts this small relaxes whole rows: its heavy phase
    // would cost a grid step for a handful of edges (distances are the same
    // least fixpoint either way)
    if (a.ctrl == kCtrlFixed && cnt <= a.full_items) full_out = 1u;
}

// The uniform state after the decision (identical in every CTA that adopts it).
__device__ __forceinline__ Uniform advance_uniform(const Uniform &U, uint32_t next, uint32_t nb) {
    Uniform N = U;
    if (U.phase == kPhPending) {
        N.pend_sel ^= 1u;
    } else if (next == kPhEdges) {
        N.logical = scan_kind(U.phase);
    } else {
        const uint32_t logical = (U.phase == kPhEdges) ? U.logical : scan_kind(U.phase);
        N.epoch += 1;
        if (logical == kPhHeavy) N.hround += 1;
    }
    if (next == kPhLightFirst) { N.b = nb; N.W = nb; }
    if (next == kPhPending) N.W = nb;
    N.phase = next;
    return N;
}

// Run by warp 0 of the deciding CTA after a phase: every other CTA has
// finished it (or is waiting while this CTA runs alone), so all counters are
// at rest.  Decides the next phase, resets the lists it appends to, records
// statistics and the trace, writes the new state to s_pub (shared memory, in
// the published layout) and says whether the next phase is small enough for
// this CTA to run alone.  In a batched launch the
// end of a run leads to FINISH, and after FINISH the group takes the next
// instance from the queue (INIT) or stops.
template <bool Batch>
__device__ inline void control_step(const SsspArgs &a, const Uniform &U, bool was_solo, bool &solo,
                                    uint32_t *s_pub, uint32_t *sc) {
    Ctl *ctl = a.ws.ctl;
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    // the error word is the one global read; it is first used at the end
    const uint32_t err = ld_relaxed(&ctl->error);
    const uint32_t ring_lo = sc[kCRing + lane];
    const uint32_t ring_hi = sc[kCRing + lane + 32];
    const uint32_t desc_cnt = sc[kCDesc];
    const uint32_t edge_cnt = sc[kCEdge];
    const uint32_t fq_next = sc[kCFq + (U.epoch + 1u) % 3u];
    const uint32_t fq_cur = sc[kCFq + U.epoch % 3u];
    const uint32_t hd_cnt = sc[kCHdesc];
    const uint32_t pc0 = sc[kCPend], pc1 = sc[kCPend + 1];
    const uint32_t pm0 = sc[kCPmin], pm1 = sc[kCPmin + 1];
    __syncwarp();   // every lane has read the counters before lane 0 resets them
    auto ring_count = [&](uint32_t bucket) {
        const uint32_t slot = bucket % kNB;
        const uint32_t lo = __shfl_sync(FULL, ring_lo, slot & 31u);
        const uint32_t hi = __shfl_sync(FULL, ring_hi, slot & 31u);
        return slot < 32 ? lo : hi;
    };
    // entries of the lists the current bucket spans (trace)
    uint32_t cur_ring;
    {
        const uint32_t c1 = ring_count(U.b + lane), c2 = ring_count(U.b + 32u + lane);
        cur_ring = (lane < U.span ? c1 : 0u) + (lane + 32u < U.span ? c2 : 0u);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cur_ring += __shfl_xor_sync(FULL, cur_ring, o);
    }

    uint32_t next = kPhDone, nb = 0;
    uint32_t ps2 = U.pend_sel;
    bool need_ring_scan = false;
    bool bucket_end = false;
    uint32_t scan_from = 0;
    bool take = false;
    if (Batch && U.phase >= kPhInit) {
        if (U.phase == kPhInit) {
            next = kPhLightFirst;   // bucket 0 holds the source
            nb = 0;
        } else {
            take = true;            // after FINISH, or at the start of the launch
        }
    } else if (U.phase == kPhPending) {
        ps2 ^= 1u;
        need_ring_scan = true;
        scan_from = U.W;
    } else if (U.phase != kPhEdges && desc_cnt > 0) {
        next = kPhEdges;
    } else {
        const uint32_t logical = (U.phase == kPhEdges) ? U.logical : scan_kind(U.phase);
        if (fq_next > 0) {
            next = kPhLight;
        } else if (logical == kPhLight && !U.full && hd_cnt > 0) {
            next = kPhHeavy;
        } else {
            bucket_end = true;
            need_ring_scan = true;
            scan_from = U.b + U.span;
        }
    }
    if (need_ring_scan) {
        // first non-empty ring bucket in [scan_from, W + kNB); at a bucket end
        // scan_from = b + span = W + span, so the slots being cleared are not read.
        const uint32_t lim = U.W + kNB;   // exclusive
        uint32_t found = 0xFFFFFFFFu;
#pragma unroll
        for (uint32_t off = 0; off < (uint32_t)kNB; off += 32u) {
            const uint32_t bk = scan_from + off + lane;
            const uint32_t c = ring_count(bk);
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
            next = Batch ? kPhFinish : kPhDone;
        }
    }
    uint32_t inst = U.inst;
    if (take) {
        if (lane == 0) inst = atomicAdd(a.queue, 1u);
        inst = __shfl_sync(FULL, inst, 0);
        next = inst < a.inst_count ? kPhInit : kPhDone;
        if (next == kPhDone) inst = kNoInst;
    }
    // whole-run limit: a run that has not finished within run_ns is stopped;
    // a learned schedule also stops at its guard (the host reruns plain)
    const unsigned long long run_t = globaltimer() - U.t0;
    if (run_t > a.run_ns) {
        next = kPhDone;
        if (lane == 0) atomicCAS(&ctl->error, 0u, (uint32_t)kErrTimeout);
    } else if (a.guard_ns && run_t > a.guard_ns) {
        next = kPhDone;
        if (lane == 0) atomicCAS(&ctl->error, 0u, (uint32_t)kErrGuard);
    }
    Uniform N = advance_uniform(U, next, nb);
    if (take) {
        N.inst = inst;
        N.hround += 1u;   // the last heavy round of the previous instance may be stamped
        // stamps restart at 1 on a fresh workspace or before they wrap; INIT
        // then clears them
        if (U.epoch == 0u || U.epoch > 0xF0000000u || U.hround > 0xF0000000u) {
            N.epoch = 1u;
            N.hround = 1u;
        }
    }
    uint32_t first_items = 0;   // LIGHT_FIRST: entries of every list the new bucket spans
    if (next == kPhLightFirst) {
        uint32_t span, full;
        decide_bucket(a, ctl, sc, nb, U.W + kNB, ring_lo, ring_hi, ps2 ? pc1 : pc0, ps2 ? pm1 : pm0, span, full,
                      first_items);
        N.span = span;
        N.full = full;
    }
    // size of the next phase's input
    uint32_t items = 0;
    switch (next) {
        case kPhLightFirst: items = first_items; break;
        case kPhLight: items = fq_next; break;
        case kPhHeavy: items = hd_cnt; break;
        case kPhEdges: items = desc_cnt; break;
        case kPhPending: items = ps2 ? pc1 : pc0; break;
        default: break;
    }
    // INIT and FINISH (batched launches) always run on the whole group; a
    // small re-bucketing of the pending list runs on this CTA like any small
    // scan
    solo = next < kPhDone && (next == kPhEdges ? items <= a.solo_desc : items <= a.solo_items);
    // an error raised anywhere ends the run (the counter resets below are
    // then moot); applied last so the global read overlaps the decision
    if (err) {
        next = kPhDone;
        N.phase = kPhDone;
        solo = false;
    }
    __syncwarp();   // the controller inputs read from sc come before the updates
    if (lane == 0) {
        if ((a.flags & GBS_F_TRACE) && a.ws.trace) {
            const uint32_t ti = ctl->trace_n;
            if (ti < a.ws.trace_cap) {
                uint32_t done_items;
                switch (U.phase) {
                    case kPhLightFirst: done_items = cur_ring; break;
                    case kPhLight: done_items = fq_cur; break;
                    case kPhHeavy: done_items = hd_cnt; break;
                    case kPhEdges: done_items = desc_cnt; break;
                    default: done_items = U.pend_sel ? pc1 : pc0; break;
                }
                TraceRec r;
                r.kind = U.phase | (was_solo ? 16u : 0u) | (U.span << 8) | (U.full << 16);
                r.bucket = U.b;
                r.items = done_items;
                r.edges = edge_cnt;
                r.pending = N.pend_sel ? pc1 : pc0;
                r.window = U.W;
                r.end_ns = globaltimer() - U.t0;
                a.ws.trace[ti] = r;
            }
            ctl->trace_n = ti + 1;
        }
        if (Batch && U.inst != kNoInst && (U.phase == kPhFinish || err)) {
            InstResult r;
            r.done = (U.phase == kPhFinish && !err) ? 1u : 0u;
            r.error = err;
            r.group = a.group;
            r.phases = sc[kSPhases];
            r.buckets = sc[kSBuckets];
            r.pending_scans = sc[kSPending];
            r.solo_phases = sc[kSSolo];
            r.pad = 0;
            r.reached = __ldcg(&ctl->st_reached);
            r.edges_reached = __ldcg(&ctl->st_edges_reached);
            r.improvements = __ldcg(&ctl->st_improvements);
            r.start_ns = ctl->inst_t0;
            r.end_ns = globaltimer();
            a.res[U.inst] = r;
        }
        if (U.phase < kPhDone) sc[kSPhases] += 1;
        if (U.phase == kPhLightFirst) sc[kSBuckets] += 1;
        if (U.phase == kPhPending) {
            sc[kSPending] += 1;
            sc[kCPend + U.pend_sel] = 0;          // the list just re-bucketed
            sc[kCPmin + U.pend_sel] = kTagInit;
        }
        if (was_solo) sc[kSSolo] += 1;
        if (next == kPhPending) sc[kCEdge] = 0;   // counts stale entries there
        if (next == kPhLight || next == kPhHeavy || next == kPhLightFirst) {
            sc[kCFq + (N.epoch + 1u) % 3u] = 0;
            sc[kCDesc] = 0;
            sc[kCEdge] = 0;
            // heavy descriptors of the next heavy round start over once the
            // last round's are relaxed, and at every new bucket
            if (U.phase == kPhHeavy || next == kPhLightFirst) sc[kCHdesc] = 0;
        }
        // the decision, in the layout the release publishes
        s_pub[kPubState] = pack_state(N);
        s_pub[kPubB] = N.b;
        s_pub[kPubW] = N.W;
        s_pub[kPubEpoch] = N.epoch;
        s_pub[kPubHround] = N.hround;
        s_pub[kPubInst] = N.inst;
        s_pub[kPubItems] = next < kPhDone ? items : kNoItems;
    }
    if (bucket_end) {   // the lists of the finished bucket
        if (lane < U.span) sc[kCRing + (U.b + lane) % kNB] = 0u;
        if (lane + 32u < U.span) sc[kCRing + (U.b + 32u + lane) % kNB] = 0u;
    }
    if (take && next == kPhInit) {
        // every list of the new instance starts empty; the source waits in
        // ring bucket 0 (list slot 0, entry 0)
        sc[kCRing + lane] = 0u;
        sc[kCRing + lane + 32] = 0u;
        __syncwarp();
        if (lane == 0) {
            sc[kCRing] = 1u;
            a.ws.ring[0] = a.inst[inst].source;
            for (int i = 0; i < 3; ++i) sc[kCFq + i] = 0u;
            sc[kCHdesc] = 0u;
            for (int i = 0; i < 2; ++i) {
                sc[kCPend + i] = 0u;
                sc[kCPmin + i] = kTagInit;
            }
            sc[kCDesc] = 0u;
            sc[kCEdge] = 0u;
            sc[kSBuckets] = 0u;
            sc[kSPhases] = 0u;
            sc[kSPending] = 0u;
            sc[kSSolo] = 0u;
            ctl->st_improvements = 0ull;
            ctl->st_reached = 0ull;
            ctl->st_edges_reached = 0ull;
            ctl->inst_t0 = globaltimer();
        }
    }
    __syncwarp();
}

// The state of s_pub (published layout) as this CTA's uniform state.
__device__ __forceinline__ void adopt_published(const uint32_t *s_pub, Uniform &U) {
    const uint32_t st = s_pub[kPubState];
    U.phase = st & 0xFFu;
    U.logical = (st >> 8) & 0xFFu;
    U.pend_sel = (st >> 16) & 1u;
    U.full = (st >> 17) & 1u;
    U.span = st >> 24;
    U.b = s_pub[kPubB];
    U.W = s_pub[kPubW];
    U.epoch = s_pub[kPubEpoch];
    U.hround = s_pub[kPubHround];
    U.inst = s_pub[kPubInst];
    U.items = s_pub[kPubItems];
}

// Grid barrier after a phase.  The CTA that arrives last decides the next
// phase (control_step); while the next phase is small it runs it alone and
// decides again, and only then releases the waiting CTAs: the decision as
// kPubWords 64-bit release stores tagged with the new generation.
// Warp 0 of a waiting CTA polls those words (one lane each) until every one
// carries the new generation, so the poll that sees the release also brings
// the state.  Every wait is bounded by a.wait_ns (globaltimer); on expiry the
// error word is set and every CTA leaves at its next check.  A solo stretch
// stops after a.wait_ns / 4 so the waiting CTAs never time out.
template <int WT, bool Batch>
__device__ __forceinline__ void barrier_and_decide(const SsspArgs &a, Uniform &U, WarpScratch *scr,
                                                   uint32_t &imp) {
    Ctl *ctl = a.ws.ctl;
    const unsigned FULL = 0xffffffffu;
    __shared__ uint32_t s_flag[2];
    __shared__ uint32_t s_pub[kPubWords];
    __shared__ uint32_t s_cnt[kCtrShared];   // the deciding CTA's copy of the list counters
    __syncthreads();
    if (threadIdx.x == 0) {
        // GBS_F_TEST_STALL: CTA 0 skips its first arrival (failure-path test)
        const bool stall = (a.flags & GBS_F_TEST_STALL) && U.gen == 0 && group_rank(a) == 0;
        uint32_t last = 0;
        if (!stall) last = atom_add_acq_rel(&ctl->bar_count, 1u) == a.group_ctas - 1u;
        s_flag[0] = last;
    }
    __syncthreads();
    const unsigned long long tag = (unsigned long long)(U.gen + 1u) << 32;
    if (s_flag[0]) {
        const unsigned long long ts = globaltimer();
        bool was_solo = false;
        // the counters, at rest, into shared memory (one round trip): every
        // decision of this barrier and every phase this CTA runs alone reads
        // and updates the copy, which goes back before the release
        if (threadIdx.x < 32) {
            uint32_t v[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t i = lane_id() + 32u * k;
                v[k] = i < (uint32_t)kCtrShared ? ld_relaxed(counter_home(ctl, i)) : 0u;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t i = lane_id() + 32u * k;
                if (i < (uint32_t)kCtrShared) s_cnt[i] = v[k];
            }
            __syncwarp();
        }
        for (;;) {
            if (threadIdx.x < 32) {
                bool solo = false;
                control_step<Batch>(a, U, was_solo, solo, s_pub, s_cnt);
                if (threadIdx.x == 0) s_flag[1] = solo && (globaltimer() - ts) < a.wait_ns / 4;
            }
            __syncthreads();
            adopt_published(s_pub, U);
            // s_pub and s_flag are written again only after the phase's
            // __syncthreads below
            if (s_flag[1] == 0) break;
            // A re-bucketing of the pending list on this CTA is fenced by
            // every thread on both sides: the phases before it wrote the
            // entries, tags and distances it reads, and the decision after it
            // reads the ring and pending counters it fills.  Without both
            // fences 200 of 432 small-width runs (grids and R-MATs, widths
            // 1-20) lost vertices or stopped early; fences inside the
            // re-bucketing and after each pending push alone were not enough
            // (measured).  The phase is rare (a few per run at most on the
            // published configurations).
            if (U.phase == kPhPending) {
                __threadfence();
                __syncthreads();
            }
            run_phase<WT>(a, U, cta_exec(), scr, imp, Ctrs{s_cnt, 1u});
            if (U.phase == kPhPending) __threadfence();
            // the decision is taken by this CTA: __syncthreads makes every
            // global access of the phase (the fire-and-forget tag and pend_min
            // reductions included) visible to all its threads, as it does for
            // the other CTAs' arrivals, where thread 0 alone fences before the
            // arrival; the release after the stretch fences before publishing
            __syncthreads();
            was_solo = true;
        }
        // the counters back to global memory, then one release store per
        // published word; lane 0's also releases the barrier counter reset
        if (threadIdx.x < 32) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t i = lane_id() + 32u * k;
                if (i < (uint32_t)kCtrShared) *counter_home(ctl, i) = s_cnt[i];
            }
            __syncwarp();
            if (threadIdx.x < kPubWords) {
                if (threadIdx.x == 0) ctl->bar_count = 0;
                st_release64(&ctl->pubw[threadIdx.x], tag | s_pub[threadIdx.x]);
            }
        }
    } else {
        if (threadIdx.x < 32) {
            const unsigned lane = lane_id();
            const unsigned long long t0 = globaltimer();
            uint32_t spins = 0;
            unsigned long long v = tag;
            bool quit = false;
            for (;;) {
                if (lane < kPubWords) v = ld_acquire64(&ctl->pubw[lane]);
                if (__all_sync(FULL, (v & 0xFFFFFFFF00000000ull) == tag)) break;
                if ((++spins & 255u) == 0) {
                    int stop = 0;
                    if (lane == 0) {
                        if (ld_relaxed(&ctl->error) != 0) {
                            stop = 1;
                        } else if (globaltimer() - t0 > a.wait_ns) {
                            atomicCAS(&ctl->error, 0u, (uint32_t)kErrTimeout);
                            stop = 1;
                        }
                    }
                    if (__shfl_sync(FULL, stop, 0)) {
                        quit = true;
                        break;
                    }
                }
            }
            if (lane < kPubWords) s_pub[lane] = (uint32_t)v;
            __syncwarp();
            // after an error or a timeout this CTA stops; an error raised
            // during the phase reaches the others through the next decision
            if (lane == 0 && quit) s_pub[kPubState] = (s_pub[kPubState] & ~0xFFu) | (uint32_t)kPhDone;
        }
        __syncthreads();
        adopt_published(s_pub, U);
    }
    __syncthreads();
    U.gen += 1;
}

template <int WT>
__global__ void __launch_bounds__(kTPB, 1) sssp_persistent(SsspArgs a) {
    Ctl *ctl = a.ws.ctl;
    __shared__ WarpScratch s_scr[kTPB / 32];
    WarpScratch *scr = &s_scr[threadIdx.x >> 5];
    Uniform U;
    U.phase = ld_relaxed(&ctl->pub_phase);
    U.logical = kPhLight;
    U.b = ld_relaxed(&ctl->pub_b);
    U.W = U.b;
    U.epoch = a.epoch0;
    U.hround = a.hround0;
    U.pend_sel = 0;
    U.inst = kNoInst;
    U.span = ld_relaxed(&ctl->pub_span);
    U.full = ld_relaxed(&ctl->pub_full);
    U.items = kNoItems;
    U.gen = 0;
    U.t0 = globaltimer();
    uint32_t imp = 0;
    while (U.phase != kPhDone) {
        run_phase<WT>(a, U, group_exec(a), scr, imp, global_ctrs(ctl));
        barrier_and_decide<WT, false>(a, U, scr, imp);
    }
    for (int o = 16; o > 0; o >>= 1) imp += __shfl_down_sync(0xffffffffu, imp, o);
    if (lane_id() == 0 && imp) atomicAdd(&ctl->st_improvements, (unsigned long long)imp);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->next_epoch = U.epoch;        // next free stamps for the following run
        ctl->next_hround = U.hround;
    }
}

// Batched launch: CTA group g (group_ctas CTAs) owns workspace ws_groups[g]
// and solves instances taken from base.queue until the queue is empty.  The
// control block of a workspace keeps the last stamps between launches.
template <int WT>
__global__ void __launch_bounds__(kTPB, 1) sssp_batch(SsspArgs base, const Workspace *__restrict__ ws_groups) {
    __shared__ SsspArgs s_a;
    __shared__ WarpScratch s_scr[kTPB / 32];
    WarpScratch *scr = &s_scr[threadIdx.x >> 5];
    const uint32_t group = blockIdx.x / base.group_ctas;
    if (threadIdx.x == 0) {
        s_a = base;
        s_a.group = group;
        s_a.ws = ws_groups[group];
    }
    __syncthreads();
    Ctl *ctl = s_a.ws.ctl;
    Uniform U;
    U.phase = kPhTake;
    U.logical = kPhLight;
    U.b = 0;
    U.W = 0;
    U.epoch = ld_relaxed(&ctl->next_epoch);
    U.hround = ld_relaxed(&ctl->next_hround);
    U.pend_sel = 0;
    U.inst = kNoInst;
    U.span = 1;
    U.full = 0;
    U.items = kNoItems;
    U.gen = 0;
    U.t0 = globaltimer();
    uint32_t loaded = kNoInst;
    uint32_t imp = 0;
    while (U.phase != kPhDone) {
        if (U.inst != loaded) {
            // a new instance: its graph, source, schedule and outputs
            if (threadIdx.x == 0) {
                const InstDesc d = s_a.inst[U.inst];
                s_a.g = d.g;
                s_a.ws.mid = const_cast<uint32_t *>(d.mid);
                s_a.source = d.source;
                s_a.delta_u = d.delta_u;
                s_a.inv_delta_f = d.inv_delta_f;
                s_a.no_heavy = d.no_heavy;
                s_a.dist_out = d.dist;
                s_a.pred_out = d.pred;
            }
            __syncthreads();
            loaded = U.inst;
            U.t0 = globaltimer();   // the run-time limit applies per instance
        }
        run_phase<WT>(s_a, U, group_exec(s_a), scr, imp, global_ctrs(ctl));
        barrier_and_decide<WT, true>(s_a, U, scr, imp);
    }
    if (group_rank(s_a) == 0 && threadIdx.x == 0) {
        // after an error the stamps in flight are unknown: 0 makes the next
        // launch clear them
        const bool err = ld_relaxed(&ctl->error) != 0;
        ctl->next_epoch = err ? 0u : U.epoch;
        ctl->next_hround = err ? 0u : U.hround;
    }
}

}  // namespace gbs
