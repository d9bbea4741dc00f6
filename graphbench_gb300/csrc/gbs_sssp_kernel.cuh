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
// Edge lists are expanded per warp: short rows by a warp-wide prefix sum,
// rows of 32+ edges by the whole warp, rows above big_threshold split into
// 512-edge chunks that every warp of the GPU shares in an extra BIG phase.
#pragma once

#include "gbs_internal.cuh"

namespace gbs {

enum Phase : uint32_t {
    kPhLightFirst = 0,
    kPhLight = 1,
    kPhHeavy = 2,
    kPhBig = 3,
    kPhPending = 4,
    kPhDone = 5,
};

// Values identical in every CTA (the kernel's uniform state).
struct Uniform {
    uint32_t phase;       // phase being executed
    uint32_t logical;     // kPhLight or kPhHeavy: the phase a BIG step belongs to
    uint32_t b;           // current bucket
    uint32_t W;           // ring window base
    uint32_t epoch;       // frontier stamp of the current frontier
    uint32_t hround;      // heavy-round stamp (selects the S list)
    uint32_t big_sel;
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

// Targets of one phase's appends.
struct Targets {
    uint32_t cur_hi;      // buckets < cur_hi belong to the current bucket
    uint32_t W;
    uint32_t stamp_next;
    uint32_t fq_next;     // index of the next-frontier list
    uint32_t pend_sel;    // pending list to append to
};

// Queue ids: -1 none, 0 next frontier, 1..kNB ring slots, kNB+1 pending.
__device__ __forceinline__ void warp_enqueue(const SsspArgs &a, const Targets &t, int q, uint32_t v) {
    const unsigned FULL = 0xffffffffu;
    if (__ballot_sync(FULL, q >= 0) == 0) return;
    const unsigned lane = lane_id();
    const unsigned grp = __match_any_sync(FULL, q);
    const int leader = __ffs(grp) - 1;
    Ctl *ctl = a.ws.ctl;
    const uint32_t n = a.g.n;
    uint32_t base = 0;
    if (q >= 0 && (int)lane == leader) {
        uint32_t *cnt;
        if (q == 0) cnt = &ctl->fq_cnt[t.fq_next];
        else if (q <= kNB) cnt = &ctl->ring_cnt[q - 1];
        else cnt = &ctl->pend_cnt[t.pend_sel];
        base = atomicAdd(cnt, (uint32_t)__popc(grp));
    }
    base = __shfl_sync(FULL, base, leader);
    if (q >= 0) {
        uint32_t pos = base + (uint32_t)__popc(grp & ((1u << lane) - 1u));
        uint32_t *buf;
        if (q == 0) buf = a.ws.fq + (size_t)t.fq_next * n;
        else if (q <= kNB) buf = a.ws.ring + (size_t)(q - 1) * n;
        else buf = a.ws.pend + (size_t)t.pend_sel * n;
        if (pos < n) buf[pos] = v;
        else atomicExch(&ctl->error, (uint32_t)kErrCapacity);
    }
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

// Relaxes edge e of u (distance bits du).  Returns the queue id for the target.
template <bool F32>
__device__ __forceinline__ int relax_edge(const SsspArgs &a, const Targets &t, uint32_t e, uint32_t u,
                                          uint32_t du, uint32_t &v_out, uint32_t &imp) {
    const uint2 ew = ld_stream(a.g.adj + e);
    const uint32_t v = ew.x;
    uint32_t nd;
    if (F32) {
        nd = __float_as_uint(__fadd_rn(__uint_as_float(du), __uint_as_float(ew.y)));
    } else {
        const unsigned long long s = (unsigned long long)du + ew.y;
        if (s >= 0xFFFFFFFFull) {
            atomicExch(&a.ws.ctl->error, (uint32_t)kErrOverflow);
            return -1;
        }
        nd = (uint32_t)s;
    }
    const unsigned long long packed = ((unsigned long long)nd << 32) | u;
    unsigned long long *dpv = a.ws.dp + v;
    if (packed >= __ldcg(dpv)) return -1;
    const unsigned long long old = atomicMin(dpv, packed);
    if (packed >= old || nd >= (uint32_t)(old >> 32)) return -1;  // no distance decrease
    ++imp;
    v_out = v;
    const uint32_t nb = bucket_of<F32>(nd, a);
    if (nb < t.cur_hi) {
        atomicMin(a.ws.tag + v, nb);
        return atomicExch(a.ws.fst + v, t.stamp_next) != t.stamp_next ? 0 : -1;
    }
    if ((unsigned long long)nb < (unsigned long long)t.W + kNB) {
        return atomicMin(a.ws.tag + v, nb) > nb ? 1 + (int)(nb % kNB) : -1;
    }
    atomicMin(&a.ws.ctl->pend_min[t.pend_sel], nb);
    return atomicMin(a.ws.tag + v, kTagPending) == kTagInit ? kNB + 1 : -1;
}

// Expands one frontier list.  vtag != kTagInit keeps only entries whose tag
// equals it (ring slots may hold entries that moved to a lower bucket).
template <bool F32>
__device__ void expand_frontier(const SsspArgs &a, const Targets &t, const uint32_t *F, uint32_t count,
                                uint32_t vtag, bool light, bool add_s, uint32_t hround,
                                uint32_t big_sel, uint32_t &imp) {
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    const uint32_t warp_g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t n = a.g.n;
    Ctl *ctl = a.ws.ctl;
    for (uint32_t base = warp_g * 32u; base < count; base += nwarps * 32u) {
        const uint32_t i = base + lane;
        uint32_t u = 0, du = 0, s = 0, e = 0;
        bool ok = false;
        if (i < count) {
            u = __ldcg(F + i);
            ok = (vtag == kTagInit) || (__ldcg(a.ws.tag + u) == vtag);
        }
        if (ok) {
            du = (uint32_t)(__ldcg(a.ws.dp + u) >> 32);
            const uint32_t r0 = __ldg(a.g.row + u);
            const uint32_t r1 = __ldg(a.g.row + u + 1);
            const uint32_t md = __ldg(a.ws.mid + u);
            s = light ? r0 : md;
            e = light ? md : r1;
        }
        bool sflag = false;
        if (ok && add_s) sflag = atomicExch(a.ws.hst + u, hround) != hround;
        warp_append(a.ws.S + (size_t)(hround & 1u) * n, &ctl->s_cnt[hround & 1u], n, sflag, u, ctl);

        uint32_t len = e - s;
        // very long rows -> shared chunk list (processed in the BIG phase)
        if (len >= a.big_threshold) {
            const uint32_t nch = (len + kChunk - 1) / kChunk;
            const uint32_t pos = atomicAdd(&ctl->big_cnt[big_sel], nch);
            if (pos + nch <= a.ws.big_cap) {
                uint4 *dst = a.ws.big + (size_t)big_sel * a.ws.big_cap + pos;
                for (uint32_t c = 0; c < nch; ++c) {
                    const uint32_t cs = s + c * kChunk;
                    const uint32_t ce = min(e, cs + kChunk);
                    dst[c] = make_uint4(u, du, cs, ce);
                }
            } else {
                atomicExch(&ctl->error, (uint32_t)kErrCapacity);
            }
            len = 0;
        }
        // rows of 32+ edges: the whole warp walks one row at a time
        unsigned mm = __ballot_sync(FULL, len >= 32u);
        if (len >= 32u) len = 0;
        while (mm) {
            const int l = __ffs(mm) - 1;
            mm &= mm - 1;
            const uint32_t su = __shfl_sync(FULL, s, l);
            const uint32_t eu = __shfl_sync(FULL, e, l);
            const uint32_t uu = __shfl_sync(FULL, u, l);
            const uint32_t duu = __shfl_sync(FULL, du, l);
            for (uint32_t j = su; j < eu; j += 32u) {
                const uint32_t ej = j + lane;
                int q = -1;
                uint32_t v = 0;
                if (ej < eu) q = relax_edge<F32>(a, t, ej, uu, duu, v, imp);
                warp_enqueue(a, t, q, v);
            }
        }
        // short rows: warp-wide prefix sum, 32 edges per step
        uint32_t incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if ((int)lane >= o) incl += y;
        }
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        const uint32_t excl = incl - len;
        for (uint32_t k0 = 0; k0 < total; k0 += 32u) {
            const uint32_t k = k0 + lane;
            int owner = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const int cand = owner + step;
                const uint32_t ex = __shfl_sync(FULL, excl, cand);
                if (ex <= k) owner = cand;
            }
            const uint32_t so = __shfl_sync(FULL, s, owner);
            const uint32_t exo = __shfl_sync(FULL, excl, owner);
            const uint32_t uo = __shfl_sync(FULL, u, owner);
            const uint32_t duo = __shfl_sync(FULL, du, owner);
            int q = -1;
            uint32_t v = 0;
            if (k < total) q = relax_edge<F32>(a, t, so + (k - exo), uo, duo, v, imp);
            warp_enqueue(a, t, q, v);
        }
    }
}

template <bool F32>
__device__ void expand_big(const SsspArgs &a, const Targets &t, uint32_t big_sel, uint32_t count,
                           uint32_t &imp) {
    const unsigned lane = lane_id();
    const uint32_t warp_g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint4 *list = a.ws.big + (size_t)big_sel * a.ws.big_cap;
    for (uint32_t c = warp_g; c < count; c += nwarps) {
        const uint4 ch = __ldcg(list + c);
        for (uint32_t j = ch.z; j < ch.w; j += 32u) {
            const uint32_t ej = j + lane;
            int q = -1;
            uint32_t v = 0;
            if (ej < ch.w) q = relax_edge<F32>(a, t, ej, ch.x, ch.y, v, imp);
            warp_enqueue(a, t, q, v);
        }
    }
}

// Moves pending vertices whose bucket entered the window [W, W+kNB) into the
// ring; the rest go to the other pending list.
template <bool F32>
__device__ void rebucket_pending(const SsspArgs &a, const Uniform &U) {
    const uint32_t n = a.g.n;
    Ctl *ctl = a.ws.ctl;
    const uint32_t count = min(__ldcg(&ctl->pend_cnt[U.pend_sel]), n);
    const uint32_t *list = a.ws.pend + (size_t)U.pend_sel * n;
    Targets t;
    t.cur_hi = 0;
    t.W = U.W;
    t.stamp_next = 0;
    t.fq_next = 0;
    t.pend_sel = U.pend_sel ^ 1u;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    for (uint32_t base = tid - lane_id(); base < count; base += nthreads) {
        const uint32_t i = base + lane_id();
        int q = -1;
        uint32_t v = 0;
        if (i < count) {
            v = __ldcg(list + i);
            if (__ldcg(a.ws.tag + v) == kTagPending) {
                const uint32_t nb = bucket_of<F32>((uint32_t)(__ldcg(a.ws.dp + v) >> 32), a);
                if ((unsigned long long)nb < (unsigned long long)U.W + kNB) {
                    a.ws.tag[v] = nb;
                    q = 1 + (int)(nb % kNB);
                } else {
                    atomicMin(&ctl->pend_min[t.pend_sel], nb);
                    q = kNB + 1;
                }
            }
        }
        warp_enqueue(a, t, q, v);
    }
}

// Run by warp 0 of the CTA that arrives last at a barrier: every other CTA
// has finished the phase, so all counters are at rest.  Decides the next
// phase, resets the lists that phase will append to, and publishes.
__device__ void control_step(const SsspArgs &a, const Uniform &U) {
    Ctl *ctl = a.ws.ctl;
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = lane_id();
    uint32_t next = kPhDone, nb = 0;
    // state after the update every CTA applies (mirrors advance_uniform)
    uint32_t e2 = U.epoch, h2 = U.hround, bs2 = U.big_sel, ps2 = U.pend_sel;
    bool need_ring_scan = false;
    uint32_t scan_from = 0;
    if (U.phase == kPhPending) {
        ps2 ^= 1u;
        need_ring_scan = true;
        scan_from = U.W;
        if (lane == 0) { ctl->pend_cnt[U.pend_sel] = 0; ctl->pend_min[U.pend_sel] = kTagInit; }
    } else {
        const uint32_t logical = (U.phase == kPhBig) ? U.logical : (U.phase == kPhHeavy ? kPhHeavy : kPhLight);
        if (U.phase != kPhBig && ld_relaxed(&ctl->big_cnt[U.big_sel]) > 0) {
            next = kPhBig;
        } else {
            e2 = U.epoch + 1;
            bs2 = U.big_sel ^ 1u;
            if (logical == kPhHeavy) h2 = U.hround + 1;
            if (ld_relaxed(&ctl->fq_cnt[e2 % 3u]) > 0) {
                next = kPhLight;
            } else if (logical == kPhLight) {
                next = kPhHeavy;
            } else {
                if (lane == 0) ctl->ring_cnt[U.b % kNB] = 0;
                need_ring_scan = true;
                scan_from = U.b + 1;
            }
        }
    }
    if (need_ring_scan) {
        // first non-empty ring bucket in [scan_from, W + kNB); at a bucket end
        // scan_from = b + 1 = W + 1, so the slot just cleared is not read.
        const uint32_t lim = U.W + kNB;   // exclusive
        uint32_t found = 0xFFFFFFFFu;
        for (uint32_t off = 0; off < (uint32_t)kNB; off += 32u) {
            const uint32_t bk = scan_from + off + lane;
            const bool nz = bk < lim && ld_relaxed(&ctl->ring_cnt[bk % kNB]) > 0;
            const unsigned m = __ballot_sync(FULL, nz);
            if (m && found == 0xFFFFFFFFu) found = scan_from + off + (uint32_t)(__ffs(m) - 1);
        }
        const uint32_t pcnt = ld_relaxed(&ctl->pend_cnt[ps2]);
        const uint32_t pm = ld_relaxed(&ctl->pend_min[ps2]);
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
    if (lane == 0) {
        if (next == kPhLight || next == kPhHeavy || next == kPhLightFirst) {
            ctl->fq_cnt[(e2 + 1u) % 3u] = 0;
            ctl->big_cnt[bs2] = 0;
            if (h2 != U.hround || next == kPhLightFirst) ctl->s_cnt[h2 & 1u] = 0;
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
    } else if (next != kPhBig) {
        const uint32_t logical = (U.phase == kPhBig) ? U.logical : (U.phase == kPhHeavy ? kPhHeavy : kPhLight);
        U.epoch += 1;
        U.big_sel ^= 1u;
        if (logical == kPhHeavy) U.hround += 1;
    } else {
        U.logical = (U.phase == kPhHeavy) ? kPhHeavy : kPhLight;
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
__global__ void __launch_bounds__(kTPB, 2) sssp_persistent(SsspArgs a) {
    Ctl *ctl = a.ws.ctl;
    Uniform U;
    U.phase = ld_relaxed(&ctl->mode);
    U.logical = kPhLight;
    U.b = ld_relaxed(&ctl->next_bucket);
    U.W = U.b;
    U.epoch = a.epoch0;
    U.hround = a.hround0;
    U.big_sel = 0;
    U.pend_sel = 0;
    U.gen = 0;
    U.t0 = globaltimer();
    uint32_t imp = 0, nphases = 0, nbuckets = 0, nscans = 0;
    const uint32_t ncap = a.g.n;   // every list holds at most n entries
    __shared__ uint32_t s_next[2];

    while (U.phase != kPhDone) {
        Targets t;
        t.cur_hi = U.b + 1;
        t.W = U.W;
        t.stamp_next = U.epoch + 1;
        t.fq_next = (U.epoch + 1) % 3u;
        t.pend_sel = U.pend_sel;
        const uint32_t n = a.g.n;
        switch (U.phase) {
            case kPhLightFirst:
                ++nbuckets;
                expand_frontier<F32>(a, t, a.ws.ring + (size_t)(U.b % kNB) * n,
                                     min(__ldcg(&ctl->ring_cnt[U.b % kNB]), ncap), U.b, true, true,
                                     U.hround, U.big_sel, imp);
                break;
            case kPhLight:
                expand_frontier<F32>(a, t, a.ws.fq + (size_t)(U.epoch % 3u) * n,
                                     min(__ldcg(&ctl->fq_cnt[U.epoch % 3u]), ncap), kTagInit, true, true,
                                     U.hround, U.big_sel, imp);
                break;
            case kPhHeavy:
                expand_frontier<F32>(a, t, a.ws.S + (size_t)(U.hround & 1u) * n,
                                     min(__ldcg(&ctl->s_cnt[U.hround & 1u]), ncap), kTagInit, false, false,
                                     U.hround, U.big_sel, imp);
                break;
            case kPhBig:
                expand_big<F32>(a, t, U.big_sel, min(__ldcg(&ctl->big_cnt[U.big_sel]), a.ws.big_cap), imp);
                break;
            case kPhPending:
                ++nscans;
                rebucket_pending<F32>(a, U);
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
        ctl->err_info = U.epoch;          // next free stamps for the following run
        ctl->pad4 = U.hround;
    }
}

}  // namespace gbs
