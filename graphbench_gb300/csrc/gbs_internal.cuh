// gbs_internal.cuh -- device data layout and helpers shared by the SSSP
// kernels of libgbsssp (sm_103a).
//
// HBM layout of one resident graph (built once by gbs_graph_create):
//   row[n+1]  uint32  exclusive row offsets (m < 2^32)
//   adj[m]    uint2   {col, weight bits}; each row sorted by (weight, col), so
//                     the light edges of any split w <= L are a row prefix
//   mid[n]    uint32  first heavy edge of each row for the cached split L
// Per-run state (workspace, reused across runs on the same graph):
//   dp[n]     uint64  (dist bits << 32) | pred; ~0 = unreached.  Non-negative
//                     float32 bit patterns order like the values, so one 64-bit
//                     atomicMin updates distance and predecessor together and
//                     keeps the smallest predecessor among equal distances.
//   tag[n]    uint32  smallest bucket the vertex was queued for (ring dedup)
//   fst[n]    uint32  frontier stamp (dedup inside one light sub-phase)
//   hst[n]    uint32  heavy-round stamp (a vertex's heavy edges are described
//                     once per heavy round)
//   ring      kNB lists of n uint32: bucket b lives in list b % kNB while it is
//                     inside the window [W, W + kNB)
//   fq        3 lists of n uint32: current-bucket frontier, rotated per step
//   pend      2 lists of n uint32: vertices whose bucket is beyond the window
//   desc      edge descriptors {u, dist(u), first edge, end edge} of one SCAN
//   hdesc     heavy-edge descriptors {u, -, first, end} of the current heavy
//             round, written by the light scans, relaxed by HEAVY
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "gbsssp.h"

namespace gbs {

constexpr int kNB = 64;                 // ring buckets (window width)
constexpr uint32_t kTagInit = 0xFFFFFFFFu;
constexpr uint32_t kTagPending = 0xFFFFFFFEu;
constexpr uint32_t kBucketMax = 0xFFFFFF00u;
constexpr unsigned long long kUnreached = ~0ull;
// Threads per CTA of the persistent SSSP kernels (one CTA per SM): 896
// leaves 72 registers a thread, and the relaxation no longer spills the way
// it did at 64 (1024 threads).  Kernel ms, 1024 / 768 / 896 threads: R-MAT 20
// 1.088 / 1.054 / 1.062, R-MAT 22 2.204 / 2.167 / 2.152, 4096^2 grid
// 214.6 / 213.2 / 210.0.
constexpr int kTPB = 896;
// Default bucket fusion rounds per warp and scan.  Plain width, 4096^2 grid
// (kernel ms): 1 231, 2 224, 4 240, 8 242; at 64 plain widths 1 96, 2 89,
// 4 83, 8 80 (the autotuner picks per graph); R-MAT 20 / 22 flat.
constexpr uint32_t kFuseRounds = 2;

enum ErrCode : uint32_t {
    kErrNone = 0,
    kErrTimeout = 1,
    kErrCapacity = 2,
    kErrOverflow = 3,
    kErrGuard = 4,          // the learned schedule ran past its time guard (host reruns the plain one)
};

// Bucket-width controller of a run.
enum CtrlMode : uint32_t {
    kCtrlFixed = 0,         // every bucket spans span_fixed base widths, split as no_heavy says
    kCtrlLearned = 1,       // the MLP picks span and split at every bucket start
};

constexpr int kFeat = 16;           // controller features
constexpr int kHid = 64;            // hidden units of each of the two layers
// Parameter block of the controller, floats:
//   mu[16] sd[16] W1[16][64] b1[64] W2[64][64] b2[64] W3[64][2] b3[2]
constexpr int kMlpW1 = 2 * kFeat;
constexpr int kMlpB1 = kMlpW1 + kFeat * kHid;
constexpr int kMlpW2 = kMlpB1 + kHid;
constexpr int kMlpB2 = kMlpW2 + kHid * kHid;
constexpr int kMlpW3 = kMlpB2 + kHid;
constexpr int kMlpB3 = kMlpW3 + kHid * 2;
constexpr int kMlpFloats = kMlpB3 + 2;
constexpr int kMlpParams = kMlpFloats - 2 * kFeat;   // trained parameters (5,378)
constexpr uint32_t kMaxSpanLog = 6;                  // a bucket spans at most 2^6 = kNB base widths
constexpr uint32_t kLearnedSpanLog = 3;              // a learned bucket spans at most 2^3 base widths

// One record per grid phase when GBS_F_TRACE is set (layout = gbs_phase_rec).
struct TraceRec {
    uint32_t kind;
    uint32_t bucket;
    uint32_t items;
    uint32_t edges;
    uint32_t pending;       // entries of the live pending list after the phase
    uint32_t window;        // ring window base during the phase
    unsigned long long end_ns;
};

// A counter alone on a 128-byte line: list counters take millions of
// appends per run, and counters sharing a line serialise at one L2 slice.
struct __align__(128) Line {
    uint32_t v;
    uint32_t pad[31];
};

// Control block in global memory.  Barrier words and every list counter sit
// on their own 128-byte lines; the block is read by the deciding CTA after
// each phase.
struct __align__(128) Ctl {
    uint32_t bar_count;
    uint32_t pad0[31];
    // the decision of each barrier, published in one line: word i holds
    // (generation << 32) | field i (kPubWords fields, see PubField), so a
    // waiting CTA's poll returns the state together with the release
    unsigned long long pubw[8];
    uint32_t pad1[16];
    uint32_t error;
    uint32_t trace_n;
    // state a launch starts from (set before the launch)
    uint32_t pub_phase;
    uint32_t pub_b;
    uint32_t pub_span;            // base widths bucket 0 spans
    uint32_t pub_full;            // 1: light scans relax whole rows, no heavy scan
    uint32_t feat_n;              // feature vectors recorded
    uint32_t pad2[25];
    Line ring_cnt[kNB];
    Line fq_cnt[3];
    Line hdesc_cnt;
    Line pend_cnt[2];
    Line pend_min[2];
    Line desc_cnt;
    Line edge_cnt;
    // statistics and carried state (written by CTA 0 at exit)
    uint32_t st_buckets;
    uint32_t st_phases;
    uint32_t st_pending_scans;
    uint32_t next_epoch;
    uint32_t next_hround;
    uint32_t st_solo_phases;      // phases run by one CTA without a grid barrier
    unsigned long long st_improvements;
    unsigned long long st_reached;
    unsigned long long st_edges_reached;
    unsigned long long inst_t0;   // globaltimer when the current instance started
};
static_assert(sizeof(Ctl) % 128 == 0, "Ctl lines");

// The list counters of Ctl (ring_cnt .. edge_cnt, consecutive Lines) by
// index.  A phase run by the whole grid reaches them in global memory, one
// Line apart; the deciding CTA keeps a copy in its shared memory while it
// decides and while it runs phases alone, one word apart, and writes it back
// before it releases the other CTAs.  Four statistics words follow the
// counters in the shared copy (their global homes are the st_* fields).
enum CtrIdx : uint32_t {
    kCRing = 0,
    kCFq = kNB,
    kCHdesc = kNB + 3,
    kCPend = kNB + 4,
    kCPmin = kNB + 6,
    kCDesc = kNB + 8,
    kCEdge = kNB + 9,
    kCtrWords = kNB + 10,
    kSPhases = kCtrWords,
    kSBuckets,
    kSPending,
    kSSolo,
    kCtrShared,
};
static_assert(offsetof(Ctl, fq_cnt) == offsetof(Ctl, ring_cnt) + 128 * kCFq, "counter order");
static_assert(offsetof(Ctl, hdesc_cnt) == offsetof(Ctl, ring_cnt) + 128 * kCHdesc, "counter order");
static_assert(offsetof(Ctl, pend_cnt) == offsetof(Ctl, ring_cnt) + 128 * kCPend, "counter order");
static_assert(offsetof(Ctl, pend_min) == offsetof(Ctl, ring_cnt) + 128 * kCPmin, "counter order");
static_assert(offsetof(Ctl, desc_cnt) == offsetof(Ctl, ring_cnt) + 128 * kCDesc, "counter order");
static_assert(offsetof(Ctl, edge_cnt) == offsetof(Ctl, ring_cnt) + 128 * kCEdge, "counter order");

// Where a phase's list counters live: counter i at base + i * stride.
struct Ctrs {
    uint32_t *base;
    uint32_t stride;   // 32 words (global Lines) or 1 (shared copy)
    __device__ __forceinline__ uint32_t *at(uint32_t i) const { return base + i * stride; }
};

struct DevGraph {
    uint32_t n;
    uint64_t m;
    gbs_weight_type wtype;
    const uint32_t *row;
    const uint2 *adj;
    const unsigned long long *w64;   // float64 graphs: the weights (adj holds the targets)
};

struct Workspace {
    unsigned long long *dp;
    uint32_t *tag, *fst, *hst, *mid;
    uint32_t *ring, *fq, *pend;
    uint4 *desc;
    uint4 *hdesc;           // heavy-edge descriptors (capacity desc_cap)
    uint32_t desc_cap;
    uint32_t n_cap;         // vertices the per-vertex arrays hold (lists use the
                            // instance's n as their stride, n <= n_cap)
    TraceRec *trace;
    uint32_t trace_cap;
    Ctl *ctl;
};

// One instance of a batched launch: a graph, a source and the bucket
// schedule; dist / pred receive the instance's result (either may be null).
struct InstDesc {
    DevGraph g;
    const uint32_t *mid;    // first heavy edge of each row (row + 1: no split)
    uint32_t source;
    uint32_t delta_u;
    float inv_delta_f;
    uint32_t no_heavy;
    uint32_t *dist;
    int32_t *pred;
};

// Written by the group that solved the instance (layout = gbs_inst_stats).
struct InstResult {
    uint32_t done;          // 1 when the instance completed
    uint32_t error;         // ErrCode of the group, if it stopped on this instance
    uint32_t group;
    uint32_t phases;
    uint32_t buckets;
    uint32_t pending_scans;
    uint32_t solo_phases;
    uint32_t pad;
    unsigned long long reached;
    unsigned long long edges_reached;
    unsigned long long improvements;
    unsigned long long start_ns;   // globaltimer at the start and end of the instance
    unsigned long long end_ns;
};

constexpr uint32_t kNoInst = 0xFFFFFFFFu;

// Everything the persistent kernel needs, passed by value.  A single-source
// launch is one group of every CTA; a batched launch cuts the grid into groups
// of group_ctas CTAs that each own a workspace and take instances from a queue.
struct SsspArgs {
    DevGraph g;
    Workspace ws;
    uint32_t source;
    uint32_t epoch0;        // first frontier stamp of this run
    uint32_t hround0;       // first heavy-round stamp of this run
    uint32_t delta_u;       // uint32 bucket width (>= 1)
    float inv_delta_f;      // float32: bucket = floor(d * inv_delta)
    double inv_delta_d;     // float64: bucket = floor(d * inv_delta)
    uint32_t flags;         // GBS_F_* of the call
    uint32_t solo_items;    // a SCAN/PENDING phase with at most this many entries runs on one CTA
    uint32_t solo_desc;     // an EDGES phase with at most this many descriptors runs on one CTA
    uint32_t no_heavy;      // the split covers every edge: light scans relax whole rows, no HEAVY phase
    uint32_t inline_max;    // rows up to this long are relaxed by the scanning warp
    uint32_t full_items;    // kCtrlFixed: a bucket whose lists hold at most this many entries when it
                            // starts relaxes whole rows (no heavy phase)
    uint32_t fuse_rounds;   // bucket fusion rounds per warp in whole-row scans (0: none)
    // bucket-width controller
    uint32_t ctrl;          // CtrlMode
    uint32_t span_fixed;    // kCtrlFixed: base widths per bucket (0 or 1 = plain delta-stepping)
    float span_bias;        // kCtrlLearned: span = 2^clamp(round(y0 + span_bias), 0, kLearnedSpanLog)
    const float *mlp;       // kCtrlLearned: parameter block (kMlpFloats)
    float gfeat[5];         // graph inputs 12..15 of the controller are gfeat[1..4] (see graph_features)
    unsigned long long guard_ns;   // kCtrlLearned: stop with kErrGuard past this run time (0 = none)
    float *feat;            // GBS_F_FEATURES: kFeat floats per bucket start
    uint32_t feat_cap;
    uint32_t group;         // this CTA's group and the CTAs in one group
    uint32_t group_ctas;
    uint32_t *dist_out;     // batched: the current instance's outputs
    int32_t *pred_out;
    const InstDesc *inst;   // batched: instances, their results, their count
    InstResult *res;
    uint32_t inst_count;
    uint32_t *queue;        // batched: next instance to take
    unsigned long long wait_ns;   // limit of one barrier wait
    unsigned long long run_ns;    // limit of the whole run
};

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// The same load through a generic address (a counter in global or shared memory).
__device__ __forceinline__ uint32_t ld_relaxed_any(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Barrier arrival: release (this CTA's phase, made visible to thread 0 by
// __syncthreads) and acquire (every earlier arrival's phase) in one atomic.
__device__ __forceinline__ uint32_t atom_add_acq_rel(uint32_t *p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Edge stream: read once per relaxation, not worth keeping in L1.
__device__ __forceinline__ uint2 ld_stream(const uint2 *p) {
    uint2 v;
    asm volatile("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];"
                 : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
// Fire-and-forget line fetches: into this SM's L1 (a row this warp reads
// soon) or into L2 (a row another SM reads in a later phase).
__device__ __forceinline__ void prefetch_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Sets the message gbs_last_error returns on the calling thread.
void set_last_error(const char *msg);

}  // namespace gbs
