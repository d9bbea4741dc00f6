// gbs_noalloc.cu -- gbs_sssp_noalloc: one SSSP that allocates no memory.
//
// Who needs it: callers that cannot call cudaMalloc/cudaFree during a query.
// Typical cases are a host application that owns every byte of device memory
// through its own pool and forbids allocations outside it, and latency-bound
// services for which cudaMalloc/cudaFree are unacceptable on the query path
// (they may synchronise the whole device and can fail with out-of-memory in
// the middle of a request).  Such a caller passes its inputs and outputs in
// device memory it already owns; every other buffer the run needs lives in
// g_noalloc_scratch below, a file-scope __device__ array that is created when
// the library is loaded and held by every GPU that loads it until the process
// exits.
//
// Limits: at most kNoAllocMaxN vertices and kNoAllocMaxM edges (the scratch
// is sized for exactly that, about 21 MB).  Larger inputs are rejected with
// GBS_ERR_INVALID_ARG before any device work.
//
// Sharing: every call uses the same array and it keeps the previous call's
// contents; each call clears what must start at zero (the frontier and
// heavy-round stamps, the control block) and re-initialises the rest.  Calls
// that overlap on the GPU (different streams, threads or processes sharing
// the context) race on the array and must be serialised by the caller.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address (cudaGetSymbolAddress; the host-side symbol is only
// a stand-in) and the persistent kernel's occupancy, and caches both.  Make
// that first call before any stream capture.
//
// Every call waits for its stream before returning: it reads the input check
// and the run's error word back into host memory.
//
// Alignment: adj_dev is read as 8-byte {target, weight} pairs, so it must be
// 8-byte aligned; row_dev, dist_dev and pred_dev 4-byte aligned.  A pointer
// that is not is refused on the host before any device work (a misaligned
// load would be a device fault that ends the context).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "gbs_sssp_persistent.cuh"

using namespace gbs;

namespace {

constexpr uint32_t kNoAllocMaxN = 65536;
constexpr uint64_t kNoAllocMaxM = 2097152;

constexpr size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kN = kNoAllocMaxN;
constexpr size_t kDescCap = kNoAllocMaxN + kNoAllocMaxM / kDescEdges + 64;
// byte offsets inside the scratch array
constexpr size_t kOffCtl = 0;
constexpr size_t kOffDp = al256(kOffCtl + sizeof(Ctl));
constexpr size_t kOffTag = al256(kOffDp + 8 * kN);
constexpr size_t kOffFst = al256(kOffTag + 4 * kN);
constexpr size_t kOffHst = al256(kOffFst + 4 * kN);
constexpr size_t kOffRing = al256(kOffHst + 4 * kN);
constexpr size_t kOffFq = al256(kOffRing + 4 * kN * kNB);
constexpr size_t kOffPend = al256(kOffFq + 4 * kN * 3);
constexpr size_t kOffDesc = al256(kOffPend + 4 * kN * 2);
constexpr size_t kOffCheck = al256(kOffDesc + sizeof(uint4) * kDescCap);
constexpr size_t kScratchBytes = al256(kOffCheck + 256);

// The only device memory the entry point uses besides the caller's buffers.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// check[0]: first bad-input code (0 = none), check[1]: max weight bits
__global__ void k_noalloc_check(const uint32_t *__restrict__ row, const uint2 *__restrict__ adj, uint32_t n,
                                uint32_t m, bool f32, uint32_t *check) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    if (tid == 0 && (row[0] != 0 || row[n] != m)) atomicCAS(&check[0], 0u, 1u);
    for (uint32_t v = tid; v < n; v += stride)
        if (row[v + 1] < row[v]) atomicCAS(&check[0], 0u, 2u);
    uint32_t wmax = 0;
    for (uint32_t e = tid; e < m; e += stride) {
        const uint2 x = adj[e];
        if (x.x >= n) atomicCAS(&check[0], 0u, 3u);
        const uint32_t wb = f32 ? (x.y == 0x80000000u ? 0u : x.y) : x.y;
        if (f32 && wb >= 0x7F800000u) atomicCAS(&check[0], 0u, 4u);   // negative, inf or NaN
        wmax = max(wmax, wb);
    }
    for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_down_sync(0xffffffffu, wmax, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&check[1], wmax);
}

__global__ void k_noalloc_reset(unsigned long long *__restrict__ dp, uint32_t *__restrict__ tag, uint32_t n,
                                uint32_t src, uint32_t *__restrict__ ring0, Ctl *ctl) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        dp[v] = (v == src) ? (unsigned long long)src : kUnreached;
        tag[v] = (v == src) ? 0u : kTagInit;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ring0[0] = src;
        ctl->ring_cnt[0].v = 1;
        ctl->pend_min[0].v = kTagInit;
        ctl->pend_min[1].v = kTagInit;
        ctl->pub_phase = kPhLightFirst;
        ctl->pub_b = 0;
        ctl->pub_span = 1;   // plain delta-stepping, no split (every edge light)
        ctl->pub_full = 1;
    }
}

template <bool F32>
__global__ void k_noalloc_unpack(const unsigned long long *__restrict__ dp, uint32_t n, uint32_t src,
                                 uint32_t *__restrict__ dist, int32_t *__restrict__ pred) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const unsigned long long x = dp[v];
        const bool reached = x != kUnreached;
        dist[v] = reached ? (uint32_t)(x >> 32) : (F32 ? 0x7F800000u : 0xFFFFFFFFu);
        if (pred) pred[v] = reached ? (v == src ? (int32_t)src : (int32_t)(uint32_t)x) : -1;
    }
}

struct DeviceSetup {
    bool ready = false;
    unsigned char *base = nullptr;   // device address of g_noalloc_scratch
    int blocks_u32 = 0, blocks_f32 = 0;
    int sms = 0;
};

constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;
gbs_status na_fail(gbs_status s, const std::string &m) {
    set_last_error(m.c_str());   // what gbs_last_error reports on this thread
    return s;
}

gbs_status setup_device(int dev, DeviceSetup **out) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    DeviceSetup &d = g_setup[dev];
    if (!d.ready) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return na_fail(GBS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        int per_u = 0, per_f = 0;
        if ((e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
            (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_u, sssp_persistent<kWU32>, kTPB, 0)) !=
                cudaSuccess ||
            (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_f, sssp_persistent<kWF32>, kTPB, 0)) !=
                cudaSuccess)
            return na_fail(GBS_ERR_CUDA, cudaGetErrorString(e));
        if (per_u < 1 || per_f < 1) return na_fail(GBS_ERR_UNSUPPORTED, "persistent kernel cannot be resident");
        d.base = static_cast<unsigned char *>(p);
        d.blocks_u32 = per_u * d.sms;
        d.blocks_f32 = per_f * d.sms;
        d.ready = true;
    }
    *out = &d;
    return GBS_OK;
}

#define NA_CUDA(call)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return na_fail(GBS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

extern "C" gbs_status gbs_sssp_noalloc(uint32_t n, uint64_t m, const uint32_t *row_dev,
                                       const uint32_t *adj_dev, gbs_weight_type wtype, uint32_t source,
                                       double delta, void *dist_dev, int32_t *pred_dev, void *stream) {
    if (!row_dev || (m && !adj_dev) || !dist_dev)
        return na_fail(GBS_ERR_INVALID_ARG, "gbs_sssp_noalloc: NULL device pointer");
    if (wtype != GBS_WEIGHT_U32 && wtype != GBS_WEIGHT_F32)
        return na_fail(GBS_ERR_INVALID_ARG, "gbs_sssp_noalloc: unknown weight type");
    if (n == 0 || n > kNoAllocMaxN || m > kNoAllocMaxM)
        return na_fail(GBS_ERR_INVALID_ARG,
                       "gbs_sssp_noalloc: needs 1 <= n <= 65536 and m <= 2097152 (its scratch is static)");
    if (source >= n) return na_fail(GBS_ERR_INVALID_ARG, "gbs_sssp_noalloc: source out of range");
    if ((reinterpret_cast<uintptr_t>(adj_dev) & 7u) || (reinterpret_cast<uintptr_t>(row_dev) & 3u) ||
        (reinterpret_cast<uintptr_t>(dist_dev) & 3u) || (reinterpret_cast<uintptr_t>(pred_dev) & 3u))
        return na_fail(GBS_ERR_INVALID_ARG,
                       "gbs_sssp_noalloc: adj_dev must be 8-byte aligned, row_dev / dist_dev / pred_dev 4-byte");
    int dev = 0;
    NA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return na_fail(GBS_ERR_UNSUPPORTED, "gbs_sssp_noalloc: device index");
    DeviceSetup *d = nullptr;
    gbs_status st = setup_device(dev, &d);
    if (st != GBS_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool f32 = wtype == GBS_WEIGHT_F32;
    unsigned char *b = d->base;
    Ctl *ctl = reinterpret_cast<Ctl *>(b + kOffCtl);
    uint32_t *check = reinterpret_cast<uint32_t *>(b + kOffCheck);
    const int tb = 256;
    const int eb = std::max(1, std::min<int>((int)((std::max<uint64_t>(n, m) + tb - 1) / tb), d->sms * 8));

    // the caller's CSR is checked on the device first: a bad row offset or
    // target would otherwise send the relaxation out of bounds
    uint32_t host_check[2] = {0, 0};
    NA_CUDA(cudaMemsetAsync(check, 0, 2 * sizeof(uint32_t), s));
    k_noalloc_check<<<eb, tb, 0, s>>>(row_dev, reinterpret_cast<const uint2 *>(adj_dev), n, (uint32_t)m, f32,
                                      check);
    NA_CUDA(cudaGetLastError());
    NA_CUDA(cudaMemcpyAsync(host_check, check, sizeof host_check, cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    if (host_check[0] != 0)
        return na_fail(GBS_ERR_INVALID_ARG, "gbs_sssp_noalloc: malformed CSR (offsets, targets or weights)");

    // bucket width: as gbs_sssp (<= 0 selects max weight / average out-degree)
    double max_w;
    if (f32) {
        float fw;
        std::memcpy(&fw, &host_check[1], 4);
        max_w = fw;
    } else {
        max_w = host_check[1];
    }
    if (!(delta > 0)) delta = (m && max_w > 0) ? max_w / ((double)m / (double)n) : 1.0;

    SsspArgs a{};
    a.g.n = n;
    a.g.m = m;
    a.g.wtype = wtype;
    a.g.row = row_dev;
    a.g.adj = reinterpret_cast<const uint2 *>(adj_dev);
    a.ws.ctl = ctl;
    a.ws.dp = reinterpret_cast<unsigned long long *>(b + kOffDp);
    a.ws.tag = reinterpret_cast<uint32_t *>(b + kOffTag);
    a.ws.fst = reinterpret_cast<uint32_t *>(b + kOffFst);
    a.ws.hst = reinterpret_cast<uint32_t *>(b + kOffHst);
    // no light/heavy split: every edge is light, so the split index of row v
    // is simply the end of the row (row_dev[v + 1]) and rows need no order
    a.ws.mid = const_cast<uint32_t *>(row_dev + 1);
    a.ws.ring = reinterpret_cast<uint32_t *>(b + kOffRing);
    a.ws.fq = reinterpret_cast<uint32_t *>(b + kOffFq);
    a.ws.pend = reinterpret_cast<uint32_t *>(b + kOffPend);
    a.ws.desc = reinterpret_cast<uint4 *>(b + kOffDesc);
    a.ws.hdesc = nullptr;   // every edge is light here: no heavy descriptors
    a.ws.desc_cap = (uint32_t)kDescCap;
    a.ws.trace = nullptr;
    a.ws.trace_cap = 0;
    a.source = source;
    a.epoch0 = 1;    // stamps restart at 1 each call: fst/hst are cleared below
    a.hround0 = 1;
    a.delta_u = (uint32_t)std::min(std::max(std::floor(delta), 1.0), 4294967295.0);
    a.inv_delta_f = (float)(1.0 / delta);
    a.flags = 0;
    a.solo_items = 1024;
    a.solo_desc = 64;
    a.no_heavy = 1;  // every edge is light (see mid above)
    a.inline_max = kInlineEdges;
    a.full_items = kFullItems;
    a.fuse_rounds = kFuseRounds;
    a.ctrl = kCtrlFixed;
    a.span_fixed = 1;
    a.wait_ns = 4000ull * 1000000ull;
    a.run_ns = a.wait_ns * 16ull;
    a.group = 0;
    a.group_ctas = (uint32_t)(f32 ? d->blocks_f32 : d->blocks_u32);
    a.ws.n_cap = n;

    NA_CUDA(cudaMemsetAsync(a.ws.fst, 0, sizeof(uint32_t) * n, s));
    NA_CUDA(cudaMemsetAsync(a.ws.hst, 0, sizeof(uint32_t) * n, s));
    NA_CUDA(cudaMemsetAsync(ctl, 0, sizeof(Ctl), s));
    k_noalloc_reset<<<eb, tb, 0, s>>>(a.ws.dp, a.ws.tag, n, source, a.ws.ring, ctl);
    NA_CUDA(cudaGetLastError());
    void *args[] = {&a};
    if (f32)
        NA_CUDA(cudaLaunchCooperativeKernel((const void *)sssp_persistent<kWF32>, dim3(d->blocks_f32), dim3(kTPB),
                                            args, 0, s));
    else
        NA_CUDA(cudaLaunchCooperativeKernel((const void *)sssp_persistent<kWU32>, dim3(d->blocks_u32), dim3(kTPB),
                                            args, 0, s));
    if (f32)
        k_noalloc_unpack<true><<<eb, tb, 0, s>>>(a.ws.dp, n, source, (uint32_t *)dist_dev, pred_dev);
    else
        k_noalloc_unpack<false><<<eb, tb, 0, s>>>(a.ws.dp, n, source, (uint32_t *)dist_dev, pred_dev);
    NA_CUDA(cudaGetLastError());
    uint32_t err = 0;
    NA_CUDA(cudaMemcpyAsync(&err, &ctl->error, sizeof err, cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    switch (err) {
        case kErrNone: return GBS_OK;
        case kErrTimeout: return na_fail(GBS_ERR_TIMEOUT, "gbs_sssp_noalloc: device-side wait limit exceeded");
        case kErrCapacity: return na_fail(GBS_ERR_CAPACITY, "gbs_sssp_noalloc: device work list overflow");
        case kErrOverflow: return na_fail(GBS_ERR_OVERFLOW, "gbs_sssp_noalloc: uint32 path sum overflow");
        default: return na_fail(GBS_ERR_INTERNAL, "gbs_sssp_noalloc: device error");
    }
}
