// gbs_batch.cu -- batched SSSP (include/gbsssp.h, "Batched SSSP"): graph
// packs, plans and their launch.
//
// A plan owns:
//   inst[count]    InstDesc: graph, split index, source, schedule, outputs
//   res[count]     InstResult written by the group that solved the instance
//   ws[groups]     one workspace per CTA group, carved from one arena
//   queue          next instance to take
//   a CUDA graph   prep (reset barrier words, queue, results) + the
//                  cooperative sssp_batch launch, captured once
// Instances are ordered largest first so the groups finish close together.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "gbs_host.hpp"

using namespace gbs;

struct gbs_pack {
    uint32_t count = 0;
    gbs_weight_type wtype = GBS_WEIGHT_U32;
    int device = 0;
    int sms = 0;
    std::vector<uint32_t> n;
    std::vector<uint64_t> m;
    std::vector<double> max_w;
    std::vector<uint64_t> voff;   // count+1: first vertex of each graph in pack-wide arrays
    std::vector<uint64_t> eoff;   // count+1: first edge of each graph
    uint32_t *d_row = nullptr;    // graph i's n_i + 1 offsets start at voff[i] + i
    uint2 *d_adj = nullptr;
};

struct gbs_plan {
    int device = 0;
    bool f32 = false;
    uint32_t count = 0;
    uint32_t groups = 0, group_ctas = 0, blocks = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    InstDesc *d_inst = nullptr;
    InstResult *d_res = nullptr;
    Workspace *d_ws = nullptr;
    uint32_t *d_queue = nullptr;
    unsigned char *d_arena = nullptr;
    uint32_t *d_mid = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<InstResult> host_res;
    std::vector<uint32_t> order;   // position i of the queue holds caller instance order[i]
    bool launched = false;
};

namespace {

__global__ void k_batch_prep(const Workspace *__restrict__ ws, uint32_t groups, InstResult *__restrict__ res,
                             uint32_t count, uint32_t *__restrict__ queue) {
    for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x) {
        Ctl *c = ws[g].ctl;
        c->bar_count = 0u;
        for (int i = 0; i < 8; ++i) c->pubw[i] = 0ull;
        c->error = 0u;
        c->trace_n = 0u;
    }
    for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
        res[i].done = 0u;
        res[i].error = 0u;
    }
    if (threadIdx.x == 0) *queue = 0u;
}

void free_plan(gbs_plan *p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    cudaFree(p->d_inst);
    cudaFree(p->d_res);
    cudaFree(p->d_ws);
    cudaFree(p->d_queue);
    cudaFree(p->d_arena);
    cudaFree(p->d_mid);
    for (auto &e : p->ev) if (e) cudaEventDestroy(e);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

void free_pack(gbs_pack *p) {
    if (!p) return;
    cudaFree(p->d_row);
    cudaFree(p->d_adj);
    delete p;
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Bytes of one group's workspace for instances of at most n_cap vertices and
// m_cap edges; carve() lays it out in the same order.
size_t workspace_bytes(uint32_t n_cap, uint64_t m_cap, uint32_t *desc_cap) {
    const size_t n = n_cap ? n_cap : 1;
    const uint64_t cap = (uint64_t)n_cap + m_cap / kDescEdges + 64;
    *desc_cap = (uint32_t)std::min<uint64_t>(cap, 0xFFFFFFF0ull);
    size_t b = 0;
    b += align_up(8 * n);                 // dp
    b += 3 * align_up(4 * n);             // tag, fst, hst
    b += align_up(4 * n * kNB);           // ring
    b += align_up(4 * n * 3);             // fq
    b += align_up(4 * n * 2);             // pend
    b += 2 * align_up(16 * (size_t)*desc_cap);   // desc, hdesc
    b += align_up(sizeof(Ctl));
    return b;
}

Workspace carve(unsigned char *base, uint32_t n_cap, uint32_t desc_cap) {
    const size_t n = n_cap ? n_cap : 1;
    Workspace w{};
    size_t o = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + o;
        o += align_up(bytes);
        return p;
    };
    w.dp = reinterpret_cast<unsigned long long *>(take(8 * n));
    w.tag = reinterpret_cast<uint32_t *>(take(4 * n));
    w.fst = reinterpret_cast<uint32_t *>(take(4 * n));
    w.hst = reinterpret_cast<uint32_t *>(take(4 * n));
    w.ring = reinterpret_cast<uint32_t *>(take(4 * n * kNB));
    w.fq = reinterpret_cast<uint32_t *>(take(4 * n * 3));
    w.pend = reinterpret_cast<uint32_t *>(take(4 * n * 2));
    w.desc = reinterpret_cast<uint4 *>(take(16 * (size_t)desc_cap));
    w.hdesc = reinterpret_cast<uint4 *>(take(16 * (size_t)desc_cap));
    w.ctl = reinterpret_cast<Ctl *>(take(sizeof(Ctl)));
    w.desc_cap = desc_cap;
    w.n_cap = n_cap;
    w.mid = nullptr;
    w.trace = nullptr;
    w.trace_cap = 0;
    return w;
}

// CTAs per group: one group per instance, as long as the groups' distance
// words (8 bytes per vertex, the target of every random access of a
// relaxation) fit in L2 together; beyond that, fewer and wider groups.  On
// R-MAT 22 (33.5 MB per group) 64 groups of 2 CTAs run 2.2x slower than 4
// groups of 38.
uint32_t auto_group_ctas(uint32_t count, uint32_t blocks, uint32_t n_cap, size_t l2_bytes) {
    const size_t per_group = std::max<size_t>(8ull * n_cap, 1);
    const size_t fit = std::max<size_t>((l2_bytes + per_group / 2) / per_group, 1);   // rounded
    const uint32_t groups = (uint32_t)std::min<size_t>({fit, (size_t)std::max(count, 1u), (size_t)blocks});
    return std::max(1u, blocks / groups);
}

// Common part of both plan kinds: groups, arena, instance table, capture.
gbs_status build_plan(gbs_plan *p, const gbs_batch_params *bp, int sms, uint32_t n_cap, uint64_t m_cap,
                      std::vector<InstDesc> &inst) {
    p->count = (uint32_t)inst.size();
    const int per_sm = persistent_ctas_per_sm(p->f32 ? GBS_WEIGHT_F32 : GBS_WEIGHT_U32, true);
    if (per_sm < 1) return fail(GBS_ERR_UNSUPPORTED, "batched kernel cannot be resident");
    const uint32_t max_blocks = (uint32_t)(per_sm * sms);
    int dev = 0, l2 = 0;
    GBS_CUDA(cudaGetDevice(&dev));
    GBS_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
    uint32_t gc = (bp && bp->group_ctas) ? bp->group_ctas : auto_group_ctas(p->count, max_blocks, n_cap, (size_t)l2);
    gc = std::min(gc, max_blocks);
    uint32_t groups = std::min(max_blocks / gc, p->count);
    uint32_t desc_cap = 0;
    const size_t ws_bytes = workspace_bytes(n_cap, m_cap, &desc_cap);
    // keep the arena within 60% of the free device memory
    size_t free_b = 0, total_b = 0;
    GBS_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t budget = free_b / 10 * 6;
    if (ws_bytes > budget) return fail(GBS_ERR_NO_MEMORY, "one group workspace exceeds the free device memory");
    groups = (uint32_t)std::min<size_t>(groups, budget / ws_bytes);
    p->group_ctas = gc;
    p->groups = groups;
    p->blocks = gc * groups;
    GBS_CUDA(cudaMalloc(&p->d_arena, ws_bytes * groups));
    GBS_CUDA(cudaMemsetAsync(p->d_arena, 0, ws_bytes * groups, p->stream));
    std::vector<Workspace> ws(groups);
    for (uint32_t g = 0; g < groups; ++g) ws[g] = carve(p->d_arena + ws_bytes * g, n_cap, desc_cap);
    GBS_CUDA(cudaMalloc(&p->d_ws, sizeof(Workspace) * groups));
    GBS_CUDA(cudaMemcpyAsync(p->d_ws, ws.data(), sizeof(Workspace) * groups, cudaMemcpyHostToDevice, p->stream));
    GBS_CUDA(cudaMalloc(&p->d_inst, sizeof(InstDesc) * p->count));
    GBS_CUDA(cudaMemcpyAsync(p->d_inst, inst.data(), sizeof(InstDesc) * p->count, cudaMemcpyHostToDevice,
                             p->stream));
    GBS_CUDA(cudaMalloc(&p->d_res, sizeof(InstResult) * p->count));
    GBS_CUDA(cudaMemsetAsync(p->d_res, 0, sizeof(InstResult) * p->count, p->stream));
    GBS_CUDA(cudaMalloc(&p->d_queue, sizeof(uint32_t)));
    GBS_CUDA(cudaStreamSynchronize(p->stream));
    p->host_res.resize(p->count);

    SsspArgs a{};
    a.flags = bp ? (bp->flags & (GBS_F_NO_SOLO | GBS_F_NO_FUSE | GBS_F_TEST_STALL)) : 0u;
    a.fuse_rounds = (a.flags & GBS_F_NO_FUSE) ? 0u : ((bp && bp->fuse_rounds) ? bp->fuse_rounds : kFuseRounds);
    const bool no_solo = (a.flags & GBS_F_NO_SOLO) != 0;
    a.solo_items = no_solo ? 0u : ((bp && bp->solo_entries) ? bp->solo_entries : 1024u);
    a.solo_desc = no_solo ? 0u : ((bp && bp->solo_descs) ? bp->solo_descs : 64u);
    a.wait_ns = (unsigned long long)((bp && bp->wait_limit_ms) ? bp->wait_limit_ms : 4000u) * 1000000ull;
    a.run_ns = a.wait_ns * 16ull;
    a.inline_max = (bp && bp->inline_edges) ? bp->inline_edges : kInlineEdges;
    a.full_items = split_full_items(n_cap);
    a.group_ctas = gc;
    a.inst = p->d_inst;
    a.res = p->d_res;
    a.inst_count = p->count;
    a.queue = p->d_queue;

    // capture: prep + cooperative persistent launch
    GBS_CUDA(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    k_batch_prep<<<1, 256, 0, p->stream>>>(p->d_ws, groups, p->d_res, p->count, p->d_queue);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(p->blocks);
        cfg.blockDim = dim3(kTPB);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = p->stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        const Workspace *wsp = p->d_ws;
        e = p->f32 ? cudaLaunchKernelEx(&cfg, sssp_batch<kWF32>, a, wsp)
                   : cudaLaunchKernelEx(&cfg, sssp_batch<kWU32>, a, wsp);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e_end = cudaStreamEndCapture(p->stream, &graph);
    if (e != cudaSuccess || e_end != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return fail(GBS_ERR_CUDA, std::string("capturing the batched launch: ") +
                                      cudaGetErrorString(e != cudaSuccess ? e : e_end));
    }
    p->graph = graph;
    GBS_CUDA(cudaGraphInstantiate(&p->exec, p->graph, 0));
    GBS_CUDA(cudaGraphUpload(p->exec, p->stream));
    return GBS_OK;
}

gbs_status new_plan(int device, bool f32, gbs_plan **out) {
    gbs_plan *p = new gbs_plan();
    p->device = device;
    p->f32 = f32;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&p->ev[0])) != cudaSuccess || (e = cudaEventCreate(&p->ev[1])) != cudaSuccess) {
        free_plan(p);
        return fail(GBS_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = p;
    return GBS_OK;
}

bool no_split(const gbs_batch_params *bp) { return bp && std::isinf(bp->light) && bp->light > 0; }

Resolved schedule_of(const gbs_batch_params *bp, gbs_weight_type wt, double max_w, uint32_t n, uint64_t m) {
    double delta = (bp && bp->delta > 0) ? bp->delta : 0.0;
    if (!(delta > 0)) {
        const double scale = (bp && bp->delta_scale > 0) ? bp->delta_scale : 1.0;
        delta = default_delta(max_w, n, m) * scale;
    }
    const double light = no_split(bp) ? INFINITY : ((bp && bp->light >= 0) ? bp->light : -1.0);
    return resolve_schedule(wt, max_w, n, m, delta, light);
}

}  // namespace

extern "C" {

gbs_status gbs_pack_create(uint32_t count, const gbs_csr_view *graphs, gbs_weight_type wtype, gbs_pack **out) {
    if (!out) return fail(GBS_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (count == 0 || !graphs) return fail(GBS_ERR_INVALID_ARG, "empty pack");
    if (wtype != GBS_WEIGHT_U32 && wtype != GBS_WEIGHT_F32)
        return fail(GBS_ERR_UNSUPPORTED, "packs take uint32 or float32 graphs");
    gbs_pack *p = new gbs_pack();
    p->count = count;
    p->wtype = wtype;
    p->n.resize(count);
    p->m.resize(count);
    p->max_w.resize(count);
    p->voff.assign(count + 1, 0);
    p->eoff.assign(count + 1, 0);
    for (uint32_t i = 0; i < count; ++i) {
        p->voff[i + 1] = p->voff[i] + graphs[i].n;
        p->eoff[i + 1] = p->eoff[i] + graphs[i].m;
    }
    const uint64_t total_rows = p->voff[count] + count;
    const uint64_t total_m = p->eoff[count];
    cudaError_t e;
    if ((e = cudaGetDevice(&p->device)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device)) != cudaSuccess ||
        (e = cudaMalloc(&p->d_row, sizeof(uint32_t) * total_rows)) != cudaSuccess ||
        (e = cudaMalloc(&p->d_adj, sizeof(uint2) * std::max<uint64_t>(total_m, 1))) != cudaSuccess) {
        free_pack(p);
        return fail(e == cudaErrorMemoryAllocation ? GBS_ERR_NO_MEMORY : GBS_ERR_CUDA, cudaGetErrorString(e));
    }
    std::vector<uint32_t> row32;
    std::vector<uint2> adj;
    for (uint32_t i = 0; i < count; ++i) {
        const gbs_csr_view &v = graphs[i];
        gbs_status st = prepare_csr(v.n, v.m, v.row_offsets, v.cols, v.weights, wtype, row32, adj, p->max_w[i]);
        if (st != GBS_OK) {
            free_pack(p);
            return fail(st, "pack graph " + std::to_string(i) + ": " + gbs_last_error());
        }
        p->n[i] = v.n;
        p->m[i] = v.m;
        if ((e = cudaMemcpy(p->d_row + p->voff[i] + i, row32.data(), sizeof(uint32_t) * (v.n + 1),
                            cudaMemcpyHostToDevice)) != cudaSuccess ||
            (v.m && (e = cudaMemcpy(p->d_adj + p->eoff[i], adj.data(), sizeof(uint2) * v.m,
                                    cudaMemcpyHostToDevice)) != cudaSuccess)) {
            free_pack(p);
            return fail(GBS_ERR_CUDA, cudaGetErrorString(e));
        }
    }
    *out = p;
    return GBS_OK;
}

gbs_status gbs_pack_destroy(gbs_pack *p) {
    if (!p) return fail(GBS_ERR_INVALID_ARG, "pack is NULL");
    cudaDeviceSynchronize();
    free_pack(p);
    return GBS_OK;
}

gbs_status gbs_pack_info(const gbs_pack *p, uint32_t *count, uint64_t *total_n, uint64_t *total_m,
                         uint64_t *vertex_offsets) {
    if (!p) return fail(GBS_ERR_INVALID_ARG, "pack is NULL");
    if (count) *count = p->count;
    if (total_n) *total_n = p->voff[p->count];
    if (total_m) *total_m = p->eoff[p->count];
    if (vertex_offsets) std::copy(p->voff.begin(), p->voff.end(), vertex_offsets);
    return GBS_OK;
}

gbs_status gbs_plan_sources(gbs_graph *g, const uint32_t *sources, uint32_t k, const gbs_batch_params *params,
                            void *dist_dev, int32_t *pred_dev, gbs_plan **out) {
    if (!out) return fail(GBS_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!g || !sources || k == 0) return fail(GBS_ERR_INVALID_ARG, "graph, sources and k > 0 are required");
    if (g->wtype == GBS_WEIGHT_F64) return fail(GBS_ERR_UNSUPPORTED, "plans take uint32 or float32 graphs");
    for (uint32_t i = 0; i < k; ++i)
        if (sources[i] >= g->n) return fail(GBS_ERR_INVALID_ARG, "source out of range");
    gbs_plan *p = nullptr;
    gbs_status st = new_plan(g->device, g->wtype == GBS_WEIGHT_F32, &p);
    if (st != GBS_OK) return st;
    const Resolved r = schedule_of(params, g->wtype, g->max_w, g->n, g->m);
    const bool no_heavy = r.light_bits >= max_weight_bits(g->wtype, g->max_w);
    const uint32_t *mid = g->d_row + 1;   // no split: the first heavy edge is the row end
    if (!no_heavy) {
        cudaError_t e = cudaMalloc(&p->d_mid, sizeof(uint32_t) * g->n);
        if (e != cudaSuccess) {
            free_plan(p);
            return fail(GBS_ERR_NO_MEMORY, cudaGetErrorString(e));
        }
        st = launch_mid(g->d_row, g->d_adj, g->n, r.light_bits, p->d_mid, g->sms, p->stream);
        if (st != GBS_OK) {
            free_plan(p);
            return st;
        }
        mid = p->d_mid;
    }
    std::vector<InstDesc> inst(k);
    for (uint32_t i = 0; i < k; ++i) {
        InstDesc &d = inst[i];
        d.g.n = g->n;
        d.g.m = g->m;
        d.g.wtype = g->wtype;
        d.g.row = g->d_row;
        d.g.adj = g->d_adj;
        d.mid = mid;
        d.source = sources[i];
        d.delta_u = r.delta_u;
        d.inv_delta_f = r.inv_delta_f;
        d.no_heavy = no_heavy ? 1u : 0u;
        d.dist = dist_dev ? static_cast<uint32_t *>(dist_dev) + (size_t)i * g->n : nullptr;
        d.pred = pred_dev ? pred_dev + (size_t)i * g->n : nullptr;
    }
    st = build_plan(p, params, g->sms, g->n, g->m, inst);
    if (st != GBS_OK) {
        free_plan(p);
        return st;
    }
    *out = p;
    return GBS_OK;
}

gbs_status gbs_plan_pack(gbs_pack *pk, const uint32_t *sources, const gbs_batch_params *params, void *dist_dev,
                         int32_t *pred_dev, gbs_plan **out) {
    if (!out) return fail(GBS_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!pk || !sources) return fail(GBS_ERR_INVALID_ARG, "pack and sources are required");
    for (uint32_t i = 0; i < pk->count; ++i)
        if (sources[i] >= pk->n[i]) return fail(GBS_ERR_INVALID_ARG, "source out of range");
    gbs_plan *p = nullptr;
    gbs_status st = new_plan(pk->device, pk->wtype == GBS_WEIGHT_F32, &p);
    if (st != GBS_OK) return st;
    std::vector<InstDesc> inst(pk->count);
    bool any_split = false;
    std::vector<Resolved> rs(pk->count);
    std::vector<bool> nh(pk->count);
    for (uint32_t i = 0; i < pk->count; ++i) {
        rs[i] = schedule_of(params, pk->wtype, pk->max_w[i], pk->n[i], pk->m[i]);
        nh[i] = rs[i].light_bits >= max_weight_bits(pk->wtype, pk->max_w[i]);
        any_split = any_split || !nh[i];
    }
    if (any_split) {
        cudaError_t e = cudaMalloc(&p->d_mid, sizeof(uint32_t) * std::max<uint64_t>(pk->voff[pk->count], 1));
        if (e != cudaSuccess) {
            free_plan(p);
            return fail(GBS_ERR_NO_MEMORY, cudaGetErrorString(e));
        }
    }
    uint32_t n_cap = 0;
    uint64_t m_cap = 0;
    for (uint32_t i = 0; i < pk->count; ++i) {
        InstDesc &d = inst[i];
        const uint32_t *row = pk->d_row + pk->voff[i] + i;
        const uint2 *adj = pk->d_adj + pk->eoff[i];
        d.g.n = pk->n[i];
        d.g.m = pk->m[i];
        d.g.wtype = pk->wtype;
        d.g.row = row;
        d.g.adj = adj;
        if (nh[i]) {
            d.mid = row + 1;
        } else {
            uint32_t *mid = p->d_mid + pk->voff[i];
            st = launch_mid(row, adj, pk->n[i], rs[i].light_bits, mid, pk->sms, p->stream);
            if (st != GBS_OK) {
                free_plan(p);
                return st;
            }
            d.mid = mid;
        }
        d.source = sources[i];
        d.delta_u = rs[i].delta_u;
        d.inv_delta_f = rs[i].inv_delta_f;
        d.no_heavy = nh[i] ? 1u : 0u;
        d.dist = dist_dev ? static_cast<uint32_t *>(dist_dev) + pk->voff[i] : nullptr;
        d.pred = pred_dev ? pred_dev + pk->voff[i] : nullptr;
        n_cap = std::max(n_cap, pk->n[i]);
        m_cap = std::max(m_cap, pk->m[i]);
    }
    // largest first: the groups that take the big graphs start them early
    std::vector<uint32_t> order(pk->count);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return pk->m[x] > pk->m[y]; });
    std::vector<InstDesc> sorted(pk->count);
    for (uint32_t i = 0; i < pk->count; ++i) sorted[i] = inst[order[i]];
    st = build_plan(p, params, pk->sms, n_cap, m_cap, sorted);
    if (st != GBS_OK) {
        free_plan(p);
        return st;
    }
    p->order = order;
    *out = p;
    return GBS_OK;
}

gbs_status gbs_plan_launch(gbs_plan *p) {
    if (!p) return fail(GBS_ERR_INVALID_ARG, "plan is NULL");
    GBS_CUDA(cudaEventRecord(p->ev[0], p->stream));
    GBS_CUDA(cudaGraphLaunch(p->exec, p->stream));
    GBS_CUDA(cudaEventRecord(p->ev[1], p->stream));
    p->launched = true;
    return GBS_OK;
}

gbs_status gbs_plan_wait(gbs_plan *p, gbs_batch_stats *stats, gbs_inst_stats *per_instance) {
    if (!p) return fail(GBS_ERR_INVALID_ARG, "plan is NULL");
    if (!p->launched) return fail(GBS_ERR_INVALID_ARG, "plan was not launched");
    GBS_CUDA(cudaStreamSynchronize(p->stream));
    GBS_CUDA(cudaMemcpy(p->host_res.data(), p->d_res, sizeof(InstResult) * p->count, cudaMemcpyDeviceToHost));
    static_assert(sizeof(InstResult) == sizeof(gbs_inst_stats), "InstResult layout = gbs_inst_stats");
    uint32_t completed = 0, max_phases = 0, first_err = 0;
    uint64_t phases = 0, reached = 0, edges = 0;
    for (uint32_t i = 0; i < p->count; ++i) {
        const InstResult &r = p->host_res[i];
        completed += r.done ? 1u : 0u;
        if (r.error && !first_err) first_err = r.error;
        if (r.done) {
            phases += r.phases;
            max_phases = std::max(max_phases, r.phases);
            reached += r.reached;
            edges += r.edges_reached;
        }
    }
    if (per_instance) {
        // back in the caller's instance order
        for (uint32_t i = 0; i < p->count; ++i) {
            const uint32_t dst = p->order.empty() ? i : p->order[i];
            std::memcpy(&per_instance[dst], &p->host_res[i], sizeof(gbs_inst_stats));
        }
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        float ms = 0.f;
        GBS_CUDA(cudaEventElapsedTime(&ms, p->ev[0], p->ev[1]));
        stats->device_ms = ms;
        stats->instances = p->count;
        stats->completed = completed;
        stats->groups = p->groups;
        stats->group_ctas = p->group_ctas;
        stats->blocks = p->blocks;
        stats->max_phases = max_phases;
        stats->phases = phases;
        stats->reached = reached;
        stats->edges_reached = edges;
    }
    switch (first_err) {
        case kErrNone: break;
        case kErrTimeout: return fail(GBS_ERR_TIMEOUT, "device-side wait limit exceeded");
        case kErrCapacity: return fail(GBS_ERR_CAPACITY, "device work list overflow");
        case kErrOverflow: return fail(GBS_ERR_OVERFLOW, "uint32 path sum overflow");
        default: return fail(GBS_ERR_INTERNAL, "device error");
    }
    if (completed < p->count) return fail(GBS_ERR_TIMEOUT, "instances left unsolved (a group stopped)");
    return GBS_OK;
}

gbs_status gbs_plan_destroy(gbs_plan *p) {
    if (!p) return fail(GBS_ERR_INVALID_ARG, "plan is NULL");
    cudaStreamSynchronize(p->stream);
    free_plan(p);
    return GBS_OK;
}

}  // extern "C"
