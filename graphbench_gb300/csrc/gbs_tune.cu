// gbs_tune.cu -- the schedule autotuner (gbs_autotune, gbs_autotune_plan_*).
//
// Host-only: candidates run through the public entry points and are timed by
// the kernel's CUDA events (single source: kernel_ms, the persistent launch
// alone; batched: the graph launch).  The result of any schedule is the same
// least fixpoint, so the search only compares times.
#include <algorithm>
#include <functional>
#include <cmath>
#include <cstring>
#include <vector>

#include "gbs_host.hpp"

using namespace gbs;

namespace {

// Width multipliers 2^e of the default width: a coarse pass over kCoarse,
// then the neighbours of the best; knob values explored around the best.
const int kCoarse[] = {0, 3, 6, 9, 12};
const int kMinExp = -3, kMaxExp = 14;
const uint32_t kInline[] = {8, 16, 64, 128};
const uint32_t kSoloEntries[] = {256, 4096, 16384};
const uint32_t kSoloDescs[] = {16, 256, 1024};
// Bucket fusion rounds besides the default: wide buckets hold longer light
// chains (4096^2 grid at 64 plain widths: 2 rounds 89 ms, 8 rounds 80 ms).
const uint32_t kFuse[] = {1, 4, 8, 16};
// A single-source candidate replaces the incumbent only when it is 2 %
// faster: the mean of a few sources moves by about that between runs, and a
// schedule picked on noise measured 0.99x of the default on the next 20
// sources (R-MAT 22).
constexpr double kWin = 0.98;

struct Budget {
    double limit_ms, used_ms = 0.0;
    bool left() const { return used_ms < limit_ms; }
};

// Mean kernel time per source of one schedule (one untimed warm-up run).
gbs_status time_single(gbs_graph *g, const std::vector<uint32_t> &src, const gbs_params &p, Budget &b,
                       uint32_t &runs, double &mean_ms) {
    gbs_stats st;
    gbs_params q = p;
    q.flags |= GBS_F_NO_STATS;
    gbs_status s = gbs_sssp_device(g, src[0], &q, nullptr, nullptr, &st);
    if (s != GBS_OK) return s;
    ++runs;
    b.used_ms += st.kernel_ms;
    double sum = 0.0;
    for (uint32_t x : src) {
        s = gbs_sssp_device(g, x, &q, nullptr, nullptr, &st);
        if (s != GBS_OK) return s;
        ++runs;
        sum += st.kernel_ms;
        b.used_ms += st.kernel_ms;
    }
    mean_ms = sum / (double)src.size();
    return GBS_OK;
}

}  // namespace

extern "C" {

gbs_status gbs_autotune(gbs_graph *g, const uint32_t *sources, uint32_t count, double budget_ms,
                        gbs_tune_report *out) {
    if (!g || !sources || count == 0 || !out) return fail(GBS_ERR_INVALID_ARG, "graph, sources and out are required");
    std::vector<uint32_t> src(sources, sources + count);
    for (uint32_t x : src)
        if (x >= g->n) return fail(GBS_ERR_INVALID_ARG, "source out of range");
    Budget b{budget_ms > 0 ? budget_ms : 4000.0};
    std::memset(out, 0, sizeof(*out));
    const double d0 = default_delta(g->max_w, g->n, g->m);
    gbs_params base{};
    base.light = -1.0;
    double best_ms = 0.0;
    gbs_status s = time_single(g, src, base, b, out->runs, best_ms);
    if (s != GBS_OK) return s;
    out->default_ms = best_ms;
    out->candidates = 1;
    gbs_params best = base;
    best.delta = d0;
    double best_scale = 1.0;
    bool best_nosplit = true;   // the default relaxes every bucket whole
    // 1. width with and without the light/heavy split of the large buckets:
    //    coarse exponents, then the neighbours of the best one (one and two
    //    steps on each side, twice)
    for (int split = 0; split < 2 && b.left(); ++split) {
        std::vector<std::pair<int, double>> seen;   // (exponent, ms)
        auto eval = [&](int e) -> gbs_status {
            if (e < kMinExp || e > kMaxExp || !b.left()) return GBS_OK;
            for (auto &q : seen)
                if (q.first == e) return GBS_OK;
            double ms = 0.0;
            if (split == 0 && e == 0) {
                ms = out->default_ms;   // the default, timed above
            } else {
                gbs_params p = base;
                p.delta = d0 * std::ldexp(1.0, e);
                if (split) p.full_items = split_full_items(g->n);
                gbs_status r = time_single(g, src, p, b, out->runs, ms);
                if (r != GBS_OK) return r;
                ++out->candidates;
                if (ms < best_ms * kWin) {
                    best_ms = ms;
                    best = p;
                    best_scale = std::ldexp(1.0, e);
                    best_nosplit = split == 0;
                }
            }
            seen.push_back({e, ms});
            return GBS_OK;
        };
        for (int e : kCoarse)
            if ((s = eval(e)) != GBS_OK) return s;
        for (int round = 0; round < 2 && !seen.empty(); ++round) {
            int be = seen[0].first;
            double bm = seen[0].second;
            for (auto &q : seen)
                if (q.second < bm) {
                    bm = q.second;
                    be = q.first;
                }
            for (int d : {-1, 1, -2, 2})
                if ((s = eval(be + d)) != GBS_OK) return s;
        }
    }
    // 2. the other knobs, one at a time around the best
    auto try_knob = [&](auto set) -> gbs_status {
        if (!b.left()) return GBS_OK;
        gbs_params p = best;
        set(p);
        double ms = 0.0;
        gbs_status r = time_single(g, src, p, b, out->runs, ms);
        if (r != GBS_OK) return r;
        ++out->candidates;
        if (ms < best_ms * kWin) {
            best_ms = ms;
            best = p;
        }
        return GBS_OK;
    };
    // 2. fusion rounds at the best width, then the widths next to it again
    //    with the rounds found
    {
        const gbs_params before = best;
        for (uint32_t v : kFuse)
            if ((s = try_knob([&](gbs_params &p) { p.fuse_rounds = v; })) != GBS_OK) return s;
        if (best.fuse_rounds != before.fuse_rounds) {
            const gbs_params at = best;
            for (double f : {0.5, 2.0}) {
                if (!b.left()) break;
                gbs_params p = at;
                p.delta = at.delta * f;
                double ms = 0.0;
                if ((s = time_single(g, src, p, b, out->runs, ms)) != GBS_OK) return s;
                ++out->candidates;
                if (ms < best_ms * kWin) {
                    best_ms = ms;
                    best = p;
                    best_scale *= f;
                }
            }
        }
    }
    // 3. the other knobs
    for (uint32_t v : kInline)
        if ((s = try_knob([&](gbs_params &p) { p.inline_edges = v; })) != GBS_OK) return s;
    for (uint32_t v : kSoloEntries)
        if ((s = try_knob([&](gbs_params &p) { p.solo_entries = v; })) != GBS_OK) return s;
    for (uint32_t v : kSoloDescs)
        if ((s = try_knob([&](gbs_params &p) { p.solo_descs = v; })) != GBS_OK) return s;
    // explicit values in the returned schedule
    if (!(best.delta > 0)) best.delta = d0;
    best.flags = 0;
    out->best = best;
    out->best_ms = best_ms;
    out->delta_scale = best_scale;
    out->no_split = best_nosplit ? 1 : 0;
    return GBS_OK;
}

}  // extern "C"

namespace {

// Creates a plan without outputs and runs it once; a run within `close_ms`
// is repeated and the faster of the two counts (a clear loser costs one run).
template <class Make>
gbs_status time_plan(Make make, const gbs_batch_params &bp, Budget &b, double close_ms, double &ms) {
    gbs_plan *plan = nullptr;
    gbs_status s = make(bp, &plan);
    if (s != GBS_OK) return s;
    gbs_batch_stats st;
    ms = INFINITY;
    for (int rep = 0; rep < 2; ++rep) {
        s = gbs_plan_launch(plan);
        if (s == GBS_OK) s = gbs_plan_wait(plan, &st, nullptr);
        if (s != GBS_OK) break;
        b.used_ms += st.device_ms;
        ms = std::min(ms, (double)st.device_ms);
        if (ms > close_ms) break;
    }
    gbs_plan_destroy(plan);
    return s;
}

// Search order: the seed schedule (when given) against the default at the
// automatic group shape; the group shape at the better of the two; the bucket
// width and split at the best shape (around the seed's width, or coarse
// exponents of the default width without a seed, then the neighbours of the
// best); the shapes next to the best one at the best schedule; the inline-row
// limit.  A candidate whose first run is 1.1x slower than the best so far is
// not run again.
template <class Make>
gbs_status tune_plan(Make make, uint32_t max_blocks, double budget_ms, const gbs_batch_params *seed,
                     gbs_batch_tune_report *out) {
    Budget b{budget_ms};
    std::memset(out, 0, sizeof(*out));
    gbs_batch_params base{};
    base.light = -1.0;
    double ms = 0.0;
    gbs_status s = time_plan(make, base, b, INFINITY, ms);
    if (s != GBS_OK) return s;
    out->default_ms = ms;
    out->candidates = 1;
    gbs_batch_params best = base;
    double best_ms = ms;
    auto consider = [&](const gbs_batch_params &p, double &t) -> gbs_status {
        t = INFINITY;
        if (!b.left()) return GBS_OK;
        gbs_status r = time_plan(make, p, b, 1.1 * best_ms, t);
        if (r == GBS_ERR_NO_MEMORY) return GBS_OK;   // a shape that does not fit is skipped
        if (r != GBS_OK) return r;
        ++out->candidates;
        if (t < best_ms) {
            best_ms = t;
            best = p;
        }
        return GBS_OK;
    };
    // width exponents e (delta_scale 2^e) for both splits around `shape`
    auto width_search = [&](const gbs_batch_params shape, const int *coarse, size_t n_coarse) -> gbs_status {
        for (int split = 0; split < 2; ++split) {
            std::vector<std::pair<int, double>> seen;
            auto eval = [&](int e) -> gbs_status {
                if (e < kMinExp || e > kMaxExp) return GBS_OK;
                for (auto &q : seen)
                    if (q.first == e) return GBS_OK;
                gbs_batch_params p = shape;
                p.delta_scale = std::ldexp(1.0, e);
                p.light = split ? INFINITY : -1.0;
                double t = 0.0;
                gbs_status r;
                const bool same = std::memcmp(&p, &best, sizeof(p)) == 0 ||
                                  (p.delta_scale == 1.0 && split == 0 && shape.delta_scale <= 0 &&
                                   shape.light < 0 && std::memcmp(&shape, &best, sizeof(p)) == 0);
                if (same) {
                    t = best_ms;
                } else if ((r = consider(p, t)) != GBS_OK) {
                    return r;
                }
                seen.push_back({e, t});
                return GBS_OK;
            };
            for (size_t i = 0; i < n_coarse; ++i)
                if ((s = eval(coarse[i])) != GBS_OK) return s;
            for (int round = 0; round < 2 && !seen.empty(); ++round) {
                int be = seen[0].first;
                double bm = seen[0].second;
                for (auto &q : seen)
                    if (q.second < bm) {
                        bm = q.second;
                        be = q.first;
                    }
                for (int d : {-1, 1})
                    if ((s = eval(be + d)) != GBS_OK) return s;
            }
        }
        return GBS_OK;
    };
    // 0. the seed
    if (seed) {
        double t;
        if ((s = consider(*seed, t)) != GBS_OK) return s;
    }
    // 1. CTAs per group (powers of two and the divisors of the SM count),
    //    widest first
    std::vector<uint32_t> shapes;
    for (uint32_t gc = 1; gc <= max_blocks; gc *= 2) shapes.push_back(gc);
    for (uint32_t d = 3; d <= max_blocks; ++d)
        if (max_blocks % d == 0 && (d & (d - 1)) != 0) shapes.push_back(d);
    std::sort(shapes.begin(), shapes.end(), std::greater<uint32_t>());
    const gbs_batch_params sched0 = best;
    for (uint32_t gc : shapes) {
        gbs_batch_params p = sched0;
        p.group_ctas = gc;
        double t;
        if ((s = consider(p, t)) != GBS_OK) return s;
    }
    // 2. schedule at the best shape
    if (seed) {
        const int e0 = seed->delta_scale > 0 ? (int)std::lround(std::log2(seed->delta_scale)) : 0;
        if ((s = width_search(best, &e0, 1)) != GBS_OK) return s;
    } else if ((s = width_search(best, kCoarse, sizeof(kCoarse) / sizeof(kCoarse[0]))) != GBS_OK) {
        return s;
    }
    // 3. the shapes next to the best one, at the best schedule
    if (best.group_ctas != 0) {
        const gbs_batch_params sched = best;
        const auto it = std::find(shapes.begin(), shapes.end(), sched.group_ctas);
        const size_t k = (size_t)(it - shapes.begin());
        for (size_t j : {k - 1, k + 1}) {
            if (it == shapes.end() || j >= shapes.size()) continue;
            gbs_batch_params p = sched;
            p.group_ctas = shapes[j];
            double t;
            if ((s = consider(p, t)) != GBS_OK) return s;
        }
    }
    // 4. inline-row limit and fusion rounds
    for (uint32_t v : kInline) {
        gbs_batch_params p = best;
        p.inline_edges = v;
        double t;
        if ((s = consider(p, t)) != GBS_OK) return s;
    }
    for (uint32_t v : kFuse) {
        gbs_batch_params p = best;
        p.fuse_rounds = v;
        double t;
        if ((s = consider(p, t)) != GBS_OK) return s;
    }
    out->best = best;
    out->best_ms = best_ms;
    return GBS_OK;
}

uint32_t batch_blocks(int device) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    return (uint32_t)std::max(1, persistent_ctas_per_sm(GBS_WEIGHT_U32, true) * sms);
}

}  // namespace

extern "C" {

gbs_status gbs_autotune_plan_sources(gbs_graph *g, const uint32_t *sources, uint32_t k, double budget_ms,
                                     gbs_batch_tune_report *out) {
    if (!g || !sources || k == 0 || !out) return fail(GBS_ERR_INVALID_ARG, "graph, sources and out are required");
    for (uint32_t i = 0; i < k; ++i)
        if (sources[i] >= g->n) return fail(GBS_ERR_INVALID_ARG, "source out of range");
    auto make = [&](const gbs_batch_params &bp, gbs_plan **plan) {
        return gbs_plan_sources(g, sources, k, &bp, nullptr, nullptr, plan);
    };
    // seed: the single-source tuner on (up to) two of the sources, with a
    // third of the budget; its width, split and knobs carry over to groups
    const double total = budget_ms > 0 ? budget_ms : 8000.0;
    gbs_tune_report sr;
    gbs_status s = gbs_autotune(g, sources, std::min(k, 2u), total / 3.0, &sr);
    if (s != GBS_OK) return s;
    gbs_batch_params seed{};
    seed.delta_scale = sr.delta_scale;
    seed.light = sr.no_split ? INFINITY : -1.0;
    seed.solo_entries = sr.best.solo_entries;
    seed.solo_descs = sr.best.solo_descs;
    seed.inline_edges = sr.best.inline_edges;
    seed.fuse_rounds = sr.best.fuse_rounds;
    return tune_plan(make, batch_blocks(g->device), total * 2.0 / 3.0, &seed, out);
}

gbs_status gbs_autotune_plan_pack(gbs_pack *pk, const uint32_t *sources, double budget_ms,
                                  gbs_batch_tune_report *out) {
    if (!pk || !sources || !out) return fail(GBS_ERR_INVALID_ARG, "pack, sources and out are required");
    int dev = 0;
    GBS_CUDA(cudaGetDevice(&dev));
    auto make = [&](const gbs_batch_params &bp, gbs_plan **plan) {
        return gbs_plan_pack(pk, sources, &bp, nullptr, nullptr, plan);
    };
    return tune_plan(make, batch_blocks(dev), budget_ms > 0 ? budget_ms : 4000.0, nullptr, out);
}

}  // extern "C"
