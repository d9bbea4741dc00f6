"""The learned bucket-width controller.

CPU: the oracle's analytic gradient agrees with finite differences (so it can
check the CUDA kernels), and the committed parameter block is well formed.
GPU: the CUDA forward/backward kernels' loss and gradient equal the oracle's
within FP32 tolerance; an Adam step equals the oracle's; training lowers the
loss; learned runs are bit-identical to plain ones, the guard falls back to
the plain schedule, the trained controller beats the plain fixed delta on
held-out graphs, and the output-bias calibration adds the best pair it timed."""
import numpy as np
import pytest

from oracle import mlp as ref

# FP32 kernels against a float64 restatement, relative to the largest entry
GRAD_RTOL = 2e-4


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(3.0, 2.0, size=(n, 16)).astype(np.float32)
    t = np.stack([rng.normal(1.0, 2.0, n), rng.integers(0, 2, n)], axis=1).astype(np.float32)
    w = rng.uniform(0.5, 2.0, n).astype(np.float32)
    return x, t, w


def test_oracle_gradient_matches_finite_differences():
    x, t, w = _data(40, 1)
    p = ref.init_params(3, mu=x.mean(0), sd=x.std(0) + 1e-3).astype(np.float64)
    _, g = ref.loss_grad(p, x, t, w)
    rng = np.random.default_rng(0)
    for k in rng.choice(len(g), 60, replace=False):
        e = np.zeros_like(p)
        e[ref.OFF_W1 + k] = 1e-6
        num = (ref.loss_grad(p + e, x, t, w)[0] - ref.loss_grad(p - e, x, t, w)[0]) / 2e-6
        assert abs(num - g[k]) <= 1e-6 + 1e-4 * abs(g[k]), (k, num, g[k])


def test_committed_controller_block(gb):
    from graphbench_gb300 import controller
    p = controller.load()
    assert p.shape == (gb.MLP_FLOATS,) and p.dtype == np.float32
    assert np.all(np.isfinite(p)) and np.all(p[16:32] > 0)


def test_label_curve_spreads_bucket_time_over_settled_vertices(gb):
    """The per-bucket labels compare schedules by the time each needs to
    settle a window of distances: a bucket's time is spread over the
    vertices it settles (their final distances are the same for every
    schedule), and flat over distances no bucket held."""
    from graphbench_gb300 import controller as c
    trace = [{"kind": "scan_bucket", "bucket": 0, "end_ns": 10}, {"kind": "relax", "bucket": 0, "end_ns": 20},
             {"kind": "scan_bucket", "bucket": 1, "end_ns": 30}, {"kind": "scan_light", "bucket": 1, "end_ns": 40},
             {"kind": "scan_bucket", "bucket": 4, "end_ns": 55}]
    curve = c.bucket_curve(trace, 2.0)
    assert curve.tolist() == [[0, 2, 0, 20], [2, 4, 20, 40], [8, 10, 40, 55]]
    fin = np.array([0.0, 0.5, 0.6, 2.5, 3.9, 9.0])
    settled = lambda d: np.searchsorted(fin, d, side="left").astype(np.float64)
    t = c.time_at(curve, np.array([0.0, 0.55, 1.0, 3.0, 5.0, 8.5, 20.0]), settled)
    assert np.allclose(t, [0.0, 20 * 2 / 3, 20.0, 30.0, 40.0, 40.0, 55.0])
    x0 = c.initial_input(1023, [4.0, 8.0, 0.5])
    assert x0[6] == 10.0 and np.all(x0[:6] == 1) and np.all(x0[7:12] == 0) and x0[15] == 0


@pytest.mark.gpu
def test_cuda_loss_and_gradient_match_oracle(gb):
    x, t, w = _data(1000, 2)
    p = ref.init_params(5, mu=x.mean(0), sd=x.std(0) + 1e-3)
    m = gb.Mlp(p)
    m.set_data(x, t, w)
    for first, count in [(0, 1000), (17, 300), (999, 1)]:
        loss, g = m.loss_grad(first, count)
        rl, rg = ref.loss_grad(p, x[first:first + count], t[first:first + count], w[first:first + count])
        assert abs(loss - rl) <= 1e-5 * max(1.0, abs(rl))
        assert np.max(np.abs(g - rg)) <= GRAD_RTOL * np.max(np.abs(rg)), (first, count)
    y = m.predict(x[:50])
    ry, _ = ref.forward(p, x[:50])
    assert np.max(np.abs(y - ry)) <= 1e-4 * max(1.0, np.max(np.abs(ry)))
    m.close()


@pytest.mark.gpu
def test_cuda_adam_step_matches_oracle(gb):
    x, t, w = _data(256, 4)
    p = ref.init_params(7, mu=x.mean(0), sd=x.std(0) + 1e-3)
    m = gb.Mlp(p)
    m.set_data(x, t, w)
    mom = np.zeros(gb.MLP_PARAMS)
    vel = np.zeros(gb.MLP_PARAMS)
    rp = p.astype(np.float64)
    for step in range(1, 4):
        m.loss_grad()
        m.adam(1e-2)
        _, rg = ref.loss_grad(rp, x, t, w)
        rp, mom, vel = ref.adam(rp, rg, mom, vel, step, 1e-2)
    got = m.params().astype(np.float64)
    assert np.max(np.abs(got - rp)) <= 1e-4 * max(1.0, np.max(np.abs(rp)))
    m.close()


@pytest.mark.gpu
def test_cuda_training_lowers_loss(gb):
    rng = np.random.default_rng(9)
    x = rng.normal(0, 1, size=(4096, 16)).astype(np.float32)
    t = np.stack([x[:, 0] * 2 - x[:, 3], (x[:, 5] > 0)], axis=1).astype(np.float32)
    m = gb.Mlp(ref.init_params(1))
    m.set_data(x, t)
    losses = m.train(epochs=30, batch=256, lr=3e-3, seed=1)
    assert losses[-1] < 0.2 * losses[0], losses[[0, -1]]
    m.close()


def _learned_graph(gb, host):
    from graphbench_gb300 import controller
    g = gb.Graph.from_host(host)
    g.set_controller(controller.load())
    return g


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["rmat", "grid"])
def test_learned_runs_bit_identical_to_plain(kind, gb, orc):
    host = gb.gen_rmat(13, 16, 31) if kind == "rmat" else gb.gen_grid(128, 160, 8, "f32")
    srcs = gb.sample_sources(host, 4, 3) if kind == "rmat" else [0, 77]
    with _learned_graph(gb, host) as g:
        for s in srcs:
            d, p, st = g.sssp(int(s), flags=gb.F_LEARNED | gb.F_TRACE)
            assert st["learned"] & 1
            tr = g.trace()
            assert all(1 <= r["span"] <= 64 for r in tr)
            d0, p0, _ = g.sssp(int(s))
            assert np.array_equal(d, d0) and np.array_equal(p, p0)
            assert np.array_equal(d, orc.dijkstra(host.row, host.col, host.w, int(s)))


@pytest.mark.gpu
def test_feature_recording(gb):
    a = gb.gen_rmat(11, 16, 4)
    with gb.Graph.from_host(a) as g:
        _, _, st = g.sssp(0, flags=gb.F_FEATURES)
        f = g.features()
    # one row per bucket start after bucket 0, whose width the host picks
    assert len(f) == st["buckets"] - 1 and f.shape[1] == gb.N_FEAT
    assert np.all(np.isfinite(f))
    assert np.all(np.diff(f[:, 8]) > 0)             # log2(1 + distance in plain widths) grows
    assert np.all(f[:, 11] <= 0)                    # log2 share of the window in the next bucket


@pytest.mark.gpu
def test_learned_guard_falls_back_to_plain(gb, orc):
    """A controller that always asks for the finest width it may (1/8 of the
    plain one: half of its clamped first prediction, 2^-2) on a grid,
    where wide buckets pay: the learned run passes its
    guard ((1 + margin) x the plain time), stops, and the plain schedule gives
    the result."""
    from graphbench_gb300 import controller
    host = gb.gen_grid(96, 96, 2, "f32")
    p = controller.load().copy()
    p[ref.OFF_W3:ref.OFF_B3] = 0.0
    p[ref.OFF_B3] = -30.0      # y0: log2(width / plain width)
    with gb.Graph.from_host(host) as g:
        g.set_controller(p, margin=1e-6)
        d, pr, st = g.sssp(0, flags=gb.F_LEARNED)   # first: times the plain schedule
        assert st["learned"] == 3
        d2, _, st2 = g.sssp(0, flags=gb.F_LEARNED)
        assert st2["learned"] == 2                  # lost here before: plain directly
        assert st["kernel_ms"] > st2["kernel_ms"]    # the first call paid for three runs
    ref_d = orc.dijkstra(host.row, host.col, host.w, 0)
    assert np.array_equal(d, ref_d) and np.array_equal(d2, ref_d)
    assert np.array_equal(pr, orc.min_tight_pred(host.row, host.col, host.w, 0, ref_d))


@pytest.mark.gpu
def test_learned_guard_longer_source_is_not_a_loss(gb, orc):
    """The guard's plain time comes from the first source.  A later source
    whose plain run alone exceeds the limit stops its learned run, but that is
    not a loss: the limit rises to that plain time and the next learned call
    runs the controller.  Graph: a 4-vertex path (timed first) beside a 200^2
    grid."""
    from graphbench_gb300 import controller
    grid = gb.gen_grid(200, 200, 5, "f32")
    gr = grid.row.astype(np.int64)
    row = np.concatenate([[0, 1, 3, 5], 6 + gr]).astype(np.uint32)
    col = np.concatenate([[1, 0, 2, 1, 3, 2], grid.col.astype(np.int64) + 4]).astype(np.uint32)
    w = np.concatenate([np.full(6, 2.0, np.float32), grid.w]).astype(np.float32)
    src = 4 + 200 * 100 + 100
    with gb.Graph(row, col, w) as g:
        g.set_controller(controller.load(), margin=10.0)
        _, _, st0 = g.sssp(0, flags=gb.F_LEARNED)      # times plain on the path
        assert st0["learned"] == 1
        d1, _, st1 = g.sssp(src, flags=gb.F_LEARNED)   # passes 11x the path's time
        assert st1["learned"] == 3
        d2, _, st2 = g.sssp(src, flags=gb.F_LEARNED)
        assert st2["learned"] == 1                     # not lost: the controller runs
    ref_d = orc.dijkstra(row, col, w, src)
    assert np.array_equal(d1, ref_d) and np.array_equal(d2, ref_d)


@pytest.mark.gpu
def test_trained_controller_beats_plain_on_held_out_graphs(gb):
    """The committed controller on graphs and seeds outside its training set
    (a 768^2 grid, R-MAT 18 and R-MAT 20 with held-out seeds): total
    kernel time of learned runs below the plain fixed delta's (a call whose
    learned run fell back is charged both runs)."""
    cases = [(gb.gen_grid(768, 768, 97, "f32"), [0]), (gb.gen_rmat(18, 16, 77), None),
             (gb.gen_rmat(20, 16, 5), None)]
    for host, srcs in cases:
        srcs = srcs if srcs is not None else [int(s) for s in gb.sample_sources(host, 6, 5)]
        with _learned_graph(gb, host) as g:
            g.sssp(srcs[0], flags=gb.F_LEARNED)   # plain timing + warm-up
            g.sssp(srcs[0])
            plain = learned = 0.0
            for s in srcs:
                for _ in range(2):
                    _, _, a = g.sssp(s, want_dist=False, want_pred=False)
                    _, _, b = g.sssp(s, want_dist=False, want_pred=False, flags=gb.F_LEARNED)
                    plain += a["kernel_ms"]
                    learned += b["kernel_ms"]   # includes any abandoned run
            assert learned < plain, (host.n, learned, plain)


@pytest.mark.gpu
@pytest.mark.parametrize("spec", [{"kind": "rmat", "scale": 12, "seed": 41}, {"kind": "grid", "side": 128, "seed": 42}])
def test_collect_graph_labels(spec, gb):
    """collect_graph: every (width, split) schedule of a small sweep runs with
    its trace and inputs; the samples are the initial state plus one per
    recorded bucket start, the width labels come from the sweep, the split
    labels are 0 / 1, and the weights sum to 1."""
    from graphbench_gb300 import controller
    c = controller.collect_graph(spec, sweep_k=(-1, 0, 1, 2), cap=500, seed=3)
    x, t, w = c["x"], c["t"], c["w"]
    assert x.shape[1] == gb.N_FEAT and len(x) == len(t) == len(w) >= 2
    assert set(np.unique(t[1:, 0])) <= {-1.0, 0.0, 1.0, 2.0}
    assert set(np.unique(t[:, 1])) <= {0.0, 1.0}
    assert abs(float(w.sum()) - 1.0) < 1e-5 and (w >= 0).all()
    bf = c["best_fixed"]
    assert bf["k"] in (-1, 0, 1, 2) and bf["split"] in (0, 1) and 0 < bf["ms"] <= bf["plain_ms"] * 1.5


@pytest.mark.gpu
def test_output_bias_calibration(gb):
    """calibrate() times every output-bias pair against plain on the given
    graphs and adds the best pair to the block (the rest of it unchanged)."""
    from graphbench_gb300 import controller
    p = controller.load()
    specs = [{"kind": "rmat", "scale": 12, "seed": 31}, {"kind": "grid", "side": 128, "seed": 32}]
    seen = []
    q, rep = controller.calibrate(p, specs, shifts=(0, -2), split_bias=(0.0, -30.0), sources=2, log=seen.append)
    assert len(seen) == 2 and rep["graphs"] == 2 and len(rep["table"]) == 4
    assert rep["geomean_speedup"] == max(rep["table"].values())
    assert q[controller.B3] == p[controller.B3] + rep["width_shift"]
    assert q[controller.B3 + 1] == p[controller.B3 + 1] + rep["split_shift"]
    assert np.array_equal(q[:controller.B3], p[:controller.B3])
