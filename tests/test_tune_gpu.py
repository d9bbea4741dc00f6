"""Autotuner (gbs_autotune, gbs_autotune_plan_*) and the knobs it turns.
Any schedule yields the same least fixpoint, so a tuned schedule must give
bit-identical distances and predecessors; the tuner reports the plain
heuristic's time beside the best, and the best is never slower than it."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(gb):
    assert gb.device_available(), "GPU tests need a CUDA device (compute capability 10.x)"


@pytest.mark.parametrize("inline_edges", [1, 8, 64, 200, 100000])
def test_inline_threshold_same_result(inline_edges, gb, orc):
    a = gb.gen_rmat(13, 16, 12)
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    with gb.Graph.from_host(a) as g:
        d, p, _ = g.sssp(src, inline_edges=inline_edges)
        d0, p0, _ = g.sssp(src)
    assert np.array_equal(d, d0) and np.array_equal(p, p0)
    assert np.array_equal(d, orc.dijkstra(a.row, a.col, a.w, src))


def test_autotune_single_source_rmat(gb):
    a = gb.gen_rmat(14, 16, 2)
    srcs = gb.sample_sources(a, 3, 5)
    with gb.Graph.from_host(a) as g:
        kw, rep = g.autotune(srcs, budget_ms=1500)
        assert rep["candidates"] >= 2 and rep["best_ms"] <= rep["default_ms"]
        assert kw["delta"] > 0
        for s in srcs:
            d, p, _ = g.sssp(int(s), **kw)
            d0, p0, _ = g.sssp(int(s))
            assert np.array_equal(d, d0) and np.array_equal(p, p0)


def test_autotune_grid_prefers_wider_buckets(gb, orc):
    """High-diameter grid: the plain width (max weight / degree 4) makes
    thousands of thin buckets; the tuner widens them."""
    a = gb.gen_grid(256, 256, 3, "f32")
    with gb.Graph.from_host(a) as g:
        kw, rep = g.autotune([0], budget_ms=3000)
        assert rep["delta_scale"] > 1.0
        assert rep["best_ms"] < rep["default_ms"]
        d, p, _ = g.sssp(0, **kw)
    ref = orc.dijkstra(a.row, a.col, a.w, 0)
    assert np.array_equal(d, ref)
    assert np.array_equal(p, orc.min_tight_pred(a.row, a.col, a.w, 0, ref))


def test_autotune_plan_sources_and_pack(gb):
    a = gb.gen_rmat(11, 16, 3)
    srcs = gb.sample_sources(a, 12, 9)
    with gb.Graph.from_host(a) as g:
        bp, rep = gb.autotune_plan(g, srcs, budget_ms=1500)
        assert rep["candidates"] >= 2 and rep["best_ms"] <= rep["default_ms"]
        with gb.Plan(g, srcs, params=bp) as plan:
            plan.run()
            D, P = plan.results()
        for i, s in enumerate(srcs):
            d, p, _ = g.sssp(int(s))
            assert np.array_equal(D[i], d) and np.array_equal(P[i], p)
    graphs = [gb.gen_rmat(7 + i % 4, 16, 50 + i) for i in range(12)]
    psrc = np.zeros(len(graphs), dtype=np.uint32)
    with gb.Pack(graphs) as pk:
        bp, rep = gb.autotune_plan(pk, psrc, budget_ms=1000)
        assert rep["best_ms"] <= rep["default_ms"]
        with gb.Plan(pk, psrc, params=bp) as plan:
            plan.run()
            D, _ = plan.results()
    for i, h in enumerate(graphs):
        with gb.Graph.from_host(h) as g:
            d, _, _ = g.sssp(0)
        assert np.array_equal(D[i], d)
