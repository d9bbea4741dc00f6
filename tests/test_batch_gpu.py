"""Batched SSSP (gbs_plan_sources / gbs_plan_pack): every instance of a
persistent multi-instance launch, replayed from its CUDA graph, must equal the
single-source call on the same graph and source bit for bit, for every group
shape; the oracle checks the single-source results independently."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(gb):
    assert gb.device_available(), "GPU tests need a CUDA device (compute capability 10.x)"


def _single(g, srcs, **kw):
    out = []
    for s in srcs:
        d, p, st = g.sssp(int(s), **kw)
        out.append((d, p, st))
    return out


@pytest.mark.parametrize("group_ctas", [0, 1, 3, 19, 152])
def test_sources_plan_matches_single(group_ctas, gb, orc):
    a = gb.gen_rmat(12, 16, 5)
    srcs = gb.sample_sources(a, 10, 3)
    with gb.Graph.from_host(a) as g:
        ref = _single(g, srcs)
        with gb.Plan(g, srcs, group_ctas=group_ctas) as plan:
            st = plan.run(per_instance=True)
            D, P = plan.results()
    assert st["completed"] == len(srcs)
    if group_ctas:
        assert st["group_ctas"] == min(group_ctas, st["blocks"])
    for i, (d, p, s1) in enumerate(ref):
        assert np.array_equal(D[i], d), f"instance {i}: distances differ"
        assert np.array_equal(P[i], p), f"instance {i}: predecessors differ"
        r = st["per_instance"][i]
        assert r["done"] == 1 and r["reached"] == s1["reached"] and r["edges_reached"] == s1["edges_reached"]
    s0 = int(srcs[0])
    assert np.array_equal(D[0], orc.dijkstra(a.row, a.col, a.w, s0))
    assert st["edges_reached"] == sum(s1["edges_reached"] for _, _, s1 in ref)


def test_sources_plan_replays_and_schedules(gb):
    """A captured plan replays with the same results; split, no split and
    explicit deltas all give the single-source answer."""
    a = gb.gen_rmat(11, 16, 9)
    srcs = gb.sample_sources(a, 6, 1)
    with gb.Graph.from_host(a) as g:
        ref = _single(g, srcs)
        for kw in [dict(), dict(light=math.inf), dict(delta=3), dict(delta_scale=8.0, light=math.inf),
                   dict(delta=40, light=10), dict(flags=gb.F_NO_SOLO)]:
            with gb.Plan(g, srcs, group_ctas=4, **kw) as plan:
                for rep in range(3):
                    st = plan.run()
                    assert st["completed"] == len(srcs)
                    D, P = plan.results()
                    for i, (d, p, _) in enumerate(ref):
                        assert np.array_equal(D[i], d), (kw, rep, i)
                        assert np.array_equal(P[i], p), (kw, rep, i)


def test_sources_plan_f32_grid(gb, orc):
    a = gb.gen_grid(48, 64, 3, "f32")
    srcs = np.array([0, 5, 100, 3071], dtype=np.uint32)
    with gb.Graph.from_host(a) as g:
        ref = _single(g, srcs)
        with gb.Plan(g, srcs, group_ctas=2) as plan:
            plan.run()
            D, P = plan.results()
    for i, (d, p, _) in enumerate(ref):
        assert np.array_equal(D[i].view(np.uint32), d.view(np.uint32))
        assert np.array_equal(P[i], p)
    assert np.array_equal(D[3], orc.dijkstra(a.row, a.col, a.w, 3071))


def _mixed_pack(gb, count, seed):
    rng = np.random.default_rng(seed)
    graphs = []
    for i in range(count):
        if i % 5 == 4:
            graphs.append(gb.gen_grid(int(rng.integers(4, 40)), int(rng.integers(4, 40)), 100 + i, "u32"))
        else:
            graphs.append(gb.gen_rmat(int(rng.integers(6, 12)), 16, 200 + i))
    return graphs


@pytest.mark.parametrize("group_ctas", [0, 1, 8])
def test_pack_plan_matches_single(group_ctas, gb, orc):
    graphs = _mixed_pack(gb, 23, 11)
    srcs = np.array([int(np.argmax(np.diff(h.row.astype(np.int64)))) for h in graphs], dtype=np.uint32)
    with gb.Pack(graphs) as pk, gb.Plan(pk, srcs, group_ctas=group_ctas) as plan:
        st = plan.run(per_instance=True)
        D, P = plan.results()
        assert st["completed"] == len(graphs)
        for i, h in enumerate(graphs):
            with gb.Graph.from_host(h) as g:
                d, p, s1 = g.sssp(int(srcs[i]))
            assert np.array_equal(D[i], d), f"graph {i}"
            assert np.array_equal(P[i], p), f"graph {i}"
            assert st["per_instance"][i]["edges_reached"] == s1["edges_reached"]
        assert np.array_equal(D[7], orc.dijkstra(graphs[7].row, graphs[7].col, graphs[7].w, int(srcs[7])))


def test_pack_plan_f32_and_isolated_sources(gb, orc):
    graphs = [gb.gen_rmat(9, 8, 30 + i, "f32") for i in range(6)] + [gb.gen_grid(9, 13, 4, "f32")]
    srcs = []
    for h in graphs[:-1]:
        deg = np.diff(h.row.astype(np.int64))
        iso = np.nonzero(deg == 0)[0]
        srcs.append(int(iso[0]) if len(iso) else 0)
    srcs.append(0)
    srcs = np.array(srcs, dtype=np.uint32)
    with gb.Pack(graphs) as pk, gb.Plan(pk, srcs, light=math.inf) as plan:
        plan.run()
        D, P = plan.results()
    for i, h in enumerate(graphs):
        ref = orc.dijkstra(h.row, h.col, h.w, int(srcs[i]))
        assert np.array_equal(D[i].view(np.uint32), ref.view(np.uint32)), f"graph {i}"
        assert np.array_equal(P[i], orc.min_tight_pred(h.row, h.col, h.w, int(srcs[i]), ref))


def test_plan_rejects_bad_input(gb):
    a = gb.gen_rmat(8, 4, 1)
    with gb.Graph.from_host(a) as g:
        with pytest.raises(gb.GbsError) as e:
            gb.Plan(g, [a.n])
        assert e.value.name == "INVALID_ARG"
        with pytest.raises(gb.GbsError):
            gb.Plan(g, [])
    with pytest.raises(TypeError):
        gb.Pack([gb.gen_rmat(6, 4, 1), gb.gen_rmat(6, 4, 2, "f32")])
