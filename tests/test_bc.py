"""Betweenness centrality (btwcentral/csr_bc.c:16-123).

CPU tests pin the oracle's Brandes restatement: hand-computed values, the
golden vectors the reference's own Brandes loop produced (tests/golden/
bc_golden.json), the reference run here where it is built, and networkx.
GPU tests run gbs_bc through the C ABI against the oracle: bit-identical for
uint32 weights (the dependency sums are added in the oracle's order), within
a relative 1e-12 for float32 / float64 weights, where two different weights
can round to the same distance and the order of the sum may differ.
"""
import hashlib
import importlib.util
import json
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
BC_GOLD = json.loads((GOLD / "bc_golden.json").read_text())
FLOAT_RTOL = 1e-12


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _mg():
    spec = importlib.util.spec_from_file_location("make_golden", GOLD / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _graph(case):
    row, col, w = _mg().bc_graph(case)
    assert sha(row) == case["row_sha"] and sha(col) == case["col_sha"] and sha(w) == case["w_sha"]
    return row, col, w


def _rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(1.0, np.abs(b)))) if len(b) else 0.0


def _csr(n, edges, wtype=np.uint32):
    edges = sorted(edges, key=lambda e: e[0])
    row = np.zeros(n + 1, dtype=np.uint64)
    for u, _, _ in edges:
        row[u + 1] += 1
    row = np.cumsum(row).astype(np.uint64)
    col = np.array([v for _, v, _ in edges], dtype=np.uint32)
    w = np.array([x for _, _, x in edges], dtype=wtype)
    return row, col, w


def _undirected(edges):
    return edges + [(v, u, w) for u, v, w in edges]


# ---------------------------------------------------------------- CPU: oracle
def test_oracle_bc_hand_values(orc):
    # path 0-1-2-3 (unit weights): ordered pairs through 1 are (0,2), (0,3),
    # (2,0), (3,0) -> 4; through 2 likewise
    row, col, w = _csr(4, _undirected([(0, 1, 1), (1, 2, 1), (2, 3, 1)]))
    assert orc.betweenness(row, col, w).tolist() == [0.0, 4.0, 4.0, 0.0]
    # 4-cycle: each pair of opposite vertices has two shortest paths, so each
    # vertex carries half of (a, c) and half of (c, a)
    row, col, w = _csr(4, _undirected([(0, 1, 1), (1, 2, 1), (2, 3, 1), (3, 0, 1)]))
    assert orc.betweenness(row, col, w).tolist() == [1.0, 1.0, 1.0, 1.0]
    # star with centre 0 and 4 leaves: 4 * 3 ordered leaf pairs pass through 0
    row, col, w = _csr(5, _undirected([(0, k, 2) for k in range(1, 5)]))
    assert orc.betweenness(row, col, w).tolist() == [12.0, 0.0, 0.0, 0.0, 0.0]
    # sources restrict the sum
    assert orc.betweenness(row, col, w, sources=[1]).tolist() == [3.0, 0.0, 0.0, 0.0, 0.0]
    assert orc.betweenness(row, col, w, sources=[0]).tolist() == [0.0] * 5


@pytest.mark.parametrize("case", BC_GOLD, ids=[c["name"] for c in BC_GOLD])
def test_oracle_bc_matches_reference_golden(case, orc):
    """The golden vectors are the reference's own Brandes loop (lists
    deduplicated where the case says so); the oracle must agree."""
    row, col, w = _graph(case)
    bc = orc.betweenness(row, col, w)
    assert _rel(bc, np.array(case["bc"])) < 1e-12


def test_oracle_bc_vs_networkx(orc):
    nx = pytest.importorskip("networkx")
    from oracle import gen
    row, col, w = gen.rmat(7, 8, 12, "u32", 1, 3)
    bc = orc.betweenness(row, col, w)
    G = nx.DiGraph()
    G.add_nodes_from(range(len(row) - 1))
    for u in range(len(row) - 1):
        for e in range(int(row[u]), int(row[u + 1])):
            G.add_edge(u, int(col[e]), weight=float(w[e]))
    ref = nx.betweenness_centrality(G, weight="weight", normalized=False)
    assert _rel(bc, np.array([ref[v] for v in range(len(row) - 1)])) < 1e-12


def test_reference_bc_live(ref_serial):
    """The reference's Brandes loop run here: with deduplicated predecessor
    lists it equals the oracle on graphs full of equal shortest paths; with
    its raw lists it equals the oracle when predecessors are unique
    (fractional float64 weights) and differs where repeats are uneven."""
    from oracle import gen
    orc = ref_serial
    row, col, w = gen.rmat(6, 8, 21, "u32", 1, 3)
    ours = orc.betweenness(row, col, w)
    ded, reps, _ = orc.ref_bc(row, col, w, delta=0.1, dedup=True)
    assert reps > 0
    assert _rel(ded, ours) < 1e-12
    raw, _, _ = orc.ref_bc(row, col, w, delta=0.1, dedup=False)
    assert _rel(raw, ours) > 1e-3      # the repeated entries change the reference's own result
    row, col, w = gen.rmat(6, 8, 22, "u32", 1, 255)
    wf = col.astype(np.float64) / 384.0 + w.astype(np.float64) / 131.0
    raw, _, _ = orc.ref_bc(row, col, wf, delta=0.5, dedup=False)
    assert _rel(raw, orc.betweenness(row, col, wf)) < 1e-12


def _diamond_chain(k):
    edges = []
    for i in range(k):
        a, b, c, d = 3 * i, 3 * i + 1, 3 * i + 2, 3 * i + 3
        edges += [(a, b, 1), (a, c, 1), (b, d, 1), (c, d, 1)]
    return _csr(3 * k + 1, edges)


def test_oracle_bc_path_counts_beyond_32_bits(orc):
    """A chain of 40 diamonds has 2^40 shortest paths from vertex 0 to its
    end: the counts need the 64-bit sums the reference uses (lint).  Each
    middle vertex of diamond i lies on half of the paths to every vertex
    after it: 0.5 * (1 + 3 * (39 - i)) for source 0."""
    row, col, w = _diamond_chain(40)
    bc = orc.betweenness(row, col, w, sources=[0])
    for i in range(40):
        assert bc[3 * i + 1] == bc[3 * i + 2] == 0.5 * (1 + 3 * (39 - i))
        if i:
            assert bc[3 * i] == 3 * (40 - i)


# ---------------------------------------------------------------- GPU
def _need_gpu(gb):
    assert gb.device_available(), "GPU tests need a CUDA device (compute capability 10.x)"


def _gpu_bc(gb, row, col, w, sources=None, **kw):
    with gb.Graph(row, col, w) as g:
        return g.betweenness(sources, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("case", BC_GOLD, ids=[c["name"] for c in BC_GOLD])
def test_gpu_bc_golden(case, gb, orc):
    _need_gpu(gb)
    row, col, w = _graph(case)
    bc, st = _gpu_bc(gb, row, col, w)
    assert st["sources"] == case["n"]
    ours = orc.betweenness(row, col, w)
    if np.asarray(w).dtype == np.uint32:
        assert np.array_equal(bc, ours), f"{int(np.sum(bc != ours))} values differ"
    else:
        assert _rel(bc, ours) < FLOAT_RTOL
    assert _rel(bc, np.array(case["bc"])) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("wmax", [2, 16, 255])
def test_gpu_bc_rmat_u32_bit_exact(wmax, gb, orc):
    _need_gpu(gb)
    from oracle import gen
    row, col, w = gen.rmat(11, 16, 5 + wmax, "u32", 1, wmax)
    src = gen.sample_sources(row, 24, 3)
    bc, st = _gpu_bc(gb, row, col, w, src)
    ours = orc.betweenness(row, col, w, src)
    assert np.array_equal(bc, ours), f"{int(np.sum(bc != ours))} values differ, rel {_rel(bc, ours):.3g}"
    assert st["tight_edges"] >= st["dag_vertices"] - len(src)
    assert st["max_levels"] > 1


@pytest.mark.gpu
def test_gpu_bc_all_sources_with_long_rows(gb, orc):
    """Every source of a skewed graph (rows longer than 32 edges take the
    warp path in every pass)."""
    _need_gpu(gb)
    from oracle import gen
    row, col, w = gen.rmat(9, 32, 8, "u32", 1, 8)
    assert int(np.max(np.diff(row.astype(np.int64)))) > 64
    bc, st = _gpu_bc(gb, row, col, w)
    assert st["sources"] == len(row) - 1
    assert np.array_equal(bc, orc.betweenness(row, col, w))


@pytest.mark.gpu
def test_gpu_bc_grid_f32(gb, orc):
    _need_gpu(gb)
    from oracle import gen
    row, col, w = gen.grid(40, 52, 3, "f32")
    src = gen.sample_sources(row, 6, 9)
    bc, st = _gpu_bc(gb, row, col, w, src)
    assert _rel(bc, orc.betweenness(row, col, w, src)) < FLOAT_RTOL
    assert st["max_levels"] >= 40


@pytest.mark.gpu
def test_gpu_bc_float64_fractional(gb, orc):
    _need_gpu(gb)
    from oracle import gen
    row, col, w = gen.rmat(10, 16, 13, "u32", 1, 255)
    wf = col.astype(np.float64) / 3072.0 + w.astype(np.float64) / 131.0
    src = gen.sample_sources(row, 12, 2)
    bc, _ = _gpu_bc(gb, row, col, wf, src)
    assert _rel(bc, orc.betweenness(row, col, wf, src)) < FLOAT_RTOL


@pytest.mark.gpu
def test_gpu_bc_edge_cases(gb, orc):
    _need_gpu(gb)
    # one vertex, no edges
    row, col, w = _csr(1, [])
    bc, _ = _gpu_bc(gb, row, col, w)
    assert bc.tolist() == [0.0]
    # a source with no out-edges, disconnected parts and a self loop
    row, col, w = _csr(6, [(1, 0, 2), (1, 2, 1), (2, 3, 1), (3, 3, 5), (4, 5, 3), (5, 4, 3)])
    bc, _ = _gpu_bc(gb, row, col, w)
    assert np.array_equal(bc, orc.betweenness(row, col, w))
    bc, _ = _gpu_bc(gb, row, col, w, [0])
    assert bc.tolist() == [0.0] * 6
    # parallel edges of equal weight double the paths through them
    row, col, w = _csr(3, [(0, 1, 1), (0, 1, 1), (1, 2, 1), (0, 2, 5)])
    bc, _ = _gpu_bc(gb, row, col, w)
    assert np.array_equal(bc, orc.betweenness(row, col, w))
    # repeated sources count twice
    row, col, w = _csr(4, _undirected([(0, 1, 1), (1, 2, 1), (2, 3, 1)]))
    bc, _ = _gpu_bc(gb, row, col, w, [0, 0])
    assert bc.tolist() == [0.0, 4.0, 2.0, 0.0]


@pytest.mark.gpu
def test_gpu_bc_path_counts_beyond_32_bits(gb, orc):
    _need_gpu(gb)
    row, col, w = _diamond_chain(40)
    bc, st = _gpu_bc(gb, row, col, w)
    assert np.array_equal(bc, orc.betweenness(row, col, w))
    assert st["max_levels"] == 81


@pytest.mark.gpu
def test_gpu_bc_rejects_zero_weights_and_bad_sources(gb):
    _need_gpu(gb)
    row, col, w = _csr(3, [(0, 1, 0), (1, 2, 1)])
    with gb.Graph(row, col, w) as g:
        with pytest.raises(gb.GbsError) as e:
            g.betweenness()
        assert e.value.status == 1
        # the same graph still runs shortest paths
        d, _, _ = g.sssp(0)
        assert d.tolist() == [0, 0, 1]
    row, col, w = _csr(3, [(0, 1, 1), (1, 2, 1)])
    with gb.Graph(row, col, w) as g:
        with pytest.raises(gb.GbsError):
            g.betweenness([5])


@pytest.mark.gpu
def test_gpu_bc_device_output_and_schedules(gb, orc):
    """gbs_bc_device leaves the result on the GPU; the result does not
    depend on the shortest-path schedule (delta, split)."""
    _need_gpu(gb)
    from oracle import gen
    row, col, w = gen.rmat(10, 16, 31, "u32", 1, 32)
    src = gen.sample_sources(row, 8, 5)
    ours = orc.betweenness(row, col, w, src)
    n = len(row) - 1
    with gb.Graph(row, col, w) as g:
        buf = gb.DeviceBuffer(8 * n)
        try:
            st = g.betweenness_device(buf.ptr, src)
            host = np.empty(n, dtype=np.float64)
            assert gb.lib.gbs_memcpy(host.ctypes.data, buf.ptr, 8 * n) == 0
        finally:
            buf.free()
        assert st["sources"] == len(src)
        assert np.array_equal(host, ours)
        for kw in ({"delta": 1.0}, {"delta": 64.0, "light": 8.0}, {"delta": 1e6}):
            bc, _ = g.betweenness(src, **kw)
            assert np.array_equal(bc, ours), kw


@pytest.mark.gpu
@pytest.mark.parametrize("wtype", ["u32", "f32"])
def test_gpu_bc_batched_equals_single(wtype, gb, orc):
    """Shortest paths solved in batched launches (more sources than one batch
    holds) or one source at a time give the same distances, hence the same
    betweenness, bit for bit."""
    _need_gpu(gb)
    from oracle import gen
    row, col, w = gen.rmat(10, 16, 41, wtype, 1, 12)
    src = gen.sample_sources(row, 70, 3)
    with gb.Graph(row, col, w) as g:
        bb, sb = g.betweenness(src)
        bs, ss = g.betweenness(src, flags=gb.F_BC_SINGLE)
    assert np.array_equal(bb, bs)
    assert np.array_equal(bb, orc.betweenness(row, col, w, src))
    assert sb["edges_reached"] == ss["edges_reached"] and sb["tight_edges"] == ss["tight_edges"]


@pytest.mark.gpu
def test_gpu_bc_rmat16_sampled(gb, orc):
    """A larger graph (R-MAT scale 16, 1M edges) with sampled sources."""
    _need_gpu(gb)
    from oracle import gen
    row, col, w = gen.rmat(16, 16, 1, "u32")
    src = gen.sample_sources(row, 4, 7)
    bc, st = _gpu_bc(gb, row, col, w, src)
    assert np.array_equal(bc, orc.betweenness(row, col, w, src))
    assert st["dag_ms"] > 0 and st["sssp_ms"] > 0
