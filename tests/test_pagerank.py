"""PageRank (pagerank/pagerank_mpi.c:667-1043 on one node) on the GPU.

The reference's MPI PageRank needs its partitioner's side files (pidx, send,
recip) and MPI, so its restatement in the oracle (or_pagerank) is pinned by
identities instead: the fixed point 0.3 + 0.7 * sum(rank(u) / deg(u)) holds
to the threshold, a cycle stops at once with every rank 1, and on graphs
without dangling vertices the ranks are n times networkx's pagerank with
alpha 0.7.  GPU results are bit-identical to the oracle (same summation
order), iteration counts equal.
"""
import numpy as np
import pytest


def _cycle(n):
    return np.arange(n + 1, dtype=np.uint64), np.array([(v - 1) % n for v in range(n)], dtype=np.uint32)


def _directed_with_sinks(seed=3, n=300, m=2400):
    rng = np.random.default_rng(seed)
    u = rng.integers(0, n, m)
    v = rng.integers(0, n, m)
    u = u[u % 7 != 0]                     # vertices divisible by 7 keep no out-edges
    v = v[: len(u)]
    order = np.argsort(u, kind="stable")
    u, v = u[order], v[order]
    row = np.zeros(n + 1, dtype=np.uint64)
    np.add.at(row, u + 1, 1)
    return np.cumsum(row).astype(np.uint64), v.astype(np.uint32)


# ---------------------------------------------------------------- CPU: oracle
def test_oracle_pagerank_cycle_and_star(orc):
    row, col = _cycle(6)
    pr, it = orc.pagerank(row, col)
    assert it == 1 and pr.tolist() == [1.0] * 6
    # symmetric star, centre 0 and 4 leaves: leaf = 0.3 + 0.7 * c / 4, c = 0.3 + 0.7 * 4 * leaf
    n = 5
    out_row = np.array([0, 4, 5, 6, 7, 8], dtype=np.uint64)
    out_col = np.array([1, 2, 3, 4, 0, 0, 0, 0], dtype=np.uint32)
    tr, tc = orc.transpose(out_row, out_col)
    pr, it = orc.pagerank(tr, tc)
    c = (0.3 + 4 * 0.7 * 0.3) / (1 - 0.49)
    leaf = 0.3 + 0.7 * c / 4
    assert abs(pr[0] - c) < 1e-5 and np.all(np.abs(pr[1:] - leaf) < 1e-5)


def test_oracle_pagerank_fixed_point_and_networkx(orc):
    nx = pytest.importorskip("networkx")
    from oracle import gen
    row, col, _ = gen.rmat(10, 8, 3, "u32")
    deg = np.diff(row.astype(np.int64))
    tr, tc = orc.transpose(row, col)
    pr, it = orc.pagerank(tr, tc)
    assert it > 3
    inflow = np.zeros(len(deg))
    src = np.repeat(np.arange(len(deg)), deg)
    np.add.at(inflow, col.astype(np.int64), pr[src] / deg[src])
    assert np.max(np.abs(pr - (0.3 + 0.7 * inflow))) < 1e-5
    # isolated vertices keep 0.3; on the rest (no sinks in a symmetric graph)
    # the ranks are n' times networkx's pagerank with alpha = 0.7
    live = np.nonzero(deg)[0]
    assert np.all(pr[deg == 0] == 0.3)
    G = nx.DiGraph()
    G.add_nodes_from(live.tolist())
    for u in live:
        for e in range(int(row[u]), int(row[u + 1])):
            G.add_edge(int(u), int(col[e]))
    x = nx.pagerank(G, alpha=0.7, tol=1e-13, max_iter=1000)
    y = np.array([x[int(v)] for v in live]) * len(live)
    assert np.max(np.abs(pr[live] - y) / y) < 1e-5


def test_oracle_transpose(orc):
    row, col = _directed_with_sinks()
    tr, tc = orc.transpose(row, col)
    assert int(tr[-1]) == len(col)
    edges = sorted(zip(np.repeat(np.arange(len(row) - 1), np.diff(row.astype(np.int64))).tolist(), col.tolist()))
    back = sorted((int(tc[e]), v) for v in range(len(tr) - 1) for e in range(int(tr[v]), int(tr[v + 1])))
    assert edges == back


# ---------------------------------------------------------------- GPU
def _need_gpu(gb):
    assert gb.device_available(), "GPU tests need a CUDA device (compute capability 10.x)"


def _gpu_pr(gb, out_row, out_col, **kw):
    with gb.DeviceCsr.from_arrays(out_row, out_col) as c, c.transpose() as t:
        tr, tc, _ = t.export()
        pr, st = t.pagerank(**kw)
    return pr, st, tr, tc


@pytest.mark.gpu
@pytest.mark.parametrize("graph", ["rmat10", "rmat12_hubs", "grid", "sinks", "cycle"])
def test_gpu_pagerank_bit_exact(graph, gb, orc):
    _need_gpu(gb)
    from oracle import gen
    if graph == "rmat10":
        row, col, _ = gen.rmat(10, 8, 3, "u32")
    elif graph == "rmat12_hubs":
        row, col, _ = gen.rmat(12, 48, 9, "u32")     # rows far longer than 8 words
        assert int(np.max(np.diff(row.astype(np.int64)))) > 32 * 32
    elif graph == "grid":
        row, col, _ = gen.grid(40, 60, 3, "f32")
    elif graph == "sinks":
        row, col = _directed_with_sinks()
    else:
        row, col = _cycle(33)
    pr, st, tr, tc = _gpu_pr(gb, row, col)
    ref_row, ref_col = orc.transpose(row, col)
    assert np.array_equal(tr, ref_row) and np.array_equal(tc, ref_col)
    ref, it = orc.pagerank(tr, tc)
    assert st["iterations"] == it and st["converged"] == 1
    assert np.array_equal(pr, ref), f"{int(np.sum(pr != ref))} ranks differ"


@pytest.mark.gpu
def test_gpu_pagerank_params_and_cap(gb, orc):
    _need_gpu(gb)
    from oracle import gen
    row, col, _ = gen.rmat(9, 8, 5, "u32")
    pr, st, tr, tc = _gpu_pr(gb, row, col, random_jump=0.15, threshold=1e-9)
    ref, it = orc.pagerank(tr, tc, 0.15, 1e-9)
    assert st["iterations"] == it and np.array_equal(pr, ref)
    pr, st, tr, tc = _gpu_pr(gb, row, col, max_iters=3)
    ref, it = orc.pagerank(tr, tc, 0.3, 1e-6, 3)
    assert st["iterations"] == 3 and st["converged"] == 0 and np.array_equal(pr, ref)


@pytest.mark.gpu
def test_gpu_pagerank_on_the_reference_reader(gb, orc):
    """The reference reads PageRank's graph with read_graph_csr(RECV): the
    in-edge CSR of the text file, as gbs_read_text(GBS_DIR_RECV) builds it."""
    _need_gpu(gb)
    from pathlib import Path
    path = Path(__file__).resolve().parent / "golden" / "ingest" / "rmat8.txt"
    with gb.DeviceCsr.read_text(path, gb.DIR_RECV) as c:
        pr, st = c.pagerank()
        row, col, _ = c.export()
    ref, it = orc.pagerank(row, col)
    assert st["iterations"] == it and np.array_equal(pr, ref)
