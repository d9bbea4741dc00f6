"""CPU tests of the oracle itself: pinned to the committed golden vectors and
to the reference's own run_sspath_arr (sssp/csr_sspath_array.c:149), built
from its sources with the D1/D2/D4 patches."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
U32MAX = 0xFFFFFFFF


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _mg():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLD / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


KNOWN = json.loads((GOLD / "known_answer.json").read_text())
SEEDED = json.loads((GOLD / "seeded.json").read_text())


@pytest.mark.parametrize("case", KNOWN, ids=[c["name"] for c in KNOWN])
def test_known_answer_oracle(case, orc):
    mg = _mg()
    row, col, w = mg.to_csr(case)
    src = case["source"]
    exp = mg.expected_dist(case)
    d = orc.dijkstra(row, col, w, src)
    assert np.array_equal(d, exp)
    ds, _ = orc.delta_stepping(row, col, w, src, case["delta"])
    d64 = d.astype(np.float64)
    if case["wtype"] == "u32":
        d64[d == U32MAX] = np.inf
    assert np.array_equal(ds.astype(np.float64), d64)
    assert orc.min_tight_pred(row, col, w, src, d).tolist() == case["pred"]


@pytest.mark.parametrize("case", SEEDED, ids=[c["name"] for c in SEEDED])
def test_seeded_oracle_pinned(case, orc):
    mg = _mg()
    row, col, w, src = mg.make_seeded(case)
    assert (sha(row), sha(col), sha(w)) == (case["row_sha"], case["col_sha"], case["w_sha"])
    assert src == case["source"]
    d = orc.dijkstra(row, col, w, src)
    assert sha(d) == case["dist_sha"]
    p = orc.min_tight_pred(row, col, w, src, d)
    assert sha(p) == case["pred_sha"]
    assert orc.check_preds(row, col, w, src, d, p) == 0


def test_rmat10_arrays_match_fixture(orc):
    mg = _mg()
    case = SEEDED[0]
    row, col, w, src = mg.make_seeded(case)
    d = orc.dijkstra(row, col, w, src)
    assert np.array_equal(d, np.load(GOLD / "rmat10_dist.npy"))
    assert np.array_equal(orc.min_tight_pred(row, col, w, src, d), np.load(GOLD / "rmat10_pred.npy"))


@pytest.mark.parametrize("delta", [1, 3, 8, 50, 300])
def test_restated_delta_stepping_any_delta(delta, orc):
    from oracle import gen
    row, col, w = gen.rmat(11, 8, 21)
    src = gen.max_degree_vertex(row)
    d = orc.dijkstra(row, col, w, src).astype(np.float64)
    d[d == U32MAX] = np.inf
    ds, _ = orc.delta_stepping(row, col, w, src, delta)
    assert np.array_equal(ds, d)


def test_restated_f32_grid(orc):
    from oracle import gen
    row, col, w = gen.grid(40, 50, 17, "f32")
    d = orc.dijkstra(row, col, w, 0)
    ds, _ = orc.delta_stepping(row, col, w, 0, 250.0)
    assert np.array_equal(ds, d)


def test_check_preds_detects_planted_error(orc):
    from oracle import gen
    row, col, w = gen.rmat(9, 8, 3)
    src = gen.max_degree_vertex(row)
    d = orc.dijkstra(row, col, w, src)
    p = orc.min_tight_pred(row, col, w, src, d)
    bad = p.copy()
    v = int(np.nonzero((d != U32MAX) & (np.arange(len(d)) != src))[0][0])
    bad[v] = (bad[v] + 1) % len(d)
    assert orc.check_preds(row, col, w, src, d, bad) >= 1


@pytest.mark.parametrize("name", ["rmat10_u32", "rmat12_u32", "grid48x80_u32"])
def test_reference_matches_oracle(name, ref_serial):
    mg = _mg()
    case = next(c for c in SEEDED if c["name"] == name)
    row, col, w, src = mg.make_seeded(case)
    rd, _ = ref_serial.ref_sssp_arr(row, col, w, src, case["delta"])
    d = ref_serial.dijkstra(row, col, w, src).astype(np.float64)
    d[d == U32MAX] = np.inf
    assert np.array_equal(rd, d)


def test_reference_list_path_tight_sets(ref_serial):
    """run_sspath (the BC caller's SSSP) keeps every tight predecessor; as a
    set it equals the oracle's tight-predecessor lists."""
    from oracle import gen
    row, col, w = gen.rmat(8, 8, 4)
    src = gen.max_degree_vertex(row)
    delta = 64.0   # run_sspath has 1000 fixed buckets
    d, cnt, lst, _ = ref_serial.ref_sssp_list(row, col, w, src, delta)
    dj = ref_serial.dijkstra(row, col, w, src).astype(np.float64)
    dj[dj == U32MAX] = np.inf
    assert np.array_equal(d, dj)
    off, preds = ref_serial.all_tight_preds(row, col, w, src, dj)
    roff = np.concatenate([[0], np.cumsum(cnt)])
    for v in range(len(dj)):
        assert sorted(set(lst[roff[v]:roff[v + 1]].tolist())) == sorted(set(preds[off[v]:off[v + 1]].tolist()))


def _edge_case_graph():
    """Multi-edges, self-loops, an isolated vertex and a vertex that only
    points into the graph (unreachable from 0):
    0->1 (5), 0->1 (3), 0->0 (2), 1->2 (1), 1->1 (4), 2->0 (7), 2->5 (255),
    4->3 (9), 5->2 (1)."""
    edges = {0: [(1, 5), (1, 3), (0, 2)], 1: [(2, 1), (1, 4)], 2: [(0, 7), (5, 255)], 3: [], 4: [(3, 9)],
             5: [(2, 1)]}
    row = [0]
    col, w = [], []
    for v in range(6):
        for t, x in edges[v]:
            col.append(t)
            w.append(x)
        row.append(len(col))
    return (np.array(row, dtype=np.uint64), np.array(col, dtype=np.uint32), np.array(w, dtype=np.uint32))


@pytest.mark.parametrize("src", [0, 3, 4])
@pytest.mark.parametrize("delta", [1, 2, 7, 1000])
def test_reference_edge_cases(src, delta, ref_serial):
    """The reference's run_sspath_arr, the oracle's restatement of it and
    Dijkstra agree on multi-edges (the lighter one counts), self-loops
    (ignored), a source without out-edges and unreachable vertices (+inf),
    for deltas below, at and far above the weights."""
    row, col, w = _edge_case_graph()
    rd, _ = ref_serial.ref_sssp_arr(row, col, w, src, float(delta))
    dj = ref_serial.dijkstra(row, col, w, src).astype(np.float64)
    dj[dj == U32MAX] = np.inf
    ds, _ = ref_serial.delta_stepping(row, col, w, src, float(delta))
    assert np.array_equal(rd, dj) and np.array_equal(ds, dj)
    if src == 0:
        assert dj.tolist() == [0.0, 3.0, 4.0, np.inf, np.inf, 259.0]
    if src == 3:
        assert dj[3] == 0.0 and np.all(np.isinf(np.delete(dj, 3)))


@pytest.mark.parametrize("delta", [0.05, 0.4, 2.5])
def test_reference_matches_oracle_float64_weights(delta, ref_serial):
    """Fractional double weights (the reference's own readers produce such
    weights): its run_sspath_arr equals the oracle's float64 Dijkstra bit for
    bit, because both take the least fixpoint of fl(d[u] + w)."""
    from oracle import gen
    row, col, _ = gen.rmat(9, 8, 13)
    rng = np.random.default_rng(5)
    w = rng.uniform(0.01, 1.0, len(col))
    src = gen.max_degree_vertex(row)
    rd, _ = ref_serial.ref_sssp_arr(row, col, w, src, delta)
    dj = ref_serial.dijkstra(row, col, w, src)
    assert np.array_equal(rd, dj)
