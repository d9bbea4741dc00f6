"""GPU parity tests: the CUDA path (through the C ABI in libgbsssp.so) against
the oracle and the committed golden vectors.  Distances must be bit-identical
(uint32, float32 and float64 alike: the least fixpoint does not depend on the
relaxation order or the bucket width), and predecessors must equal the
smallest tight in-neighbour, which the oracle computes independently."""
import hashlib
import importlib.util
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
U32MAX = 0xFFFFFFFF
KNOWN = json.loads((GOLD / "known_answer.json").read_text())
SEEDED = json.loads((GOLD / "seeded.json").read_text())


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _mg():
    spec = importlib.util.spec_from_file_location("make_golden", GOLD / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(gb):
    assert gb.device_available(), "GPU tests need a CUDA device (compute capability 10.x)"


def run_and_check(gb, orc, row, col, w, src, **kw):
    with gb.Graph(row, col, w) as g:
        d, p, st = g.sssp(src, **kw)
    ref = orc.dijkstra(row, col, w, src)
    assert np.array_equal(d, ref), f"{int(np.sum(d != ref))} distances differ"
    rp = orc.min_tight_pred(row, col, w, src, ref)
    assert np.array_equal(p, rp), f"{int(np.sum(p != rp))} predecessors differ"
    assert orc.check_preds(row, col, w, src, d, p) == 0
    return d, p, st


@pytest.mark.parametrize("case", KNOWN, ids=[c["name"] for c in KNOWN])
def test_known_answer(case, gb):
    mg = _mg()
    row, col, w = mg.to_csr(case)
    with gb.Graph(row, col, w) as g:
        for kw in ({}, dict(full_items=1)):   # whole rows / the split in every bucket
            d, p, _ = g.sssp(case["source"], delta=case["delta"], **kw)
            assert np.array_equal(d, mg.expected_dist(case)), kw
            assert p.tolist() == case["pred"], kw


@pytest.mark.parametrize("case", SEEDED, ids=[c["name"] for c in SEEDED])
def test_seeded_golden(case, gb):
    mg = _mg()
    row, col, w, src = mg.make_seeded(case)
    with gb.Graph(row, col, w) as g:
        d, p, st = g.sssp(src, delta=case["delta"])
    assert sha(d) == case["dist_sha"]
    assert sha(p) == case["pred_sha"]
    assert st["reached"] == case["reached"]
    assert st["edges_reached"] == case["edges_reached"]


@pytest.mark.parametrize("delta,light", [(None, None), (1, None), (3, None), (40, None), (255, None),
                                         (10000, None), (8, 0), (8, 64), (2, 300)])
def test_rmat_deltas_and_splits(delta, light, gb, orc):
    """Widths and light bounds, with whole rows in every bucket (the default)
    and with the split in every bucket (full_items 1)."""
    a = gb.gen_rmat(13, 16, 3)
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    run_and_check(gb, orc, a.row, a.col, a.w, src, delta=delta, light=light)
    run_and_check(gb, orc, a.row, a.col, a.w, src, delta=delta, light=light, full_items=1)


def test_rmat16_many_sources_one_graph(gb, orc):
    """Repeated runs on one resident graph (stamps carried across runs)."""
    a = gb.gen_rmat(16, 16, 1)
    srcs = gb.sample_sources(a, 6, 7)
    with gb.Graph.from_host(a) as g:
        for s in srcs:
            d, p, st = g.sssp(int(s))
            ref = orc.dijkstra(a.row, a.col, a.w, int(s))
            assert np.array_equal(d, ref)
            assert np.array_equal(p, orc.min_tight_pred(a.row, a.col, a.w, int(s), ref))
            assert st["buckets"] >= 1 and st["phases"] >= 2


def test_hub_rows_split_into_descriptors(gb, orc):
    """Hub rows (thousands of edges) are cut into 128-edge descriptors that
    many warps relax; a huge delta puts every edge in the light part."""
    a = gb.gen_rmat(14, 32, 5)
    assert np.diff(a.row.astype(np.int64)).max() > 1000
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    run_and_check(gb, orc, a.row, a.col, a.w, src)
    run_and_check(gb, orc, a.row, a.col, a.w, src, delta=100000)


@pytest.mark.parametrize("mode", ["grid_only", "default", "all_solo", "all_solo_no_fuse", "no_fuse", "split",
                                  "all_solo_split"])
def test_solo_phases_same_result(mode, gb, orc):
    """Phases run by one CTA (small inputs) or by the whole grid give the same
    result; 'all_solo' makes every phase after the first run on one CTA;
    the no_fuse modes turn bucket fusion off; the split modes keep the
    light/heavy split in every bucket (heavy phases)."""
    kw = {"grid_only": dict(flags=gb.F_NO_SOLO),
          "default": {},
          "all_solo": dict(solo_entries=1 << 30, solo_descs=1 << 30),
          "all_solo_no_fuse": dict(solo_entries=1 << 30, solo_descs=1 << 30, flags=gb.F_NO_FUSE),
          "no_fuse": dict(flags=gb.F_NO_FUSE),
          "split": dict(full_items=1),
          "all_solo_split": dict(solo_entries=1 << 30, solo_descs=1 << 30, full_items=1)}[mode]
    a = gb.gen_rmat(13, 16, 11)
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    _, _, st = run_and_check(gb, orc, a.row, a.col, a.w, src, **kw)
    if mode == "grid_only":
        assert st["solo_phases"] == 0
    if mode.startswith("all_solo"):
        assert st["solo_phases"] >= st["phases"] - 2
    g2 = gb.gen_grid(64, 96, 5, "f32")
    _, _, st2 = run_and_check(gb, orc, g2.row, g2.col, g2.w, 0, **kw)
    if mode == "default":
        assert st2["solo_phases"] > 0
    # pending traffic (weights up to 255, width 2): the re-bucketing of the
    # pending list runs on one CTA in the solo modes
    g3 = gb.gen_grid(60, 90, 11, "u32")
    for src in (0, 2777):
        _, _, st3 = run_and_check(gb, orc, g3.row, g3.col, g3.w, src, delta=2, **kw)
        assert st3["pending_scans"] >= 1


@pytest.mark.parametrize("full_items", [1, 1024, 0, 1 << 30])
def test_whole_row_threshold_same_result(full_items, gb, orc):
    """Buckets of up to full_items entries relax whole rows (0: the default,
    every bucket); 1 splits every bucket but the source's, 1024 the large
    ones, 2^30 relaxes every bucket whole.  Distances and predecessors stay
    the oracle's, and on R-MAT the heavy phases disappear when every bucket
    is whole."""
    a = gb.gen_rmat(14, 16, 21)
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    _, _, st = run_and_check(gb, orc, a.row, a.col, a.w, src, full_items=full_items)
    _, _, st1 = run_and_check(gb, orc, a.row, a.col, a.w, src, full_items=1)
    if full_items in (0, 1 << 30):
        assert st["phases"] < st1["phases"]
    g2 = gb.gen_grid(48, 80, 7, "f32")
    run_and_check(gb, orc, g2.row, g2.col, g2.w, 0, full_items=full_items)


def test_phase_trace(gb, orc):
    """GBS_F_TRACE records one entry per grid phase; scans are followed by a
    relaxation of the edges they emitted, and device time is monotone."""
    a = gb.gen_rmat(12, 16, 2)
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    with gb.Graph.from_host(a) as g:
        d, _, st = g.sssp(src, flags=gb.F_TRACE)
        tr = g.trace()
        assert len(tr) == st["phases"]
        assert sum(1 for r in tr if r["kind"] == "scan_bucket") == st["buckets"]
        assert all(tr[i]["end_ns"] <= tr[i + 1]["end_ns"] for i in range(len(tr) - 1))
        for i, r in enumerate(tr[:-1]):
            if r["kind"].startswith("scan") and r["edges"] > 0:
                assert tr[i + 1]["kind"] == "relax"
                assert tr[i + 1]["edges"] == r["edges"]
        # tracing changes nothing in the result
        d2, _, _ = g.sssp(src)
    assert np.array_equal(d, d2) and np.array_equal(d, orc.dijkstra(a.row, a.col, a.w, src))


@pytest.mark.parametrize("wtype", ["u32", "f32"])
def test_split_covering_all_edges_skips_heavy(wtype, gb, orc):
    """A light bound at or above the largest weight leaves no heavy edge: the
    light scans relax whole rows and no heavy scan runs; a bound just below
    the largest weight keeps the heavy scans."""
    a = gb.gen_rmat(12, 16, 21, wtype)
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    wmax = float(a.w.max())
    with gb.Graph.from_host(a) as g:
        for light, heavy_expected in [(wmax, False), (wmax * 4, False), (wmax - 1, True)]:
            d, p, st = g.sssp(src, delta=wmax / 8, light=light, flags=gb.F_TRACE, full_items=1)
            kinds = {r["kind"] for r in g.trace()}
            assert ("heavy" in kinds) == heavy_expected, (light, kinds)
            ref = orc.dijkstra(a.row, a.col, a.w, src)
            assert np.array_equal(d, ref)
            assert np.array_equal(p, orc.min_tight_pred(a.row, a.col, a.w, src, ref))


def test_pending_list_small_delta(gb, orc):
    """delta = 1 with weights up to 255 pushes vertices past the 64-bucket
    ring window, exercising the pending list and its re-bucketing."""
    a = gb.gen_grid(40, 60, 11, "u32")
    _, _, st = run_and_check(gb, orc, a.row, a.col, a.w, 0, delta=1)
    assert st["pending_scans"] >= 1


@pytest.mark.parametrize("mode", ["default", "all_solo", "no_fuse", "split"])
def test_pending_rebucketing_on_one_cta(mode, gb, orc):
    """Widths far below the largest weight push most vertices past the ring
    window; their re-bucketing runs on the deciding CTA when the pending list
    is small.  Every run must give the oracle's distances and predecessors
    (before the re-bucketing fenced its tag stores and the pending minimum,
    half of these runs on one CTA stopped early or skipped vertices)."""
    kw = {"default": {}, "all_solo": dict(solo_entries=1 << 30, solo_descs=1 << 30),
          "no_fuse": dict(flags=gb.F_NO_FUSE), "split": dict(full_items=1)}[mode]
    cases = [(gb.gen_grid(54, 83, 107, "u32"), [1, 2, 3]), (gb.gen_grid(47, 71, 205, "f32"), [2.0, 20.0]),
             (gb.gen_rmat(12, 16, 302), [1, 4])]
    pend = 0
    for a, deltas in cases:
        for src in [int(x) for x in gb.sample_sources(a, 2, 5)]:
            for d in deltas:
                _, _, st = run_and_check(gb, orc, a.row, a.col, a.w, src, delta=d, **kw)
                pend += st["pending_scans"]
    assert pend > 20


@pytest.mark.parametrize("wtype", ["u32", "f32"])
def test_bucket_fusion_fewer_phases_same_result(wtype, gb, orc):
    """Whole-row scans relax the vertices they improve into the current bucket
    later in the same phase (bucket fusion).  On a grid, whose buckets hold
    long chains of light hops, that takes fewer phases than waiting for the
    next frontier scan each hop; with and without it, on one CTA and on the
    whole grid, the distances and predecessors are the oracle's."""
    a = gb.gen_grid(80, 120, 9, wtype)
    for src in (0, 120 * 40 + 57):
        for base in (0, gb.F_NO_SOLO):
            _, _, on = run_and_check(gb, orc, a.row, a.col, a.w, src, flags=base)
            _, _, off = run_and_check(gb, orc, a.row, a.col, a.w, src, flags=base | gb.F_NO_FUSE)
            assert on["phases"] < off["phases"], (on["phases"], off["phases"])


@pytest.mark.parametrize("delta", [None, 50.0, 1000.0, 1e6])
def test_grid_f32(delta, gb, orc):
    a = gb.gen_grid(96, 128, 3, "f32")
    run_and_check(gb, orc, a.row, a.col, a.w, 0, delta=delta)


def test_f32_rmat_random_sources(gb, orc):
    a = gb.gen_rmat(12, 16, 9, "f32")
    for s in gb.sample_sources(a, 3, 2):
        run_and_check(gb, orc, a.row, a.col, a.w, int(s))


def test_isolated_source_and_unreached(gb, orc):
    a = gb.gen_rmat(10, 4, 1)
    deg = np.diff(a.row.astype(np.int64))
    iso = int(np.nonzero(deg == 0)[0][0])
    d, p, st = run_and_check(gb, orc, a.row, a.col, a.w, iso)
    assert st["reached"] == 1 and d[iso] == 0 and p[iso] == iso
    assert np.all(d[np.arange(a.n) != iso] == U32MAX) and np.all(p[np.arange(a.n) != iso] == -1)


def test_multi_source_rows_match_single(gb, orc):
    a = gb.gen_rmat(12, 16, 4)
    srcs = gb.sample_sources(a, 4, 3)
    with gb.Graph.from_host(a) as g:
        D, P, st = g.sssp_multi(srcs, want_pred=True)
        for i, s in enumerate(srcs):
            d, p, _ = g.sssp(int(s))
            assert np.array_equal(D[i], d) and np.array_equal(P[i], p)


def test_device_outputs(gb, orc):
    """gbs_sssp_device writes into caller-owned device memory (torch tensors
    here, used only as device allocations)."""
    torch = pytest.importorskip("torch")
    a = gb.gen_rmat(11, 16, 6)
    dd = torch.empty(a.n, dtype=torch.int32, device="cuda")
    pd = torch.empty(a.n, dtype=torch.int32, device="cuda")
    with gb.Graph.from_host(a) as g:
        g.sssp_device(5, dd.data_ptr(), pd.data_ptr())
        d, p, _ = g.sssp(5)
    assert np.array_equal(dd.cpu().numpy().view(np.uint32), d)
    assert np.array_equal(pd.cpu().numpy(), p)


def test_invalid_source(gb):
    a = gb.gen_rmat(8, 4, 1)
    with gb.Graph.from_host(a) as g:
        with pytest.raises(gb.GbsError) as e:
            g.sssp(a.n)
        assert e.value.name == "INVALID_ARG"


def test_wait_limit_returns_timeout_and_device_recovers(gb, orc):
    """One CTA never arrives at the first barrier (GBS_F_TEST_STALL): every
    bounded wait runs out, the call reports TIMEOUT, and the next run on the
    same graph is correct."""
    a = gb.gen_rmat(10, 16, 2)
    with gb.Graph.from_host(a) as g:
        with pytest.raises(gb.GbsError) as e:
            g.sssp(3, flags=0x80000000, wait_limit_ms=200)
        assert e.value.name == "TIMEOUT"
        d, p, _ = g.sssp(3)
    ref = orc.dijkstra(a.row, a.col, a.w, 3)
    assert np.array_equal(d, ref)


def _fractional(a):
    """Fractional double weights in (0, 2): not float32-exact in general."""
    return a.col.astype(np.float64) / 3072.0 + a.w.astype(np.float64) / 131.0


@pytest.mark.parametrize("delta,light", [(None, None), (0.05, None), (0.4, None), (2.5, None),
                                         (0.4, 0.0), (0.4, 10.0), (100.0, None)])
def test_float64_rmat_deltas_and_splits(delta, light, gb, orc):
    """float64 weights: distances bit-identical to the float64 oracle (one
    rounding per relaxation, as the reference computes), predecessors the
    smallest tight in-neighbour found by the pass after the run."""
    a = gb.gen_rmat(12, 16, 13)
    w = _fractional(a)
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    d, p, st = run_and_check(gb, orc, a.row, a.col, w, src, delta=delta, light=light)
    assert d.dtype == np.float64 and st["reached"] == int(np.isfinite(d).sum())
    run_and_check(gb, orc, a.row, a.col, w, src, delta=delta, light=light, full_items=1)


def test_float64_grid_multi_and_device_outputs(gb, orc):
    torch = pytest.importorskip("torch")
    a = gb.gen_grid(40, 56, 5, "f32")
    w = a.w.astype(np.float64) / 7.0
    srcs = np.array([0, 17, 2239], dtype=np.uint32)
    with gb.Graph(a.row, a.col, w) as g:
        D, P, _ = g.sssp_multi(srcs, want_pred=True)
        dd = torch.empty(a.n, dtype=torch.float64, device="cuda")
        pd = torch.empty(a.n, dtype=torch.int32, device="cuda")
        g.sssp_device(17, dd.data_ptr(), pd.data_ptr())
        with pytest.raises(gb.GbsError) as e:
            gb.Plan(g, srcs)
        assert e.value.name == "UNSUPPORTED"
    for i, s in enumerate(srcs):
        ref = orc.dijkstra(a.row, a.col, w, int(s))
        assert np.array_equal(D[i], ref)
        assert np.array_equal(P[i], orc.min_tight_pred(a.row, a.col, w, int(s), ref))
    assert np.array_equal(dd.cpu().numpy(), D[1]) and np.array_equal(pd.cpu().numpy(), P[1])


@pytest.mark.parametrize("wtype", ["u32", "f32", "f64"])
def test_pinned_host_outputs(wtype, gb, orc):
    """gbs_sssp writes page-locked host outputs from the device directly and
    copies into any other host memory.  Pinned, pageable, mixed and single
    outputs all give the oracle's distances and predecessors."""
    a = gb.gen_rmat(12, 16, 23)
    w = {"u32": a.w, "f32": a.w.astype(np.float32) / 3.0, "f64": _fractional(a)}[wtype]
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    ref = orc.dijkstra(a.row, a.col, w, src)
    rp = orc.min_tight_pred(a.row, a.col, w, src, ref)
    with gb.Graph(a.row, a.col, w) as g:
        hd = gb.PinnedBuffer(a.n, g.dist_dtype)
        hp = gb.PinnedBuffer(a.n, np.int32)
        plain_d = np.empty(a.n, dtype=g.dist_dtype)
        plain_p = np.empty(a.n, dtype=np.int32)
        for od, op in ((hd.array, hp.array), (plain_d, plain_p), (hd.array, plain_p), (plain_d, hp.array)):
            od.fill(0)
            op.fill(0)
            g.sssp(src, out_dist=od, out_pred=op)
            assert np.array_equal(od, ref) and np.array_equal(op, rp)
        hd.array.fill(0)
        hp.array.fill(0)
        g.sssp(src, out_dist=hd.array, want_pred=False)
        assert np.array_equal(hd.array, ref) and not hp.array.any()
        g.sssp(src, want_dist=False, out_pred=hp.array)
        assert np.array_equal(hp.array, rp)
        hd.free()
        hp.free()


def test_reference_mirror_fractional_weights(gb, orc, ref_serial):
    """The Python mirror with fractional double weights returns the
    reference's own run_sspath_arr doubles bit for bit."""
    a = gb.gen_rmat(11, 16, 8)
    w = _fractional(a)
    gs = gb.TCsr(a.row[1:].astype(np.int64), a.col.astype(np.int64), w)
    out = gb.run_sspath_arr(gs, 17, 0.4)
    refd, _ = ref_serial.ref_sssp_arr(a.row, a.col, w, 17, 0.4)
    assert np.array_equal(out, refd)


def test_reference_mirror_run_sspath_arr(gb, orc):
    """The Python mirror of run_sspath_arr over a t_csr-shaped CSR (inclusive
    int64 end offsets, double weights) returns the reference's doubles."""
    a = gb.gen_rmat(11, 16, 8)
    gs = gb.TCsr(a.row[1:].astype(np.int64), a.col.astype(np.int64), a.w.astype(np.float64))
    out = gb.run_sspath_arr(gs, 17, 9.0)
    ref = orc.dijkstra(a.row, a.col, a.w, 17).astype(np.float64)
    ref[ref == U32MAX] = np.inf
    assert np.array_equal(out, ref) and np.array_equal(gs.weight, ref)
