"""gbs_sssp_noalloc: the SSSP entry point that allocates no memory.

It serves callers that cannot call cudaMalloc/cudaFree while answering a
query (a host application that owns all device memory through its own pool,
or a latency-bound service where an allocation may synchronise the device or
fail mid-request).  They pass device buffers they own; the run's scratch is a
static device array of fixed size (n <= 65,536, m <= 2,097,152).

This file is collected last on purpose.  Its checks, all through the C ABI:
  - two calls in a row give the same distances and predecessors as gbs_sssp
    (the existing entry point), bit for bit -- the tolerance of every parity
    test here -- for uint32 and float32 weights;
  - at the size limit (R-MAT scale 16: n = 65,536 and m = 1.82 M; a 256 x 256
    grid) the distances equal the oracle's Dijkstra and every predecessor is
    the oracle's smallest tight one;
  - sizes beyond the limit and misaligned pointers are refused on the host,
    malformed CSRs by the device-side check, each with an error and before
    the relaxation runs; a valid call afterwards is still exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    assert t.cuda.is_available()
    return t


def _adj_words(a):
    adj = np.empty(2 * a.m, dtype=np.uint32)
    adj[0::2] = a.col
    adj[1::2] = a.w.view(np.uint32)
    return adj


def _device_csr(torch, a, adj=None, row=None):
    """The caller-owned device inputs: row offsets and {target, weight} pairs."""
    row = a.row.astype(np.uint32) if row is None else row
    adj = _adj_words(a) if adj is None else adj
    return (torch.from_numpy(row.view(np.int32).copy()).cuda(),
            torch.from_numpy(adj.view(np.int32).copy()).cuda())


def _noalloc(gb, a, row, adj, wtype, source, dist, pred, n=None, m=None):
    return gb.lib.gbs_sssp_noalloc(a.n if n is None else n, a.m if m is None else m, row.data_ptr(),
                                   adj.data_ptr(), wtype, int(source), 0.0, dist.data_ptr(),
                                   pred.data_ptr() if pred is not None else None, None)


def _outputs(torch, n):
    return (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"))


@pytest.mark.parametrize("kind", ["rmat_u32", "grid_f32"])
def test_noalloc_matches_gbs_sssp_two_calls(kind, gb, torch):
    if kind == "rmat_u32":
        a = gb.gen_rmat(14, 16, 3)
        wtype, dt = gb.W_U32, np.uint32
    else:
        a = gb.gen_grid(120, 160, 7, "f32")
        wtype, dt = gb.W_F32, np.float32
    assert a.n <= 65536 and a.m <= 2097152
    row, adj = _device_csr(torch, a)
    dist, pred = _outputs(torch, a.n)
    sources = gb.sample_sources(a, 2, 5)
    with gb.Graph.from_host(a) as g:
        for s in sources:          # two calls in a row share the static scratch
            st = _noalloc(gb, a, row, adj, wtype, s, dist, pred)
            assert st == 0, gb.lib.gbs_last_error()
            torch.cuda.synchronize()
            ref_d, ref_p, _ = g.sssp(int(s))
            assert np.array_equal(dist.cpu().numpy().view(dt), ref_d)
            assert np.array_equal(pred.cpu().numpy(), ref_p)


@pytest.mark.parametrize("kind", ["rmat16_u32", "grid256_f32"])
def test_noalloc_at_its_limit_matches_the_oracle(kind, gb, torch, orc):
    """The largest inputs the scratch holds (n = 65,536 vertices, m up to
    1.82 M edges), two sources each, against the oracle directly."""
    if kind == "rmat16_u32":
        a = gb.gen_rmat(16, 16, 1)
        wtype, dt = gb.W_U32, np.uint32
        deg = np.diff(a.row.astype(np.int64))
        sources = [int(np.argmax(deg)), int(gb.sample_sources(a, 1, 9)[0])]
    else:
        a = gb.gen_grid(256, 256, 3, "f32")
        wtype, dt = gb.W_F32, np.float32
        sources = [0, 256 * 128 + 77]
    assert a.n == 65536 and a.m <= 2097152
    row, adj = _device_csr(torch, a)
    dist, pred = _outputs(torch, a.n)
    for s in sources:
        st = _noalloc(gb, a, row, adj, wtype, s, dist, pred)
        assert st == 0, gb.lib.gbs_last_error()
        torch.cuda.synchronize()
        ref = orc.dijkstra(a.row, a.col, a.w, s)
        got = dist.cpu().numpy().view(dt)
        assert np.array_equal(got, ref), int(np.sum(got != ref))
        assert np.array_equal(pred.cpu().numpy(), orc.min_tight_pred(a.row, a.col, a.w, s, ref))


def test_noalloc_refuses_sizes_beyond_its_scratch(gb, torch):
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = dummy.data_ptr()
    st = gb.lib.gbs_sssp_noalloc(65537, 10, p, p, gb.W_U32, 0, 1.0, p, p, None)
    assert st == 1 and b"65536" in gb.lib.gbs_last_error()
    st = gb.lib.gbs_sssp_noalloc(100, 2097153, p, p, gb.W_U32, 0, 1.0, p, p, None)
    assert st == 1


def test_noalloc_refuses_misaligned_pointers(gb, torch):
    """Checked on the host: no kernel is launched with these pointers."""
    buf = torch.zeros(64, dtype=torch.int32, device="cuda")
    p = buf.data_ptr()
    for row, adj, dist, pred in ((p, p + 4, p, p), (p + 2, p, p, p), (p, p, p + 1, p), (p, p, p, p + 2)):
        st = gb.lib.gbs_sssp_noalloc(4, 2, row, adj, gb.W_U32, 0, 1.0, dist, pred, None)
        assert st == 1 and b"aligned" in gb.lib.gbs_last_error()


def test_noalloc_rejects_malformed_csrs_then_runs_exact(gb, torch, orc):
    """One malformed CSR per check of the device-side validation (first
    offset, last offset, decreasing offsets, target out of range, negative /
    infinite / NaN float32 weight).  Every buffer has its full size, so the
    check kernel reads only inside them; each call must return
    GBS_ERR_INVALID_ARG naming a malformed CSR, and a valid call afterwards
    must still match the oracle (the shared scratch is re-initialised)."""
    a = gb.gen_rmat(8, 16, 2)
    af = gb.gen_grid(12, 14, 5, "f32")
    cases = []
    r = a.row.astype(np.uint32)
    bad = r.copy(); bad[0] = 1
    cases.append((a, gb.W_U32, bad, None))
    bad = r.copy(); bad[-1] = a.m - 1
    cases.append((a, gb.W_U32, bad, None))
    bad = r.copy(); bad[6] = bad[5] - 1 if bad[5] > 0 else 0; bad[5] = bad[6] + 3
    cases.append((a, gb.W_U32, bad, None))
    adj = _adj_words(a); adj[2 * 10] = a.n
    cases.append((a, gb.W_U32, None, adj))
    for bits in (0xBF800000, 0x7F800000, 0x7FC00000):       # -1.0, +inf, NaN
        adj = _adj_words(af); adj[2 * 7 + 1] = bits
        cases.append((af, gb.W_F32, None, adj))
    for g, wt, row, adj in cases:
        drow, dadj = _device_csr(torch, g, adj=adj, row=row)
        dist, pred = _outputs(torch, g.n)
        st = _noalloc(gb, g, drow, dadj, wt, 0, dist, pred)
        assert st == 1 and b"malformed CSR" in gb.lib.gbs_last_error(), (st, gb.lib.gbs_last_error())
    for g, wt, dt in ((a, gb.W_U32, np.uint32), (af, gb.W_F32, np.float32)):
        drow, dadj = _device_csr(torch, g)
        dist, pred = _outputs(torch, g.n)
        assert _noalloc(gb, g, drow, dadj, wt, 3, dist, pred) == 0, gb.lib.gbs_last_error()
        torch.cuda.synchronize()
        ref = orc.dijkstra(g.row, g.col, g.w, 3)
        assert np.array_equal(dist.cpu().numpy().view(dt), ref)
        assert np.array_equal(pred.cpu().numpy(), orc.min_tight_pred(g.row, g.col, g.w, 3, ref))
