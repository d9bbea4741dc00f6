"""gbs_sssp_noalloc: the SSSP entry point that allocates no memory.

It serves callers that cannot call cudaMalloc/cudaFree while answering a
query (a host application that owns all device memory through its own pool,
or a latency-bound service where an allocation may synchronise the device or
fail mid-request).  They pass device buffers they own; the run's scratch is a
static device array of fixed size (n <= 65,536, m <= 2,097,152).

This file is collected last on purpose.  Its checks: two calls in a row
through the C ABI give the same distances and predecessors as gbs_sssp (the
existing entry point, bit for bit -- the tolerance of every parity test
here), for uint32 and float32 weights, and sizes beyond the limit are refused
with an error before any device work.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    assert t.cuda.is_available()
    return t


def _device_csr(torch, a):
    """The caller-owned device inputs: row offsets and {target, weight} pairs."""
    row = torch.from_numpy(a.row.astype(np.uint32).view(np.int32)).cuda()
    adj = np.empty(2 * a.m, dtype=np.uint32)
    adj[0::2] = a.col
    adj[1::2] = a.w.view(np.uint32)
    adj = torch.from_numpy(adj.view(np.int32)).cuda()
    return row, adj


def _noalloc(gb, torch, a, row, adj, wtype, source, dist, pred):
    st = gb.lib.gbs_sssp_noalloc(a.n, a.m, row.data_ptr(), adj.data_ptr(), wtype, int(source), 0.0,
                                 dist.data_ptr(), pred.data_ptr(), None)
    return st


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
    dist = torch.empty(a.n, dtype=torch.int32, device="cuda")
    pred = torch.empty(a.n, dtype=torch.int32, device="cuda")
    sources = gb.sample_sources(a, 2, 5)
    with gb.Graph.from_host(a) as g:
        for s in sources:          # two calls in a row share the static scratch
            st = _noalloc(gb, torch, a, row, adj, wtype, s, dist, pred)
            assert st == 0, gb.lib.gbs_last_error()
            torch.cuda.synchronize()
            ref_d, ref_p, _ = g.sssp(int(s))
            assert np.array_equal(dist.cpu().numpy().view(dt), ref_d)
            assert np.array_equal(pred.cpu().numpy(), ref_p)


def test_noalloc_refuses_sizes_beyond_its_scratch(gb, torch):
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = dummy.data_ptr()
    st = gb.lib.gbs_sssp_noalloc(65537, 10, p, p, gb.W_U32, 0, 1.0, p, p, None)
    assert st == 1 and b"65536" in gb.lib.gbs_last_error()
    st = gb.lib.gbs_sssp_noalloc(100, 2097153, p, p, gb.W_U32, 0, 1.0, p, p, None)
    assert st == 1
