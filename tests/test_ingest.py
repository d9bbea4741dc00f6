"""Graph ingest (graph/csr.c readers, duplicate removal) on the GPU.

CPU tests pin the oracle's restatement of the readers against the golden
CSRs the reference's own readers produced (tests/golden/ingest_golden.json,
input files in tests/golden/ingest/) and, where the reference is built here,
against its readers run live.  GPU tests parse the same files through the C
ABI and compare the exported CSR bit for bit (offsets, columns, weights),
check the rejected inputs, and run shortest paths and betweenness on graphs
built on the device against graphs uploaded from the host.
"""
import hashlib
import json
import struct
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
FILES = GOLD / "ingest"
CASES = json.loads((GOLD / "ingest_golden.json").read_text())


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _oracle_read(orc, case):
    data = (FILES / case["file"]).read_bytes()
    if case["kind"] == "text":
        return orc.read_text(data, case["direction"])
    return orc.read_bin(data, case["direction"], 1, case["dedup"])


def _ids(c):
    return f"{c['file']}-{'send' if c['direction'] else 'recv'}{'-dedup' if c['dedup'] else ''}"


def _bin(v_num, offset, pairs):
    return struct.pack("<4q", v_num, len(pairs), offset, v_num) + b"".join(struct.pack("<2q", a, b) for a, b in pairs)


# ---------------------------------------------------------------- CPU: oracle
@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_oracle_reader_matches_reference_golden(case, orc):
    row, col, w, _ = _oracle_read(orc, case)
    assert (sha(row), sha(col), sha(w)) == (case["row_sha"], case["col_sha"], case["w_sha"])
    if "row" in case:
        assert row.tolist() == case["row"] and col.tolist() == case["col"] and w.tolist() == case["w"]


def test_reference_readers_live(ref_serial, tmp_path):
    """The reference's scan_csr_idx + read_graph_csr and read_csr_bin, run here
    on a file out of row order: rows keep file order, the text weights sit at
    the file-order positions, the binary weights alternate 0.1 / 0.2."""
    orc = ref_serial
    txt = b"p sp 4 5 1 4\na 2 1 9\na 1 3 9\na 4 2 9\na 1 2 9\na 3 4 9\n"
    p = tmp_path / "t.txt"
    p.write_bytes(txt)
    re, cl, wt = orc.ref_read_graph(p, False, 1)
    row, col, w, _ = orc.read_text(txt, 1)
    assert re.tolist() == row[1:].astype(np.int64).tolist() == [2, 3, 4, 5]
    assert cl.tolist() == col.tolist() == [2, 1, 0, 3, 1]
    assert wt.tolist() == w.tolist() == [0.25, 0.75, 0.5, 0.5, 1.0]
    b = _bin(4, 1, [(2, 1), (1, 3), (4, 2), (1, 2)])
    p = tmp_path / "t.bin"
    p.write_bytes(b)
    re, cl, wt = orc.ref_read_graph(p, True, 0)
    row, col, w, _ = orc.read_bin(b, 0)
    assert re.tolist() == row[1:].astype(np.int64).tolist()
    assert cl.tolist() == col.tolist() and wt.tolist() == w.tolist() == [0.1, 0.2, 0.1, 0.2]


def test_oracle_dedup_keeps_first_occurrence(orc):
    a = np.array([3, 1, 3, 1, 2, 1], dtype=np.int64)
    b = np.array([1, 2, 1, 2, 2, 5], dtype=np.int64)
    x, y = orc.dedup_pairs(a, b)
    assert list(zip(x.tolist(), y.tolist())) == [(3, 1), (1, 2), (2, 2), (1, 5)]


# ---------------------------------------------------------------- GPU
def _need_gpu(gb):
    assert gb.device_available(), "GPU tests need a CUDA device (compute capability 10.x)"


def _gpu_read(gb, case, from_bytes=False):
    """from_bytes: False reads the file, True parses its bytes, "pinned"
    parses them from a page-locked uint8 array."""
    path = FILES / case["file"]
    data = path.read_bytes()
    if from_bytes == "pinned":
        pin = gb.PinnedBuffer(len(data), np.uint8)
        pin.array[:] = np.frombuffer(data, dtype=np.uint8)
        data = pin.array
    if case["kind"] == "text":
        if from_bytes:
            return gb.DeviceCsr.parse_text(data, case["direction"])
        return gb.DeviceCsr.read_text(path, case["direction"])
    if from_bytes:
        return gb.DeviceCsr.parse_bin(data, case["direction"], 1, case["dedup"])
    return gb.DeviceCsr.read_bin(path, case["direction"], 1, case["dedup"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_gpu_reader_matches_reference_golden(case, gb):
    _need_gpu(gb)
    for from_bytes in (False, True, "pinned"):
        with _gpu_read(gb, case, from_bytes) as c:
            row, col, w = c.export()
            assert (sha(row), sha(col), sha(w)) == (case["row_sha"], case["col_sha"], case["w_sha"])
            assert c.n == case["n"] and c.m == case["m"]
            if case["dedup"]:
                assert c.info["duplicates"] == c.info["records"] - case["m"] > 0


@pytest.mark.gpu
def test_gpu_text_large_generated(gb, orc, tmp_path):
    """R-MAT scale 14 written as text, rows out of order: the GPU parse equals
    the oracle's restatement; the binary form of the same edges too."""
    _need_gpu(gb)
    from oracle import gen
    u, v = gen.rmat_edges(14, 8, 23)
    u = u.astype(np.int64)
    v = v.astype(np.int64)
    lines = [b"p sp 16384 %d 1 16384" % len(u)] + [b"a %d %d 1" % (a + 1, b + 1) for a, b in zip(u, v)]
    txt = b"\n".join(lines) + b"\n"
    p = tmp_path / "r.txt"
    p.write_bytes(txt)
    for d in (gb.DIR_SEND, gb.DIR_RECV):
        with gb.DeviceCsr.read_text(p, d) as c:
            row, col, w = c.export()
        r2, c2, w2, _ = orc.read_text(txt, d)
        assert np.array_equal(row, r2) and np.array_equal(col, c2) and np.array_equal(w, w2)
    b = _bin(16384, 1, list(zip((u + 1).tolist(), (v + 1).tolist())))
    for dedup in (False, True):
        with gb.DeviceCsr.parse_bin(b, gb.DIR_SEND, 1, dedup) as c:
            row, col, w = c.export()
        r2, c2, w2, _ = orc.read_bin(b, 1, 1, dedup)
        assert np.array_equal(row, r2) and np.array_equal(col, c2) and np.array_equal(w, w2)


@pytest.mark.gpu
def test_gpu_ingest_rejects_bad_input(gb, tmp_path):
    _need_gpu(gb)
    bad = [
        b"a 1 2 3\np sp 3 1 1 3\n",               # record before the header
        b"c nothing here\n",                       # no header
        b"p sp 3 1 1 3\na 1 x 3\n",                # not an integer
        b"p sp 3 1 1 3\na 1 4 3\n",                # column past v_num
        b"p sp 3 1 1 3\na 0 2 3\n",                # row below 0 after the offset
    ]
    for data in bad:
        with pytest.raises(gb.GbsError) as e:
            gb.DeviceCsr.parse_text(data)
        assert e.value.status == 1
    with pytest.raises(gb.GbsError):
        gb.DeviceCsr.parse_bin(b"\x00" * 16)       # short header
    with pytest.raises(gb.GbsError):
        gb.DeviceCsr.parse_bin(_bin(3, 1, [(1, 2)])[:-8])   # truncated pairs
    with pytest.raises(gb.GbsError):
        gb.DeviceCsr.parse_bin(_bin(3, 1, [(1, 9)]))        # column past v_num
    with pytest.raises(gb.GbsError):
        gb.DeviceCsr.read_text(tmp_path / "missing.txt")
    # uint32 graphs need integer weights; the text weights are fractions
    with gb.DeviceCsr.parse_text(b"p sp 3 2 1 3\na 1 2 1\na 2 3 1\n") as c:
        with pytest.raises(gb.GbsError):
            c.graph(gb.W_U32)


@pytest.mark.gpu
@pytest.mark.parametrize("wtype", ["f64", "f32"])
def test_gpu_graph_from_device_csr_equals_host_upload(wtype, gb, orc):
    """A graph built on the device from the ingested CSR gives the same
    shortest paths (distances and predecessors) as the same CSR uploaded from
    the host, and the same betweenness."""
    _need_gpu(gb)
    data = (FILES / "rmat8.txt").read_bytes()
    with gb.DeviceCsr.parse_text(data) as c:
        row, col, w = c.export()
        wt = {"f64": gb.W_F64, "f32": gb.W_F32}[wtype]
        wh = w if wtype == "f64" else w.astype(np.float32)
        with c.graph(wt) as gd, gb.Graph(row, col, wh) as gh:
            assert gd.n == gh.n and gd.m == gh.m
            src = [int(s) for s in np.nonzero(np.diff(row.astype(np.int64)))[0][:6]]
            for s in src:
                d1, p1, _ = gd.sssp(s)
                d2, p2, _ = gh.sssp(s)
                assert np.array_equal(d1, d2) and np.array_equal(p1, p2)
                assert np.array_equal(d1, orc.dijkstra(row, col, wh, s))
            b1, _ = gd.betweenness(src)
            b2, _ = gh.betweenness(src)
            assert np.array_equal(b1, b2)


@pytest.mark.gpu
def test_gpu_graph_from_bin_integer_weights(gb, orc):
    """Binary graphs carry 0.1 / 0.2 weights; the device build sorts every
    row by (weight, column) as the host upload does."""
    _need_gpu(gb)
    with gb.DeviceCsr.read_bin(FILES / "rmat8.bin", gb.DIR_SEND, 1, True) as c:
        row, col, w = c.export()
        with c.graph(gb.W_F64) as g:
            d, p, _ = g.sssp(int(np.argmax(np.diff(row.astype(np.int64)))))
            ref = orc.dijkstra(row, col, w, int(np.argmax(np.diff(row.astype(np.int64)))))
            assert np.array_equal(d, ref)
