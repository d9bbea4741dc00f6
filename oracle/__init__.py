"""CPU oracle for the delta-stepping SSSP path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg (and ``bench.py --impl reference``) may import this package, and only as
the checker or the timed CPU baseline.  The product library
(``graphbench_gb300``) never imports it.

Contents:

* ``gen``               -- numpy restatement of the synthetic graph generators.
* ``liboracle.so``      -- ``oracle.c``: serial delta-stepping restated from
                           sssp/csr_sspath_array.c, Dijkstra, predecessor
                           rules and checkers (built by ``build()``).
* ``_ref/libref_*.so``  -- the reference's own sources (patched D1, D2, D4,
                           P0), built by ``build_ref.py``; ``ref_sssp_arr`` /
                           ``ref_sssp_list`` call them through
                           ``ref_driver.c``.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from pathlib import Path

import numpy as np

from . import gen  # noqa: F401  (re-exported)

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"

_P = ctypes.c_void_p
_u32, _i64, _i32, _dbl = ctypes.c_uint32, ctypes.c_int64, ctypes.c_int32, ctypes.c_double


def build(force: bool = False) -> Path:
    """Compile oracle.c into liboracle.so (seconds; no GPU needed)."""
    src = HERE / "oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-fno-fast-math",
                        "-ffp-contract=off", "-o", str(LIB_PATH), str(src), "-lm"],
                       check=True)
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        for name in ("or_dijkstra_u32", "or_dijkstra_f32", "or_dijkstra_f64"):
            getattr(L, name).argtypes = [_u32, _P, _P, _P, _u32, _P]
            getattr(L, name).restype = ctypes.c_int
        for name in ("or_min_tight_pred_u32", "or_min_tight_pred_f32", "or_min_tight_pred_f64"):
            getattr(L, name).argtypes = [_u32, _P, _P, _P, _u32, _P, _P]
            getattr(L, name).restype = ctypes.c_int
        for name in ("or_check_preds_u32", "or_check_preds_f32", "or_check_preds_f64"):
            getattr(L, name).argtypes = [_u32, _P, _P, _P, _u32, _P, _P]
            getattr(L, name).restype = _i64
        for name in ("or_delta_stepping_u32", "or_delta_stepping_f32", "or_delta_stepping_f64"):
            getattr(L, name).argtypes = [_u32, _P, _P, _P, _u32, _dbl, _P, _P]
            getattr(L, name).restype = ctypes.c_int
        L.or_pagerank.argtypes = [_u32, _P, _P, ctypes.c_double, ctypes.c_double, _u32, _P]
        L.or_pagerank.restype = ctypes.c_int
        for name in ("or_bc_u32", "or_bc_f32", "or_bc_f64"):
            getattr(L, name).argtypes = [_u32, _P, _P, _P, _u32, _P, _P]
            getattr(L, name).restype = ctypes.c_int
        L.or_count_tight_preds_f64.argtypes = [_u32, _P, _P, _P, _u32, _P, _P]
        L.or_fill_tight_preds_f64.argtypes = [_u32, _P, _P, _P, _u32, _P, _P, _P, _P]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _prep(row, col, w):
    row = np.ascontiguousarray(row, dtype=np.uint64)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    w = np.ascontiguousarray(w)
    if w.dtype not in (np.uint32, np.float32, np.float64):
        raise TypeError(f"weights must be uint32, float32 or float64, not {w.dtype}")
    return row, col, w


def dijkstra(row, col, w, src: int) -> np.ndarray:
    """Least-fixpoint distances in the weight type (u32: UINT32_MAX unreached;
    f32 / f64: +inf unreached)."""
    row, col, w = _prep(row, col, w)
    n = len(row) - 1
    if w.dtype == np.uint32:
        d = np.empty(n, dtype=np.uint32)
        rc = lib().or_dijkstra_u32(n, _ptr(row), _ptr(col), _ptr(w), src, _ptr(d))
    elif w.dtype == np.float64:
        d = np.empty(n, dtype=np.float64)
        rc = lib().or_dijkstra_f64(n, _ptr(row), _ptr(col), _ptr(w), src, _ptr(d))
    else:
        d = np.empty(n, dtype=np.float32)
        rc = lib().or_dijkstra_f32(n, _ptr(row), _ptr(col), _ptr(w.astype(np.float32)), src, _ptr(d))
    if rc != 0:
        raise RuntimeError(f"oracle dijkstra failed ({rc})")
    return d


def delta_stepping(row, col, w, src: int, delta: float):
    """Restated serial run_sspath_arr.  Returns (dist, buckets_walked); dist is
    float64 for u32/f64 weights and float32 for f32 weights."""
    row, col, w = _prep(row, col, w)
    n = len(row) - 1
    phases = np.zeros(1, dtype=np.int64)
    if w.dtype == np.uint32:
        d = np.empty(n, dtype=np.float64)
        fn = lib().or_delta_stepping_u32
    elif w.dtype == np.float32:
        d = np.empty(n, dtype=np.float32)
        fn = lib().or_delta_stepping_f32
    else:
        d = np.empty(n, dtype=np.float64)
        fn = lib().or_delta_stepping_f64
    rc = fn(n, _ptr(row), _ptr(col), _ptr(w), src, float(delta), _ptr(d), _ptr(phases))
    if rc != 0:
        raise RuntimeError(f"oracle delta_stepping failed ({rc})")
    return d, int(phases[0])


def min_tight_pred(row, col, w, src: int, dist) -> np.ndarray:
    row, col, w = _prep(row, col, w)
    n = len(row) - 1
    p = np.empty(n, dtype=np.int32)
    if w.dtype == np.uint32:
        lib().or_min_tight_pred_u32(n, _ptr(row), _ptr(col), _ptr(w), src,
                                    _ptr(np.ascontiguousarray(dist, dtype=np.uint32)), _ptr(p))
    elif w.dtype == np.float64:
        lib().or_min_tight_pred_f64(n, _ptr(row), _ptr(col), _ptr(w), src,
                                    _ptr(np.ascontiguousarray(dist, dtype=np.float64)), _ptr(p))
    else:
        lib().or_min_tight_pred_f32(n, _ptr(row), _ptr(col), _ptr(w.astype(np.float32)), src,
                                    _ptr(np.ascontiguousarray(dist, dtype=np.float32)), _ptr(p))
    return p


def check_preds(row, col, w, src: int, dist, pred) -> int:
    """Number of predecessor violations (0 = every reached vertex's pred edge
    is tight in the weight type and unreached vertices have pred -1)."""
    row, col, w = _prep(row, col, w)
    n = len(row) - 1
    pred = np.ascontiguousarray(pred, dtype=np.int32)
    if w.dtype == np.uint32:
        return int(lib().or_check_preds_u32(n, _ptr(row), _ptr(col), _ptr(w), src,
                                            _ptr(np.ascontiguousarray(dist, dtype=np.uint32)), _ptr(pred)))
    if w.dtype == np.float64:
        return int(lib().or_check_preds_f64(n, _ptr(row), _ptr(col), _ptr(w), src,
                                            _ptr(np.ascontiguousarray(dist, dtype=np.float64)), _ptr(pred)))
    return int(lib().or_check_preds_f32(n, _ptr(row), _ptr(col), _ptr(w.astype(np.float32)), src,
                                        _ptr(np.ascontiguousarray(dist, dtype=np.float32)), _ptr(pred)))


def all_tight_preds(row, col, w, src: int, dist):
    """(offsets, preds): every tight in-edge source per vertex, in increasing
    source order, computed in float64 (the reference's arithmetic)."""
    row = np.ascontiguousarray(row, dtype=np.uint64)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    wd = np.ascontiguousarray(w, dtype=np.float64)
    dd = np.ascontiguousarray(dist, dtype=np.float64)
    n = len(row) - 1
    cnt = np.zeros(n, dtype=np.uint64)
    lib().or_count_tight_preds_f64(n, _ptr(row), _ptr(col), _ptr(wd), src, _ptr(dd), _ptr(cnt))
    off = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum(cnt, out=off[1:])
    cur = np.empty(n, dtype=np.uint64)
    out = np.empty(int(off[-1]), dtype=np.uint32)
    lib().or_fill_tight_preds_f64(n, _ptr(row), _ptr(col), _ptr(wd), src, _ptr(dd),
                                  _ptr(off[:-1].copy()), _ptr(cur), _ptr(out))
    return off, out


# ----------------------------------------------------------- the reference
_ref_libs: dict[str, ctypes.CDLL] = {}


def ref_available(variant: str = "serial") -> bool:
    return (REF_DIR / f"libref_{variant}.so").exists()


def ref_lib(variant: str = "serial") -> ctypes.CDLL:
    if variant not in _ref_libs:
        path = REF_DIR / f"libref_{variant}.so"
        L = ctypes.CDLL(str(path), mode=os.RTLD_LOCAL | os.RTLD_NOW)
        L.gbref_sssp_arr.argtypes = [_i64, _i64, _P, _P, _P, _i64, _dbl, ctypes.c_int,
                                     ctypes.c_int, _dbl, _P, _P]
        L.gbref_sssp_arr.restype = ctypes.c_int
        L.gbref_sssp_list.argtypes = [_i64, _i64, _P, _P, _P, _i64, _dbl, _P, _P, _P, _i64, _P]
        L.gbref_sssp_list.restype = ctypes.c_int
        L.gbref_bc.argtypes = [_i64, _i64, _P, _P, _P, _i64, _P, _dbl, ctypes.c_int, _P, _P, _P]
        L.gbref_bc.restype = ctypes.c_int
        L.gbref_read_graph.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _i64,
                                       _i64, _P, _P, _P, _P]
        L.gbref_read_graph.restype = ctypes.c_int
        _ref_libs[variant] = L
    return _ref_libs[variant]


def ref_bucket_count(maxdist: float, delta: float) -> int:
    return int(math.floor(maxdist / delta)) + 2


def ref_sssp_arr(row, col, w, src: int, delta: float, *, variant: str = "serial",
                 threads: int = 1, buckets: int | None = None, cap_mult: float = 2.0,
                 maxdist: float | None = None):
    """The reference's run_sspath_arr (patched) on this CSR.  Returns
    (dist float64, seconds).  ``buckets`` defaults to a count derived from
    ``maxdist`` (computed with the oracle's Dijkstra when not given)."""
    row64 = np.ascontiguousarray(row, dtype=np.int64)
    col64 = np.ascontiguousarray(col, dtype=np.int64)
    wd = np.ascontiguousarray(w, dtype=np.float64)
    n = len(row64) - 1
    if buckets is None:
        if maxdist is None:
            d = dijkstra(row, col, w, src).astype(np.float64)
            if np.asarray(w).dtype == np.uint32:
                d[d == np.float64(0xFFFFFFFF)] = np.inf
            fin = d[np.isfinite(d)]
            maxdist = float(fin.max()) if len(fin) else 0.0
        buckets = ref_bucket_count(maxdist, delta)
    out = np.empty(n, dtype=np.float64)
    secs = np.zeros(1, dtype=np.float64)
    rc = ref_lib(variant).gbref_sssp_arr(n, int(row64[-1]), _ptr(row64), _ptr(col64), _ptr(wd),
                                         int(src), float(delta), int(threads), int(buckets),
                                         float(cap_mult), _ptr(out), _ptr(secs))
    if rc != 0:
        raise RuntimeError(f"reference run_sspath_arr failed (code {rc})")
    return out, float(secs[0])


def ref_sssp_list(row, col, w, src: int, delta: float, pred_cap: int | None = None):
    """The reference's run_sspath (list variant) with predecessor lists.
    Returns (dist float64, pred_counts int64[n], preds int64[...], seconds)."""
    row64 = np.ascontiguousarray(row, dtype=np.int64)
    col64 = np.ascontiguousarray(col, dtype=np.int64)
    wd = np.ascontiguousarray(w, dtype=np.float64)
    n = len(row64) - 1
    m = int(row64[-1])
    cap = pred_cap if pred_cap is not None else 4 * m + 16
    dist = np.empty(n, dtype=np.float64)
    cnt = np.empty(n, dtype=np.int64)
    lst = np.empty(cap, dtype=np.int64)
    secs = np.zeros(1, dtype=np.float64)
    rc = ref_lib("serial").gbref_sssp_list(n, m, _ptr(row64), _ptr(col64), _ptr(wd), int(src),
                                           float(delta), _ptr(dist), _ptr(cnt), _ptr(lst), cap,
                                           _ptr(secs))
    if rc != 0:
        raise RuntimeError(f"reference run_sspath failed (code {rc})")
    return dist, cnt, lst[: int(cnt.sum())], float(secs[0])


def ref_bc(row, col, w, sources=None, delta: float = 0.1, dedup: bool = False):
    """The reference's Brandes loop (btwcentral/csr_bc.c:40-59: run_sspath,
    q_sort_double, comp_num_spath, comp_delta) on this CSR.  Returns
    (bc float64[n], duplicated predecessor entries, seconds).  run_sspath
    allocates 1000 buckets, so every distance must stay below 1000 * delta.
    ``dedup`` drops repeated entries of each predecessor list before the
    path counts (run_sspath appends a predecessor again whenever it
    re-relaxes an edge to an equal distance)."""
    row64 = np.ascontiguousarray(row, dtype=np.int64)
    col64 = np.ascontiguousarray(col, dtype=np.int64)
    wd = np.ascontiguousarray(w, dtype=np.float64)
    n = len(row64) - 1
    src = None if sources is None else np.ascontiguousarray(sources, dtype=np.int64)
    k = n if src is None else len(src)
    bc = np.empty(n, dtype=np.float64)
    dups = np.zeros(1, dtype=np.int64)
    secs = np.zeros(1, dtype=np.float64)
    rc = ref_lib("serial").gbref_bc(n, int(row64[-1]), _ptr(row64), _ptr(col64), _ptr(wd), k,
                                    _ptr(src) if src is not None else None, float(delta),
                                    int(bool(dedup)), _ptr(bc), _ptr(dups), _ptr(secs))
    if rc != 0:
        raise RuntimeError(f"reference BC failed (code {rc})")
    return bc, int(dups[0]), float(secs[0])


def ref_read_graph(path, binary: bool, direction: int, cap_n: int = 1 << 20, cap_m: int = 1 << 22):
    """The reference's own readers on a file (graph/csr.c: scan_csr_idx +
    read_graph_csr for text, read_csr_bin for binary; direction 1 = SEND,
    0 = RECV).  Returns (row_end int64[n] inclusive, col int64[m],
    weight float64[m]) exactly as the reference leaves them in its t_csr."""
    p = Path(path).resolve()
    nm = np.zeros(2, dtype=np.int64)
    re = np.zeros(cap_n + 1, dtype=np.int64)
    cl = np.zeros(cap_m + 1, dtype=np.int64)
    wt = np.zeros(cap_m + 1, dtype=np.float64)
    rc = ref_lib("serial").gbref_read_graph(str(p.parent).encode() + b"/", p.name.encode(), int(bool(binary)),
                                            int(direction), cap_n, cap_m, _ptr(nm), _ptr(re), _ptr(cl), _ptr(wt))
    if rc != 0:
        raise RuntimeError(f"reference reader failed (code {rc})")
    n, m = int(nm[0]), int(nm[1])
    return re[:n].copy(), cl[:m].copy(), wt[:m].copy()


def betweenness(row, col, w, sources=None) -> np.ndarray:
    """Brandes betweenness over shortest paths summed over `sources` (all
    vertices when None), restating btwcentral/csr_bc.c:16-123 with each tight
    predecessor counted once.  Weights must be positive."""
    row, col, w = _prep(row, col, w)
    n = len(row) - 1
    bc = np.zeros(n, dtype=np.float64)
    src = None if sources is None else np.ascontiguousarray(sources, dtype=np.uint32)
    k = n if src is None else len(src)
    fn = {np.dtype(np.uint32): lib().or_bc_u32, np.dtype(np.float32): lib().or_bc_f32,
          np.dtype(np.float64): lib().or_bc_f64}[w.dtype]
    rc = fn(n, _ptr(row), _ptr(col), _ptr(w), k, _ptr(src) if src is not None else None, _ptr(bc))
    if rc != 0:
        raise RuntimeError(f"oracle betweenness failed ({rc})")
    return bc


# ------------------------------------------------------------ graph readers
def _text_records(data: bytes):
    """Header and "a" records of a text graph, line by line (graph/csr.c:
    scan_csr_idx :136-202 and read_graph_csr :4-60 read the same tokens)."""
    hdr = None
    recs = []
    for raw in data.split(b"\n"):
        tok = raw.split()
        if not tok:
            continue
        if tok[0] == b"p" and hdr is None:
            if recs:
                raise ValueError("an \"a\" line before the \"p\" line")
            hdr = [int(t) for t in tok[2:6]]
        elif tok[0] == b"a":
            if hdr is None:
                raise ValueError("an \"a\" line before the \"p\" line")
            if len(tok) < 4:
                raise ValueError("an \"a\" line without three integers")
            recs.append((int(tok[1]), int(tok[2]), int(tok[3])))
    if hdr is None:
        raise ValueError("no \"p\" line")
    return hdr, recs[: hdr[1]]


def _stable_csr(rows, cols, n):
    """Rows filled in input order (the reference's v_idx_tmp placement)."""
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    order = np.argsort(rows, kind="stable")
    row = np.zeros(n + 1, dtype=np.uint64)
    np.add.at(row, rows + 1, 1)
    return np.cumsum(row).astype(np.uint64), cols[order].astype(np.uint32)


def read_text(data: bytes, direction: int):
    """Restates scan_csr_idx + read_graph_csr (graph/csr.c:4-202) on the bytes
    of a text graph.  direction 1 = SEND (row = v_id - offset, column = v_to - 1),
    0 = RECV (row = v_to - offset, column = v_id - 1).  Weights: the k-th
    record's v_to / v_num at CSR position k (edge_info[e_num_read], :46).
    Returns (row_offsets uint64[n+1] exclusive, cols uint32[m], weights
    float64[m], header)."""
    hdr, recs = _text_records(data)
    v_num, offset = hdr[0], hdr[2]
    a = np.array([r[0] for r in recs], dtype=np.int64)
    b = np.array([r[1] for r in recs], dtype=np.int64)
    if direction == 1:
        rows, cols = a - offset, b - 1
    else:
        rows, cols = b - offset, a - 1
    if len(recs) and (rows.min() < 0 or rows.max() >= v_num or cols.min() < 0 or cols.max() >= v_num):
        raise ValueError("a row or column outside [0, v_num)")
    row, col = _stable_csr(rows, cols, v_num)
    w = b.astype(np.float64) / float(v_num)
    return row, col, w, hdr


def dedup_pairs(a, b):
    """remove_duplicate (partition/csr_partition_bin_mpi.c:47-105): keep the
    first occurrence of every (from, to) pair, in file order."""
    seen = set()
    keep = []
    for i, p in enumerate(zip(a.tolist(), b.tolist())):
        if p not in seen:
            seen.add(p)
            keep.append(i)
    keep = np.array(keep, dtype=np.int64)
    return a[keep], b[keep]


def read_bin(data: bytes, direction: int, target_offset: int = 1, dedup: bool = False):
    """Restates read_csr_bin (graph/csr.c:211-299): int64 header v_num, e_num,
    offset, g_v_size and e_num int64 (from, to) pairs.  SEND: row = from -
    offset, column = to - target_offset; RECV: row = to - offset, column = from
    - target_offset.  Weight of CSR position p: 0.1 if p is even, else 0.2."""
    hdr = np.frombuffer(data[:32], dtype="<i8").tolist()
    v_num, e_num, offset = hdr[0], hdr[1], hdr[2]
    pairs = np.frombuffer(data[32:32 + 16 * e_num], dtype="<i8").reshape(-1, 2)
    a, b = pairs[:, 0].copy(), pairs[:, 1].copy()
    if dedup:
        a, b = dedup_pairs(a, b)
    if direction == 1:
        rows, cols = a - offset, b - target_offset
    else:
        rows, cols = b - offset, a - target_offset
    if len(a) and (rows.min() < 0 or rows.max() >= v_num or cols.min() < 0 or cols.max() >= v_num):
        raise ValueError("a row or column outside [0, v_num)")
    row, col = _stable_csr(rows, cols, v_num)
    w = np.where(np.arange(len(col)) % 2 == 0, 0.1, 0.2)
    return row, col, w, hdr


def pagerank(in_row, in_col, random_jump: float = 0.3, threshold: float = 1e-6, max_iters: int = 10000):
    """The reference's PageRank iteration on an in-edge CSR (row v lists the
    sources of the edges into v), restating pagerank/pagerank_mpi.c:667-1043
    on one node.  Returns (rank float64[n], iterations)."""
    row = np.ascontiguousarray(in_row, dtype=np.uint64)
    col = np.ascontiguousarray(in_col, dtype=np.uint32)
    n = len(row) - 1
    out = np.empty(n, dtype=np.float64)
    it = lib().or_pagerank(n, _ptr(row), _ptr(col), float(random_jump), float(threshold), int(max_iters), _ptr(out))
    if it < 0:
        raise RuntimeError("oracle pagerank failed")
    return out, it


def transpose(row, col):
    """In-edge CSR of an out-edge CSR: row v of the result lists the u with an
    edge u -> v, in the order the out-edge CSR lists them (by u, then
    position)."""
    row = np.asarray(row, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    n = len(row) - 1
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(row))
    order = np.argsort(col, kind="stable")
    t_row = np.zeros(n + 1, dtype=np.uint64)
    np.add.at(t_row, col + 1, 1)
    return np.cumsum(t_row).astype(np.uint64), src[order].astype(np.uint32)
