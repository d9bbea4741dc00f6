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
