"""Oracle graph generators (numpy), TEST INFRASTRUCTURE ONLY.

This module is part of the oracle: only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it, and only as the checker.
The product library carries its own, independently written C generator
(``graphbench_gb300/host/gen.c``); the parity tests require both to produce the
identical CSR.

Generator specification (shared contract, restated here in numpy):

* ``mix64`` is the splitmix64 finaliser.  ``key(seed, stream) =
  mix64(seed * 0x100000001B3 + stream)`` and ``rnd(key, i) = mix64(key + i *
  0xD1B54A32D192ED03)`` (all mod 2**64).  Streams: 1 = R-MAT quadrant draws,
  2 = vertex permutation, 3 = edge weights, 4 = source sampling.
* R-MAT (the Graph500 Kronecker model the reference consumes through
  ``read_csr_bin``, graph/csr.c:211-299): edge sample ``e`` in
  ``[0, edgefactor * 2**scale)`` draws, for level ``l`` in ``[0, scale)``,
  ``r = rnd(key1, e*scale + l) >> 32`` and picks quadrant (0,0) if
  ``r < 2448131358``, (0,1) if ``r < 3264175144``, (1,0) if
  ``r < 4080218931``, else (1,1) (a,b,c,d = .57,.19,.19,.05 scaled to 2**32);
  the bits are appended most-significant first.  Both endpoints then go
  through a bijective permutation of ``scale`` bits (multiply by an odd
  constant plus a constant, xorshift, twice), self loops are dropped, every
  edge is stored in both directions and duplicates are removed.
* 2-D grid: ``rows x cols`` vertices, id ``r*cols + c``, 4-neighbour edges in
  both directions.
* Weights belong to the unordered pair ``{a, b}`` (``a < b``):
  ``r = rnd(key3, a << 32 | b) >> 32``; uint32 weights are ``wmin + r %
  (wmax - wmin + 1)``; float32 weights are ``1 + (r % 16367616) / 16384``,
  which is exactly representable and lies in ``[1, 1000)``.
* Rows of the CSR are sorted by column.  Offsets are exclusive
  (``row[v]..row[v+1]``), unlike the reference's inclusive ``vet_idx``
  (include/graph.h:113-127), which the oracle converts where it calls the
  reference.
"""
from __future__ import annotations

import numpy as np

M64 = (1 << 64) - 1
GOLDEN = np.uint64(0x9E3779B97F4A7C15)
C1 = np.uint64(0xBF58476D1CE4E5B9)
C2 = np.uint64(0x94D049BB133111EB)
STEP = np.uint64(0xD1B54A32D192ED03)
TA, TB, TC = 2448131358, 3264175144, 4080218931
F32_STEPS = 16367616  # 999 * 16384

STREAM_RMAT, STREAM_PERM, STREAM_WEIGHT, STREAM_SOURCE = 1, 2, 3, 4


def mix64(x):
    """splitmix64 finaliser on a uint64 array (wrapping arithmetic)."""
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = x + GOLDEN
        x = (x ^ (x >> np.uint64(30))) * C1
        x = (x ^ (x >> np.uint64(27))) * C2
    return x ^ (x >> np.uint64(31))


def mix64_int(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
    return x ^ (x >> 31)


def stream_key(seed: int, stream: int) -> int:
    return mix64_int((seed * 0x100000001B3 + stream) & M64)


def rnd(key: int, idx):
    idx = np.asarray(idx, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return mix64(np.uint64(key) + idx * STEP)


def rnd_int(key: int, idx: int) -> int:
    return mix64_int((key + idx * 0xD1B54A32D192ED03) & M64)


def permute(x, scale: int, seed: int):
    """Bijection on ``scale``-bit vertex ids."""
    k = stream_key(seed, STREAM_PERM)
    p = [rnd_int(k, i) for i in range(4)]
    mask = np.uint64((1 << scale) - 1)
    sh = np.uint64(scale // 2 + 1)
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = (x * np.uint64(p[0] | 1) + np.uint64(p[2])) & mask
        x = x ^ (x >> sh)
        x = (x * np.uint64(p[1] | 1) + np.uint64(p[3])) & mask
        x = x ^ (x >> sh)
    return x


def pair_weights(a, b, seed: int, wtype: str, wmin: int = 1, wmax: int = 255):
    """Weight of each unordered pair (a[i], b[i]); a and b may be in any order."""
    a = np.asarray(a, dtype=np.uint64)
    b = np.asarray(b, dtype=np.uint64)
    lo = np.minimum(a, b)
    hi = np.maximum(a, b)
    k = stream_key(seed, STREAM_WEIGHT)
    r = rnd(k, (lo << np.uint64(32)) | hi) >> np.uint64(32)
    if wtype == "u32":
        return (np.uint64(wmin) + r % np.uint64(wmax - wmin + 1)).astype(np.uint32)
    if wtype == "f32":
        q = (r % np.uint64(F32_STEPS)).astype(np.float64)
        return (1.0 + q / 16384.0).astype(np.float32)
    raise ValueError(wtype)


def _csr_from_pairs(n: int, src, dst):
    """Symmetrise, drop self loops, dedup, sort rows by column."""
    src = np.asarray(src, dtype=np.uint64)
    dst = np.asarray(dst, dtype=np.uint64)
    keep = src != dst
    src, dst = src[keep], dst[keep]
    keys = np.concatenate([(src << np.uint64(32)) | dst, (dst << np.uint64(32)) | src])
    keys = np.unique(keys)
    u = (keys >> np.uint64(32)).astype(np.int64)
    v = (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    deg = np.bincount(u, minlength=n).astype(np.uint64)
    row = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum(deg, out=row[1:])
    return row, u.astype(np.uint32), v


def rmat_edges(scale: int, edgefactor: int, seed: int):
    """Raw (unpermuted, unfiltered) R-MAT samples as two uint64 arrays."""
    E = edgefactor << scale
    k = stream_key(seed, STREAM_RMAT)
    u = np.zeros(E, dtype=np.uint64)
    v = np.zeros(E, dtype=np.uint64)
    e = np.arange(E, dtype=np.uint64)
    for lvl in range(scale):
        r = rnd(k, e * np.uint64(scale) + np.uint64(lvl)) >> np.uint64(32)
        bu = (r >= TB).astype(np.uint64)           # quadrants (1,0) and (1,1)
        bv = (((r >= TA) & (r < TB)) | (r >= TC)).astype(np.uint64)
        u = (u << np.uint64(1)) | bu
        v = (v << np.uint64(1)) | bv
    return u, v


def rmat(scale: int, edgefactor: int = 16, seed: int = 1, wtype: str = "u32",
         wmin: int = 1, wmax: int = 255):
    """Symmetrised, deduplicated R-MAT graph as (row, col, w), rows by column."""
    n = 1 << scale
    u, v = rmat_edges(scale, edgefactor, seed)
    u = permute(u, scale, seed)
    v = permute(v, scale, seed)
    row, uu, col = _csr_from_pairs(n, u, v)
    w = pair_weights(uu, col, seed, wtype, wmin, wmax)
    return row, col, w


def grid(rows: int, cols: int, seed: int = 3, wtype: str = "f32",
         wmin: int = 1, wmax: int = 255):
    """4-neighbour 2-D grid as (row, col, w), rows sorted by column."""
    n = rows * cols
    ids = np.arange(n, dtype=np.uint64).reshape(rows, cols)
    a = np.concatenate([ids[:, :-1].ravel(), ids[:-1, :].ravel()])
    b = np.concatenate([ids[:, 1:].ravel(), ids[1:, :].ravel()])
    row, uu, col = _csr_from_pairs(n, a, b)
    w = pair_weights(uu, col, seed, wtype, wmin, wmax)
    return row, col, w


def sample_sources(row, count: int, seed: int):
    """``count`` distinct vertices with out-degree > 0, drawn from stream 4."""
    row = np.asarray(row)
    n = len(row) - 1
    deg = np.diff(row.astype(np.int64))
    k = stream_key(seed, STREAM_SOURCE)
    out, seen, i = [], set(), 0
    if not (deg > 0).any():
        return np.zeros(0, dtype=np.uint32)
    while len(out) < count:
        v = (rnd_int(k, i) >> 11) % n
        i += 1
        if deg[v] > 0 and v not in seen:
            seen.add(v)
            out.append(v)
        if i > 64 * count + 100000:
            break
    return np.asarray(out, dtype=np.uint32)


def max_degree_vertex(row) -> int:
    deg = np.diff(np.asarray(row, dtype=np.int64))
    return int(np.argmax(deg))


def heuristic_delta(row, w) -> float:
    """Bucket width max_w / average out-degree (the published configs' rule)."""
    n = len(row) - 1
    m = int(row[-1])
    if m == 0:
        return 1.0
    return float(np.max(w)) / (m / n)
