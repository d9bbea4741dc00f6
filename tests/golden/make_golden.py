"""Generates the committed golden fixtures in tests/golden/.

Run from the repository root where the reference tree is present, naming
it in GBREF_TREE:

    GBREF_TREE=<path of the GRAPHBENCH tree> python tests/golden/make_golden.py

1. ``known_answer.json``: small hand-built graphs with hand-computed distances
   and predecessors.  Before writing, every case is checked against the
   oracle's Dijkstra, the oracle's restated serial delta-stepping, and (for
   integer weights) the reference's own run_sspath_arr (patched D1, D2, D4, P0)
   and, where it applies, run_sspath's predecessor lists.
2. ``seeded.json``: seeded R-MAT / grid instances of the published configs'
   families at sizes the CPU finishes in seconds: CSR checksums, source,
   delta, and the SHA-256 of the oracle's distances and predecessors, each
   cross-checked against the reference (uint32) or the reference's double
   result within float32 rounding (float32).
3. ``rmat10_dist.npy`` / ``rmat10_pred.npy``: the full arrays of the first
   seeded case, for diagnostics.
4. ``bc_golden.json``: betweenness centrality over every source of small
   graphs, computed by the reference's own Brandes loop (run_sspath,
   q_sort_double, comp_num_spath, comp_delta; btwcentral/csr_bc.c:40-59).
   Where a vertex has several shortest-path predecessors the reference's
   lists repeat entries unevenly, so those cases are recorded from the
   reference with each list deduplicated (``dedup``); every case is checked
   against the oracle's Brandes restatement before it is written.
"""
from __future__ import annotations

import hashlib
import json
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from oracle import build_ref, gen  # noqa: E402

INF = math.inf
U32MAX = 0xFFFFFFFF

# (name, n, directed edge list (u, v, w), weight type, source, delta,
#  expected dist, expected min-tight pred, expected all tight preds or None)
KNOWN = [
    dict(name="path", n=5, undirected=True, wtype="u32", source=0, delta=2,
         edges=[(0, 1, 3), (1, 2, 1), (2, 3, 4), (3, 4, 1)],
         dist=[0, 3, 4, 8, 9], pred=[0, 0, 1, 2, 3]),
    dict(name="star", n=6, undirected=True, wtype="u32", source=3, delta=2,
         edges=[(0, 1, 5), (0, 2, 4), (0, 3, 3), (0, 4, 2), (0, 5, 1)],
         dist=[3, 8, 7, 0, 5, 4], pred=[3, 0, 0, 3, 0, 0]),
    dict(name="diamond_ties", n=5, undirected=False, wtype="u32", source=0, delta=2,
         edges=[(0, 1, 2), (0, 2, 1), (1, 3, 1), (2, 3, 2), (3, 4, 5), (0, 4, 8)],
         dist=[0, 2, 1, 3, 8], pred=[0, 0, 0, 1, 0],
         all_preds={3: [1, 2], 4: [0, 3]}),
    dict(name="sink_source", n=3, undirected=False, wtype="u32", source=0, delta=1,
         edges=[(1, 0, 1), (2, 1, 1)],
         dist=[0, None, None], pred=[0, -1, -1]),
    dict(name="disconnected", n=4, undirected=True, wtype="u32", source=2, delta=3,
         edges=[(0, 1, 2), (2, 3, 5)],
         dist=[None, None, 0, 5], pred=[-1, -1, 2, 2]),
    dict(name="parallel_edges", n=3, undirected=False, wtype="u32", source=0, delta=4,
         edges=[(0, 1, 7), (0, 1, 3), (1, 2, 2), (0, 2, 9), (0, 2, 5)],
         dist=[0, 3, 5], pred=[0, 0, 0]),
    dict(name="zero_weights_selfloop", n=3, undirected=False, wtype="u32", source=0, delta=1,
         edges=[(0, 1, 0), (1, 2, 0), (0, 2, 1), (2, 2, 3)],
         dist=[0, 0, 0], pred=[0, 0, 1]),
    dict(name="single_vertex", n=1, undirected=False, wtype="u32", source=0, delta=1,
         edges=[], dist=[0], pred=[0]),
    dict(name="long_light_chain", n=6, undirected=False, wtype="u32", source=0, delta=10,
         edges=[(0, 5, 9), (0, 1, 1), (1, 2, 1), (2, 3, 1), (3, 4, 1), (4, 5, 1)],
         dist=[0, 1, 2, 3, 4, 5], pred=[0, 0, 1, 2, 3, 4]),
    dict(name="heavy_reentry", n=4, undirected=False, wtype="u32", source=0, delta=4,
         edges=[(0, 1, 5), (0, 2, 3), (2, 1, 1), (1, 3, 6), (2, 3, 9)],
         dist=[0, 4, 3, 10], pred=[0, 2, 0, 1]),
    # float32 arithmetic: fl32(2^24 + 1) == 2^24, so the double reference differs
    dict(name="f32_rounding", n=4, undirected=False, wtype="f32", source=0, delta=8.0,
         edges=[(0, 1, 16777216.0), (1, 2, 1.0), (2, 3, 1.0), (0, 3, 16777218.0)],
         dist=[0.0, 16777216.0, 16777216.0, 16777216.0], pred=[0, 0, 1, 2]),
    dict(name="f32_fractional", n=4, undirected=True, wtype="f32", source=1, delta=0.75,
         edges=[(0, 1, 0.5), (1, 2, 0.25), (2, 3, 1.5), (0, 3, 1.25)],
         dist=[0.5, 0.0, 0.25, 1.75], pred=[1, 1, 1, 0]),
]


def to_csr(case):
    n = case["n"]
    edges = list(case["edges"])
    if case["undirected"]:
        edges = edges + [(v, u, w) for (u, v, w) in edges]
    # stable order: by source, then insertion order
    edges = sorted(enumerate(edges), key=lambda t: (t[1][0], t[0]))
    edges = [e for _, e in edges]
    row = np.zeros(n + 1, dtype=np.uint64)
    for (u, _, _) in edges:
        row[u + 1] += 1
    row = np.cumsum(row).astype(np.uint64)
    col = np.array([v for (_, v, _) in edges], dtype=np.uint32)
    dt = np.uint32 if case["wtype"] == "u32" else np.float32
    w = np.array([wt for (_, _, wt) in edges], dtype=dt)
    return row, col, w


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def expected_dist(case):
    if case["wtype"] == "u32":
        return np.array([U32MAX if d is None else d for d in case["dist"]], dtype=np.uint32)
    return np.array([np.inf if d is None else d for d in case["dist"]], dtype=np.float32)


def check_known(have_ref: bool):
    out = []
    for case in KNOWN:
        row, col, w = to_csr(case)
        src, delta = case["source"], case["delta"]
        exp = expected_dist(case)
        dj = oracle.dijkstra(row, col, w, src)
        assert np.array_equal(dj, exp), (case["name"], dj, exp)
        ds, _ = oracle.delta_stepping(row, col, w, src, delta)
        dj64 = dj.astype(np.float64)
        if case["wtype"] == "u32":
            dj64[dj == U32MAX] = np.inf
        assert np.array_equal(ds.astype(np.float64), dj64), (case["name"], ds, dj)
        pred = oracle.min_tight_pred(row, col, w, src, dj)
        assert pred.tolist() == case["pred"], (case["name"], pred, case["pred"])
        assert oracle.check_preds(row, col, w, src, dj, pred) == 0
        if have_ref and case["wtype"] == "u32":
            rd, _ = oracle.ref_sssp_arr(row, col, w, src, delta)
            assert np.array_equal(rd, dj64), (case["name"], "reference", rd, dj64)
            if "all_preds" in case:
                d2, cnt, lst, _ = oracle.ref_sssp_list(row, col, w, src, delta)
                assert np.array_equal(d2, dj64)
                off = np.concatenate([[0], np.cumsum(cnt)])
                for v, pl in case["all_preds"].items():
                    # run_sspath appends a predecessor on every relaxation with
                    # new <= old (sssp/csr_sspath.c:116-118), so a tight edge
                    # relaxed twice appears twice; compare as sets
                    got = sorted(set(lst[off[v]:off[v + 1]].tolist()))
                    assert got == pl, (case["name"], v, got, pl)
        rec = dict(case)
        rec["edges"] = [list(e) for e in case["edges"]]
        out.append(rec)
    return out


SEEDED = [
    dict(name="rmat10_u32", kind="rmat", scale=10, edgefactor=16, seed=1, wtype="u32"),
    dict(name="rmat12_u32", kind="rmat", scale=12, edgefactor=16, seed=1, wtype="u32"),
    dict(name="rmat14_u32", kind="rmat", scale=14, edgefactor=16, seed=1, wtype="u32"),
    dict(name="rmat16_u32", kind="rmat", scale=16, edgefactor=16, seed=1, wtype="u32"),
    dict(name="rmat12_f32", kind="rmat", scale=12, edgefactor=16, seed=5, wtype="f32"),
    dict(name="grid64_f32", kind="grid", rows=64, cols=64, seed=3, wtype="f32"),
    dict(name="grid48x80_u32", kind="grid", rows=48, cols=80, seed=9, wtype="u32"),
]


def make_seeded(case):
    if case["kind"] == "rmat":
        row, col, w = gen.rmat(case["scale"], case["edgefactor"], case["seed"], case["wtype"])
        src = gen.max_degree_vertex(row)
    else:
        row, col, w = gen.grid(case["rows"], case["cols"], case["seed"], case["wtype"])
        src = 0
    return row, col, w, src


def check_seeded(have_ref: bool):
    out = []
    for case in SEEDED:
        row, col, w, src = make_seeded(case)
        delta = gen.heuristic_delta(row, w)
        dj = oracle.dijkstra(row, col, w, src)
        pred = oracle.min_tight_pred(row, col, w, src, dj)
        assert oracle.check_preds(row, col, w, src, dj, pred) == 0
        ds, phases = oracle.delta_stepping(row, col, w, src, delta)
        dj64 = dj.astype(np.float64)
        if case["wtype"] == "u32":
            dj64[dj == U32MAX] = np.inf
            reached = int((dj != U32MAX).sum())
        else:
            reached = int(np.isfinite(dj).sum())
        assert np.array_equal(ds.astype(np.float64), dj64), case["name"]
        rec = dict(case)
        rec.update(n=int(len(row) - 1), m=int(row[-1]), source=int(src), delta=delta,
                   row_sha=sha(row), col_sha=sha(col), w_sha=sha(w),
                   dist_sha=sha(dj), pred_sha=sha(pred), reached=reached,
                   edges_reached=int(sum(int(row[v + 1] - row[v]) for v in np.nonzero(np.isfinite(dj64))[0])),
                   max_dist=float(dj64[np.isfinite(dj64)].max()), oracle_buckets=phases)
        if have_ref:
            rd, secs = oracle.ref_sssp_arr(row, col, w, src, delta)
            if case["wtype"] == "u32":
                assert np.array_equal(rd, dj64), (case["name"], "reference mismatch")
                rec["reference"] = "bit-exact"
            else:
                fin = np.isfinite(dj64)
                assert np.array_equal(np.isfinite(rd), fin)
                rel = float(np.max(np.abs(rd[fin] - dj64[fin]) / np.maximum(1.0, rd[fin])))
                rec["reference"] = f"double result within relative {rel:.3g} of the float32 fixpoint"
                assert rel < 1e-5
        out.append(rec)
        if case["name"] == "rmat10_u32":
            np.save(HERE / "rmat10_dist.npy", dj)
            np.save(HERE / "rmat10_pred.npy", pred)
    return out


# (name, graph, dedup): u32 cases with small weight ranges have many equal
# shortest paths (sigma > 1); the float64 case has fractional weights and
# unique predecessors, where the reference's raw lists give Brandes' result.
BC_CASES = [
    dict(name="bc_path5", kind="known", known="path"),
    dict(name="bc_diamond", kind="known", known="diamond_ties"),
    dict(name="bc_star", kind="known", known="star"),
    dict(name="bc_disconnected", kind="known", known="disconnected"),
    dict(name="bc_parallel", kind="known", known="parallel_edges"),
    dict(name="bc_rmat7_w1_4", kind="rmat", scale=7, edgefactor=8, seed=3, wtype="u32", wmax=4),
    dict(name="bc_rmat8_w1_255", kind="rmat", scale=8, edgefactor=8, seed=4, wtype="u32", wmax=255),
    dict(name="bc_grid8x9_w1_2", kind="grid", rows=8, cols=9, seed=5, wtype="u32", wmax=2),
    dict(name="bc_rmat7_f64", kind="rmat_f64", scale=7, edgefactor=8, seed=6),
]


def bc_graph(case):
    if case["kind"] == "known":
        kc = next(k for k in KNOWN if k["name"] == case["known"])
        return to_csr(kc)
    if case["kind"] == "rmat":
        return gen.rmat(case["scale"], case["edgefactor"], case["seed"], "u32", 1, case["wmax"])
    if case["kind"] == "grid":
        return gen.grid(case["rows"], case["cols"], case["seed"], "u32", 1, case["wmax"])
    row, col, w = gen.rmat(case["scale"], case["edgefactor"], case["seed"], "u32", 1, 255)
    return row, col, col.astype(np.float64) / 384.0 + w.astype(np.float64) / 131.0


def check_bc(have_ref: bool):
    out = []
    for case in BC_CASES:
        row, col, w = bc_graph(case)
        if np.asarray(w).dtype == np.float64:
            w = np.asarray(w, dtype=np.float64)
        bc = oracle.betweenness(row, col, w)
        rec = dict(case)
        rec.update(n=int(len(row) - 1), m=int(row[-1]), row_sha=sha(row), col_sha=sha(col), w_sha=sha(w))
        if have_ref:
            maxd = 0.0
            for s in range(len(row) - 1):
                d = oracle.dijkstra(row, col, w, s).astype(np.float64)
                if np.asarray(w).dtype == np.uint32:
                    d[d == float(U32MAX)] = np.inf
                fin = d[np.isfinite(d)]
                maxd = max(maxd, float(fin.max()) if len(fin) else 0.0)
            delta = max(0.1, maxd / 900.0)
            dedup = np.asarray(w).dtype != np.float64
            ref, dups, _ = oracle.ref_bc(row, col, w, delta=delta, dedup=dedup)
            rel = float(np.max(np.abs(ref - bc) / np.maximum(1.0, np.abs(ref))))
            assert rel < 1e-12, (case["name"], rel)
            rec.update(reference_delta=delta, reference_dedup=bool(dedup), reference_repeats=dups,
                       max_rel_vs_oracle=rel)
            rec["bc"] = [float(x) for x in ref]
        else:
            rec["bc"] = [float(x) for x in bc]
        rec["from_reference"] = bool(have_ref)
        out.append(rec)
    return out


# ------------------------------------------------------------ graph files
INGEST_DIR = HERE / "ingest"

# The reference reads whitespace-separated tokens, so a comment holding a
# lone "a" or "p" token is taken for a record (its reader crashed on one);
# the comments below avoid such tokens.
HAND_TEXT = (b"c hand-made graph: comments, blank lines, CRLF endings, records out of\r\n"
             b"c row order, leading blanks, and one record past e_num\r\n"
             b"p sp 6 7 1 6\r\n"
             b"\r\n"
             b"a 3 1 7\r\n"
             b"a 1 2 4\r\n"
             b"  a 1 6 9\r\n"
             b"a 2 3 1\r\n"
             b"c in the middle\r\n"
             b"a 6 4 2\r\n"
             b"a\t3 4 8\r\n"
             b"a 5 5 3\r\n"
             b"a 4 1 5\r\n")


def _bin_bytes(v_num, offset, pairs):
    import struct
    out = struct.pack("<4q", v_num, len(pairs), offset, v_num)
    for a, b in pairs:
        out += struct.pack("<2q", a, b)
    return out


def ingest_files():
    """(name, kind, bytes): hand-made and seeded graph files."""
    files = [("hand.txt", "text", HAND_TEXT)]
    u, v = gen.rmat_edges(8, 8, 17)          # raw samples: self loops and repeats included
    u = u.astype(np.int64)
    v = v.astype(np.int64)
    rng = np.random.default_rng(5)
    w = rng.integers(1, 100, len(u))
    lines = [b"c R-MAT scale 8 samples, file order as generated", b"p sp 256 %d 1 256" % len(u)]
    lines += [b"a %d %d %d" % (a + 1, b + 1, c) for a, b, c in zip(u.tolist(), v.tolist(), w.tolist())]
    files.append(("rmat8.txt", "text", b"\n".join(lines) + b"\n"))
    files.append(("hand.bin", "bin", _bin_bytes(5, 1, [(3, 1), (1, 2), (1, 5), (2, 3), (5, 4), (3, 4), (1, 2),
                                                        (3, 1), (4, 5)])))
    files.append(("rmat8.bin", "bin", _bin_bytes(256, 1, list(zip((u + 1).tolist(), (v + 1).tolist())))))
    return files


def make_ingest(have_ref: bool):
    """Expected CSRs of the graph files: the reference's own readers
    (scan_csr_idx + read_graph_csr, read_csr_bin) when it is built, checked
    against the oracle's restatement; duplicate removal restated (the
    reference's remove_duplicate needs its MPI driver) and then read by the
    reference's read_csr_bin."""
    INGEST_DIR.mkdir(exist_ok=True)
    out = []
    for name, kind, data in ingest_files():
        (INGEST_DIR / name).write_bytes(data)
        for direction in (1, 0):
            for dedup in ((False, True) if kind == "bin" else (False,)):
                if kind == "text":
                    row, col, w, hdr = oracle.read_text(data, direction)
                else:
                    row, col, w, hdr = oracle.read_bin(data, direction, 1, dedup)
                rec = dict(file=name, kind=kind, direction=direction, dedup=dedup, n=int(len(row) - 1),
                           m=int(len(col)), row_sha=sha(row), col_sha=sha(col), w_sha=sha(w))
                if have_ref:
                    path = INGEST_DIR / name
                    if dedup:
                        a = np.frombuffer(data[32:], dtype="<i8").reshape(-1, 2)
                        x, y = oracle.dedup_pairs(a[:, 0].copy(), a[:, 1].copy())
                        tmp = Path("/tmp") / f"gb_dedup_{name}"
                        tmp.write_bytes(_bin_bytes(hdr[0], hdr[2], list(zip(x.tolist(), y.tolist()))))
                        path = tmp
                    re, cl, wt = oracle.ref_read_graph(path, kind == "bin", direction)
                    assert np.array_equal(row[1:].astype(np.int64), re), (name, direction, "rows")
                    assert np.array_equal(col.astype(np.int64), cl), (name, direction, "cols")
                    assert np.array_equal(w, wt), (name, direction, "weights")
                    rec["reference"] = "bit-exact"
                if len(col) <= 16:
                    rec.update(row=row.tolist(), col=col.tolist(), w=w.tolist())
                out.append(rec)
    return out


def main():
    have_ref = build_ref.stage()
    if have_ref:
        build_ref.compile_ref()
    known = check_known(have_ref)
    seeded = check_seeded(have_ref)
    bc = check_bc(have_ref)
    ingest = make_ingest(have_ref)
    (HERE / "ingest_golden.json").write_text(json.dumps(ingest, indent=1) + "\n")
    (HERE / "bc_golden.json").write_text(json.dumps(bc) + "\n")
    (HERE / "known_answer.json").write_text(json.dumps(known, indent=1) + "\n")
    (HERE / "seeded.json").write_text(json.dumps(seeded, indent=1) + "\n")
    print(f"wrote {len(known)} known-answer, {len(seeded)} seeded and {len(bc)} betweenness cases; "
          f"reference checked: {have_ref}")


if __name__ == "__main__":
    main()
