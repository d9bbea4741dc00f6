"""The reference-named entry points of libgbsssp_compat.so (run_sspath_arr,
run_sspath over t_csr), exercised through a C program written like the
reference's caller (tests/compat_driver.c).

CPU: the library exports every name its header declares, the mirrored
structures have the reference's layout, and bad inputs take the reference's
error exit.  GPU: distances equal the oracle's and the reference's own
run_sspath_arr bit for bit (as doubles); predecessor lists hold the smallest
tight predecessor (array path) or every tight predecessor (list path)."""
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "graphbench_gb300"
INCLUDE = ROOT / "include"
COMPAT_LIB = PKG / "libgbsssp_compat.so"


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    out = tmp_path_factory.mktemp("compat") / "compat_driver"
    subprocess.run(["gcc", "-O2", "-std=c11", "-I", str(INCLUDE), str(ROOT / "tests" / "compat_driver.c"),
                    "-o", str(out), "-L", str(PKG), "-lgbsssp_compat", "-lgbsssp",
                    f"-Wl,-rpath,{PKG}"], check=True, capture_output=True, text=True)
    return out


def write_input(path, row, col, w, src, delta):
    n = len(row) - 1
    with open(path, "wb") as f:
        np.array([n, len(col), src], dtype=np.int64).tofile(f)
        np.array([delta], dtype=np.float64).tofile(f)
        np.asarray(row[1:], dtype=np.int64).tofile(f)          # inclusive row ends (vet_idx)
        np.asarray(col, dtype=np.int64).tofile(f)
        np.asarray(w, dtype=np.float64).tofile(f)


def read_output(path, n):
    raw = np.fromfile(path, dtype=np.uint8)
    dist = raw[: 8 * n].view(np.float64).copy()
    rest = raw[8 * n:].view(np.int64)
    lists, i = [], 0
    for _ in range(n):
        c = int(rest[i])
        lists.append(rest[i + 1: i + 1 + c].tolist())
        i += 1 + c
    return dist, lists


def run_driver(driver, tmp_path, row, col, w, src, delta, mode="arr", reps=1, extra=()):
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    write_input(inp, row, col, w, src, delta)
    r = subprocess.run([str(driver), str(inp), str(out), mode, str(reps), *extra],
                       capture_output=True, text=True, timeout=600)
    return r, out


# ------------------------------------------------------------------ CPU
def test_compat_exports_every_declared_function():
    text = (INCLUDE / "gbsssp_compat.h").read_text()
    declared = set(re.findall(r"^(?:void|gbs_status)\s+(\w+)\s*\(", text, re.M))
    assert {"run_sspath_arr", "run_sspath"} <= declared
    nm = subprocess.run(["nm", "-D", "--defined-only", str(COMPAT_LIB)], capture_output=True, text=True,
                        check=True).stdout
    exported = {ln.split()[-1] for ln in nm.splitlines() if " T " in ln}
    assert declared <= exported, declared - exported


PROBE = r"""
#include <stddef.h>
#include <stdio.h>
%s
int main(void) {
    printf("%%zu %%zu %%zu %%zu\n", sizeof(t_csr), sizeof(t_vi), sizeof(t_e), sizeof(t_list));
    printf("%%zu %%zu %%zu %%zu %%zu %%zu %%zu\n", offsetof(t_csr, vet_idx), offsetof(t_csr, edge_idx),
           offsetof(t_csr, vet_info), offsetof(t_csr, edge_info), offsetof(t_csr, v_size),
           offsetof(t_csr, e_size), offsetof(t_csr, global_v_size));
    printf("%%zu %%zu %%zu\n", offsetof(t_vi, weight), offsetof(t_e, edge_weight), offsetof(t_list, next));
    return 0;
}
"""


def _probe(tmp_path, name, include, flags):
    src = tmp_path / f"{name}.c"
    exe = tmp_path / name
    src.write_text(PROBE % include)
    subprocess.run(["gcc", "-std=gnu11", *flags, str(src), "-o", str(exe)], check=True, capture_output=True,
                   text=True)
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout


def test_compat_structs_match_reference_layout(tmp_path):
    staged = ROOT / "oracle" / "_ref" / "src" / "include"
    if not (staged / "list.h").exists():
        pytest.skip("the reference's headers are not staged (oracle/_ref)")
    stubs = ROOT / "oracle" / "stubs"
    ours = _probe(tmp_path, "ours", '#include "gbsssp_compat.h"', ["-I", str(INCLUDE)])
    ref = _probe(tmp_path, "ref", '#include "list.h"',
                 ["-include", str(stubs / "prelude.h"), "-I", str(stubs), "-I", str(staged), "-fopenmp"])
    assert ours == ref


def test_compat_driver_links(driver):
    assert driver.exists()


def test_compat_rejects_bad_input_like_the_reference(driver, tmp_path):
    """A negative or NaN weight, or a source out of range: the reference's
    ERROR_PRINT behaviour (message, exit 123), or a status with
    gbs_compat_set_exit(0).  Rejected before any device work."""
    row = np.array([0, 1, 2], dtype=np.int64)
    col = np.array([1, 0], dtype=np.int64)
    r, _ = run_driver(driver, tmp_path, row, col, np.array([0.5, -1.0]), 0, 0.4)
    assert r.returncode == 123 and "Error:" in r.stderr and "run_sspath_arr" in r.stderr
    r, _ = run_driver(driver, tmp_path, row, col, np.array([np.nan, 1.0]), 0, 0.4, extra=("noexit",))
    assert r.returncode == 0 and "status 1" in r.stdout
    r, _ = run_driver(driver, tmp_path, row, col, np.array([1.0, 2.0]), 5, 1.0, mode="list", extra=("noexit",))
    assert "status 1" in r.stdout   # source out of range


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("delta", [9.0, 0.4, 64.0])
def test_run_sspath_arr_matches_oracle_and_reference(delta, driver, tmp_path, gb, orc, ref_serial):
    a = gb.gen_rmat(12, 16, 4)
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    r, out = run_driver(driver, tmp_path, a.row, a.col, a.w, src, delta, reps=2)
    assert r.returncode == 0 and "status 0" in r.stdout, r.stderr
    dist, lists = read_output(out, a.n)
    ref = orc.dijkstra(a.row, a.col, a.w, src).astype(np.float64)
    ref[ref == np.float64(0xFFFFFFFF)] = np.inf
    assert np.array_equal(dist, ref)
    refd, _ = ref_serial.ref_sssp_arr(a.row, a.col, a.w, src, max(delta, 1.0))
    assert np.array_equal(dist, refd)
    mp = orc.min_tight_pred(a.row, a.col, a.w, src, orc.dijkstra(a.row, a.col, a.w, src))
    for v in range(a.n):
        if v == src or not np.isfinite(dist[v]):
            assert lists[v] == []
        else:
            assert lists[v] == [int(mp[v])]


@pytest.mark.gpu
def test_run_sspath_lists_every_tight_predecessor(driver, tmp_path, gb, orc):
    a = gb.gen_rmat(11, 16, 6, wmin=1, wmax=8)   # small weights: many ties
    src = 3
    r, out = run_driver(driver, tmp_path, a.row, a.col, a.w, src, 4.0, mode="list")
    assert r.returncode == 0 and "status 0" in r.stdout, r.stderr
    dist, lists = read_output(out, a.n)
    d32 = orc.dijkstra(a.row, a.col, a.w, src)
    ref = d32.astype(np.float64)
    ref[d32 == 0xFFFFFFFF] = np.inf
    assert np.array_equal(dist, ref)
    off, preds = orc.all_tight_preds(a.row, a.col, a.w, src, ref)
    multi = 0
    for v in range(a.n):
        want = sorted(set(preds[off[v]:off[v + 1]].tolist())) if np.isfinite(ref[v]) else []
        assert sorted(lists[v]) == want, v
        multi += len(want) > 1
    assert multi > 10


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["arr", "list"])
def test_fractional_weights_match_the_reference_doubles(mode, driver, tmp_path, gb, orc, ref_serial):
    """Weights like the reference's own reader makes (v_to / v_num,
    graph/csr.c:42): fractional doubles run in float64 and every distance
    equals the reference's run_sspath_arr bit for bit."""
    a = gb.gen_rmat(11, 16, 7)
    w = a.col.astype(np.float64) / 2048.0 + a.w.astype(np.float64) / 255.0
    src = int(np.argmax(np.diff(a.row.astype(np.int64))))
    r, out = run_driver(driver, tmp_path, a.row, a.col, w, src, 0.4, mode=mode, reps=2)
    assert r.returncode == 0 and "status 0" in r.stdout, r.stderr
    dist, lists = read_output(out, a.n)
    refd, _ = ref_serial.ref_sssp_arr(a.row, a.col, w, src, 0.4)
    assert np.array_equal(dist, refd)
    assert np.array_equal(dist, orc.dijkstra(a.row, a.col, w, src))
    if mode == "arr":
        mp = orc.min_tight_pred(a.row, a.col, w, src, dist)
        for v in range(a.n):
            assert lists[v] == ([] if v == src or not np.isfinite(dist[v]) else [int(mp[v])])
    else:
        off, preds = orc.all_tight_preds(a.row, a.col, w, src, dist)
        for v in range(a.n):
            want = sorted(set(preds[off[v]:off[v + 1]].tolist())) if np.isfinite(dist[v]) else []
            assert sorted(lists[v]) == want, v


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["arr", "list"])
def test_large_integer_weights_whose_sums_pass_uint32(mode, driver, tmp_path, gb, orc, ref_serial):
    """Integer weights of 3e9 on a multi-hop path: the sums pass 2^32 - 1, so
    the uint32 run overflows and the call reruns in float64.  The distances
    must equal the reference's doubles (integer sums below 2^53 are exact)."""
    # path 0 -> 1 -> ... -> 7 of weight 3e9 each, plus a cheap shortcut
    # 0 -> 5 of weight 1 and a back edge 7 -> 0
    edges = [(i, i + 1, 3.0e9) for i in range(7)] + [(0, 5, 1.0), (7, 0, 2.0)]
    n = 8
    edges.sort()
    row = np.zeros(n + 1, dtype=np.int64)
    for u, _, _ in edges:
        row[u + 1] += 1
    row = np.cumsum(row)
    col = np.array([v for _, v, _ in edges], dtype=np.int64)
    w = np.array([x for _, _, x in edges], dtype=np.float64)
    r, out = run_driver(driver, tmp_path, row, col, w, 0, 1.0e9, mode=mode, reps=2)
    assert r.returncode == 0 and "status 0" in r.stdout, r.stderr
    dist, lists = read_output(out, n)
    want = np.array([0, 3e9, 6e9, 9e9, 12e9, 1.0, 1.0 + 3e9, 1.0 + 6e9])
    assert np.array_equal(dist, want)
    refd, _ = ref_serial.ref_sssp_arr(row, col, w, 0, 1.0e9)
    assert np.array_equal(dist, refd)
    assert np.array_equal(dist, orc.dijkstra(row.astype(np.uint64), col.astype(np.uint32), w, 0))
    for v in range(1, n):
        assert lists[v] == [v - 1 if v != 5 else 0], (v, lists[v])


@pytest.mark.gpu
def test_run_sspath_arr_float32_grid(driver, tmp_path, gb, orc):
    a = gb.gen_grid(40, 50, 3, "f32")
    r, out = run_driver(driver, tmp_path, a.row, a.col, a.w.astype(np.float64), 0, 250.0, extra=("f32",))
    assert r.returncode == 0 and "status 0" in r.stdout, r.stderr
    dist, _ = read_output(out, a.n)
    assert np.array_equal(dist, orc.dijkstra(a.row, a.col, a.w, 0).astype(np.float64))


# ------------------------------------------------- readers and run_bc
GOLD = ROOT / "tests" / "golden"


@pytest.fixture(scope="module")
def io_driver(tmp_path_factory):
    out = tmp_path_factory.mktemp("compat_io") / "compat_io_driver"
    subprocess.run(["gcc", "-O2", "-std=c11", "-I", str(INCLUDE), str(ROOT / "tests" / "compat_io_driver.c"),
                    "-o", str(out), "-L", str(PKG), "-lgbsssp_compat", "-lgbsssp",
                    f"-Wl,-rpath,{PKG}"], check=True, capture_output=True, text=True)
    return out


def test_compat_io_driver_links(io_driver):
    assert io_driver.exists()


def _read_tcsr(path):
    raw = np.fromfile(path, dtype=np.uint8)
    hdr = raw[:32].view(np.int64)
    n, m = int(hdr[0]), int(hdr[1])
    per_v = raw[32:32 + 40 * n].reshape(n, 40)
    vet_idx = per_v[:, 0:8].copy().view(np.int64).ravel()
    weight = per_v[:, 8:16].copy().view(np.float64).ravel()
    wb = per_v[:, 16:24].copy().view(np.float64).ravel()
    recip = per_v[:, 24:32].copy().view(np.float64).ravel()
    deg = per_v[:, 32:40].copy().view(np.int64).ravel()
    per_e = raw[32 + 40 * n:].reshape(m, 16)
    col = per_e[:, 0:8].copy().view(np.int64).ravel()
    ew = per_e[:, 8:16].copy().view(np.float64).ravel()
    return hdr.tolist(), vet_idx, weight, wb, recip, deg, col, ew


@pytest.mark.gpu
@pytest.mark.parametrize("name,kind", [("hand.txt", "text"), ("rmat8.txt", "text"), ("hand.bin", "bin"),
                                       ("rmat8.bin", "bin")])
@pytest.mark.parametrize("direction", [1, 0])
def test_compat_readers_fill_tcsr_like_the_reference(name, kind, direction, io_driver, tmp_path, orc):
    out = tmp_path / "tcsr.bin"
    r = subprocess.run([str(io_driver), kind, str(GOLD / "ingest") + "/", name, str(direction), str(out)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    hdr, vet_idx, weight, wb, recip, deg, col, ew = _read_tcsr(out)
    data = (GOLD / "ingest" / name).read_bytes()
    row, c2, w2, h2 = orc.read_text(data, direction) if kind == "text" else orc.read_bin(data, direction)
    assert hdr == [h2[0], h2[1], h2[2], h2[3]]
    assert np.array_equal(vet_idx, row[1:].astype(np.int64))
    assert np.array_equal(col[: len(c2)], c2.astype(np.int64)) and np.array_equal(ew[: len(w2)], w2)
    d = np.diff(row.astype(np.int64))
    if kind == "text":   # scan_csr_idx's vertex fields
        assert np.all(weight == 1.0) and np.all(wb == 0) and np.array_equal(deg, d)
        with np.errstate(divide="ignore"):
            assert np.array_equal(recip, 1.0 / d.astype(np.float64))
    else:                # read_csr_bin's
        assert np.all(np.isinf(weight)) and np.all(wb == 0) and np.all(recip == 0) and np.all(deg == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hand.txt", "rmat8.txt"])
def test_compat_run_bc_prints_the_reference_report(name, io_driver, orc):
    """run_bc(file, dir): the reference's printout, values equal to the
    oracle's Brandes on the graph the reference's text reader builds."""
    r = subprocess.run([str(io_driver), "bc", str(GOLD / "ingest") + "/", name], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "the final result for betweeness centrality is:"
    pairs = [t.split(":") for t in lines[1].split()]
    row, col, w, _ = orc.read_text((GOLD / "ingest" / name).read_bytes(), 1)
    ours = orc.betweenness(row, col, w)
    assert [int(p[0]) for p in pairs] == list(range(1, len(row)))
    assert [p[1] for p in pairs] == ["%f" % x for x in ours]
