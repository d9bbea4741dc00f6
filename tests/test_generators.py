"""The product's C generators (libgbsssp) against the oracle's numpy
restatement of the same specification: bit-identical CSR and weights."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import gen

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("scale,ef,seed,wt", [(6, 4, 1, "u32"), (10, 16, 1, "u32"), (12, 16, 7, "u32"),
                                              (11, 8, 5, "f32"), (14, 16, 1, "u32")])
def test_rmat_matches_oracle(scale, ef, seed, wt, gb):
    a = gb.gen_rmat(scale, ef, seed, wt)
    r, c, w = gen.rmat(scale, ef, seed, wt)
    assert np.array_equal(a.row, r) and np.array_equal(a.col, c) and np.array_equal(a.w, w)


@pytest.mark.parametrize("rows,cols,wt", [(1, 1, "f32"), (1, 7, "u32"), (9, 1, "f32"), (33, 65, "f32"), (20, 30, "u32")])
def test_grid_matches_oracle(rows, cols, wt, gb):
    a = gb.gen_grid(rows, cols, 3, wt)
    r, c, w = gen.grid(rows, cols, 3, wt)
    assert np.array_equal(a.row, r) and np.array_equal(a.col, c) and np.array_equal(a.w, w)
    assert a.m == 2 * (rows * (cols - 1) + (rows - 1) * cols)


def test_weight_ranges(gb):
    a = gb.gen_rmat(12, 16, 2, "u32")
    assert a.w.min() >= 1 and a.w.max() <= 255
    g = gb.gen_grid(64, 64, 3, "f32")
    assert g.w.min() >= 1.0 and g.w.max() < 1000.0
    assert np.all((g.w.astype(np.float64) * 16384) == np.floor(g.w.astype(np.float64) * 16384))


def test_symmetric_no_selfloops_no_dups(gb):
    a = gb.gen_rmat(10, 16, 3)
    u = np.repeat(np.arange(a.n), np.diff(a.row.astype(np.int64)))
    assert not np.any(u == a.col)
    keys = u.astype(np.uint64) << np.uint64(32) | a.col.astype(np.uint64)
    assert len(np.unique(keys)) == len(keys)
    rkeys = a.col.astype(np.uint64) << np.uint64(32) | u.astype(np.uint64)
    assert np.array_equal(np.sort(keys), np.sort(rkeys))


def test_sources_match_oracle(gb):
    a = gb.gen_rmat(12, 16, 1)
    assert np.array_equal(gb.sample_sources(a, 64, 7), gen.sample_sources(a.row, 64, 7))


def test_seeded_fixture_graphs(gb):
    import hashlib
    sha = lambda x: hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()
    for case in json.loads((GOLD / "seeded.json").read_text()):
        if case["kind"] == "rmat":
            a = gb.gen_rmat(case["scale"], case["edgefactor"], case["seed"], case["wtype"])
        else:
            a = gb.gen_grid(case["rows"], case["cols"], case["seed"], case["wtype"])
        assert (sha(a.row), sha(a.col), sha(a.w)) == (case["row_sha"], case["col_sha"], case["w_sha"]), case["name"]
