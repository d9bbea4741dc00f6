"""The ctypes mirrors of graphbench_gb300 match the C structs of
include/gbsssp.h: size and the offset of every field, from a small C program
compiled here with gcc against the header.  A field added on one side only
(the way gbs_params.fuse_rounds was added to both) would shift every later
field the library reads."""
import ctypes
import shutil
import subprocess
from pathlib import Path

import pytest

import graphbench_gb300 as gb

ROOT = Path(__file__).resolve().parents[1]

MIRRORS = {
    "gbs_params": gb.Params,
    "gbs_phase_rec": gb.PhaseRec,
    "gbs_stats": gb.Stats,
    "gbs_bc_stats": gb.BcStats,
    "gbs_ingest_info": gb.IngestInfo,
    "gbs_pagerank_params": gb.PagerankParams,
    "gbs_pagerank_stats": gb.PagerankStats,
    "gbs_csr_view": gb.CsrView,
    "gbs_batch_params": gb.BatchParams,
    "gbs_inst_stats": gb.InstStats,
    "gbs_batch_stats": gb.BatchStats,
    "gbs_tune_report": gb.TuneReport,
    "gbs_batch_tune_report": gb.BatchTuneReport,
    "gbs_host_csr": gb.HostCsr,
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gbsssp.h"', "int main(void) {"]
    for cname, py in MIRRORS.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    d = tmp_path_factory.mktemp("layout")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        cname, key, val = line.split()
        got[(cname, key)] = int(val)
    return got


@pytest.mark.parametrize("cname", sorted(MIRRORS))
def test_mirror_matches_header(cname, c_layout):
    py = MIRRORS[cname]
    assert ctypes.sizeof(py) == c_layout[(cname, "size")], cname
    for fname, _ in py._fields_:
        assert getattr(py, fname).offset == c_layout[(cname, fname)], (cname, fname)
