"""Build recipe for the reference's own SSSP code (the oracle's second leg).

TEST INFRASTRUCTURE ONLY.  Two stages:

1. ``stage(tree)`` (needs the read-only GRAPHBENCH tree: the argument, or
   the ``GBREF_TREE`` environment variable): copies the few source files the
   SSSP path needs into
   ``oracle/_ref/src/`` and applies the minimal patches listed in ``PATCHES``
   there.  Nothing is written outside ``oracle/_ref/``; the tree itself is
   never modified.
2. ``compile_ref()`` (anywhere gcc is, including a machine without the
   reference tree): compiles ``oracle/_ref/src`` plus ``oracle/ref_driver.c``
   into ``oracle/_ref/libref_serial.so`` and ``oracle/_ref/libref_omp.so``
   (the latter with ``-DUSE_OMP``, the reference's OpenMP build).

Patches (each anchor must match exactly once):

* D1  sssp/csr_sspath_array.c:444-446 -- relax_arr_single rewrote the
  vertex's bucket index even when it did not move; now only on insertion.
* D2  sssp/csr_sspath_array.c:427-430 -- re-inserting a vertex that
  remember_arr_single had already moved to S did not count it in b_total.
* D4  sssp/csr_sspath_array.c:194,202-204 -- request/S arrays were sized by
  the edge count although S can hold a vertex more than once; they are sized
  by ``GBREF_REQ_CAP`` (prelude) instead.
* P0  sssp/csr_sspath_array.c:352, sssp/csr_sspath.c:74 -- the per-phase
  dump of every bucket to ./data/log is skipped unless ``gbref_log_buckets``
  is set (it is debug output, and it would dominate a timed run).
* D3 (separate_csr increments uninitialised degree counters,
  graph/csr.c:76-94) needs no source change: the ``_mm_malloc`` stand-in in
  ``oracle/stubs/immintrin.h`` returns zeroed memory.

D5 (the OpenMP relax keeps only the first request per target, ordered by edge
weight) is structural and deliberately left alone: the OpenMP build is timed
as the reference's parallel CPU path and its mismatches are counted.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SRC_OUT = OUT / "src"
STUBS = HERE / "stubs"
def _default_tree() -> Path | None:
    """The reference tree named by GBREF_TREE, if any."""
    t = os.environ.get("GBREF_TREE")
    return Path(t) if t else None

SOURCES = [
    "graph/csr.c",
    "sssp/csr_sspath_array.c",
    "sssp/csr_sspath.c",
    "structs/array.c",
    "structs/list.c",
    "utils/timer.c",
    "utils/utils.c",
    "btwcentral/csr_bc.c",
]
HEADERS = ["array.h", "barrier.h", "csr.h", "csr_bc.h", "csr_sspath.h",
           "csr_sspath_array.h", "graph.h", "list.h", "timer.h", "utils.h"]

# (file, anchor lines (whitespace-stripped), replacement lines)
PATCHES = [
    ("sssp/csr_sspath_array.c",  # D1
     ["//change vidx",
      "vidx[target_idx].buck_id = new_buck;",
      "vidx[target_idx].buck_pos = B[new_buck]->idx-1;"],
     ["\t\t\t//change vidx (GBREF D1: only when the vertex was inserted)",
      "\t\t\tif(target_ori_val==INFINITY || vidx[target_idx].buck_id!=new_buck){",
      "\t\t\tvidx[target_idx].buck_id = new_buck;",
      "\t\t\tvidx[target_idx].buck_pos = B[new_buck]->idx-1;",
      "\t\t\t}"]),
    ("sssp/csr_sspath_array.c",  # D2
     ["remove_find_arr(B[old_buck], vidx[target_idx].buck_pos);",
      "B[old_buck]->num--;",
      "}"],
     ["\t\t\t\t\t\tremove_find_arr(B[old_buck], vidx[target_idx].buck_pos);",
      "\t\t\t\t\t\tB[old_buck]->num--;",
      "\t\t\t\t\t}",
      "\t\t\t\t\telse (*b_total)+=1; /* GBREF D2 */"]),
    ("sssp/csr_sspath_array.c",  # D4 (tmp)
     ["double *tmp = (double*)_mm_malloc(sizeof(double)*gs->e_size, 64);"],
     ["\tdouble *tmp = (double*)_mm_malloc(sizeof(double)*GBREF_REQ_CAP(gs), 64); /* GBREF D4 */"]),
    ("sssp/csr_sspath_array.c",  # D4 (R, tmp_R, S)
     ["create_arr(R, gs->e_size);",
      "create_arr(tmp_R, gs->e_size);",
      "create_arr(S, gs->e_size);"],
     ["\tcreate_arr(R, GBREF_REQ_CAP(gs)); /* GBREF D4 */",
      "\tcreate_arr(tmp_R, GBREF_REQ_CAP(gs));",
      "\tcreate_arr(S, GBREF_REQ_CAP(gs));"]),
    ("sssp/csr_sspath_array.c",  # P0
     ["print_B_map(log, B, iter);"],
     ["\t\tif(gbref_log_buckets) print_B_map(log, B, iter); /* GBREF P0 */"]),
    ("sssp/csr_sspath.c",  # P0
     ["print_B(B, log, iter);"],
     ["\t\tif(gbref_log_buckets) print_B(B, log, iter); /* GBREF P0 */"]),
]


def _apply(lines: list[str], anchor: list[str], repl: list[str], name: str) -> list[str]:
    stripped = [ln.strip() for ln in lines]
    hits = [i for i in range(len(lines) - len(anchor) + 1)
            if stripped[i:i + len(anchor)] == anchor]
    if len(hits) != 1:
        raise RuntimeError(f"patch anchor in {name} matched {len(hits)} times: {anchor[0]!r}")
    i = hits[0]
    return lines[:i] + repl + lines[i + len(anchor):]


def stage(ref_tree: Path | None = None) -> bool:
    """Copy + patch the reference sources into oracle/_ref/src.  Returns False
    when no reference tree is given (argument or GBREF_TREE) or it is absent
    (e.g. on a machine that only compiles the staged sources)."""
    ref_tree = Path(ref_tree) if ref_tree is not None else _default_tree()
    if ref_tree is None or not (ref_tree / "sssp" / "csr_sspath_array.c").exists():
        return False
    (SRC_OUT / "include").mkdir(parents=True, exist_ok=True)
    for h in HEADERS:
        shutil.copyfile(ref_tree / "include" / h, SRC_OUT / "include" / h)
    texts = {}
    for rel in SOURCES:
        raw = (ref_tree / rel).read_bytes().decode("latin-1")
        texts[rel] = raw.replace("\r\n", "\n").split("\n")
    for rel, anchor, repl in PATCHES:
        texts[rel] = _apply(texts[rel], anchor, repl, rel)
    for rel, lines in texts.items():
        dst = SRC_OUT / rel.replace("/", "__")
        dst.write_text("\n".join(lines), encoding="latin-1")
    return True


def _cc(args):
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + " ".join(args) + "\n" + r.stderr[-4000:])


def compile_ref(jobs: int = 8) -> list[Path]:
    """Compile the staged sources into the serial and OpenMP shared objects."""
    if not SRC_OUT.exists():
        raise FileNotFoundError("oracle/_ref/src is not staged; run stage() where the reference tree exists")
    srcs = sorted(SRC_OUT.glob("*.c"))
    common = ["gcc", "-O2", "-fPIC", "-fopenmp", "-w", "-std=gnu99", "-DREV_STATS",
              "-include", str(STUBS / "prelude.h"), "-I", str(STUBS),
              "-I", str(SRC_OUT / "include")]
    outs = []
    for variant, extra in (("serial", []), ("omp", ["-DUSE_OMP"])):
        objdir = OUT / f"obj_{variant}"
        objdir.mkdir(parents=True, exist_ok=True)
        cmds, objs = [], []
        for s in srcs + [HERE / "ref_driver.c"]:
            o = objdir / (s.stem + ".o")
            objs.append(o)
            cmds.append(common + extra + ["-c", str(s), "-o", str(o)])
        with ThreadPoolExecutor(jobs) as ex:
            list(ex.map(_cc, cmds))
        lib = OUT / f"libref_{variant}.so"
        _cc(["gcc", "-shared", "-fopenmp", "-o", str(lib)] + [str(o) for o in objs] + ["-lm"])
        outs.append(lib)
    return outs


def build(ref_tree: Path | None = None) -> list[Path]:
    stage(ref_tree)
    return compile_ref()


if __name__ == "__main__":
    print(build(Path(sys.argv[1]) if len(sys.argv) > 1 else None))
