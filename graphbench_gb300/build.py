"""Builds libgbsssp.so in-tree (graphbench_gb300/libgbsssp.so).

CUDA sources are compiled for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``); host C sources with gcc.  Object files go
to ``graphbench_gb300/_build``.  Translation units compile in parallel and are
rebuilt only when a source or header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libgbsssp.so"
# run_sspath_arr / run_sspath over the reference's t_csr (include/gbsssp_compat.h)
COMPAT_LIB = PKG / "libgbsssp_compat.so"
COMPAT_SOURCES = ["host/compat.c"]

CUDA_SOURCES = ["csrc/gbs_api.cu", "csrc/gbs_batch.cu", "csrc/gbs_tune.cu", "csrc/gbs_mlp.cu", "csrc/gbs_noalloc.cu",
                "csrc/gbs_bc.cu", "csrc/gbs_ingest.cu", "csrc/gbs_pagerank.cu"]
C_SOURCES = ["host/gen.c"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise FileNotFoundError("nvcc not found")


def _deps() -> list[Path]:
    out = [INCLUDE / h for h in os.listdir(INCLUDE)]
    for sub in ("csrc", "host"):
        out += list((PKG / sub).glob("*"))
    return out


def _stale() -> bool:
    if not LIB.exists() or not COMPAT_LIB.exists():
        return True
    t = min(LIB.stat().st_mtime, COMPAT_LIB.stat().st_mtime)
    return any(p.stat().st_mtime > t for p in _deps() if p.is_file())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout[-3000:] + r.stderr[-6000:])


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cmds, objs = [], []
    for src in CUDA_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
               "-I", str(INCLUDE), "-c", str(PKG / src), "-o", str(obj)]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
        cmds.append(cmd)
        objs.append(obj)
    for src in C_SOURCES:
        obj = BUILD / (Path(src).stem + "_c.o")
        cmds.append(["gcc", "-O2", "-fPIC", "-std=c11", "-D_GNU_SOURCE", "-pthread",
                     "-I", str(INCLUDE), "-c", str(PKG / src), "-o", str(obj)])
        objs.append(obj)
    with ThreadPoolExecutor(max(1, min(len(cmds), os.cpu_count() or 1))) as ex:
        list(ex.map(_run, cmds))
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-pthread"])
    os.replace(tmp, LIB)
    ctmp = COMPAT_LIB.with_suffix(".so.tmp")
    _run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-D_GNU_SOURCE", "-pthread", "-I", str(INCLUDE),
          *[str(PKG / c) for c in COMPAT_SOURCES], "-o", str(ctmp), "-L", str(PKG), "-lgbsssp",
          "-Wl,-rpath,$ORIGIN", "-lm"])
    os.replace(ctmp, COMPAT_LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
