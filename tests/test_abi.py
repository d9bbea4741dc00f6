"""C-ABI checks that need no GPU: the library loads, exports every symbol the
headers in include/ declare, and rejects malformed input with a status code
before touching the device."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

INCLUDE = Path(__file__).resolve().parent.parent / "include"


def declared_functions(header: Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M)
    return sorted({n for n in names if n not in ("if", "for", "while", "sizeof", "defined")})


@pytest.mark.parametrize("header", sorted(p.name for p in INCLUDE.glob("*.h")))
def test_library_exports_header_symbols(header, gb):
    names = declared_functions(INCLUDE / header)
    assert names, header
    # the reference-named entry points live in their own library
    path = gb.COMPAT_LIB_PATH if header == "gbsssp_compat.h" else gb.LIB_PATH
    lib = ctypes.CDLL(str(path))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_export_list_matches_header(gb):
    assert sorted(gb.EXPORTS) == declared_functions(INCLUDE / "gbsssp.h")


def test_status_strings(gb):
    gb.lib.gbs_status_string.restype = ctypes.c_char_p
    assert gb.lib.gbs_status_string(0) == b"ok"
    assert gb.lib.gbs_status_string(5) == b"device wait limit exceeded"
    assert gb.lib.gbs_abi_version() == 1


def _create(gb, row, col, w, wtype):
    h = ctypes.c_void_p()
    st = gb.lib.gbs_graph_create(len(row) - 1, len(col), gb._ptr(row), gb._ptr(col) if len(col) else None,
                                 gb._ptr(w) if len(w) else None, wtype, ctypes.byref(h))
    return st, h


@pytest.mark.parametrize("bad", ["row0", "rowend", "decreasing", "col", "negw", "nanw", "n0"])
def test_graph_create_rejects_malformed(bad, gb):
    row = np.array([0, 2, 3, 3], dtype=np.uint64)
    col = np.array([1, 2, 0], dtype=np.uint32)
    w = np.array([1.0, 2.0, 3.0], dtype=np.float32)
    if bad == "row0":
        row[0] = 1
    elif bad == "rowend":
        row[-1] = 2
    elif bad == "decreasing":
        row[1], row[2] = 3, 2
    elif bad == "col":
        col[1] = 3
    elif bad == "negw":
        w[0] = -1.0
    elif bad == "nanw":
        w[2] = np.nan
    elif bad == "n0":
        row = np.array([0], dtype=np.uint64)
        col = np.array([], dtype=np.uint32)
        w = np.array([], dtype=np.float32)
    st, h = _create(gb, row, col, w, gb.W_F32)
    assert st == 1 and not h.value
    assert gb.lib.gbs_last_error()


def test_null_arguments(gb):
    assert gb.lib.gbs_graph_create(3, 0, None, None, None, 0, None) == 1
    assert gb.lib.gbs_sssp(None, 0, None, None, None, None) == 1
    assert gb.lib.gbs_graph_destroy(None) == 1


def test_host_mirror_weight_rules(gb):
    """Negative or non-finite double weights are refused before any device
    work (fractional ones run in float64, the reference's arithmetic)."""
    for bad in (-0.5, np.nan, np.inf):
        gs = gb.TCsr(np.array([1, 1], dtype=np.int64), np.array([1], dtype=np.int64), np.array([bad]))
        with pytest.raises(gb.GbsError) as e:
            gb.run_sspath_arr(gs, 0, 0.4)
        assert e.value.name == "INVALID_ARG"
