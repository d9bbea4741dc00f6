"""graphbench_gb300 -- GB300-native delta-stepping SSSP (Python host side).

Thin ctypes layer over ``libgbsssp.so`` (the C ABI declared in
``include/gbsssp.h``), mirroring the reference's SSSP entry points
(``run_sspath_arr`` sssp/csr_sspath_array.c:149, ``run_sspath``
sssp/csr_sspath.c:38) and its CSR (``t_csr`` include/graph.h:113-127).

The compute path is the CUDA library; there is no CPU fallback.  Loading the
package does not need a GPU, but any SSSP call raises ``GbsError`` with
status ``UNSUPPORTED`` (or a CUDA error) when no usable GPU is present, and
``ImportError`` is raised if the shared library has not been built
(``python -m graphbench_gb300.build``).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libgbsssp.so"
COMPAT_LIB_PATH = _PKG / "libgbsssp_compat.so"   # run_sspath_arr / run_sspath over t_csr

STATUS = {
    0: "OK", 1: "INVALID_ARG", 2: "CUDA", 3: "NO_MEMORY", 4: "CAPACITY",
    5: "TIMEOUT", 6: "OVERFLOW", 7: "UNSUPPORTED", 8: "INTERNAL",
}
W_U32, W_F32, W_F64 = 0, 1, 2
F_NO_STATS = 0x1

# Every symbol include/gbsssp.h declares (tests check the library exports them).
EXPORTS = [
    "gbs_status_string", "gbs_last_error", "gbs_abi_version", "gbs_device_available",
    "gbs_graph_create", "gbs_graph_destroy", "gbs_graph_info", "gbs_sssp", "gbs_sssp_device",
    "gbs_sssp_multi", "gbs_bc", "gbs_bc_device", "gbs_trace",
    "gbs_read_text", "gbs_parse_text", "gbs_read_bin", "gbs_parse_bin", "gbs_device_csr_info",
    "gbs_device_csr_export", "gbs_graph_from_device_csr", "gbs_device_csr_destroy",
    "gbs_pagerank", "gbs_device_csr_transpose", "gbs_sssp_noalloc", "gbs_host_alloc", "gbs_host_free",
    "gbs_pack_create", "gbs_pack_destroy", "gbs_pack_info", "gbs_plan_sources", "gbs_plan_pack",
    "gbs_plan_launch", "gbs_plan_wait", "gbs_plan_destroy",
    "gbs_autotune", "gbs_autotune_plan_sources", "gbs_autotune_plan_pack",
    "gbs_graph_set_controller", "gbs_features", "gbs_mlp_create", "gbs_mlp_destroy", "gbs_mlp_set_params",
    "gbs_mlp_get_params", "gbs_mlp_set_data", "gbs_mlp_loss_grad", "gbs_mlp_adam", "gbs_mlp_train",
    "gbs_mlp_predict",
    "gbs_device_alloc", "gbs_device_free",
    "gbs_device_synchronize", "gbs_memcpy",
    "gbs_gen_rmat", "gbs_gen_grid", "gbs_sample_sources", "gbs_host_csr_free",
]


class GbsError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str = ""):
        self.status = status
        self.name = STATUS.get(status, str(status))
        super().__init__(f"{where}: {self.name}" + (f" ({msg})" if msg else ""))


class Params(ctypes.Structure):
    _fields_ = [("delta", ctypes.c_double), ("light", ctypes.c_double),
                ("flags", ctypes.c_uint32), ("wait_limit_ms", ctypes.c_uint32),
                ("solo_entries", ctypes.c_uint32), ("solo_descs", ctypes.c_uint32),
                ("inline_edges", ctypes.c_uint32), ("full_items", ctypes.c_uint32),
                ("fuse_rounds", ctypes.c_uint32)]


class PhaseRec(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("bucket", ctypes.c_uint32), ("items", ctypes.c_uint32),
                ("edges", ctypes.c_uint32), ("pending", ctypes.c_uint32), ("window", ctypes.c_uint32),
                ("end_ns", ctypes.c_uint64)]


PHASE_KINDS = {0: "scan_bucket", 1: "scan_light", 2: "heavy", 3: "relax", 4: "pending",
               8: "bc_count", 9: "bc_forward", 10: "bc_backward", 11: "bc_backward_words"}
F_TRACE = 0x2
F_NO_SOLO = 0x4
F_BC_SINGLE = 0x20
F_NO_FUSE = 0x40
F_FEATURES = 0x8
F_LEARNED = 0x10
N_FEAT = 16
MLP_FLOATS = 5410      # controller block: means, scales, W1, b1, W2, b2, W3, b3
MLP_PARAMS = 5378      # the trained part
F_TEST_STALL = 0x80000000


class Stats(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("kernel_ms", ctypes.c_double),
                ("reached", ctypes.c_uint64), ("edges_reached", ctypes.c_uint64),
                ("improvements", ctypes.c_uint64), ("buckets", ctypes.c_uint32),
                ("phases", ctypes.c_uint32), ("pending_scans", ctypes.c_uint32),
                ("blocks", ctypes.c_uint32), ("delta_used", ctypes.c_double),
                ("light_used", ctypes.c_double), ("solo_phases", ctypes.c_uint32),
                ("learned", ctypes.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class BcStats(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("sssp_ms", ctypes.c_double), ("dag_ms", ctypes.c_double),
                ("edges_reached", ctypes.c_uint64), ("tight_edges", ctypes.c_uint64),
                ("dag_vertices", ctypes.c_uint64), ("max_levels", ctypes.c_uint32),
                ("sources", ctypes.c_uint32), ("blocks", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class IngestInfo(ctypes.Structure):
    _fields_ = [("v_num", ctypes.c_int64), ("e_num", ctypes.c_int64), ("offset", ctypes.c_int64),
                ("g_v_size", ctypes.c_int64), ("records", ctypes.c_uint64), ("edges", ctypes.c_uint64),
                ("duplicates", ctypes.c_uint64), ("read_ms", ctypes.c_double), ("parse_ms", ctypes.c_double),
                ("build_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class PagerankParams(ctypes.Structure):
    _fields_ = [("random_jump", ctypes.c_double), ("threshold", ctypes.c_double),
                ("max_iters", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class PagerankStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_uint32), ("converged", ctypes.c_uint32),
                ("device_ms", ctypes.c_double), ("edges", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class CsrView(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("m", ctypes.c_uint64), ("row_offsets", ctypes.c_void_p),
                ("cols", ctypes.c_void_p), ("weights", ctypes.c_void_p)]


class BatchParams(ctypes.Structure):
    _fields_ = [("delta", ctypes.c_double), ("delta_scale", ctypes.c_double), ("light", ctypes.c_double),
                ("group_ctas", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("wait_limit_ms", ctypes.c_uint32), ("solo_entries", ctypes.c_uint32),
                ("solo_descs", ctypes.c_uint32), ("inline_edges", ctypes.c_uint32),
                ("fuse_rounds", ctypes.c_uint32)]


class InstStats(ctypes.Structure):
    _fields_ = [("done", ctypes.c_uint32), ("error", ctypes.c_uint32), ("group", ctypes.c_uint32),
                ("phases", ctypes.c_uint32), ("buckets", ctypes.c_uint32), ("pending_scans", ctypes.c_uint32),
                ("solo_phases", ctypes.c_uint32), ("pad", ctypes.c_uint32), ("reached", ctypes.c_uint64),
                ("edges_reached", ctypes.c_uint64), ("improvements", ctypes.c_uint64),
                ("start_ns", ctypes.c_uint64), ("end_ns", ctypes.c_uint64)]


class BatchStats(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("instances", ctypes.c_uint32), ("completed", ctypes.c_uint32),
                ("groups", ctypes.c_uint32), ("group_ctas", ctypes.c_uint32), ("blocks", ctypes.c_uint32),
                ("max_phases", ctypes.c_uint32), ("phases", ctypes.c_uint64), ("reached", ctypes.c_uint64),
                ("edges_reached", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class TuneReport(ctypes.Structure):
    _fields_ = [("best", Params), ("best_ms", ctypes.c_double), ("default_ms", ctypes.c_double),
                ("delta_scale", ctypes.c_double), ("candidates", ctypes.c_uint32), ("runs", ctypes.c_uint32),
                ("no_split", ctypes.c_int32), ("reserved", ctypes.c_uint32)]


class BatchTuneReport(ctypes.Structure):
    _fields_ = [("best", BatchParams), ("best_ms", ctypes.c_double), ("default_ms", ctypes.c_double),
                ("candidates", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


def _struct_dict(s) -> dict:
    return {k: getattr(s, k) for k, _ in s._fields_}


class HostCsr(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("m", ctypes.c_uint64),
                ("row_offsets", ctypes.POINTER(ctypes.c_uint64)),
                ("cols", ctypes.POINTER(ctypes.c_uint32)),
                ("weights", ctypes.c_void_p), ("wtype", ctypes.c_int)]


def _load() -> ctypes.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m graphbench_gb300.build`")
    L = ctypes.CDLL(str(LIB_PATH))
    P = ctypes.c_void_p
    L.gbs_status_string.restype = ctypes.c_char_p
    L.gbs_last_error.restype = ctypes.c_char_p
    L.gbs_graph_create.argtypes = [ctypes.c_uint32, ctypes.c_uint64, P, P, P, ctypes.c_int,
                                   ctypes.POINTER(P)]
    L.gbs_graph_destroy.argtypes = [P]
    L.gbs_graph_info.argtypes = [P, P, P, P, P, P]
    L.gbs_sssp.argtypes = [P, ctypes.c_uint32, ctypes.POINTER(Params), P, P, ctypes.POINTER(Stats)]
    L.gbs_sssp_device.argtypes = [P, ctypes.c_uint32, ctypes.POINTER(Params), P, P,
                                  ctypes.POINTER(Stats)]
    L.gbs_sssp_multi.argtypes = [P, P, ctypes.c_uint32, ctypes.POINTER(Params), P, P,
                                 ctypes.POINTER(Stats)]
    L.gbs_bc.argtypes = [P, P, ctypes.c_uint32, ctypes.POINTER(Params), P, ctypes.POINTER(BcStats)]
    L.gbs_bc_device.argtypes = [P, P, ctypes.c_uint32, ctypes.POINTER(Params), P, ctypes.POINTER(BcStats)]
    L.gbs_read_text.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(P), ctypes.POINTER(IngestInfo)]
    L.gbs_parse_text.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(P),
                                 ctypes.POINTER(IngestInfo)]
    L.gbs_read_bin.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(P),
                               ctypes.POINTER(IngestInfo)]
    L.gbs_parse_bin.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int64, ctypes.c_int,
                                ctypes.POINTER(P), ctypes.POINTER(IngestInfo)]
    L.gbs_device_csr_info.argtypes = [P, P, P]
    L.gbs_device_csr_export.argtypes = [P, P, P, P]
    L.gbs_graph_from_device_csr.argtypes = [P, ctypes.c_int, ctypes.POINTER(P)]
    L.gbs_device_csr_destroy.argtypes = [P]
    L.gbs_pagerank.argtypes = [P, ctypes.POINTER(PagerankParams), P, ctypes.POINTER(PagerankStats)]
    L.gbs_device_csr_transpose.argtypes = [P, ctypes.POINTER(P)]
    L.gbs_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(P)]
    L.gbs_host_free.argtypes = [P]
    L.gbs_device_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(P)]
    L.gbs_device_free.argtypes = [P]
    L.gbs_memcpy.argtypes = [P, P, ctypes.c_size_t]
    L.gbs_gen_rmat.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int,
                               ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.POINTER(HostCsr))]
    L.gbs_gen_grid.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int,
                               ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.POINTER(HostCsr))]
    L.gbs_sample_sources.argtypes = [ctypes.POINTER(HostCsr), ctypes.c_uint32, ctypes.c_uint64, P, P]
    L.gbs_host_csr_free.argtypes = [ctypes.POINTER(HostCsr)]
    L.gbs_trace.argtypes = [P, P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
    # no-allocation variant: device pointers in, device pointers out
    L.gbs_sssp_noalloc.argtypes = [ctypes.c_uint32, ctypes.c_uint64, P, P, ctypes.c_int, ctypes.c_uint32,
                                   ctypes.c_double, P, P, P]
    # batched launches
    L.gbs_pack_create.argtypes = [ctypes.c_uint32, P, ctypes.c_int, ctypes.POINTER(P)]
    L.gbs_pack_destroy.argtypes = [P]
    L.gbs_pack_info.argtypes = [P, P, P, P, P]
    L.gbs_plan_sources.argtypes = [P, P, ctypes.c_uint32, ctypes.POINTER(BatchParams), P, P, ctypes.POINTER(P)]
    L.gbs_plan_pack.argtypes = [P, P, ctypes.POINTER(BatchParams), P, P, ctypes.POINTER(P)]
    L.gbs_plan_launch.argtypes = [P]
    L.gbs_plan_wait.argtypes = [P, ctypes.POINTER(BatchStats), P]
    L.gbs_plan_destroy.argtypes = [P]
    L.gbs_autotune.argtypes = [P, P, ctypes.c_uint32, ctypes.c_double, ctypes.POINTER(TuneReport)]
    L.gbs_graph_set_controller.argtypes = [P, P, ctypes.c_uint32, ctypes.c_double]
    L.gbs_features.argtypes = [P, P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
    L.gbs_mlp_create.argtypes = [ctypes.POINTER(P)]
    L.gbs_mlp_destroy.argtypes = [P]
    L.gbs_mlp_set_params.argtypes = [P, P]
    L.gbs_mlp_get_params.argtypes = [P, P]
    L.gbs_mlp_set_data.argtypes = [P, P, P, P, ctypes.c_uint32]
    L.gbs_mlp_loss_grad.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_double), P]
    L.gbs_mlp_adam.argtypes = [P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float]
    L.gbs_mlp_train.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_uint64, P]
    L.gbs_mlp_predict.argtypes = [P, P, ctypes.c_uint32, P]
    L.gbs_autotune_plan_sources.argtypes = [P, P, ctypes.c_uint32, ctypes.c_double,
                                            ctypes.POINTER(BatchTuneReport)]
    L.gbs_autotune_plan_pack.argtypes = [P, P, ctypes.c_double, ctypes.POINTER(BatchTuneReport)]
    return L


lib = _load()


def _check(status: int, where: str) -> None:
    if status != 0:
        raise GbsError(status, where, lib.gbs_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def device_available() -> bool:
    return bool(lib.gbs_device_available())


class DeviceBuffer:
    """cudaMalloc'd bytes owned by Python (outputs of Graph.sssp_device)."""

    def __init__(self, nbytes: int):
        p = ctypes.c_void_p()
        _check(lib.gbs_device_alloc(nbytes, ctypes.byref(p)), "gbs_device_alloc")
        self.ptr, self.nbytes = p, nbytes

    def free(self) -> None:
        if self.ptr:
            lib.gbs_device_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PinnedBuffer:
    """Page-locked host array (fast device-to-host copies)."""

    def __init__(self, count: int, dtype):
        dtype = np.dtype(dtype)
        p = ctypes.c_void_p()
        _check(lib.gbs_host_alloc(max(1, count * dtype.itemsize), ctypes.byref(p)), "gbs_host_alloc")
        self.ptr = p
        buf = (ctypes.c_char * max(1, count * dtype.itemsize)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=count)

    def free(self) -> None:
        if self.ptr:
            self.array = None
            lib.gbs_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def synchronize() -> None:
    _check(lib.gbs_device_synchronize(), "gbs_device_synchronize")


# ------------------------------------------------------------ generators
@dataclass
class HostGraph:
    """A CSR in host memory: exclusive uint64 offsets, uint32 columns,
    uint32 or float32 weights."""
    row: np.ndarray
    col: np.ndarray
    w: np.ndarray

    @property
    def n(self) -> int:
        return len(self.row) - 1

    @property
    def m(self) -> int:
        return int(self.row[-1])


def _take_host_csr(p) -> HostGraph:
    c = p.contents
    n, m = int(c.n), int(c.m)
    row = np.ctypeslib.as_array(c.row_offsets, shape=(n + 1,)).copy()
    col = np.ctypeslib.as_array(c.cols, shape=(max(m, 1),))[:m].copy()
    wt = np.float32 if c.wtype == W_F32 else np.uint32
    wp = ctypes.cast(c.weights, ctypes.POINTER(ctypes.c_float if wt is np.float32 else ctypes.c_uint32))
    w = np.ctypeslib.as_array(wp, shape=(max(m, 1),))[:m].copy()
    lib.gbs_host_csr_free(p)
    return HostGraph(row, col, w)


def gen_rmat(scale: int, edgefactor: int = 16, seed: int = 1, wtype: str = "u32",
             wmin: int = 1, wmax: int = 255) -> HostGraph:
    p = ctypes.POINTER(HostCsr)()
    _check(lib.gbs_gen_rmat(scale, edgefactor, seed, W_F32 if wtype == "f32" else W_U32,
                            wmin, wmax, ctypes.byref(p)), "gbs_gen_rmat")
    return _take_host_csr(p)


def gen_grid(rows: int, cols: int, seed: int = 3, wtype: str = "f32",
             wmin: int = 1, wmax: int = 255) -> HostGraph:
    p = ctypes.POINTER(HostCsr)()
    _check(lib.gbs_gen_grid(rows, cols, seed, W_F32 if wtype == "f32" else W_U32,
                            wmin, wmax, ctypes.byref(p)), "gbs_gen_grid")
    return _take_host_csr(p)


def sample_sources(g: HostGraph, count: int, seed: int) -> np.ndarray:
    hc = HostCsr(g.n, g.m, g.row.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                 g.col.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                 g.w.ctypes.data, W_F32 if g.w.dtype == np.float32 else W_U32)
    out = np.zeros(count, dtype=np.uint32)
    got = np.zeros(1, dtype=np.uint32)
    _check(lib.gbs_sample_sources(ctypes.byref(hc), count, seed, _ptr(out), _ptr(got)),
           "gbs_sample_sources")
    return out[: int(got[0])]


def heuristic_delta(g: HostGraph) -> float:
    """max_w / average out-degree."""
    if g.m == 0:
        return 1.0
    return float(np.max(g.w)) / (g.m / g.n)


# ----------------------------------------------------------------- graph
class Graph:
    """A device-resident CSR (gbs_graph).  Replaces the t_csr that
    scan_csr_idx/read_graph_csr or read_csr_bin build (graph/csr.c)."""

    def __init__(self, row, col, w):
        row = np.ascontiguousarray(row, dtype=np.uint64)
        col = np.ascontiguousarray(col, dtype=np.uint32)
        w = np.ascontiguousarray(w)
        if w.dtype == np.float32:
            self.wtype = W_F32
        elif w.dtype == np.uint32:
            self.wtype = W_U32
        elif w.dtype == np.float64:
            self.wtype = W_F64
        else:
            raise TypeError("weights must be uint32, float32 or float64")
        self.n = len(row) - 1
        self.m = int(row[-1]) if len(row) else 0
        self.dist_dtype = {W_F32: np.float32, W_U32: np.uint32, W_F64: np.float64}[self.wtype]
        h = ctypes.c_void_p()
        _check(lib.gbs_graph_create(self.n, len(col), _ptr(row), _ptr(col), _ptr(w), self.wtype,
                                    ctypes.byref(h)), "gbs_graph_create")
        self._h = h

    @classmethod
    def from_host(cls, g: HostGraph) -> "Graph":
        return cls(g.row, g.col, g.w)

    @classmethod
    def _adopt(cls, handle: ctypes.c_void_p, wtype: int) -> "Graph":
        g = cls.__new__(cls)
        n, m = ctypes.c_uint32(), ctypes.c_uint64()
        wt, mw = ctypes.c_int(), ctypes.c_double()
        _check(lib.gbs_graph_info(handle, ctypes.byref(n), ctypes.byref(m), ctypes.byref(wt), ctypes.byref(mw),
                                  None), "gbs_graph_info")
        g.n, g.m, g.wtype = n.value, m.value, wtype
        g.dist_dtype = {W_F32: np.float32, W_U32: np.uint32, W_F64: np.float64}[wtype]
        g._h = handle
        return g

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.gbs_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def info(self) -> dict:
        n, m, wt, mw, dd = (ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_int(), ctypes.c_double(),
                            ctypes.c_double())
        _check(lib.gbs_graph_info(self._h, ctypes.byref(n), ctypes.byref(m), ctypes.byref(wt),
                                  ctypes.byref(mw), ctypes.byref(dd)), "gbs_graph_info")
        return {"n": n.value, "m": m.value, "wtype": wt.value, "max_weight": mw.value,
                "default_delta": dd.value}

    @staticmethod
    def params(delta: float | None = None, light: float | None = None, flags: int = 0,
               wait_limit_ms: int = 0, solo_entries: int = 0, solo_descs: int = 0,
               inline_edges: int = 0, full_items: int = 0, fuse_rounds: int = 0) -> Params:
        p = Params()
        p.delta = float(delta) if delta else 0.0
        p.light = float(light) if light is not None else -1.0
        p.flags = flags
        p.wait_limit_ms = wait_limit_ms
        p.solo_entries = solo_entries
        p.solo_descs = solo_descs
        p.inline_edges = inline_edges
        p.full_items = full_items
        p.fuse_rounds = fuse_rounds
        return p

    def trace(self) -> list[dict]:
        """Per-phase records of the last run made with flags=F_TRACE."""
        cnt = ctypes.c_uint32()
        _check(lib.gbs_trace(self._h, None, 0, ctypes.byref(cnt)), "gbs_trace")
        recs = (PhaseRec * max(1, cnt.value))()
        _check(lib.gbs_trace(self._h, recs, cnt.value, ctypes.byref(cnt)), "gbs_trace")
        return [{"kind": PHASE_KINDS.get(r.kind & 15, r.kind), "solo": bool(r.kind & 16),
                 "span": (r.kind >> 8) & 0xFF, "full": bool((r.kind >> 16) & 1),
                 "bucket": r.bucket, "items": r.items, "edges": r.edges, "pending": r.pending,
                 "window": r.window, "end_ns": r.end_ns}
                for r in recs[: cnt.value]]

    def set_controller(self, params: np.ndarray | None, margin: float = 0.0) -> None:
        """Installs the learned bucket-width controller (MLP_FLOATS float32
        values) used by runs with flags=F_LEARNED; None removes it."""
        if params is None:
            _check(lib.gbs_graph_set_controller(self._h, None, 0, 0.0), "gbs_graph_set_controller")
            return
        p = np.ascontiguousarray(params, dtype=np.float32)
        _check(lib.gbs_graph_set_controller(self._h, _ptr(p), len(p), float(margin)), "gbs_graph_set_controller")

    def features(self) -> np.ndarray:
        """Controller inputs recorded by the last run made with F_FEATURES
        (one row of N_FEAT per bucket start)."""
        cnt = ctypes.c_uint32()
        _check(lib.gbs_features(self._h, None, 0, ctypes.byref(cnt)), "gbs_features")
        out = np.empty((cnt.value, N_FEAT), dtype=np.float32)
        if cnt.value:
            _check(lib.gbs_features(self._h, _ptr(out), cnt.value, ctypes.byref(cnt)), "gbs_features")
        return out

    def sssp(self, source: int, delta: float | None = None, light: float | None = None,
             out_dist: np.ndarray | None = None, out_pred: np.ndarray | None = None,
             want_dist: bool = True, want_pred: bool = True, **kw):
        """One SSSP; returns (dist, pred, stats dict).  dist is uint32
        (UINT32_MAX unreached) or float32 (+inf unreached); pred is int32
        (pred[source] = source, -1 unreached)."""
        p = self.params(delta, light, **kw)
        st = Stats()
        dist = out_dist if out_dist is not None else (np.empty(self.n, dtype=self.dist_dtype) if want_dist else None)
        pred = out_pred if out_pred is not None else (np.empty(self.n, dtype=np.int32) if want_pred else None)
        _check(lib.gbs_sssp(self._h, int(source), ctypes.byref(p),
                            _ptr(dist) if dist is not None else None,
                            _ptr(pred) if pred is not None else None, ctypes.byref(st)), "gbs_sssp")
        return dist, pred, st.as_dict()

    def sssp_device(self, source: int, dist_ptr: int | None = None, pred_ptr: int | None = None,
                    delta: float | None = None, light: float | None = None, **kw) -> dict:
        """Run with outputs left in caller-owned device memory (raw pointers)."""
        p = self.params(delta, light, **kw)
        st = Stats()
        _check(lib.gbs_sssp_device(self._h, int(source), ctypes.byref(p), dist_ptr, pred_ptr,
                                   ctypes.byref(st)), "gbs_sssp_device")
        return st.as_dict()

    def autotune(self, sources, budget_ms: float = 0.0):
        """Fastest schedule on these sources (gbs_autotune).  Returns (kwargs
        for sssp / sssp_device, report dict)."""
        src = np.ascontiguousarray(sources, dtype=np.uint32)
        rep = TuneReport()
        _check(lib.gbs_autotune(self._h, _ptr(src), len(src), float(budget_ms), ctypes.byref(rep)), "gbs_autotune")
        b = rep.best
        kw = {"delta": b.delta, "light": b.light, "solo_entries": b.solo_entries, "solo_descs": b.solo_descs,
              "inline_edges": b.inline_edges, "fuse_rounds": b.fuse_rounds, "full_items": b.full_items}
        r = {k: getattr(rep, k) for k, _ in TuneReport._fields_ if k != "best"}
        r["best"] = dict(kw)
        return kw, r

    def betweenness(self, sources=None, delta: float | None = None, light: float | None = None,
                    out: np.ndarray | None = None, **kw):
        """Betweenness centrality summed over `sources` (every vertex when
        None), as run_bc computes it (btwcentral/csr_bc.c:16-64).  Returns
        (bc float64[n], stats dict)."""
        p = self.params(delta, light, **kw)
        st = BcStats()
        bc = out if out is not None else np.empty(self.n, dtype=np.float64)
        src = None if sources is None else np.ascontiguousarray(sources, dtype=np.uint32)
        _check(lib.gbs_bc(self._h, _ptr(src) if src is not None else None,
                          len(src) if src is not None else 0, ctypes.byref(p), _ptr(bc),
                          ctypes.byref(st)), "gbs_bc")
        return bc, st.as_dict()

    def betweenness_device(self, bc_ptr: int, sources=None, delta: float | None = None,
                           light: float | None = None, **kw) -> dict:
        """Betweenness into caller-owned device memory (n doubles)."""
        p = self.params(delta, light, **kw)
        st = BcStats()
        src = None if sources is None else np.ascontiguousarray(sources, dtype=np.uint32)
        _check(lib.gbs_bc_device(self._h, _ptr(src) if src is not None else None,
                                 len(src) if src is not None else 0, ctypes.byref(p), bc_ptr,
                                 ctypes.byref(st)), "gbs_bc_device")
        return st.as_dict()

    def sssp_multi(self, sources, delta: float | None = None, light: float | None = None,
                   want_dist: bool = True, want_pred: bool = False, **kw):
        src = np.ascontiguousarray(sources, dtype=np.uint32)
        k = len(src)
        p = self.params(delta, light, **kw)
        st = Stats()
        dist = np.empty((k, self.n), dtype=self.dist_dtype) if want_dist else None
        pred = np.empty((k, self.n), dtype=np.int32) if want_pred else None
        _check(lib.gbs_sssp_multi(self._h, _ptr(src), k, ctypes.byref(p),
                                  _ptr(dist) if dist is not None else None,
                                  _ptr(pred) if pred is not None else None, ctypes.byref(st)),
               "gbs_sssp_multi")
        return dist, pred, st.as_dict()


# ------------------------------------------------------------ graph ingest
DIR_RECV, DIR_SEND = 0, 1


def _bytes_arg(data):
    """(pointer, length) of a bytes object or a contiguous uint8 array."""
    if isinstance(data, np.ndarray):
        if data.dtype != np.uint8 or not data.flags["C_CONTIGUOUS"]:
            raise TypeError("file image arrays must be contiguous uint8")
        return ctypes.c_void_p(data.ctypes.data), data.nbytes
    data = bytes(data) if not isinstance(data, bytes) else data
    return ctypes.cast(ctypes.c_char_p(data), ctypes.c_void_p), len(data)


class DeviceCsr:
    """A graph read on the GPU (gbs_read_text / gbs_read_bin and the parse_*
    variants over bytes), laid out as the reference's readers lay out their
    t_csr (graph/csr.c): rows in file order, weights where the reference
    stores them."""

    def __init__(self, handle: ctypes.c_void_p, info: IngestInfo):
        self._h = handle
        self.info = info.as_dict()
        n, m = ctypes.c_uint32(), ctypes.c_uint64()
        _check(lib.gbs_device_csr_info(handle, ctypes.byref(n), ctypes.byref(m)), "gbs_device_csr_info")
        self.n, self.m = n.value, m.value

    @classmethod
    def read_text(cls, path, direction: int = DIR_SEND) -> "DeviceCsr":
        h, info = ctypes.c_void_p(), IngestInfo()
        _check(lib.gbs_read_text(str(path).encode(), direction, ctypes.byref(h), ctypes.byref(info)), "gbs_read_text")
        return cls(h, info)

    @classmethod
    def parse_text(cls, data, direction: int = DIR_SEND) -> "DeviceCsr":
        """data: bytes, or a contiguous uint8 array (e.g. a PinnedBuffer's)."""
        h, info = ctypes.c_void_p(), IngestInfo()
        ptr, n = _bytes_arg(data)
        _check(lib.gbs_parse_text(ptr, n, direction, ctypes.byref(h), ctypes.byref(info)), "gbs_parse_text")
        return cls(h, info)

    @classmethod
    def read_bin(cls, path, direction: int = DIR_SEND, target_offset: int = 1, dedup: bool = False) -> "DeviceCsr":
        h, info = ctypes.c_void_p(), IngestInfo()
        _check(lib.gbs_read_bin(str(path).encode(), direction, target_offset, int(bool(dedup)), ctypes.byref(h),
                                ctypes.byref(info)), "gbs_read_bin")
        return cls(h, info)

    @classmethod
    def parse_bin(cls, data, direction: int = DIR_SEND, target_offset: int = 1,
                  dedup: bool = False) -> "DeviceCsr":
        """data: bytes, or a contiguous uint8 array (e.g. a PinnedBuffer's)."""
        h, info = ctypes.c_void_p(), IngestInfo()
        ptr, n = _bytes_arg(data)
        _check(lib.gbs_parse_bin(ptr, n, direction, target_offset, int(bool(dedup)), ctypes.byref(h),
                                 ctypes.byref(info)), "gbs_parse_bin")
        return cls(h, info)

    def export(self):
        """(row_offsets uint64[n+1] exclusive, cols uint32[m], weights float64[m])."""
        row = np.empty(self.n + 1, dtype=np.uint64)
        col = np.empty(self.m, dtype=np.uint32)
        w = np.empty(self.m, dtype=np.float64)
        _check(lib.gbs_device_csr_export(self._h, _ptr(row), _ptr(col), _ptr(w)), "gbs_device_csr_export")
        return row, col, w

    def transpose(self) -> "DeviceCsr":
        h = ctypes.c_void_p()
        _check(lib.gbs_device_csr_transpose(self._h, ctypes.byref(h)), "gbs_device_csr_transpose")
        return DeviceCsr(h, IngestInfo())

    def pagerank(self, random_jump: float = 0.0, threshold: float = 0.0, max_iters: int = 0):
        """PageRank with this CSR as the in-edge lists (gbs_pagerank).
        Returns (rank float64[n], stats dict)."""
        p = PagerankParams(random_jump, threshold, max_iters, 0)
        st = PagerankStats()
        out = np.empty(self.n, dtype=np.float64)
        _check(lib.gbs_pagerank(self._h, ctypes.byref(p), _ptr(out), ctypes.byref(st)), "gbs_pagerank")
        return out, st.as_dict()

    @classmethod
    def from_arrays(cls, row, col, w=None) -> "DeviceCsr":
        """A device CSR from host arrays (exclusive offsets, columns, weights),
        through the binary reader's in-memory form."""
        row = np.asarray(row, dtype=np.int64)
        col = np.asarray(col, dtype=np.int64)
        n = len(row) - 1
        src = np.repeat(np.arange(n, dtype=np.int64), np.diff(row))
        pairs = np.empty((len(col), 2), dtype="<i8")
        pairs[:, 0] = src + 1
        pairs[:, 1] = col + 1
        data = np.array([n, len(col), 1, n], dtype="<i8").tobytes() + pairs.tobytes()
        return cls.parse_bin(data, DIR_SEND, 1, False)

    def graph(self, wtype: int = W_F64) -> "Graph":
        """A resident graph built on the device (rows sorted by (weight, column))."""
        h = ctypes.c_void_p()
        _check(lib.gbs_graph_from_device_csr(self._h, wtype, ctypes.byref(h)), "gbs_graph_from_device_csr")
        return Graph._adopt(h, wtype)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.gbs_device_csr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# ------------------------------------------------ reference-shaped mirror
@dataclass
class TCsr:
    """Python mirror of the reference's t_csr (include/graph.h:113-127):
    vet_idx[v] is the INCLUSIVE end offset of row v (row v starts at
    vet_idx[v-1], 0 for v = 0), edge_idx the targets, edge_weight the doubles
    of edge_info[].edge_weight, and weight (vet_info[].weight) receives the
    distances."""
    vet_idx: np.ndarray
    edge_idx: np.ndarray
    edge_weight: np.ndarray
    weight: np.ndarray | None = None

    @property
    def v_size(self) -> int:
        return len(self.vet_idx)


def _tcsr_to_graph(gs: TCsr) -> Graph:
    ends = np.asarray(gs.vet_idx, dtype=np.int64)
    row = np.zeros(len(ends) + 1, dtype=np.uint64)
    row[1:] = ends
    w = np.asarray(gs.edge_weight, dtype=np.float64)
    if np.all(w == np.floor(w)) and (len(w) == 0 or (w.min() >= 0 and w.max() < 2**32 - 1)):
        return Graph(row, gs.edge_idx, w.astype(np.uint32))
    return Graph(row, gs.edge_idx, w)


def run_sspath_arr(gs: TCsr, source: int, delta: float) -> np.ndarray:
    """Mirror of run_sspath_arr(gs, predecesor, source, delta)
    (sssp/csr_sspath_array.c:149): fills gs.weight with float64 distances
    (inf for unreached) and returns them.  Integer weights run on the uint32
    path (exact in double); other weights on the float64 path, the
    reference's own arithmetic."""
    with _tcsr_to_graph(gs) as g:
        dist, _, _ = g.sssp(int(source), delta=float(delta), want_pred=False)
    out = dist.astype(np.float64)
    if g.wtype == W_U32:
        out[dist == np.uint32(0xFFFFFFFF)] = math.inf
    gs.weight = out
    return out


# --------------------------------------------------------------- batched
def batch_params(delta: float | None = None, delta_scale: float | None = None, light: float | None = None,
                 group_ctas: int = 0, flags: int = 0, wait_limit_ms: int = 0, solo_entries: int = 0,
                 solo_descs: int = 0, inline_edges: int = 0, fuse_rounds: int = 0) -> BatchParams:
    """light=None: light bound = delta; light=math.inf: no light/heavy split."""
    p = BatchParams()
    p.delta = float(delta) if delta else 0.0
    p.delta_scale = float(delta_scale) if delta_scale else 0.0
    p.light = float(light) if light is not None else -1.0
    p.group_ctas = group_ctas
    p.flags = flags
    p.wait_limit_ms = wait_limit_ms
    p.solo_entries = solo_entries
    p.solo_descs = solo_descs
    p.inline_edges = inline_edges
    p.fuse_rounds = fuse_rounds
    return p


class Pack:
    """Independent graphs uploaded together (gbs_pack) for batched SSSP."""

    def __init__(self, graphs: list[HostGraph]):
        if not graphs:
            raise ValueError("empty pack")
        dt = graphs[0].w.dtype
        if any(g.w.dtype != dt for g in graphs):
            raise TypeError("every graph of a pack has the same weight type")
        self.wtype = W_F32 if dt == np.float32 else W_U32
        self.dist_dtype = np.float32 if self.wtype == W_F32 else np.uint32
        self._keep = [(np.ascontiguousarray(g.row, dtype=np.uint64), np.ascontiguousarray(g.col, dtype=np.uint32),
                       np.ascontiguousarray(g.w)) for g in graphs]
        views = (CsrView * len(graphs))()
        for i, (r, c, w) in enumerate(self._keep):
            views[i] = CsrView(len(r) - 1, len(c), r.ctypes.data, c.ctypes.data, w.ctypes.data)
        h = ctypes.c_void_p()
        _check(lib.gbs_pack_create(len(graphs), views, self.wtype, ctypes.byref(h)), "gbs_pack_create")
        self._h = h
        self._keep = None
        cnt, tn, tm = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint64()
        offs = np.zeros(len(graphs) + 1, dtype=np.uint64)
        _check(lib.gbs_pack_info(h, ctypes.byref(cnt), ctypes.byref(tn), ctypes.byref(tm), _ptr(offs)),
               "gbs_pack_info")
        self.count, self.total_n, self.total_m = cnt.value, tn.value, tm.value
        self.vertex_offsets = offs

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.gbs_pack_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Plan:
    """A batched launch captured in a CUDA graph (gbs_plan).  Outputs stay in
    device memory owned by the plan object: dist (and pred) hold every
    instance's arrays back to back."""

    def __init__(self, target, sources, params: BatchParams | None = None, want_pred: bool = True, **kw):
        src = np.ascontiguousarray(sources, dtype=np.uint32)
        params = params if params is not None else batch_params(**kw)
        if isinstance(target, Graph):
            self.k, n = len(src), target.n
            self.offsets = np.arange(self.k + 1, dtype=np.uint64) * np.uint64(n)
            self.dist_dtype = target.dist_dtype
        elif isinstance(target, Pack):
            if len(src) != target.count:
                raise ValueError("one source per pack graph")
            self.k = target.count
            self.offsets = target.vertex_offsets.copy()
            self.dist_dtype = target.dist_dtype
        else:
            raise TypeError("target must be a Graph or a Pack")
        total = int(self.offsets[-1])
        self.dist = DeviceBuffer(max(4, 4 * total))
        self.pred = DeviceBuffer(max(4, 4 * total)) if want_pred else None
        h = ctypes.c_void_p()
        pp = self.pred.ptr if self.pred else None
        if isinstance(target, Graph):
            _check(lib.gbs_plan_sources(target.handle, _ptr(src), self.k, ctypes.byref(params), self.dist.ptr, pp,
                                        ctypes.byref(h)), "gbs_plan_sources")
        else:
            _check(lib.gbs_plan_pack(target._h, _ptr(src), ctypes.byref(params), self.dist.ptr, pp,
                                     ctypes.byref(h)), "gbs_plan_pack")
        self._h = h
        self.target = target

    def launch(self) -> None:
        _check(lib.gbs_plan_launch(self._h), "gbs_plan_launch")

    def wait(self, per_instance: bool = False):
        st = BatchStats()
        inst = (InstStats * self.k)() if per_instance else None
        _check(lib.gbs_plan_wait(self._h, ctypes.byref(st), inst), "gbs_plan_wait")
        d = st.as_dict()
        if per_instance:
            d["per_instance"] = [{k: getattr(r, k) for k, _ in InstStats._fields_} for r in inst]
        return d

    def run(self, per_instance: bool = False):
        self.launch()
        return self.wait(per_instance)

    def results(self, want_pred: bool = True):
        """Copies the outputs to the host: lists of per-instance arrays."""
        total = int(self.offsets[-1])
        dist = np.empty(total, dtype=self.dist_dtype)
        _check(lib.gbs_memcpy(_ptr(dist), self.dist.ptr, 4 * total), "gbs_memcpy")
        pred = None
        if want_pred and self.pred is not None:
            pred = np.empty(total, dtype=np.int32)
            _check(lib.gbs_memcpy(_ptr(pred), self.pred.ptr, 4 * total), "gbs_memcpy")
        o = [int(x) for x in self.offsets]
        ds = [dist[o[i]:o[i + 1]] for i in range(self.k)]
        ps = [pred[o[i]:o[i + 1]] for i in range(self.k)] if pred is not None else None
        return ds, ps

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.gbs_plan_destroy(self._h)
            self._h = None
        for b in (getattr(self, "dist", None), getattr(self, "pred", None)):
            if b is not None:
                b.free()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def autotune_plan(target, sources, budget_ms: float = 0.0):
    """Fastest batched parameters (CTAs per group, schedule) for a Plan over
    target (Graph or Pack) and sources.  Returns (BatchParams, report dict)."""
    src = np.ascontiguousarray(sources, dtype=np.uint32)
    rep = BatchTuneReport()
    if isinstance(target, Graph):
        _check(lib.gbs_autotune_plan_sources(target.handle, _ptr(src), len(src), float(budget_ms),
                                             ctypes.byref(rep)), "gbs_autotune_plan_sources")
    else:
        _check(lib.gbs_autotune_plan_pack(target._h, _ptr(src), float(budget_ms), ctypes.byref(rep)),
               "gbs_autotune_plan_pack")
    best = BatchParams()
    ctypes.memmove(ctypes.byref(best), ctypes.byref(rep.best), ctypes.sizeof(BatchParams))
    r = {"best_ms": rep.best_ms, "default_ms": rep.default_ms, "candidates": rep.candidates,
         "best": _struct_dict(best)}
    return best, r


# ---------------------------------------------------- controller training
class Mlp:
    """The controller network on the GPU (gbs_mlp): parameters, gradient,
    Adam state and a training set, with the library's CUDA kernels."""

    def __init__(self, params: np.ndarray | None = None):
        h = ctypes.c_void_p()
        _check(lib.gbs_mlp_create(ctypes.byref(h)), "gbs_mlp_create")
        self._h = h
        self.n = 0
        if params is not None:
            self.set_params(params)

    def set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.shape == (MLP_FLOATS,)
        _check(lib.gbs_mlp_set_params(self._h, _ptr(p)), "gbs_mlp_set_params")

    def params(self) -> np.ndarray:
        p = np.empty(MLP_FLOATS, dtype=np.float32)
        _check(lib.gbs_mlp_get_params(self._h, _ptr(p)), "gbs_mlp_get_params")
        return p

    def set_data(self, x: np.ndarray, t: np.ndarray, w: np.ndarray | None = None) -> None:
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        w = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
        assert x.ndim == 2 and x.shape[1] == N_FEAT and t.shape == (len(x), 2)
        self.n = len(x)
        _check(lib.gbs_mlp_set_data(self._h, _ptr(x), _ptr(t), _ptr(w) if w is not None else None, len(x)),
               "gbs_mlp_set_data")

    def loss_grad(self, first: int = 0, count: int | None = None):
        count = self.n - first if count is None else count
        loss = ctypes.c_double()
        g = np.empty(MLP_PARAMS, dtype=np.float32)
        _check(lib.gbs_mlp_loss_grad(self._h, first, count, ctypes.byref(loss), _ptr(g)), "gbs_mlp_loss_grad")
        return loss.value, g

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        _check(lib.gbs_mlp_adam(self._h, lr, beta1, beta2, eps), "gbs_mlp_adam")

    def train(self, epochs: int, batch: int, lr: float, seed: int = 0) -> np.ndarray:
        losses = np.zeros(epochs, dtype=np.float64)
        _check(lib.gbs_mlp_train(self._h, epochs, batch, lr, seed, _ptr(losses)), "gbs_mlp_train")
        return losses

    def predict(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((len(x), 2), dtype=np.float32)
        _check(lib.gbs_mlp_predict(self._h, _ptr(x), len(x), _ptr(y)), "gbs_mlp_predict")
        return y

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.gbs_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
