#!/usr/bin/env python3
"""bench.py -- GTEPS of delta-stepping SSSP on GB300.

Default workload (the published GPU configuration): R-MAT scale 22, edge
factor 16, a/b/c/d = .57/.19/.19/.05, symmetrised and deduplicated, uint32
weights uniform in [1, 255], 64 sources drawn with seed 7, each timed
separately; delta = max weight / average out-degree.  One step = one SSSP
from the next source (plain fixed-delta delta-stepping, one cooperative
persistent launch).  Inputs are synthetic (seeded generator in the library).

  value  = sum(edges reached) / sum(device time of the steps)  [GTEPS]
           device time = CUDA events around reset + kernel + output unpack,
           graph resident in HBM
  e2e    = same metric through gbs_sssp with pinned HOST output buffers
           (device->host copy of dist + pred inside the timed call)

Beside the plain kernel, on the same resident graph and the same sources:
  learned    every step with the learned bucket-width controller (the
             committed block, flags=F_LEARNED; a run past its guard reruns
             plain and the step is charged both runs; after that the graph
             runs plain)
  autotuned  every step with the schedule gbs_autotune picked on 4 sources
  batched    all sources in one persistent launch replayed from a CUDA graph
             (gbs_plan_sources with the parameters gbs_autotune_plan_sources
             picked), dist/pred of every source kept on the device
Each reports GTEPS and its ratio to the plain value.
  betweenness  gbs_bc over 16 of the sources (batched shortest paths, then
             the path-count / dependency passes per source), with a bit-exact
             check of one more source against the oracle at full scale
  pagerank   gbs_pagerank on the same graph (in-edges), to convergence
  ingest     the same edges as a shuffled binary edge list parsed on the GPU
             with duplicate removal, CSR and resident graph built there

The other published configurations, each its own record with a parity field
(oracle Dijkstra and smallest-tight-predecessor rule, run in host threads
while the GPU works, compared bit for bit; learned / autotuned / batched
results compared with the plain ones):
  grid4096_f32   4096 x 4096 grid, float32 weights in [1, 1000), source 0:
                 plain, autotuned, learned, and 8 sources batched
  rmat24_u32     R-MAT scale 24, 8 sources: plain, learned, autotuned, batched
  rmat20_512src  R-MAT scale 20, 512 sources in one batched launch vs plain
  pack1024       1,024 R-MAT graphs of scales 10..16 (seed 11), one source
                 each, in one batched launch vs plain one graph at a time
The plain R-MAT 22 steps are also checked: two of their sources are re-run
after the timed loop and compared with the oracle.

Multi-GPU: one process per GPU (torchrun); every rank runs the whole workload
on its own GPU (replicas: a single SSSP does not shard); value = sum over
ranks / max time.  ``--impl reference`` times the reference's own CPU code.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "rmat22": dict(kind="rmat", scale=22, edgefactor=16, seed=1, wtype="u32", sources=64, source_seed=7),
    "rmat20": dict(kind="rmat", scale=20, edgefactor=16, seed=1, wtype="u32", sources=64, source_seed=7),
    "rmat16": dict(kind="rmat", scale=16, edgefactor=16, seed=1, wtype="u32", sources=64, source_seed=7),
    "rmat24": dict(kind="rmat", scale=24, edgefactor=16, seed=1, wtype="u32", sources=8, source_seed=7),
    "grid4096": dict(kind="grid", rows=4096, cols=4096, seed=3, wtype="f32", sources=1, source_seed=0),
    "grid1024": dict(kind="grid", rows=1024, cols=1024, seed=3, wtype="f32", sources=1, source_seed=0),
}
L2_BYTES = 129 * 1024 * 1024


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def make_workload(gb, wl):
    if wl["kind"] == "rmat":
        g = gb.gen_rmat(wl["scale"], wl["edgefactor"], wl["seed"], wl["wtype"])
        srcs = gb.sample_sources(g, wl["sources"], wl["source_seed"])
    else:
        g = gb.gen_grid(wl["rows"], wl["cols"], wl["seed"], wl["wtype"])
        srcs = np.zeros(1, dtype=np.uint32)
    return g, srcs


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel: str, workload: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    rec = d.get(f"{kernel}:{workload}")
    return rec


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init_group(world, rank):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allreduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------ CPU baseline
def cpu_baseline_port(g, srcs, delta, budget_s: float):
    """The oracle's C restatement of the reference's serial run_sspath_arr
    (kind "port"), one thread, on whole single-source runs of this workload
    until the budget is spent (at least one)."""
    import oracle
    done, edges, t_total = 0, 0, 0.0
    deg = np.diff(g.row.astype(np.int64))
    while done < len(srcs) and (done == 0 or t_total < budget_s):
        s = int(srcs[done])
        t0 = time.perf_counter()
        d, _ = oracle.delta_stepping(g.row, g.col, g.w, s, delta)
        t_total += time.perf_counter() - t0
        edges += int(deg[np.isfinite(d)].sum())
        done += 1
    return {"value": edges / t_total / 1e9, "unit": "GTEPS", "cores": 1, "kind": "port",
            "sample": f"{done} source(s) of this workload, whole SSSP each, oracle restatement of "
                      f"run_sspath_arr (serial), {t_total:.1f} s"}


def arm_learned(gb, g, order, W, K, par=None):
    from graphbench_gb300 import controller
    g.set_controller(controller.load())
    if par is not None:   # bit-exact against the plain schedule on the first timed source
        par.equal("arms", "plain (learned schedule)", g.sssp(order[W], flags=gb.F_LEARNED)[:2],
                  g.sssp(order[W])[:2])
    for i in range(W):
        g.sssp_device(order[i], flags=gb.F_LEARNED)
    ms = edges = 0.0
    counts = {1: 0, 2: 0, 3: 0}
    for i in range(W, W + K):
        st = g.sssp_device(order[i], flags=gb.F_LEARNED)
        ms += st["device_ms"]          # includes any abandoned learned run
        edges += st["edges_reached"]
        counts[st["learned"]] = counts.get(st["learned"], 0) + 1
    g.set_controller(None)
    return {"value": edges / ms / 1e6, "unit": "GTEPS", "ms_per_step": ms / K, "steps": K,
            "learned_steps": counts[1], "fell_back_steps": counts[3], "plain_after_loss_steps": counts[2],
            "path": "gbs_sssp_device, flags=GBS_F_LEARNED, committed controller block"}


def arm_autotuned(gb, g, order, W, K, srcs, par=None):
    t0 = time.time()
    kw, rep = g.autotune([int(s) for s in srcs[:8]], budget_ms=3000)
    tune_s = time.time() - t0
    if par is not None:
        par.equal("arms", "plain (autotuned schedule)", g.sssp(order[W], **kw)[:2], g.sssp(order[W])[:2])
    for i in range(W):
        g.sssp_device(order[i], **kw)
    ms = edges = 0.0
    for i in range(W, W + K):
        st = g.sssp_device(order[i], **kw)
        ms += st["device_ms"]
        edges += st["edges_reached"]
    return {"value": edges / ms / 1e6, "unit": "GTEPS", "ms_per_step": ms / K, "steps": K,
            "schedule": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in kw.items()},
            "delta_scale": rep["delta_scale"], "no_split": rep["no_split"], "tune_seconds": round(tune_s, 1)}


def arm_batched(gb, g, srcs, reps: int = 5, par=None):
    t0 = time.time()
    bp, rep = gb.autotune_plan(g, srcs, budget_ms=8000)
    tune_s = time.time() - t0
    with gb.Plan(g, srcs, params=bp) as plan:
        for _ in range(2):
            plan.run()
        if par is not None:
            ds, ps = plan.results()
            last = len(srcs) - 1
            par.equal("arms", "plain (batched instance 0)", (ds[0], ps[0]), g.sssp(int(srcs[0]))[:2])
            par.equal("arms", f"plain (batched instance {last})", (ds[last], ps[last]), g.sssp(int(srcs[last]))[:2])
            del ds, ps
        ms = edges = 0.0
        for _ in range(reps):
            st = plan.run()
            ms += st["device_ms"]
            edges += st["edges_reached"]
    return {"value": edges / ms / 1e6, "unit": "GTEPS", "ms_per_launch": ms / reps, "instances": len(srcs),
            "launches": reps, "group_ctas": st["group_ctas"], "groups": st["groups"],
            "params": dict(rep["best"]), "tune_seconds": round(tune_s, 1),
            "path": "gbs_plan_sources + gbs_plan_launch (CUDA graph), outputs on the device"}


def arm_betweenness(gb, g, hg, srcs, cpu: bool, n_src: int = 16):
    """Betweenness centrality (gbs_bc) over the first n_src sources of the
    workload: batched shortest paths + the DAG passes, rate in edges out of
    reached vertices per second summed over sources.  One more source is run
    alone and compared bit for bit with the oracle's Brandes restatement, whose
    single-thread time on it is the CPU baseline."""
    src = [int(x) for x in srcs[:n_src]]
    g.betweenness(src[:2])
    bc, st = g.betweenness(src)
    k = len(src)
    out = {"value": st["edges_reached"] / st["device_ms"] / 1e6, "unit": "GTEPS",
           "sources": k, "ms_per_source": st["device_ms"] / k,
           "sssp_ms_per_source": st["sssp_ms"] / k, "dag_ms_per_source": st["dag_ms"] / k,
           "max_levels": st["max_levels"], "tight_edges_per_source": st["tight_edges"] / k,
           "path": "gbs_bc (C ABI): batched gbs_plan_sources launches of up to 64 sources, then one "
                   "cooperative bc_dag launch per source; result accumulated on the device"}
    if cpu:
        import oracle
        one = [int(srcs[n_src % len(srcs)])]
        ours, st1 = g.betweenness(one)
        t0 = time.perf_counter()
        ref = oracle.betweenness(hg.row, hg.col, hg.w, one)
        secs = time.perf_counter() - t0
        out["parity_one_source"] = {"bit_identical": bool(np.array_equal(ours, ref)),
                                    "max_rel": float(np.max(np.abs(ours - ref) / np.maximum(1.0, np.abs(ref))))}
        out["cpu_baseline"] = {"value": st1["edges_reached"] / secs / 1e9, "unit": "GTEPS", "cores": 1,
                               "kind": "port", "sample": f"1 source, oracle Brandes (Dijkstra + path counts + "
                                                         f"dependencies), {secs:.1f} s"}
    return out


def arm_pagerank(gb, hg, cpu: bool):
    """PageRank (gbs_pagerank) on the workload's graph as in-edges (the graph
    is symmetric), from a device CSR built by the ingest path; the oracle's
    restatement on R-MAT 18 is the CPU baseline."""
    with gb.DeviceCsr.from_arrays(hg.row, hg.col) as c, c.transpose() as t:
        t.pagerank(max_iters=2)
        _, st = t.pagerank()
    out = {"value": st["edges"] * st["iterations"] / st["device_ms"] / 1e6, "unit": "G edge-updates/s",
           "iterations": st["iterations"], "converged": st["converged"], "ms": st["device_ms"],
           "ms_per_iteration": st["device_ms"] / max(st["iterations"], 1),
           "path": "gbs_device_csr_transpose + gbs_pagerank (RDM_JMP 0.3, THRESH 1e-6, float64)"}
    if cpu:
        import oracle
        from oracle import gen
        row, col, _ = gen.rmat(18, 16, 1, "u32")
        tr, tc = oracle.transpose(row, col)
        t0 = time.perf_counter()
        _, it = oracle.pagerank(tr, tc)
        secs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": int(row[-1]) * it / secs / 1e9, "unit": "G edge-updates/s", "cores": 1,
                               "kind": "port", "sample": f"R-MAT 18, {it} iterations, oracle or_pagerank, {secs:.1f} s"}
    return out


def arm_ingest(gb, hg, cpu: bool):
    """The binary edge-list reader (gbs_parse_bin: read_csr_bin's layout, with
    duplicate removal) and the device build of the resident graph, on the
    workload's edges in shuffled file order, from host memory."""
    n, m = hg.n, hg.m
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(hg.row.astype(np.int64)))
    perm = np.random.default_rng(1).permutation(m)
    pairs = np.empty((m, 2), dtype="<i8")
    pairs[:, 0] = src[perm] + 1
    pairs[:, 1] = hg.col.astype(np.int64)[perm] + 1
    data = np.array([n, m, 1, n], dtype="<i8").tobytes() + pairs.tobytes()
    del pairs, src, perm
    # the file image in pinned host memory, as gbs_read_bin reads a file
    pin = gb.PinnedBuffer(len(data), np.uint8)
    pin.array[:] = np.frombuffer(data, dtype=np.uint8)
    with gb.DeviceCsr.parse_bin(pin.array, gb.DIR_SEND, 1, True):
        pass
    with gb.DeviceCsr.parse_bin(pin.array, gb.DIR_SEND, 1, True) as c:
        info = dict(c.info)
        t0 = time.perf_counter()
        g = c.graph(gb.W_F64)
        gb.synchronize()
        graph_ms = (time.perf_counter() - t0) * 1e3
        g.close()
    dev_ms = info["parse_ms"] + info["build_ms"]
    out = {"value": len(data) / dev_ms / 1e6, "unit": "GB/s of file parsed and built (device)",
           "bytes": len(data), "pairs": m, "duplicates": info["duplicates"], "parse_ms": info["parse_ms"],
           "build_ms": info["build_ms"], "resident_graph_ms": graph_ms,
           "path": "gbs_parse_bin (dedup) + gbs_graph_from_device_csr; file image in pinned host memory "
                   "(host-to-device copy inside parse_ms)"}
    if cpu:
        import oracle
        k = min(m, 8_000_000)
        sample = np.array([n, k, 1, n], dtype="<i8").tobytes() + data[32:32 + 16 * k]
        t0 = time.perf_counter()
        oracle.read_bin(sample, 1, 1, False)
        secs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": len(sample) / secs / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                               "sample": f"first {k} pairs, oracle read_bin (numpy), {secs:.1f} s"}
    pin.free()
    return out


# --------------------------------------------------------------- parity
def _oracle_check(row, col, w, src, dist, pred):
    """Bit-for-bit comparison of one GPU result with the oracle: Dijkstra in
    the weight type and the smallest tight predecessor of every vertex."""
    import oracle
    ref = oracle.dijkstra(row, col, w, int(src))
    dm = int(np.count_nonzero(dist != ref))
    pm = None
    if pred is not None:
        pm = int(np.count_nonzero(pred != oracle.min_tight_pred(row, col, w, int(src), ref)))
    return {"source": int(src), "dist_mismatches": dm, "pred_mismatches": pm}


class Parity:
    """Oracle checks run in host threads while the GPU carries on (the
    oracle's C calls release the GIL); collect() waits for them."""

    def __init__(self, workers: int):
        self.pool = cf.ThreadPoolExecutor(max_workers=max(1, workers))
        self.jobs: dict[str, list] = {}

    def oracle(self, key: str, hg, src, dist, pred):
        fut = self.pool.submit(_oracle_check, hg.row, hg.col, hg.w, src, dist, pred)
        self.jobs.setdefault(key, []).append(fut)

    def equal(self, key: str, what: str, a, b):
        """A result that must equal another one (learned / autotuned /
        batched against plain), recorded like an oracle check."""
        fut = cf.Future()
        fut.set_result({"compared_with": what, "dist_mismatches": int(np.count_nonzero(a[0] != b[0])),
                        "pred_mismatches": int(np.count_nonzero(a[1] != b[1]))})
        self.jobs.setdefault(key, []).append(fut)

    def collect(self, key: str) -> dict:
        recs = [f.result() for f in self.jobs.pop(key, [])]
        bad = sum(r["dist_mismatches"] + (r["pred_mismatches"] or 0) for r in recs)
        return {"result": ("bit-identical" if bad == 0 else "MISMATCH") if recs else "not checked",
                "checks": recs}

    def close(self):
        self.pool.shutdown(wait=True)


def _timed_runs(g, srcs, reps=1, **kw):
    """Device-timed single-source runs (CUDA events of the library); returns
    (GTEPS, ms per run, runs, per-run stats)."""
    ms = edges = 0.0
    per = []
    for _ in range(reps):
        for s in srcs:
            st = g.sssp_device(int(s), **kw)
            ms += st["device_ms"]
            edges += st["edges_reached"]
            per.append(st)
    return edges / ms / 1e6, ms / len(per), len(per), per


def _plan_timed(gb, plan, launches):
    plan.run()
    ms = edges = 0.0
    for _ in range(launches):
        st = plan.run()
        ms += st["device_ms"]
        edges += st["edges_reached"]
    return edges / ms / 1e6, ms / launches, st


def config_grid4096(gb, par: Parity, steps: int):
    """C3: the 4096 x 4096 grid, float32 weights [1, 1000) (seed 3), source 0:
    plain fixed delta against the autotuned schedule and the learned
    controller; batching on 8 sources (corner + 7 seeded) of the same grid
    against those 8 run plain one after another."""
    from graphbench_gb300 import controller
    hg = gb.gen_grid(4096, 4096, 3, "f32")
    out = {"workload": "grid4096_f32", "n": hg.n, "m": hg.m}
    with gb.Graph.from_host(hg) as g:
        g.sssp_device(0)
        v, ms, k, per = _timed_runs(g, [0], reps=max(1, steps))
        out["plain"] = {"value": v, "unit": "GTEPS", "ms_per_sssp": ms, "runs": k, "phases": per[0]["phases"],
                        "buckets": per[0]["buckets"], "delta": per[0]["delta_used"]}
        d0, p0, _ = g.sssp(0)
        par.oracle("grid4096", hg, 0, d0, p0)
        t0 = time.time()
        kw, rep = g.autotune([0], budget_ms=8000)
        tune_s = time.time() - t0
        v2, ms2, k2, _ = _timed_runs(g, [0], reps=max(1, steps), **kw)
        out["autotuned"] = {"value": v2, "unit": "GTEPS", "ms_per_sssp": ms2, "runs": k2, "vs_plain": v2 / v,
                            "schedule": {a: (round(b, 4) if isinstance(b, float) else b) for a, b in kw.items()},
                            "tune_seconds": round(tune_s, 1)}
        par.equal("grid4096", "plain (autotuned schedule)", g.sssp(0, **kw)[:2], (d0, p0))
        g.set_controller(controller.load())
        # the first learned call on a graph also times the plain schedule
        # once (its guard); that run is not part of a learned step
        g.sssp_device(0, flags=gb.F_LEARNED)
        lv, lms, lk, lper = _timed_runs(g, [0], reps=max(1, steps), flags=gb.F_LEARNED)
        out["learned"] = {"value": lv, "unit": "GTEPS", "ms_per_sssp": lms, "runs": lk, "vs_plain": lv / v,
                          "learned_runs": sum(1 for s in lper if s["learned"] == 1),
                          "fell_back_runs": sum(1 for s in lper if s["learned"] != 1)}
        par.equal("grid4096", "plain (learned schedule)", g.sssp(0, flags=gb.F_LEARNED)[:2], (d0, p0))
        g.set_controller(None)
        srcs = np.concatenate([[0], gb.sample_sources(hg, 7, 3)]).astype(np.uint32)
        pv, pms, _, _ = _timed_runs(g, srcs[1:], reps=1)
        plain8 = (pms * 7 + ms) / 8
        bp, brep = gb.autotune_plan(g, srcs, budget_ms=8000)
        with gb.Plan(g, srcs, params=bp) as plan:
            bv, bms, bst = _plan_timed(gb, plan, 2)
            ds, ps = plan.results()
        par.equal("grid4096", "plain (batched instance 0)", (ds[0], ps[0]), (d0, p0))
        par.oracle("grid4096", hg, int(srcs[7]), ds[7].copy(), ps[7].copy())
        del ds, ps
        out["batched"] = {"value": bv, "unit": "GTEPS", "ms_per_launch": bms, "instances": len(srcs),
                          "plain_ms_for_the_same_sources": plain8 * 8, "vs_plain": (plain8 * 8) / bms,
                          "groups": bst["groups"], "group_ctas": bst["group_ctas"], "params": brep["best"]}
    out["parity"] = par.collect("grid4096")
    return out


def config_rmat24(gb, par: Parity, steps: int):
    """C5: R-MAT scale 24 (edge factor 16, uint32 [1, 255]), 8 sources of seed
    7: plain, learned, autotuned and batched; every learned / autotuned result
    compared with the plain one, two plain ones with the oracle."""
    from graphbench_gb300 import controller
    hg = gb.gen_rmat(24, 16, 1)
    srcs = gb.sample_sources(hg, 8, 7)
    out = {"workload": "rmat24_u32", "n": hg.n, "m": hg.m, "sources": len(srcs)}
    reps = max(1, steps // len(srcs))
    with gb.Graph.from_host(hg) as g:
        for s in srcs[:2]:
            g.sssp_device(int(s))
        v, ms, k, per = _timed_runs(g, srcs, reps=reps)
        out["plain"] = {"value": v, "unit": "GTEPS", "ms_per_sssp": ms, "runs": k,
                        "avg_phases": sum(p["phases"] for p in per) / k, "delta": per[0]["delta_used"]}
        ref = {}
        for s in srcs[:2]:
            d, p, _ = g.sssp(int(s))
            ref[int(s)] = (d, p)
            par.oracle("rmat24", hg, int(s), d, p)
        g.set_controller(controller.load())
        g.sssp_device(int(srcs[0]), flags=gb.F_LEARNED)   # the guard's plain timing run
        lv, lms, lk, lper = _timed_runs(g, srcs, reps=reps, flags=gb.F_LEARNED)
        out["learned"] = {"value": lv, "unit": "GTEPS", "ms_per_sssp": lms, "runs": lk, "vs_plain": lv / v,
                          "learned_runs": sum(1 for s in lper if s["learned"] == 1),
                          "fell_back_runs": sum(1 for s in lper if s["learned"] == 3),
                          "plain_after_loss_runs": sum(1 for s in lper if s["learned"] == 2)}
        for s in srcs[:2]:
            par.equal("rmat24", "plain (learned schedule)", g.sssp(int(s), flags=gb.F_LEARNED)[:2], ref[int(s)])
        g.set_controller(None)
        t0 = time.time()
        kw, rep = g.autotune([int(x) for x in srcs[:2]], budget_ms=4000)
        tune_s = time.time() - t0
        av, ams, ak, _ = _timed_runs(g, srcs, reps=reps, **kw)
        out["autotuned"] = {"value": av, "unit": "GTEPS", "ms_per_sssp": ams, "runs": ak, "vs_plain": av / v,
                            "schedule": {a: (round(b, 4) if isinstance(b, float) else b) for a, b in kw.items()},
                            "tune_seconds": round(tune_s, 1)}
        for s in srcs[:2]:
            par.equal("rmat24", "plain (autotuned schedule)", g.sssp(int(s), **kw)[:2], ref[int(s)])
        t0 = time.time()
        bp, brep = gb.autotune_plan(g, srcs, budget_ms=8000)
        tune_b = time.time() - t0
        with gb.Plan(g, srcs, params=bp) as plan:
            bv, bms, bst = _plan_timed(gb, plan, 2)
            ds, ps = plan.results()
        for i in range(2):
            par.equal("rmat24", f"plain (batched instance {i})", (ds[i], ps[i]), ref[int(srcs[i])])
        del ds, ps
        out["batched"] = {"value": bv, "unit": "GTEPS", "ms_per_launch": bms, "instances": len(srcs),
                          "vs_plain": bv / v, "groups": bst["groups"], "group_ctas": bst["group_ctas"],
                          "params": brep["best"], "tune_seconds": round(tune_b, 1)}
    out["parity"] = par.collect("rmat24")
    return out


def config_rmat20_512(gb, par: Parity):
    """C4a: 512 sources (seed 7) on R-MAT scale 20 in one persistent batched
    launch replayed from a CUDA graph, against the same 512 run plain one
    after another; two instances checked with the oracle."""
    hg = gb.gen_rmat(20, 16, 1)
    srcs = gb.sample_sources(hg, 512, 7)
    out = {"workload": "rmat20_512src_u32", "n": hg.n, "m": hg.m, "sources": len(srcs)}
    with gb.Graph.from_host(hg) as g:
        for s in srcs[:3]:
            g.sssp_device(int(s))
        v, ms, k, _ = _timed_runs(g, srcs)
        out["plain"] = {"value": v, "unit": "GTEPS", "ms_total": ms * k, "runs": k}
        t0 = time.time()
        bp, brep = gb.autotune_plan(g, srcs, budget_ms=6000)
        tune_b = time.time() - t0
        with gb.Plan(g, srcs, params=bp) as plan:
            bv, bms, bst = _plan_timed(gb, plan, 3)
            ds, ps = plan.results()
        for i in (0, 511):
            par.oracle("rmat20_512", hg, int(srcs[i]), ds[i].copy(), ps[i].copy())
        del ds, ps
    out["batched"] = {"value": bv, "unit": "GTEPS", "ms_per_launch": bms, "vs_plain": bv / v,
                      "groups": bst["groups"], "group_ctas": bst["group_ctas"], "params": brep["best"],
                      "tune_seconds": round(tune_b, 1),
                      "path": "gbs_plan_sources + gbs_plan_launch (CUDA graph), 512 dist/pred arrays on the device"}
    out["parity"] = par.collect("rmat20_512")
    return out


def config_pack1024(gb, par: Parity):
    """C4b: 1,024 independent R-MAT graphs, scales uniform in [10, 16] (seed
    11), one seeded source each, in one batched launch, against the same
    graphs run one after another (each its own resident graph, plain
    schedule); two instances checked with the oracle."""
    rng = np.random.default_rng(11)
    scales = rng.integers(10, 17, size=1024)
    graphs, srcs = [], []
    for i, sc in enumerate(scales):
        h = gb.gen_rmat(int(sc), 16, 11 + i)
        graphs.append(h)
        srcs.append(int(gb.sample_sources(h, 1, 11 + i)[0]))
    srcs = np.array(srcs, dtype=np.uint32)
    out = {"workload": "pack1024_u32", "graphs": len(graphs), "scales": [int(scales.min()), int(scales.max())],
           "total_n": int(sum(h.n for h in graphs)), "total_m": int(sum(h.m for h in graphs))}
    ms = edges = 0.0
    for h, s in zip(graphs, srcs):
        with gb.Graph.from_host(h) as g:
            g.sssp_device(int(s))
            st = g.sssp_device(int(s))
            ms += st["device_ms"]
            edges += st["edges_reached"]
    out["plain"] = {"value": edges / ms / 1e6, "unit": "GTEPS", "ms_total": ms,
                    "path": "one resident graph and one gbs_sssp_device run per pack graph"}
    with gb.Pack(graphs) as pk:
        t0 = time.time()
        bp, brep = gb.autotune_plan(pk, srcs, budget_ms=6000)
        tune_b = time.time() - t0
        with gb.Plan(pk, srcs, params=bp) as plan:
            bv, bms, bst = _plan_timed(gb, plan, 3)
            ds, ps = plan.results()
        big = int(np.argmax([h.m for h in graphs]))
        for i in (0, big):
            par.oracle("pack1024", graphs[i], int(srcs[i]), ds[i].copy(), ps[i].copy())
        del ds, ps
    out["batched"] = {"value": bv, "unit": "GTEPS", "ms_per_launch": bms, "vs_plain": bv / out["plain"]["value"],
                      "groups": bst["groups"], "group_ctas": bst["group_ctas"], "params": brep["best"],
                      "tune_seconds": round(tune_b, 1),
                      "path": "gbs_pack_create + gbs_plan_pack + gbs_plan_launch (CUDA graph)"}
    out["parity"] = par.collect("pack1024")
    return out


CONFIGS = {"grid4096_f32": config_grid4096, "rmat24_u32": config_rmat24,
           "rmat20_512src": config_rmat20_512, "pack1024": config_pack1024}


# ----------------------------------------------------------------- our arm
def run_ours(args):
    world, rank, local = dist_env()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = init_group(world, rank)
    import runpy
    runpy.run_path(str(ROOT / "graphbench_gb300" / "build.py"))["build"]()
    import graphbench_gb300 as gb
    if not gb.device_available():
        raise SystemExit("no usable GPU")
    wl = WORKLOADS[args.workload]
    t0 = time.time()
    hg, srcs = make_workload(gb, wl)
    log(f"[rank {rank}] generated {args.workload}: n={hg.n} m={hg.m} in {time.time() - t0:.1f}s")
    t0 = time.time()
    g = gb.Graph.from_host(hg)
    log(f"[rank {rank}] uploaded in {time.time() - t0:.1f}s")
    delta = args.delta if args.delta else None
    light = args.light if args.light is not None else None
    K, W = args.steps, args.warmup
    order = [int(srcs[i % len(srcs)]) for i in range(W + K)]
    dd = gb.DeviceBuffer(4 * hg.n)
    pd = gb.DeviceBuffer(4 * hg.n)
    for i in range(W):
        g.sssp_device(order[i], dd.ptr, pd.ptr, delta=delta, light=light)
    gb.synchronize()
    sampler = ClockSampler(local if world > 1 else int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0))
    sampler.start()
    barrier(dist)
    gb.synchronize()
    wall0 = time.perf_counter()
    per = []
    for i in range(W, W + K):
        st = g.sssp_device(order[i], dd.ptr, pd.ptr, delta=delta, light=light)
        per.append(st)
    gb.synchronize()
    barrier(dist)
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    dev_s = sum(s["device_ms"] for s in per) / 1e3
    ker_s = sum(s["kernel_ms"] for s in per) / 1e3
    edges = sum(s["edges_reached"] for s in per)
    verts = sum(s["reached"] for s in per)
    # e2e: the public call with pinned host outputs (dist + pred copied back)
    hd = gb.PinnedBuffer(hg.n, g.dist_dtype)
    hp = gb.PinnedBuffer(hg.n, np.int32)
    ke = min(K, args.e2e_steps)
    e2e_t, e2e_edges = 0.0, 0
    for i in range(ke):
        t = time.perf_counter()
        _, _, st = g.sssp(order[W + i], delta=delta, light=light, out_dist=hd.array, out_pred=hp.array)
        e2e_t += time.perf_counter() - t
        e2e_edges += st["edges_reached"]
    # parity of the plain steps: the first two timed sources again, results
    # to the host, against the oracle (host threads; the GPU carries on)
    par = Parity(min(8, os.cpu_count() or 1)) if rank == 0 else None
    if par is not None and not args.no_parity:
        for src in order[W:W + 2]:
            d, p, _ = g.sssp(src, delta=delta, light=light)
            par.oracle("plain", hg, src, d, p)
    # whole-job aggregates
    dev_max = allreduce_max(dist, dev_s)
    wall_max = allreduce_max(dist, wall)
    edges_all = allreduce_sum(dist, float(edges))
    e2e_max = allreduce_max(dist, e2e_t)
    e2e_edges_all = allreduce_sum(dist, float(e2e_edges))
    result = None
    if rank == 0:
        peak, peak_src = measured_peaks()
        algo_bytes = 16.0 * edges + 24.0 * verts           # per-launch sum over the K launches
        achieved = algo_bytes / ker_s / 1e9
        st0 = per[0]
        traffic = profiled_traffic("sssp_persistent", args.workload)
        wlc = dict(wl)
        wlc.update(n=hg.n, m=hg.m, delta=st0["delta_used"], light=st0["light_used"],
                   blocks=st0["blocks"], source_rule="seeded sample of vertices with out-degree > 0"
                   if wl["kind"] == "rmat" else "corner vertex 0",
                   l2=f"inputs larger than L2: CSR {(hg.m * 8 + hg.n * 4) / 1e9:.2f} GB vs 0.135 GB L2; "
                      "per-step device time from CUDA events on the library's stream",
                   avg_buckets=sum(s["buckets"] for s in per) / K,
                   avg_phases=sum(s["phases"] for s in per) / K,
                   avg_kernel_ms=ker_s * 1e3 / K,
                   avg_device_ms=dev_s * 1e3 / K,
                   wall_ms_per_step=wall * 1e3 / K)
        result = {
            "metric": "GTEPS SSSP, learned/batched vs plain fixed-delta on 1 GB300; % HBM roofline",
            "value_is": "plain fixed-delta delta-stepping (learned / autotuned / batched: see those keys)",
            "value": edges_all / dev_max / 1e9,
            "unit": "GTEPS",
            "n_gpus": world,
            "steps": K,
            "warmup": W,
            "ms_per_step": dev_max * 1e3 / K,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": wl["wtype"],
            "data": "synthetic (seeded R-MAT / grid generator, no dataset)",
            "config": {"workload": f"{args.workload}_{wl['wtype']}", **wlc,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"
                         if peak_src == "measured" else "fallback 6.8 TB/s",
                         "kernel": "sssp_persistent",
                         "algorithmic_bytes_per_launch": algo_bytes / K,
                         "traffic": traffic.get("bytes_per_launch") if traffic else None,
                         "traffic_source": traffic.get("source") if traffic else None},
            "e2e": {"value": e2e_edges_all / e2e_max / 1e9 if e2e_max > 0 else None, "unit": "GTEPS",
                    "h2d_bytes_per_step": 4,
                    "d2h_bytes_per_step": hg.n * 8 + 1024,
                    "steps": ke,
                    "path": "gbs_sssp (C ABI) -> pinned host dist + pred; graph resident"},
            "gpu_launches": 4 * K,
            "clocks": clocks,
            "wall_ms_per_step": wall_max * 1e3 / K,
        }
        if world == 1 and not args.no_arms:
            plain = result["value"]
            for name, fn in (("learned", lambda: arm_learned(gb, g, order, W, K, par)),
                             ("autotuned", lambda: arm_autotuned(gb, g, order, W, K, srcs, par)),
                             ("batched", lambda: arm_batched(gb, g, srcs, par=par))):
                try:
                    arm = fn()
                    arm["vs_plain"] = arm["value"] / plain
                except Exception as e:  # pragma: no cover
                    arm = {"value": None, "error": str(e)}
                result[name] = arm
                log(f"[rank 0] {name}: {arm.get('value')}")
            result["arms_parity"] = par.collect("arms")
        if world == 1 and not args.no_bc:
            try:
                result["betweenness"] = arm_betweenness(gb, g, hg, srcs, cpu=not args.no_cpu_baseline)
            except Exception as e:  # pragma: no cover
                result["betweenness"] = {"value": None, "error": str(e)}
            log(f"[rank 0] betweenness: {result['betweenness'].get('value')}")
        # the oracle checks of the plain steps finish before the host-bound
        # ingest measurement starts
        result["parity"] = par.collect("plain")
        if world == 1 and not args.no_bc:
            for name, fn in (("pagerank", lambda: arm_pagerank(gb, hg, not args.no_cpu_baseline)),
                             ("ingest", lambda: arm_ingest(gb, hg, not args.no_cpu_baseline))):
                try:
                    result[name] = fn()
                except Exception as e:  # pragma: no cover
                    result[name] = {"value": None, "error": str(e)}
                log(f"[rank 0] {name}: {result[name].get('value')}")
        if world == 1 and not args.no_cpu_baseline:
            try:
                result["cpu_baseline"] = cpu_baseline_port(hg, srcs, st0["delta_used"], args.cpu_budget_s)
            except Exception as e:  # pragma: no cover
                result["cpu_baseline"] = {"value": None, "unavailable": str(e)}
    dd.free()
    pd.free()
    hd.free()
    hp.free()
    g.close()
    if rank == 0 and world == 1 and args.configs != "none":
        names = list(CONFIGS) if args.configs == "all" else [c for c in args.configs.split(",") if c]
        for name in names:
            t0 = time.time()
            try:
                fn = CONFIGS[name]
                rec = fn(gb, par, args.config_steps) if name in ("grid4096_f32", "rmat24_u32") else fn(gb, par)
            except Exception as e:  # pragma: no cover
                rec = {"value": None, "error": f"{type(e).__name__}: {e}"}
            rec["wall_s"] = round(time.time() - t0, 1)
            result[name] = rec
            log(f"[rank 0] {name}: {json.dumps({k: v.get('value') for k, v in rec.items() if isinstance(v, dict) and 'value' in v})} "
                f"parity {rec.get('parity', {}).get('result')} in {rec['wall_s']} s")
    if par is not None:
        par.close()
    if dist is not None:
        dist.destroy_process_group()
    if result is not None:
        print(json.dumps(result), flush=True)


# ------------------------------------------------------------ reference arm
def _ref_worker(args_tuple):
    """Runs in a forked child: one reference run_sspath_arr, returns
    (edges_reached, seconds)."""
    import oracle
    row, col, w, src, delta, maxd = args_tuple
    d, secs = oracle.ref_sssp_arr(row, col, w, src, delta, maxdist=maxd, cap_mult=2.0)
    deg = np.diff(row.astype(np.int64))
    return int(deg[np.isfinite(d)].sum()), secs


def _child_call(q, fn, args):
    try:
        q.put(("ok", fn(*args)))
    except BaseException as e:  # pragma: no cover - reported to the parent
        q.put(("error", f"{type(e).__name__}: {e}"))


def _in_child(ctx, fn, args, timeout_s):
    """fn(*args) in a forked child (the reference keeps globals and never
    frees, and its OpenMP build can crash): (status, value-or-message)."""
    q = ctx.Queue()
    pr = ctx.Process(target=_child_call, args=(q, fn, args))
    pr.start()
    try:
        status, val = q.get(timeout=timeout_s)
    except Exception:
        status, val = "error", "no result within the time limit" if pr.is_alive() else f"exit code {pr.exitcode}"
    pr.join(timeout=5)
    if pr.is_alive():
        pr.kill()
        pr.join()
    return status, val


def _ref_omp(row, col, w, src, delta, maxd, threads):
    import oracle
    return oracle.ref_sssp_arr(row, col, w, src, delta, variant="omp", threads=threads, maxdist=maxd, cap_mult=4.0)


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    import oracle
    from oracle import build_ref, gen
    try:
        if not (oracle.ref_available("serial") and oracle.ref_available("omp")):
            build_ref.stage()
            build_ref.compile_ref()
        # mapped in this process before the workers fork, so the process
        # that prints the line has the compiled reference loaded
        oracle.ref_lib("serial")
        oracle.ref_lib("omp")
    except Exception as e:
        print(json.dumps({"impl": "reference", "unavailable": f"reference build failed: {e}"}))
        return
    wl = WORKLOADS[args.workload]
    # Bounded sample: the reference's serial run_sspath_arr costs ~120 s per
    # source at scale 20 on one core (measured), so each step runs one source
    # per host core on the same R-MAT family at --ref-scale (default 16, the
    # reference's own CPU-runnable configuration).
    scale = args.ref_scale if wl["kind"] == "rmat" else None
    if scale is None:
        print(json.dumps({"impl": "reference", "unavailable": "reference arm implemented for the R-MAT workloads"}))
        return
    row, col, w = gen.rmat(scale, wl["edgefactor"], wl["seed"], wl["wtype"])
    srcs = gen.sample_sources(row, 64, wl["source_seed"])
    delta = gen.heuristic_delta(row, w)
    exact = {}
    maxd = 0.0
    for s in srcs[:4]:
        dj = oracle.dijkstra(row, col, w, int(s))
        exact[int(s)] = dj
        maxd = max(maxd, float(dj[dj != 0xFFFFFFFF].max()))
    maxd *= 1.5
    host_cores = os.cpu_count() or 1
    cores = max(1, min(host_cores, args.ref_procs))
    ctx = mp.get_context("fork")
    K, W = args.steps, args.warmup
    i = 0

    def one_step(pool):
        nonlocal i
        batch = [(row, col, w, int(srcs[(i + j) % len(srcs)]), delta, maxd) for j in range(cores)]
        i += cores
        t0 = time.perf_counter()
        res = pool.map(_ref_worker, batch)
        return sum(r[0] for r in res), time.perf_counter() - t0

    budget = args.ref_budget_s
    with ctx.Pool(cores) as pool:
        for _ in range(W):
            one_step(pool)
        done, edges, secs = 0, 0, 0.0
        t_start = time.perf_counter()
        while done < K and (done == 0 or time.perf_counter() - t_start < budget):
            e, s = one_step(pool)
            edges += e
            secs += s
            done += 1
    val = edges / secs / 1e9
    # the reference's OpenMP build (-DUSE_OMP), all host cores on one source
    # at a time; its relax keeps one request per target ordered by edge
    # weight (structural defect D5), so its distances are counted against
    # the exact ones
    deg = np.diff(row.astype(np.int64))
    omp = {"threads": host_cores, "runs": []}
    t_omp = 0.0
    e_omp = 0
    for s in list(exact)[:4]:
        st, res = _in_child(ctx, _ref_omp, (row, col, w, s, delta, maxd, host_cores), 120)
        if st != "ok":
            omp["runs"].append({"source": s, "status": res})
            continue
        d, sec = res
        ex = exact[s].astype(np.float64)
        ex[exact[s] == 0xFFFFFFFF] = np.inf
        omp["runs"].append({"source": s, "seconds": sec, "distance_mismatches": int(np.count_nonzero(d != ex))})
        t_omp += sec
        e_omp += int(deg[np.isfinite(ex)].sum())
    omp["value"] = e_omp / t_omp / 1e9 if t_omp > 0 else None
    omp["unit"] = "GTEPS"
    omp["note"] = ("reported beside the serial value, not as it: the OpenMP build is inexact by design "
                   "(one request per target, ordered by edge weight)")
    sample = (f"{done} step(s) x {cores} concurrent single-source runs of the reference's serial "
              f"run_sspath_arr (patched D1/D2/D4, logging off) on R-MAT scale {scale} (same generator, "
              f"edge factor, weights, delta rule and source seed as {args.workload}); stand-in size because "
              f"one scale-{wl.get('scale')} run takes minutes on one core")
    print(json.dumps({
        "impl": "reference", "metric": "GTEPS SSSP, learned/batched vs plain fixed-delta on 1 GB300; % HBM roofline",
        "value_is": "the reference's serial run_sspath_arr, plain fixed delta", "value": val,
        "unit": "GTEPS", "n_gpus": world, "steps": done, "warmup": W, "ms_per_step": secs * 1e3 / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 (reference doubles)",
        "data": "synthetic", "config": {"workload": f"{args.workload}_{wl['wtype']}", "reference_scale": scale,
                                        "delta": delta, "processes": cores, "host_cores": host_cores},
        "cpu_baseline": {"value": val, "unit": "GTEPS", "cores": cores, "kind": "reference", "sample": sample},
        "openmp": omp,
        "e2e": {"value": val, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=64)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="rmat22")
    ap.add_argument("--delta", type=float, default=0.0)
    ap.add_argument("--light", type=float, default=None)
    ap.add_argument("--e2e-steps", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-arms", action="store_true", help="skip the learned / autotuned / batched arms")
    ap.add_argument("--no-bc", action="store_true", help="skip the betweenness, PageRank and ingest measurements")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle checks of the plain steps")
    ap.add_argument("--configs", default="all",
                    help="comma-separated list of " + ", ".join(CONFIGS) + "; 'all' (default) or 'none'")
    ap.add_argument("--config-steps", type=int, default=2,
                    help="timed runs per source in the grid4096_f32 / rmat24_u32 records")
    ap.add_argument("--cpu-budget-s", type=float, default=20.0)
    ap.add_argument("--ref-scale", type=int, default=16)
    ap.add_argument("--ref-procs", type=int, default=16)
    ap.add_argument("--ref-budget-s", type=float, default=120.0)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        log("note: fewer than 3 warm-up steps")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
