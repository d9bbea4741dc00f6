"""The learned bucket-width controller: data collection, training, storage.

The network (an FP32 MLP, 16 inputs -> 64 -> 64 -> 2) runs inside the SSSP
kernel at every bucket start of a ``flags=F_LEARNED`` run (see
``gbs_graph_set_controller`` in include/gbsssp.h for its inputs and outputs).
It is trained here, on the GPU, with the library's own CUDA forward, backward
and Adam kernels (``Mlp``), on traces of the plain method:

1. for each seeded training graph, the autotuner sweeps the bucket width
   (powers of two times the plain width max_weight / average degree) with and
   without the light/heavy split and keeps the fastest (``collect_graph``);
2. fixed-width runs around that best width record the controller inputs at
   every bucket start (``GBS_F_FEATURES``);
3. every recorded input is labelled with the graph's best (log2 width
   scale, split); samples are weighted so that each graph counts once.
   Every width at or above the largest distance gives the same schedule (one
   bucket), so the label is capped at the first such width: otherwise small
   graphs, where every width past that point ties, give labels spread over
   the whole flat end of the sweep.

4. the two output biases are calibrated on the held-out graphs
   (``calibrate``): learned runs with output 0 shifted by 0 .. -4 (every
   predicted width divided by up to 16) and output 1 shifted by -30 / 0 / +30
   (always whole rows / as predicted / always split) are timed against the
   plain schedule, and the pair with the best geometric-mean speed-up is
   added to the block.  The labels are the best FIXED width of a graph, but
   the controller re-decides at every bucket start, and a width that is best
   for the whole run is too wide for most buckets taken one at a time.

Distances never depend on the width, so the controller can only change the
run time; the library checks that by falling back to the plain schedule when
a learned run takes longer than (1 + margin) times the plain one.

``python -m graphbench_gb300.controller --out FILE`` runs the whole pipeline
(200 graphs: R-MAT scales 14-20 and 1024^2-2048^2 grids) and writes the
parameter block; the committed block is ``delta_mlp.bin`` beside this file.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time
from pathlib import Path

import numpy as np

import graphbench_gb300 as gb

DEFAULT_PATH = Path(__file__).resolve().parent / "delta_mlp.bin"
MAGIC = b"GBSMLP01"


def save(params: np.ndarray, path: Path | str = DEFAULT_PATH) -> None:
    p = np.ascontiguousarray(params, dtype="<f4")
    assert p.shape == (gb.MLP_FLOATS,)
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.array([gb.MLP_FLOATS], dtype="<u4").tobytes())
        f.write(p.tobytes())


def load(path: Path | str = DEFAULT_PATH) -> np.ndarray:
    raw = Path(path).read_bytes()
    if raw[:8] != MAGIC:
        raise ValueError(f"{path}: not a controller block")
    n = int(np.frombuffer(raw[8:12], dtype="<u4")[0])
    if n != gb.MLP_FLOATS:
        raise ValueError(f"{path}: {n} floats, expected {gb.MLP_FLOATS}")
    return np.frombuffer(raw[12:12 + 4 * n], dtype="<f4").astype(np.float32).copy()


# ----------------------------------------------------------------- data
def training_specs(count: int = 200, seed: int = 2024) -> list[dict]:
    """R-MAT scales 14-20 (uint32 weights 1..255) and square grids with
    sides 1024-2048 (float32 weights), three R-MATs for every grid."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        if i % 4 == 3:
            side = int(rng.integers(1024, 2049))
            specs.append({"kind": "grid", "side": side, "seed": 5000 + i})
        else:
            specs.append({"kind": "rmat", "scale": int(rng.integers(14, 21)), "seed": 1000 + i})
    return specs


def make_graph(spec: dict) -> gb.HostGraph:
    if spec["kind"] == "grid":
        return gb.gen_grid(spec["side"], spec["side"], spec["seed"], "f32")
    return gb.gen_rmat(spec["scale"], 16, spec["seed"])


def collect_graph(spec: dict, tune_budget_ms: float = 800.0, feature_scales=(1 / 8, 1 / 2, 1, 2, 8)) -> dict:
    """Best plain schedule of one graph and the inputs recorded around it."""
    host = make_graph(spec)
    srcs = [0] if spec["kind"] == "grid" else [int(s) for s in gb.sample_sources(host, 2, spec["seed"])]
    with gb.Graph.from_host(host) as g:
        _, rep = g.autotune(srcs, budget_ms=tune_budget_ms)
        best = float(rep["delta_scale"])
        split = 0.0 if rep["no_split"] else 1.0
        d0 = g.info()["default_delta"]
        d, _, _ = g.sssp(srcs[0], want_pred=False)
        unreached = np.float32(np.inf) if d.dtype == np.float32 else np.uint32(0xFFFFFFFF)
        fin = d[d != unreached].astype(np.float64)
        maxdist = float(fin.max()) if len(fin) else d0
        one_bucket = 2.0 ** math.ceil(math.log2(max(maxdist / d0, 1.0)))
        best = min(best, one_bucket)
        rows = []
        for f in sorted(set([*feature_scales, 1.0 / best])):
            light = None if split else math.inf
            g.sssp(srcs[0], delta=d0 * best * f, light=light, flags=gb.F_FEATURES, want_dist=False,
                   want_pred=False)
            x = g.features()
            if len(x):
                # the state the host predicts from before bucket 0 (the source
                # alone in its bucket, nothing done yet), with this run's
                # graph inputs
                first = np.concatenate([np.ones(7), np.zeros(4), x[0, 11:]]).astype(np.float32)
                rows.append(first[None, :])
            rows.append(x)
    x = np.concatenate(rows) if rows else np.zeros((0, gb.N_FEAT), np.float32)
    return {"spec": spec, "best_scale": best, "split": split, "default_ms": rep["default_ms"],
            "best_ms": rep["best_ms"], "x": x}


def dataset(collected: list[dict]):
    """(inputs, targets, weights) with every graph's samples weighing 1 in all."""
    xs, ts, ws = [], [], []
    for c in collected:
        k = len(c["x"])
        if not k:
            continue
        xs.append(c["x"])
        ts.append(np.tile([math.log2(c["best_scale"]), c["split"]], (k, 1)))
        ws.append(np.full(k, 1.0 / k))
    return (np.concatenate(xs).astype(np.float32), np.concatenate(ts).astype(np.float32),
            np.concatenate(ws).astype(np.float32))


# ------------------------------------------------------------- training
def init_block(x: np.ndarray, seed: int) -> np.ndarray:
    """He-initialised parameter block standardising the inputs of x."""
    rng = np.random.default_rng(seed)
    F, H = gb.N_FEAT, 64
    p = np.zeros(gb.MLP_FLOATS, dtype=np.float64)
    p[:F] = x.mean(0)
    p[F:2 * F] = np.maximum(x.std(0), 1e-3)
    o = 2 * F
    p[o:o + F * H] = rng.normal(0, math.sqrt(2 / F), F * H)
    o += F * H + H
    p[o:o + H * H] = rng.normal(0, math.sqrt(2 / H), H * H)
    o += H * H + H
    p[o:o + H * 2] = rng.normal(0, math.sqrt(1 / H), H * 2)
    return p.astype(np.float32)


def fit(x, t, w, epochs: int = 80, batch: int = 512, lr: float = 2e-3, seed: int = 0):
    """Adam on the GPU kernels; returns (parameter block, per-epoch loss)."""
    m = gb.Mlp(init_block(x, seed))
    m.set_data(x, t, w)
    losses = m.train(epochs, batch, lr, seed)
    p = m.params()
    m.close()
    return p, losses


def evaluate(params, x, t, w) -> float:
    m = gb.Mlp(params)
    m.set_data(x, t, w)
    loss, _ = m.loss_grad()
    m.close()
    return loss


B3 = gb.MLP_FLOATS - 2   # output biases: b3[0] (log2 width scale), b3[1] (split logit)


def calibrate(params: np.ndarray, specs: list[dict], shifts=(0, -1, -2, -3, -4),
              split_bias=(0.0, -30.0, 30.0), sources: int = 4, log=print) -> tuple[np.ndarray, dict]:
    """Output-bias pair with the best geometric-mean speed-up of learned over
    plain runs (kernel time, guard off) on the graphs of `specs`; returns the
    block with that pair added and a report."""
    speed = {(a, b): [] for a in shifts for b in split_bias}
    for spec in specs:
        host = make_graph(spec)
        srcs = [0] if spec["kind"] == "grid" else [int(x) for x in gb.sample_sources(host, sources, spec["seed"])]
        with gb.Graph.from_host(host) as g:
            g.sssp_device(srcs[0])
            plain = float(np.mean([g.sssp_device(x)["kernel_ms"] for x in srcs]))
            row = {}
            for (a, b) in speed:
                q = params.copy()
                q[B3] += a
                q[B3 + 1] += b
                g.set_controller(q, margin=1000.0)
                g.sssp_device(srcs[0], flags=gb.F_LEARNED)
                ms = float(np.mean([g.sssp_device(x, flags=gb.F_LEARNED)["kernel_ms"] for x in srcs]))
                g.set_controller(None)
                speed[(a, b)].append(plain / ms)
                row[f"{a}/{b:g}"] = round(plain / ms, 3)
        log(json.dumps({**spec, "plain_ms": round(plain, 3), "speedup": row}))
    gm = {k: float(np.exp(np.mean(np.log(v)))) for k, v in speed.items()}
    best = max(gm, key=gm.get)
    out = params.copy()
    out[B3] += best[0]
    out[B3 + 1] += best[1]
    report = {"graphs": len(specs), "width_shift": best[0], "split_shift": best[1],
              "geomean_speedup": round(gm[best], 4), "geomean_uncalibrated": round(gm[(0, 0.0)], 4),
              "table": {f"{a}/{b:g}": round(v, 4) for (a, b), v in gm.items()}}
    return out, report


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="train the bucket-width controller")
    ap.add_argument("--out", default=str(DEFAULT_PATH))
    ap.add_argument("--graphs", type=int, default=200)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--epochs", type=int, default=80)
    ap.add_argument("--summary", default=None, help="JSON summary file")
    ap.add_argument("--calibrate", default=None, metavar="BLOCK",
                    help="only calibrate the output biases of an existing block on the held-out graphs")
    args = ap.parse_args(argv)
    t0 = time.time()
    specs = training_specs(args.graphs, args.seed)
    held_out = [s for i, s in enumerate(specs) if i % 10 == 9]
    if args.calibrate:
        params, rep = calibrate(load(args.calibrate), held_out)
        save(params, args.out)
        rep["seconds"] = round(time.time() - t0, 1)
        if args.summary:
            Path(args.summary).write_text(json.dumps(rep, indent=1))
        print(json.dumps({k: v for k, v in rep.items() if k != "table"}), flush=True)
        return 0
    collected = []
    for i, s in enumerate(specs):
        c = collect_graph(s, tune_budget_ms=8000.0 if s["kind"] == "grid" else 800.0)
        collected.append(c)
        print(json.dumps({"i": i, **s, "best_scale": c["best_scale"], "split": c["split"],
                          "samples": len(c["x"]), "default_ms": round(c["default_ms"], 3),
                          "best_ms": round(c["best_ms"], 3)}), flush=True)
    # every tenth graph is held out for validation
    tr = [c for i, c in enumerate(collected) if i % 10 != 9]
    va = [c for i, c in enumerate(collected) if i % 10 == 9]
    x, t, w = dataset(tr)
    params, losses = fit(x, t, w, epochs=args.epochs)
    vx, vt, vw = dataset(va)
    vloss = evaluate(params, vx, vt, vw)
    params, cal = calibrate(params, held_out)
    save(params, args.out)
    summary = {"graphs": len(specs), "samples": int(len(x)), "train_loss_first": float(losses[0]),
               "train_loss_last": float(losses[-1]), "val_loss": float(vloss), "calibration": cal,
               "seconds": round(time.time() - t0, 1),
               "per_graph": [{**c["spec"], "best_scale": c["best_scale"], "split": c["split"],
                              "default_ms": c["default_ms"], "best_ms": c["best_ms"]} for c in collected]}
    if args.summary:
        Path(args.summary).write_text(json.dumps(summary, indent=1))
    print(json.dumps({k: v for k, v in summary.items() if k != "per_graph"}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
