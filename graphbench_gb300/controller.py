"""The learned bucket-width controller: data collection, training, storage.

The network (an FP32 MLP, 16 inputs -> 64 -> 64 -> 2) runs inside the SSSP
kernel at every bucket start of a ``flags=F_LEARNED`` run (see
``gbs_graph_set_controller`` in include/gbsssp.h for its inputs and outputs).
It is trained here, on the GPU, with the library's own CUDA forward, backward
and Adam kernels (``Mlp``), on traces of the plain method:

1. for each seeded training graph, the plain method runs at every width
   d * 2^k (k = -2 .. 8, d the plain width max_weight / average degree),
   with and without the light/heavy split, recording its phase trace and the
   controller inputs at every bucket start (``collect_graph``);
2. each run's trace gives the time at which every distance was settled
   (inside a bucket, its time is spread over the vertices it settles, whose
   final distances every schedule shares); a recorded bucket start at
   distance D is labelled with the (k, split) whose run covered the next
   HORIZON plain widths [D, D + 8 d) fastest.  The initial state (the source
   alone; the host predicts the run's base width from it) is labelled with
   the graph's best fixed (k, split) and carries the vertex count.  The
   controller re-decides at every bucket start, so it learns the width that
   pays from that point on (narrow where the buckets are large, wide in the
   sparse tail), not one width per graph.  Samples weigh by the time their
   window costs at its best width; each graph counts once;
3. training (``fit``) minimises the squared error of output 0 against k and
   the logistic loss of output 1 against the split;
4. the two output biases are calibrated on the held-out graphs
   (``calibrate``): learned runs with output 0 shifted by 0 .. -4 (every
   predicted width divided by up to 16) and output 1 shifted by -30 / 0 / +30
   (always whole rows / as predicted / always split) are timed against the
   plain schedule, and the pair with the best geometric-mean speed-up is
   added to the block.

None of the inputs grows with the vertex count by itself (occupancies are
absolute entry counts, which is what a phase's fixed cost is amortised
over), so graphs larger than the training ones do not push the network past
the range of its inputs along the graph size.

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
    """R-MAT scales 14-22 (uint32 weights 1..255) and square grids with
    sides 1024-2048 (float32 weights), three R-MATs for every grid.  Scales
    21 and 22 are there for the vertex-count input of the first prediction:
    trained on 14-20 alone, it carried the wide widths that win up to scale 20
    (4-8 plain widths, 1.4x) to scale 22, where 2 plain widths is best."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        if i % 4 == 3:
            side = int(rng.integers(1024, 2049))
            specs.append({"kind": "grid", "side": side, "seed": 5000 + i})
        else:
            specs.append({"kind": "rmat", "scale": int(rng.integers(14, 23)), "seed": 1000 + i})
    return specs


def make_graph(spec: dict) -> gb.HostGraph:
    if spec["kind"] == "grid":
        return gb.gen_grid(spec["side"], spec["side"], spec["seed"], "f32")
    return gb.gen_rmat(spec["scale"], 16, spec["seed"])


SWEEP_K = tuple(range(-2, 9))     # log2(width / plain width) of the delta sweep
HORIZON = 8.0                     # label window, in plain widths


def bucket_curve(trace: list[dict], width: float) -> np.ndarray:
    """(distance start, distance end, time start, time end) of every bucket a
    fixed-width run processed, from its phase trace (a bucket's time runs from
    the end of the phase before its first scan to the end of its last phase,
    so the pending re-bucketing before a bucket counts towards it)."""
    starts = [i for i, r in enumerate(trace) if r["kind"] == "scan_bucket"]
    out = []
    for j, i in enumerate(starts):
        t0 = trace[i - 1]["end_ns"] if i > 0 else 0
        last = (starts[j + 1] if j + 1 < len(starts) else len(trace)) - 1
        b = trace[i]["bucket"]
        out.append((b * width, (b + 1) * width, t0, trace[last]["end_ns"]))
    return np.array(out, dtype=np.float64).reshape(-1, 4)


def time_at(curve: np.ndarray, dist: np.ndarray, settled=None) -> np.ndarray:
    """Time at which a run had finished every distance below dist, flat over
    distances no bucket held.  Inside a bucket the time is spread over the
    vertices it settles: settled(D) counts the vertices whose final distance
    is below D (the same for every schedule), so a wide bucket is charged in
    a window in proportion to the vertices that window holds, not to its
    width (uniform spreading when settled is None)."""
    d0, d1, t0, t1 = curve.T
    i = np.searchsorted(d0, dist, side="right") - 1
    out = np.zeros(len(dist))
    ok = i >= 0
    ii = np.clip(i, 0, None)
    inside = ok & (dist < d1[ii])
    if settled is None:
        frac = np.clip((dist - d0[ii]) / np.maximum(d1[ii] - d0[ii], 1e-30), 0.0, 1.0)
    else:
        lo, hi = settled(d0[ii]), settled(d1[ii])
        frac = np.clip((settled(dist) - lo) / np.maximum(hi - lo, 1.0), 0.0, 1.0)
    out[ok] = t1[ii][ok]
    out[inside] = (t0[ii] + (t1[ii] - t0[ii]) * frac)[inside]
    return out


def initial_input(n: int, gfeat) -> np.ndarray:
    """The controller input the host predicts the run's base width from,
    before bucket 0 (the source alone in the window): the window entries
    input (6) carries log2(1 + n), the vertices the run will settle, so the
    base width can follow the graph's size; the kernel's own inputs at later
    bucket starts grow with no size by themselves."""
    x = np.zeros(gb.N_FEAT, np.float32)
    x[0:6] = 1.0
    x[6] = math.log2(1.0 + n)
    x[12:15] = gfeat
    return x


def collect_graph(spec: dict, sweep_k=SWEEP_K, horizon: float = HORIZON, cap: int = 3000, seed: int = 0) -> dict:
    """Per-bucket labels from a delta sweep of the plain method on one graph.

    Every width d * 2^k (k in sweep_k, d the plain width) runs with and
    without the light/heavy split, recording the phase trace and the
    controller inputs at every bucket start.  Each run gives a curve of time
    against the distance settled.  A recorded bucket start at distance D gets
    as label the (k, split) whose run covered [D, D + horizon * d) fastest:
    the width that pays best from that point of the run on, not one width for
    the whole graph.  Samples weigh by the time that window costs at its best
    width, so the expensive stretches of a run count most; a graph's samples
    weigh 1 in all."""
    host = make_graph(spec)
    src = 0 if spec["kind"] == "grid" else int(gb.sample_sources(host, 1, spec["seed"])[0])
    runs = {}
    with gb.Graph.from_host(host) as g:
        d = g.info()["default_delta"]
        fin, _, _ = g.sssp(src, want_pred=False)
        fin = fin[fin != np.uint32(0xFFFFFFFF)] if fin.dtype == np.uint32 else fin[np.isfinite(fin)]
        fin = np.sort(fin.astype(np.float64))
        settled = lambda dd: np.searchsorted(fin, dd, side="left").astype(np.float64)
        g.sssp_device(src)
        # split 1: the light/heavy split at the width in every bucket above
        # max(1024, n / 16) entries (the fixed schedule's split rule)
        split_items = max(1024, host.n // 16)
        for k in sweep_k:
            for split in (0, 1):
                kw = dict(light=None, full_items=split_items) if split else dict(light=math.inf)
                g.sssp_device(src, delta=d * 2.0 ** k, **kw)          # warm-up
                st = g.sssp_device(src, delta=d * 2.0 ** k, flags=gb.F_TRACE | gb.F_FEATURES, **kw)
                tr = g.trace()
                x = g.features()
                runs[(k, split)] = (bucket_curve(tr, st["delta_used"]), x, st["kernel_ms"])
    keys = list(runs)
    xs, labels, costs = [], [], []
    for key in keys:
        curve, x, _ = runs[key]
        # feature row j belongs to the bucket start j + 1 (bucket 0's width is
        # the host's first prediction, made before the run)
        if len(x) != len(curve) - 1 or not len(x):
            continue
        dist = curve[1:, 0]
        h = horizon * d
        c = np.stack([time_at(runs[q][0], dist + h, settled) - time_at(runs[q][0], dist, settled) for q in keys])
        best = np.argmin(c, axis=0)
        xs.append(x)
        labels.append(np.array([[keys[b][0], keys[b][1]] for b in best], dtype=np.float32))
        costs.append(c[best, np.arange(len(best))])
    if not xs:
        return {"spec": spec, "x": np.zeros((0, gb.N_FEAT), np.float32), "t": np.zeros((0, 2), np.float32),
                "w": np.zeros(0, np.float32), "best_fixed": None}
    x = np.concatenate(xs)
    t = np.concatenate(labels)
    w = np.concatenate(costs) + 1e-3
    if len(x) > cap:
        keep = np.random.default_rng(seed).choice(len(x), cap, replace=False)
        x, t, w = x[keep], t[keep], w[keep]
    total = {q: runs[q][2] for q in keys}
    best_fixed = min(total, key=total.get)
    # the initial state, labelled with the graph's best fixed schedule: the
    # base width the host derives from it bounds every later bucket's
    # width to 1/8 .. 8x of that prediction; it weighs as much as all the
    # graph's bucket starts together
    avg = host.m / max(host.n, 1)
    wmax = float(host.w.max()) if host.m else 1.0
    gfeat = [math.log2(max(avg, 1e-3)), math.log2(max(wmax, 1e-30)),
             float(host.w.astype(np.float64).mean() / wmax) if host.m else 0.0]
    x0 = initial_input(host.n, gfeat)[None, :]
    x = np.concatenate([x0, x])
    t = np.concatenate([np.array([[best_fixed[0], best_fixed[1]]], np.float32), t])
    w = np.concatenate([[1.0], w / w.sum()])
    return {"spec": spec, "x": x.astype(np.float32), "t": t, "w": (w / w.sum()).astype(np.float32),
            "best_fixed": {"k": best_fixed[0], "split": best_fixed[1], "ms": total[best_fixed],
                           "plain_ms": total[(0, 0)]}}


def dataset(collected: list[dict]):
    """(inputs, targets, weights); every graph's samples weigh 1 in all."""
    xs = [c["x"] for c in collected if len(c["x"])]
    ts = [c["t"] for c in collected if len(c["x"])]
    ws = [c["w"] for c in collected if len(c["x"])]
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
        c = collect_graph(s, seed=i)
        collected.append(c)
        print(json.dumps({"i": i, **s, "samples": len(c["x"]), "best_fixed": c["best_fixed"],
                          "label_k_mean": round(float(np.average(c["t"][:, 0], weights=c["w"])), 2)
                          if len(c["x"]) else None}), flush=True)
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
               "per_graph": [{**c["spec"], "samples": int(len(c["x"])), "best_fixed": c["best_fixed"]}
                             for c in collected]}
    if args.summary:
        Path(args.summary).write_text(json.dumps(summary, indent=1))
    print(json.dumps({k: v for k, v in summary.items() if k != "per_graph"}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
