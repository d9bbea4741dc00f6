"""Several GPUs: replicas only.  The path does not shard (one SSSP is one
graph on one device), so ``bench.py --gpus N`` runs one independent replica
per rank and only its timings cross ranks: a barrier around the timed region
and a max / sum over ranks, on a gloo process group.  These tests run that
host path here on the CPU with two ranks, and the reference arm under
torchrun, where rank 0 alone measures and prints."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    world, r, _ = bench.dist_env()
    dist = bench.init_group(world, r)
    bench.barrier(dist)
    q.put((r, bench.allreduce_max(dist, 1.5 + r), bench.allreduce_sum(dist, 1.5 + r)))
    bench.barrier(dist)
    dist.destroy_process_group()


def test_gloo_two_ranks_barrier_and_reductions():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    assert out == [(0, 2.5, 4.0), (1, 2.5, 4.0)]


def test_single_rank_needs_no_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.init_group(1, 0) is None
    assert bench.allreduce_max(None, 3.0) == 3.0 and bench.allreduce_sum(None, 3.0) == 3.0


def test_reference_arm_under_torchrun_prints_once():
    """torchrun with two ranks: rank 0 times the reference's CPU path and
    prints the one JSON line, rank 1 exits without work."""
    pytest.importorskip("torch")
    import oracle
    if not oracle.ref_available("serial"):
        pytest.skip("the reference's own SSSP is not built here")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--steps", "1", "--warmup", "0", "--ref-scale", "10", "--ref-procs", "2", "--ref-budget-s", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "reference"
