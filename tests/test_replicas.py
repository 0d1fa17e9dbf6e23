"""The multi-process side of bench.py on CPU (gloo, world size 2).

The path does not shard: under torchrun every rank runs an independent
replica, the timed region is bracketed by barriers and the reported time is
the maximum over ranks; the reference arm runs on rank 0 alone and the other
ranks exit without work.  These run here without a GPU.
"""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out: str) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    w, r, _, dist = bench.dist_setup()
    bench.barrier(dist)
    m = bench.dist_max(dist, 1.5 + r)   # each rank's "time"; the line reports the slowest
    with open(f"{out}.{r}", "w") as f:
        json.dump({"world": w, "rank": r, "max": m}, f)
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    out = str(tmp_path / "rank")
    mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
    for r in range(2):
        with open(f"{out}.{r}") as f:
            d = json.load(f)
        assert d == {"world": 2, "rank": r, "max": 2.5}
    assert torch is not None


def test_reference_arm_under_torchrun_prints_one_line():
    pytest.importorskip("torch")
    from oracle.pyoracle import build
    build(ref=False)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT,
                       env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "node-evals/s"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port", "reference")
