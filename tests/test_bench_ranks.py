"""The multi-process side of bench.py on CPU: the max-over-ranks timing with
two gloo ranks, and the reference arm under torchrun with two ranks (rank 0
prints the one JSON line, the other rank exits without work)."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local = [2.0, 3.5][rank]                      # each rank's total seconds
    slowest = bench.max_over_ranks(local, dist, "cpu")
    out.put((rank, slowest, bench.job_rate(world, 1000, 4, slowest)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    # every rank sees the slowest rank's time; the rate counts both ranks' keys
    assert [r[1] for r in res] == [3.5, 3.5]
    assert res[0][2] == pytest.approx(2 * 1000 * 4 / 3.5)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(1.25, None, "cpu") == 1.25
    assert bench.job_rate(1, 10, 2, 4.0) == 5.0


def test_reference_arm_under_torchrun(oracle_mod):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--keys", "200000"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
