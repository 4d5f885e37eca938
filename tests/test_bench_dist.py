"""The multi-rank contract of bench.py on CPU (gloo, world size 2): process
group set-up, barrier and max over ranks, and the reference arm under
torchrun printing one line from rank 0 only."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
torch = pytest.importorskip("torch")


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(REPO))
    import bench
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    out.put((r, bench.allmax(w, 10.0 + r)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_dist_setup_barrier_and_max_over_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 11.0), (1, 11.0)]


def test_reference_arm_under_torchrun_prints_one_line():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(REPO / "bench.py"),
           "--impl", "reference", "--config", "channel-128x64x64", "--steps", "1", "--warmup", "3", "--cpu-budget", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=REPO, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2


def test_reference_arm_loads_only_the_oracle():
    """The reference arm times the oracle alone: the product library is never
    mapped into that process, and it prints the GPU arm's metric and unit."""
    script = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3', '--cpu-budget', '1']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('MAPPED', 'liblbm_gb300' in maps, 'liblbm_oracle' in maps)\n")
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, timeout=300, cwd=REPO, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    assert "MAPPED False True" in p.stdout
    d = json.loads(next(ln for ln in p.stdout.splitlines() if ln.startswith("{")))
    sys.path.insert(0, str(REPO))
    import bench
    assert d["metric"] == bench.METRIC and d["unit"] == "GLUPS" and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and "fluid nodes" in d["cpu_baseline"]["sample"]
