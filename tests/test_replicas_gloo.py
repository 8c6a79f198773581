"""The N > 1 path of bench.py on the CPU: ranks over gloo on 127.0.0.1, the
max-over-ranks timing reduction, and the reference arm launched by torchrun with
two ranks (rank 0 alone runs and prints its one JSON line; the other exits 0)."""
import json
import os
import socket
import subprocess
import sys

import pytest

import conftest


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, conftest.REPO)
    import bench
    r, world, local, dist = bench.dist_setup(2)
    bench.barrier(dist)
    q.put((r, world, bench.max_over_ranks(dist, float(10 * (r + 1)))))
    bench.barrier(dist)
    dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=180) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 20.0), (1, 2, 20.0)]


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch")
    subprocess.run(["make", "-s", "-C", os.path.join(conftest.REPO, "oracle")], check=True)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(conftest.REPO, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=conftest.REPO)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
