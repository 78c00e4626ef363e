"""The bench's multi-rank plumbing on CPU with the gloo backend (world size
2, rendezvous on 127.0.0.1): the max over ranks of the per-rank times, the
barrier, and the reference arm under torchrun, where rank 0 alone prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": "2",
                       "RANK": str(rank), "LOCAL_RANK": str(rank), "FCC_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    ws, r, _ = bench.dist_setup()
    m = bench.dist_max(10.0 * (rank + 1), ws)
    bench.barrier(ws)
    out.put((r, ws, m))
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 20.0), (1, 2, 20.0)]


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, FCC_BACKEND="gloo")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3",
           "--nnz", "200000"]
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
