"""The N-GPU bench path is replicas only: every rank solves its own volumes
and the ranks meet only in a barrier and a max-over-ranks of the timer.
Run here as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    got_ws, got_rank, local = bench.dist_init()
    bench.barrier(got_ws)
    m = bench.max_over_ranks(1.5 + rank, got_ws)     # per-rank timer, max taken
    # The reference arm runs on rank 0 only; other ranks leave without work.
    class A:
        steps = 1
        warmup = 0
        gpus = ws
    out = "skipped" if rank != 0 else "rank0"
    if rank != 0:
        bench.run_reference(A(), got_ws, got_rank)
    bench.barrier(got_ws)
    dist.destroy_process_group()
    q.put((rank, got_ws, local, m, out))


def test_two_gloo_ranks_barrier_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    assert all(r[1] == 2 for r in res)
    assert all(r[3] == 2.5 for r in res)     # both ranks see the slowest rank's time


def test_bench_starts_its_own_replicas():
    """`bench.py --gpus 2` without torchrun starts two ranks itself; they meet
    in the barrier and the max over ranks, and rank 0 alone prints."""
    import json
    import subprocess
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--replica-check"],
                         capture_output=True, text=True, timeout=300, env=env)
    assert out.returncode == 0, out.stderr
    lines = [json.loads(ln) for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert lines == [{"replica_check": True, "world_size": 2, "max_over_ranks": 2.5}]
