"""The multi-GPU form is replicas only: one process per GPU, no exchange
within a pattern. Its host side runs here as two gloo ranks on the CPU: the
whole-job time is the max over ranks, and the reference arm's non-zero
ranks exit at once without work."""
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


def _rank(rank, ws, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, ROOT)
    import bench
    got = bench.job_times([1.0 + rank, 10.0 - rank, 0.5 * rank], ws)
    dist.destroy_process_group()
    q.put((rank, got))


def test_job_time_is_the_max_over_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0] == out[1] == [2.0, 10.0, 0.5]


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_times([3.0, 4.0], 1) == [3.0, 4.0]


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"),
                        "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
