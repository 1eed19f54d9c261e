"""Replicas under torch.distributed on CPU (gloo, world size 2): the bench's whole-job aggregation
(slowest rank's time, all ranks' rays) and the reference arm's rank discipline."""
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


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, ROOT)
        import bench

        ms, rays = bench.aggregate_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1), "cpu")
        q.put((rank, ms, rays))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_aggregate_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 15.0, 3000.0), (1, 15.0, 3000.0)]


def test_aggregate_single_process_is_identity():
    pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench

    assert bench.aggregate_ranks(7.5, 123, "cpu") == (7.5, 123)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
