"""bench.py's multi-rank aggregation (replicas, max-over-ranks time) with
world_size 2 on the gloo backend, CPU only."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    value, ms = bench.combine_ranks(world, 1000, 10, 100.0 + 50.0 * rank, dist, device="cpu")
    out.put((rank, value, ms))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms in res:
        assert ms == 150.0
        assert abs(value - 2 * 1000 * 10 / 0.150 / 1e6) < 1e-12


def test_single_rank_value():
    sys.path.insert(0, ROOT)
    import bench
    v, ms = bench.combine_ranks(1, 4194304, 50, 500.0)
    assert ms == 500.0 and abs(v - 4194304 * 50 / 0.5 / 1e6) < 1e-9


def test_launch_count_per_form():
    """The kernels of one step that bench.py's gpu_launches counts: stage (a) and the flux
    kernel, plus the ghost pass of f-bar-plus in FP64 and in the 16-bit forms with periodic x."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.launches_per_step("fp64", periodic_x=False) == 3
    assert bench.launches_per_step("fp32", periodic_x=False) == 2
    assert bench.launches_per_step("fp16", periodic_x=False) == 2
    assert bench.launches_per_step("bf16", periodic_x=True) == 3
