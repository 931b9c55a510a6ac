"""bench.py's multi-rank path on the CPU: two gloo ranks (one replica each) agree on the
job time (maximum over ranks) and the whole-job value; the reference arm runs on rank 0
only."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    sys.path.insert(0, REPO)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.job_time_ms(100.0 + 50.0 * rank, dist)
    out[rank] = (ms, bench.job_value(1000, 5, ms, world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_agree_on_job_time_and_value():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    assert out[0] == out[1]
    ms, value = out[0]
    assert ms == 150.0
    assert value == pytest.approx(2 * 1000 * 5 / 0.150)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, REPO)
    import bench
    args = type("A", (), dict(n=16, gpus=2, steps=1, warmup=0))()
    bench.run_reference(args, rank=1, world=2)
    assert capsys.readouterr().out == ""
