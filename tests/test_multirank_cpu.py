"""The benchmark's multi-rank bookkeeping over torch.distributed (gloo, CPU).

Under torchrun every rank advances its own replica of the system (the time
step has no data-parallel split); the job time is the slowest rank's and the
job throughput counts every rank's atoms.  Two gloo ranks on 127.0.0.1.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
    ms_max = bench.max_over_ranks(ms, dist, "cpu")
    out[rank] = (ms_max, bench.job_throughput(1000, 10, ms_max, world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 150.0
    assert res[0][1] == pytest.approx(2 * 1000 * 10 / 0.150)


def test_single_rank_is_identity():
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_throughput(10, 4, 2.0, 1) == pytest.approx(20000.0)
