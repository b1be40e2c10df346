"""Independent systems spread over ranks (parm_gb300.shard), on the CPU.

The split balances the work estimate N_s * (1 + neighbours per atom) with the
greedy longest-processing-time rule; every system lands on exactly one rank;
the per-system results gathered over two gloo ranks equal a one-rank run of
the whole batch (the per-system computation here is the oracle's damped
minimisation, standing in for the GPU handle of each rank).
"""
import os
import socket

import numpy as np
import pytest

from parm_gb300 import shard, workloads as W

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def test_partition_covers_and_balances():
    w = W.packings(nsys=4096, nmin=64, nmax=4096, seed=3)
    wt = shard.system_weights(w.sizes, w.L, 1.4 + w.skin)
    for nr in (1, 2, 4, 8):
        parts = shard.partition(wt, nr)
        allsys = sorted(s for p in parts for s in p)
        assert allsys == list(range(4096))
        assert shard.imbalance(wt, parts) < 1.002, nr
    # a few heavy systems: the heaviest sits alone, the rest fill the others
    parts = shard.partition([10.0, 1.0, 1.0, 1.0, 1.0], 2)
    assert parts == [[0], [1, 2, 3, 4]]


def test_select_keeps_system_order():
    w = W.packings(nsys=6, nmin=10, nmax=30, seed=5)
    sub = shard.select(w, [4, 1])
    off = np.concatenate([[0], np.cumsum(w.sizes)])
    assert sub.sizes == [w.sizes[4], w.sizes[1]]
    np.testing.assert_array_equal(sub.x[: w.sizes[4]], w.x[off[4]:off[5]])
    np.testing.assert_array_equal(sub.L[1], w.L[1])


def _per_system(wl):
    """Per-system energies and box-relative final position sums after 30 damped oracle steps."""
    from oracle.oracle import Oracle
    E, X = [], []
    off = np.concatenate([[0], np.cumsum(wl.sizes)]).astype(int)
    for s in range(len(wl.sizes)):
        sl = slice(off[s], off[s + 1])
        o = Oracle(wl.sizes[s], 3)
        o.set_box(wl.L[s])
        o.set_state(x=wl.x[sl], v=wl.v[sl], m=wl.m[sl])
        o.set_interaction(wl.kind, wl.params[sl], wl.skin)
        o.initialize()
        o.damped(0.01, 1.0, 30)
        E.append(o.energy())
        X.append(o.get_state()["x"].sum(0))
    return {"E": np.array(E), "X": np.array(X)}


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    from parm_gb300 import shard as S, workloads as WW
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = WW.packings(nsys=9, nmin=20, nmax=120, phi_lo=0.5, phi_hi=0.6, seed=8)
    parts = S.partition(S.system_weights(w.sizes, w.L, 1.4 + w.skin), world)
    mine = parts[rank]
    local = _per_system(S.select(w, mine))
    res = S.gather_results(local, mine, len(w.sizes), dist)
    if rank == 0:
        out["E"] = res["E"].tolist()
        out["X"] = res["X"].tolist()
        out["parts"] = parts
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_equals_one_rank():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    w = W.packings(nsys=9, nmin=20, nmax=120, phi_lo=0.5, phi_hi=0.6, seed=8)
    ref = _per_system(w)
    assert all(len(p) > 0 for p in res["parts"])
    np.testing.assert_array_equal(np.array(res["E"]), ref["E"])
    np.testing.assert_array_equal(np.array(res["X"]), ref["X"])
