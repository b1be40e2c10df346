"""Independent systems spread over GPUs (one process per GPU).

A batch of independent systems (packings, Langevin replicas) has no exchange
between systems, so N GPUs run disjoint subsets with no collective in the
data path.  The work of a system is about proportional to its atoms times its
neighbours per atom (N_s * rho_s * list volume), so systems are assigned by a
greedy longest-processing-time rule on that weight: heaviest first, each to
the currently lightest rank.  Results are per system; `gather_results` brings
them back to rank 0 in the batch's original order (one host-side gather at
the end, over torch.distributed's object collectives).
"""
from __future__ import annotations

from typing import Sequence

import numpy as np


def system_weights(sizes: Sequence[int], boxes: np.ndarray, list_radius: float, ndim: int = 3) -> np.ndarray:
    """Work estimate per system: N_s times the expected neighbours per atom within the list radius."""
    sizes = np.asarray(sizes, dtype=np.float64)
    boxes = np.asarray(boxes, dtype=np.float64).reshape(len(sizes), -1)
    vol = np.prod(boxes[:, :ndim], axis=1)
    ball = (4.0 / 3.0) * np.pi * list_radius ** 3 if ndim == 3 else np.pi * list_radius ** 2
    return sizes * (1.0 + sizes / vol * ball)


def partition(weights: Sequence[float], nranks: int) -> list[list[int]]:
    """Greedy balanced split: systems in decreasing weight, each to the lightest rank so far.
    Returns, per rank, its systems in increasing index order."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    w = np.asarray(weights, dtype=np.float64)
    order = sorted(range(len(w)), key=lambda i: (-w[i], i))
    load = np.zeros(nranks)
    parts: list[list[int]] = [[] for _ in range(nranks)]
    for i in order:
        r = int(np.argmin(load))
        parts[r].append(i)
        load[r] += w[i]
    return [sorted(p) for p in parts]


def imbalance(weights: Sequence[float], parts: list[list[int]]) -> float:
    """Largest rank load over the mean rank load (1.0 is a perfect split)."""
    w = np.asarray(weights, dtype=np.float64)
    loads = np.array([w[p].sum() for p in parts])
    return float(loads.max() / loads.mean()) if loads.mean() > 0 else 1.0


def select(workload, systems: Sequence[int]):
    """The sub-workload holding `systems` (in that order) of a batched workload."""
    from .workloads import Workload
    off = np.concatenate([[0], np.cumsum(workload.sizes)]).astype(np.int64)
    idx = np.concatenate([np.arange(off[s], off[s + 1]) for s in systems]) if len(systems) else np.zeros(0, int)
    return Workload(workload.name, workload.ndim, [workload.sizes[s] for s in systems], workload.L[list(systems)],
                    workload.x[idx], workload.v[idx], workload.m[idx], workload.kind, workload.params[idx],
                    workload.skin, dict(workload.extra))


def gather_results(local: dict, systems: Sequence[int], nsys: int, dist=None):
    """Per-system results of every rank in batch order on rank 0 (None elsewhere).

    `local` maps a name to an array whose first axis runs over this rank's
    `systems`.  With no process group (one rank) the arrays are returned as
    they are."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return {k: np.asarray(v) for k, v in local.items()}
    payload = (list(systems), {k: np.asarray(v) for k, v in local.items()})
    world = dist.get_world_size()
    got = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(payload, got, dst=0)
    if dist.get_rank() != 0:
        return None
    out = {}
    for k in local:
        first = next(p[1][k] for p in got if len(p[0]))
        arr = np.zeros((nsys,) + first.shape[1:], dtype=first.dtype)
        for sysl, vals in got:
            if len(sysl):
                arr[np.asarray(sysl)] = vals[k]
        out[k] = arr
    return out
