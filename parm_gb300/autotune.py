"""Autotuner of a batched workload's run parameters: neighbour-list skin, cell
width and pair-kernel variant.

The skin trades list rebuilds against pairs per atom, the cell width trades
candidates per rebuild against cells, and the kernel variant (threads per
atom, shared-memory staging) depends on density and system sizes; none of
them changes results beyond rounding.  `tune` builds a probe of the workload
(its first systems, up to a number of atoms), and for every (skin, cell scale)
pair lets the library pick its kernel variant (parm_autotune) and times the
workload's own steps with synchronised wall clocks after a warm-up; the
fastest combination is returned with the whole table.
"""
from __future__ import annotations

import time
from dataclasses import replace
from typing import Callable, Sequence

from . import shard


def probe_systems(sizes: Sequence[int], max_atoms: int, max_systems: int = 256) -> list[int]:
    """The first systems of a batch, up to `max_atoms` atoms and `max_systems` systems."""
    out, tot = [], 0
    for s, n in enumerate(sizes):
        if out and (tot + n > max_atoms or len(out) >= max_systems):
            break
        out.append(s)
        tot += int(n)
    return out


def tune(workload, make: Callable, step: Callable, skins: Sequence[float], cell_scales: Sequence[float] = (1.0,),
         prepare: Callable | None = None, steps: int = 200, warm: int = 50, max_atoms: int = 400_000) -> dict:
    """Time `step(handle, steps)` on a probe of `workload` for each skin and cell scale.

    make(workload) returns a handle with the workload's atoms and interaction
    (its list skin is the workload's); prepare(handle), when given, sets up
    the integrator after the kernel variant is chosen; step(handle, n) runs n
    steps of the workload's integrator.  Returns {"skin", "cell_scale",
    "variant", "seconds_per_step", "table", ...}.
    """
    probe = shard.select(workload, probe_systems(workload.sizes, max_atoms))
    table = []
    for skin in skins:
        for cs in cell_scales:
            g = make(replace(probe, skin=float(skin)))
            g.set_cell_scale(cs)
            variant = g.autotune() if g.precision == "mixed" else 0
            if prepare is not None:
                prepare(g)
            step(g, warm)
            g.sync()
            t0 = time.perf_counter()
            step(g, steps)
            g.sync()
            dt = (time.perf_counter() - t0) / steps
            table.append({"skin": float(skin), "cell_scale": float(cs), "variant": int(variant),
                          "seconds_per_step": dt, "probe_atoms": probe.n, "probe_systems": len(probe.sizes)})
            g.close()
    best = min(table, key=lambda r: r["seconds_per_step"])
    return {**best, "table": table}


def summarise(result: dict) -> dict:
    """The chosen values and the per-combination step times (microseconds), for a JSON line."""
    return {"skin": result["skin"], "cell_scale": result["cell_scale"], "kernel_variant": result["variant"],
            "probe_atoms": result["probe_atoms"], "probe_systems": result["probe_systems"],
            "us_per_step": {f"skin={r['skin']:g},cell={r['cell_scale']:g}": round(1e6 * r["seconds_per_step"], 1)
                            for r in result["table"]}}
