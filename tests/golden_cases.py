"""Loading and replaying the golden fixtures produced by the reference itself.

Each ``tests/golden/<case>.npz`` holds an input deck (box, atoms, pair
parameters, insertion order, exclusions, integrator and step counts) and the
reference's outputs for it: the neighbour pair list after ``update_list(true)``,
forces, accelerations, energy, pressure, stress, contacts and overlaps after
``Collection::initialize`` (src/collection.cpp:13-19), and positions,
velocities, accelerations, forces, energy, kinetic energy and the list's
``which()`` counter at the recorded steps.  The conjugate-gradient cases
(CollectionNLCG / CollectionNLCGV) add their parameter vector ``cg`` and, per
recorded step, the box (``box_steps``) and the minimiser's state
(``cg_state_steps``: Knew, k, vl, fl, al, alpha, beta, betaused, dxsum,
alphavmax, sec).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
VERLET, DAMPED, SOL, NLCG, NLCGV = 0, 1, 2, 3, 4


def names() -> list[str]:
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        d = {k: z[k] for k in z.files}
    d["name"] = name
    d["ndim"] = int(d["L"].shape[0])
    d["n"] = int(d["m"].shape[0])
    for k in ("kind", "integ", "nsteps"):
        d[k] = int(d[k])
    for k in ("dt", "damping", "T", "skin"):
        d[k] = float(d[k])
    return d


def pair_set(pairs: np.ndarray) -> set:
    return {(int(a), int(b)) if a < b else (int(b), int(a)) for a, b in pairs}
