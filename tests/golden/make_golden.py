"""Generate the golden fixtures in this folder from the reference itself.

The reference's own sources (vecrand.cpp, box.cpp, trackers.cpp,
collection.cpp and the headers they include) are compiled where they lie by
``oracle/refbuild/Makefile`` against a restatement of the Eigen/Boost subset
they use (``oracle/refbuild/shim``), together with ``ref_driver.cpp``, which
drives ``OriginBox``, ``AtomVec``, ``NListed<A,P>``, ``NeighborList`` and
``CollectionVerlet`` / ``CollectionDamped`` / ``CollectionSol`` exactly as a
reference program does.  Each case below is a seeded input deck; the driver's
output (pair list, initial forces, energies, stresses, trajectories) is
stored with the deck in ``<case>.npz``.

Run from the repository root (needs the reference sources)::

    python tests/golden/make_golden.py [--ref-src /path/to/parm/src]

Positions and velocities come from numpy's seeded generators, so the decks
are reproducible; the reference's own random streams (Boost.Random) are not
used: Langevin cases run at T = 0, where the noise term vanishes.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REFBUILD = ROOT / "oracle" / "refbuild"
REFOUT = ROOT / "oracle" / "_ref"

VERLET, DAMPED, SOL, NLCG, NLCGV = 0, 1, 2, 3, 4
LJCUT, REPULSION, LJREPULSE, LJATTRACT = 0, 1, 2, 3
LOISOHERN, LOISOHERN_MIN, LOISLIN, LOISLIN_MIN, EISMCLACHLAN, REPULSIONDRAG = 4, 5, 6, 7, 8, 9
LJCUT_IEPSISIG, LJATTRACT_IEPSISIG, LJATTRACT_IEPS, LJATTRACTREPULSE, LJATTRACTFIXEDREPULSE, LJISH = range(10, 16)
REPULSION_IEPSISIG = 16
LJATTRACTREPULSESIGS = 17
SIG_PRIME = 2.0 ** (-1.0 / 6.0)


def _deck(c: dict) -> str:
    nd = c["L"].shape[0]
    lees = "le_gamma" in c   # a LeesEdwardsBox: kind + 100 and the shear after the box
    out = [f"{c['kind'] + (100 if lees else 0)} {c['integ']} {c['nsteps']} {c['dt']!r} {c['damping']!r} "
           f"{c['T']!r} {c['skin']!r}",
           " ".join(repr(float(q)) for q in c["L"]) + (f" {float(c['le_gamma'])!r}" if lees else ""),
           str(len(c["m"]))]
    for i in range(len(c["m"])):
        prm = c["deck_params"][i] if "deck_params" in c else c["params"][i]
        vals = list(c["x"][i]) + list(c["v"][i]) + [c["m"][i]] + list(prm)
        out.append(" ".join(repr(float(q)) for q in vals))
    if "pair_eps" in c:   # the indexed kinds' tables
        nt = c["pair_eps"].shape[0]
        out.append(f"{nt} " + " ".join(repr(float(q)) for q in c["pair_eps"].reshape(-1)) + " "
                   + " ".join(repr(float(q)) for q in c["pair_sig"].reshape(-1)))
    out.append(f"{len(c['order'])} " + " ".join(str(int(q)) for q in c["order"]))
    ig = c["ignores"].reshape(-1)
    out.append(f"{len(ig) // 2} " + " ".join(str(int(q)) for q in ig))
    out.append(f"{len(c['out_steps'])} " + " ".join(str(int(q)) for q in c["out_steps"]))
    if c["integ"] >= NLCG:
        out.append(" ".join(repr(float(q)) for q in c["cg"]))
    assert nd in (2, 3)
    return "\n".join(out) + "\n"


def _parse(text: str, n: int, nd: int) -> dict:
    lines = text.splitlines()
    pos = 0

    def nxt():
        nonlocal pos
        pos += 1
        return lines[pos - 1].split()

    h = nxt()
    assert h[0] == "PAIRS"
    k = int(h[1])
    pairs = np.array([[int(t) for t in nxt()] for _ in range(k)], dtype=np.uint32).reshape(k, 2)
    h = nxt()
    assert h[0] == "INIT"
    init = np.array([float(h[1]), float(h[2])])
    counts = np.array([int(h[3]), int(h[4]), int(h[5])], dtype=np.int64)
    stress = np.array([float(t) for t in nxt()]).reshape(nd, nd)
    fa = np.array([[float(t) for t in nxt()] for _ in range(n)]).reshape(n, 2 * nd)
    steps, which, energy, ke, st, cgl = [], [], [], [], [], []
    while pos < len(lines):
        h = nxt()
        assert h[0] == "STEP"
        steps.append(int(h[1]))
        which.append(int(h[2]))
        energy.append(float(h[3]))
        ke.append(float(h[4]))
        if pos < len(lines) and lines[pos].startswith("NLCG"):
            cgl.append([float(t) for t in nxt()[1:]])
        st.append(np.array([[float(t) for t in nxt()] for _ in range(n)]).reshape(n, 4 * nd))
    st = np.array(st).reshape(len(steps), n, 4 * nd)
    extra = {}
    if cgl:
        cg = np.array(cgl)
        extra = {"box_steps": cg[:, :nd], "cg_state_steps": cg[:, nd:]}
    return {**extra, "pairs": pairs, "init": init, "init_counts": counts, "stress": stress,
            "f0": fa[:, :nd], "a0": fa[:, nd:], "steps": np.array(steps, dtype=np.int64),
            "which_steps": np.array(which, dtype=np.int64), "energy_steps": np.array(energy),
            "ke_steps": np.array(ke), "x_steps": st[:, :, 0:nd], "v_steps": st[:, :, nd:2 * nd],
            "a_steps": st[:, :, 2 * nd:3 * nd], "f_steps": st[:, :, 3 * nd:4 * nd]}


def _case(name, kind, integ, nsteps, dt, L, x, v, m, params, skin, out_steps, damping=0.0, T=0.0,
          order=None, ignores=None, cg=None, deck_params=None, pair_eps=None, pair_sig=None, le_gamma=None):
    """deck_params: the atoms' constructor arguments when they differ from the stored fields
    (LoisLinAtom takes depth and width and stores f = depth / width and l = width)."""
    n = len(m)
    extra = {} if cg is None else {"cg": np.asarray(cg, dtype=np.float64)}
    if deck_params is not None:
        extra["deck_params"] = np.asarray(deck_params, dtype=np.float64).reshape(n, -1)
    if le_gamma is not None:
        extra["le_gamma"] = np.float64(le_gamma)
    if pair_eps is not None:
        extra["pair_eps"] = np.asarray(pair_eps, dtype=np.float64)
        extra["pair_sig"] = (np.asarray(pair_sig, dtype=np.float64) if pair_sig is not None
                             else np.zeros_like(extra["pair_eps"]))
    return {**extra, "name": name, "kind": kind, "integ": integ, "nsteps": nsteps, "dt": float(dt),
            "damping": float(damping), "T": float(T), "skin": float(skin),
            "L": np.asarray(L, dtype=np.float64), "x": np.asarray(x, dtype=np.float64),
            "v": np.asarray(v, dtype=np.float64), "m": np.asarray(m, dtype=np.float64),
            "params": np.asarray(params, dtype=np.float64).reshape(n, -1),
            "order": np.arange(n, dtype=np.int64) if order is None else np.asarray(order, dtype=np.int64),
            "ignores": np.zeros((0, 2), np.int64) if ignores is None else np.asarray(ignores, np.int64),
            "out_steps": np.asarray(out_steps, dtype=np.int64)}


def lj_lattice_deck(shape, seed, T=1.0):
    """Config-0 style: simple-cubic lattice at rho' = 0.8, +-0.05 sigma' jitter."""
    rng = np.random.default_rng(seed)
    rho = 0.8 / SIG_PRIME ** 3
    a = (1.0 / rho) ** (1.0 / 3.0)
    g = np.stack(np.meshgrid(*[np.arange(s) for s in shape], indexing="ij"), -1).reshape(-1, len(shape))
    x = (g + 0.5) * a + rng.uniform(-0.05 * SIG_PRIME, 0.05 * SIG_PRIME, size=g.shape)
    v = rng.normal(0.0, np.sqrt(T), size=g.shape)
    v -= v.mean(axis=0)
    L = np.array(shape, dtype=np.float64) * a
    return L, x, v


def cases() -> list[dict]:
    out = []
    cut = 2.5 * SIG_PRIME
    # 1. LJ, 1000 atoms, the plain FP64 configuration: 1000 Verlet steps
    L, x, v = lj_lattice_deck((10, 10, 10), 12345)
    n = len(x)
    out.append(_case("lj1000_verlet", LJCUT, VERLET, 1000, 0.001, L, x, v, np.ones(n),
                     np.tile([1.0, 1.0, cut], (n, 1)), 0.4 * SIG_PRIME, [1, 10, 100, 1000]))
    # 2. the 12-atom Hertzian fixture of pyparm/tests.py (PairedCollectionTest,
    #    RandomHertzianVerletTest): legacy numpy stream seeded 131
    N = 12
    sig = np.array([1.0] * (N // 2) + [1.4] * (N - N // 2))
    Lh = float((np.sum((sig / 2) ** 3) * 4 / 3 * np.pi / 0.3) ** (1 / 3))
    rs = np.random.RandomState(131)
    xs, vs = [], []
    for s in sig:
        xs.append(rs.uniform(0.0, Lh, size=(3,)))
        vs.append(rs.normal(size=(3,)) / s ** 3)
        rs.normal(size=(3,))   # the fixture also draws a force it never uses
    out.append(_case("hertz12_verlet", REPULSION, VERLET, 2000, 0.01, [Lh] * 3, xs, vs, sig ** 3,
                     np.stack([np.full(N, 1.2), sig, np.full(N, 2.0)], 1), 0.4, [1, 10, 100, 1000, 2000]))
    # 3. 3D soft spheres, exponent 2.5, damped minimisation steps
    rng = np.random.default_rng(7)
    n = 200
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Lc = (np.sum(np.pi * sig ** 3 / 6) / 0.64) ** (1 / 3)
    out.append(_case("spheres200_damped", REPULSION, DAMPED, 300, 0.01, [Lc] * 3,
                     rng.uniform(0, Lc, (n, 3)), np.zeros((n, 3)), np.ones(n),
                     np.stack([np.ones(n), sig, np.full(n, 2.5)], 1), 0.1, [1, 10, 100, 300], damping=0.5))
    # 4. 2D harmonic disks at phi = 0.84, damped
    rng = np.random.default_rng(8)
    n = 256
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Ld = np.sqrt(np.sum(np.pi * sig ** 2 / 4) / 0.84)
    out.append(_case("disks256_damped", REPULSION, DAMPED, 300, 0.01, [Ld, Ld],
                     rng.uniform(0, Ld, (n, 2)), np.zeros((n, 2)), np.ones(n),
                     np.stack([np.ones(n), sig, np.full(n, 2.0)], 1), 0.1, [1, 10, 100, 300], damping=1.0))
    # 5. WCA fluid under CollectionSol at T = 0 (the noise term vanishes)
    L, x, v = lj_lattice_deck((6, 6, 6), 99)
    n = len(x)
    out.append(_case("wca216_sol", LJREPULSE, SOL, 300, 0.001, L, x, v, np.ones(n),
                     np.tile([1.0, 1.0, 0.0], (n, 1)), 0.3, [1, 10, 100, 300], damping=1.0))
    # 6. 2D LJ, Verlet
    L, x, v = lj_lattice_deck((20, 20), 5)
    n = len(x)
    L = L * (0.8 / SIG_PRIME ** 3) ** (1 / 3) / (0.8 / SIG_PRIME ** 2) ** (1 / 2)   # rho' = 0.8 in 2D
    x = x * L[0] / (20 * (1.0 / (0.8 / SIG_PRIME ** 3)) ** (1 / 3))
    out.append(_case("lj400_2d_verlet", LJCUT, VERLET, 300, 0.002, L, x, v, np.ones(n),
                     np.tile([1.0, 1.0, cut], (n, 1)), 0.3, [1, 10, 100, 300]))
    # 7. bidisperse LJ with shuffled insertion order, non-member atoms,
    #    exclusions, immobile atoms (mass 0 and inf)
    rng = np.random.default_rng(21)
    L, x, v = lj_lattice_deck((8, 8, 8), 21)
    n = len(x)
    eps = rng.choice([0.8, 1.2], n)
    sg = rng.choice([1.0, 1.2], n)
    order = rng.permutation(n)[: n - 7]
    ign = np.array([[order[0], order[1]], [order[5], order[2]], [3, 4], [10, 11]])
    m = np.ones(n)
    m[order[3]] = 0.0
    m[order[4]] = np.inf
    out.append(_case("ljmix512_order_excl", LJCUT, VERLET, 200, 0.001, L, x, v, m,
                     np.stack([eps, sg, 2.5 * sg], 1), 0.3, [1, 10, 100, 200], order=order, ignores=ign))
    # 8. boundary cases: atoms exactly at +-L/2 and beyond the box, a pair
    #    separated by exactly cut + skin (the list test is a strict '<')
    rng = np.random.default_rng(33)
    n = 64
    Lb = np.array([8.0, 8.0, 8.0])
    x = rng.uniform(-4.0, 4.0, (n, 3))
    x[0] = [4.0, -4.0, 0.5]
    x[1] = [-4.0, 4.0, 26.5]          # unwrapped: 26.5 = 2.5 + 3 L
    x[2] = [1.0, 1.0, 1.0]
    x[3] = [1.0 + 2.5, 1.0, 1.0]      # |x3 - x2| = 2.0 + 0.5 exactly
    x[4] = [-3.0, -3.0, -3.0]
    x[5] = [-3.0, -3.0, -3.0 + 2.5 - 2.0 ** -40]
    params = np.tile([1.0, 2.0, 2.0], (n, 1))     # cut = sigma = 2.0, list radius 2.5
    out.append(_case("edges64_pairs", REPULSION, VERLET, 50, 0.005, Lb, x, rng.normal(0, 0.3, (n, 3)),
                     np.ones(n), params, 0.5, [1, 20, 50]))
    # 12. LJAttractCutPair (pyparm's LJAttractCut): attraction only, per-atom epsilon and sigma,
    #     Verlet from a jittered lattice
    rng = np.random.default_rng(51)
    L, x, v = lj_lattice_deck((8, 8, 8), 51)
    n = len(x)
    eps = rng.choice([0.8, 1.2], n)
    sg = rng.choice([1.0, 1.2], n)
    out.append(_case("ljattract512_verlet", LJATTRACT, VERLET, 300, 0.002, L, x, v, np.ones(n),
                     np.stack([eps, sg, np.full(n, cut)], 1), 0.3, [1, 10, 100, 300]))
    # 9. CollectionNLCG (box and positions), 3D harmonic spheres from phi = 0.4 at the goal
    #    pressure 1e-3, set up as pyparm's packmin.Minimizer (dt 0.1, kappa 10, kmax 1000,
    #    secmax 40, seceps 1e-20, alphamax 2, dxmax 100, stepmax 1e-3); one immobile atom
    rng = np.random.default_rng(41)
    n = 64
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Lp = (np.sum(np.pi * sig ** 3 / 6) / 0.4) ** (1 / 3)
    m = np.ones(n)
    m[5] = np.inf
    cg = [0.1, 1e-3, 10.0, 1000, 40, 1e-20, 2.0, 0.0, 100.0, 1e-3, 0.0]
    out.append(_case("nlcg64_pack", REPULSION, NLCG, 200, 0.1, [Lp] * 3, rng.uniform(0, Lp, (n, 3)),
                     np.zeros((n, 3)), m, np.stack([np.ones(n), sig, np.full(n, 2.0)], 1), 0.4,
                     [0, 1, 2, 3, 5, 10, 30, 100, 200], cg=cg))
    # 10. CollectionNLCG in 2D, Hertzian (exponent 2.5) disks from phi = 0.6, goal pressure 1e-2
    rng = np.random.default_rng(42)
    n = 80
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Lq = np.sqrt(np.sum(np.pi * sig ** 2 / 4) / 0.6)
    cg = [0.1, 1e-2, 10.0, 1000, 40, 1e-20, 2.0, 0.0, 100.0, 1e-3, 0.0]
    out.append(_case("nlcg80_2d_pack", REPULSION, NLCG, 150, 0.1, [Lq, Lq], rng.uniform(0, Lq, (n, 2)),
                     np.zeros((n, 2)), np.ones(n), np.stack([np.ones(n), sig, np.full(n, 2.5)], 1), 0.4,
                     [0, 1, 2, 5, 10, 50, 150], cg=cg))
    # 11. CollectionNLCGV (positions only, fixed box), 3D harmonic spheres at phi = 0.7,
    #     the constructor's defaults (kmax 1000, secmax 10, seceps 1e-4)
    rng = np.random.default_rng(43)
    n = 100
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Lv = (np.sum(np.pi * sig ** 3 / 6) / 0.7) ** (1 / 3)
    cg = [0.01, 0.0, 1.0, 1000, 10, 1e-4, 0.0, 0.0, 0.0, 0.0, 0.0]
    out.append(_case("nlcgv100_fixed", REPULSION, NLCGV, 200, 0.01, [Lv] * 3, rng.uniform(0, Lv, (n, 3)),
                     np.zeros((n, 3)), np.ones(n), np.stack([np.ones(n), sig, np.full(n, 2.0)], 1), 0.3,
                     [0, 1, 2, 5, 10, 50, 200], cg=cg))
    # 13. LoisOhernPair (sticky spheres: harmonic repulsion, linear attraction out to
    #     sigma (1 + C + l)), per-atom C and l averaged, 3D, damped from random positions
    rng = np.random.default_rng(61)
    n = 216
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Lo = (np.sum(np.pi * sig ** 3 / 6) / 0.5) ** (1 / 3)
    C = rng.choice([0.05, 0.1], n)
    ll = rng.choice([0.02, 0.05], n)
    out.append(_case("loisohern216_damped", LOISOHERN, DAMPED, 300, 0.01, [Lo] * 3, rng.uniform(0, Lo, (n, 3)),
                     rng.normal(0, 0.05, (n, 3)), np.ones(n), np.stack([np.ones(n), sig, C, ll], 1), 0.2,
                     [1, 10, 100, 300], damping=0.5))
    # 14. LoisOhernPairMinCLs (the smaller C and l of the two atoms) in 2D, Verlet
    rng = np.random.default_rng(62)
    n = 150
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Lo2 = np.sqrt(np.sum(np.pi * sig ** 2 / 4) / 0.7)
    C = rng.choice([0.04, 0.08], n)
    ll = rng.choice([0.03, 0.06], n)
    eps = rng.choice([0.5, 2.0], n)
    out.append(_case("loisohernmin150_2d_verlet", LOISOHERN_MIN, VERLET, 400, 0.005, [Lo2, Lo2],
                     rng.uniform(0, Lo2, (n, 2)), rng.normal(0, 0.1, (n, 2)), np.ones(n),
                     np.stack([eps, sig, C, ll], 1), 0.2, [1, 10, 100, 400]))
    # 15. LoisLinPair (harmonic repulsion, a fixed attractive force f = depth / width out to
    #     sigma + width), 3D, damped; the fixture keeps the atoms' fields (eps, sigma, f, l)
    rng = np.random.default_rng(63)
    n = 200
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Ll = (np.sum(np.pi * sig ** 3 / 6) / 0.55) ** (1 / 3)
    depth = rng.choice([0.001, 0.003], n)
    width = rng.choice([0.05, 0.1], n)
    f = depth / width
    out.append(_case("loislin200_damped", LOISLIN, DAMPED, 300, 0.01, [Ll] * 3, rng.uniform(0, Ll, (n, 3)),
                     np.zeros((n, 3)), np.ones(n), np.stack([np.ones(n), sig, f, width], 1), 0.2,
                     [1, 10, 100, 300], damping=0.5, deck_params=np.stack([np.ones(n), sig, depth, width], 1)))
    # 16. LoisLinPairMin (the smaller f and l) in 2D, Verlet, one atom with width 0 (f = 0)
    rng = np.random.default_rng(64)
    n = 120
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Ll2 = np.sqrt(np.sum(np.pi * sig ** 2 / 4) / 0.75)
    depth = rng.choice([0.002, 0.004], n)
    width = rng.choice([0.04, 0.08], n)
    width[7] = 0.0
    f = np.where(width > 0, depth / np.where(width > 0, width, 1.0), 0.0)
    out.append(_case("loislinmin120_2d_verlet", LOISLIN_MIN, VERLET, 400, 0.005, [Ll2, Ll2],
                     rng.uniform(0, Ll2, (n, 2)), rng.normal(0, 0.1, (n, 2)), np.ones(n),
                     np.stack([np.ones(n), sig, f, width], 1), 0.2, [1, 10, 100, 400],
                     deck_params=np.stack([np.ones(n), sig, depth, width], 1)))
    # 17. EisMclachlanPair (implicit solvation, E = c0/R + c1 + c2 R out to dist_i + dist_j),
    #     per-atom dist and solvation parameter of either sign, 3D, damped
    rng = np.random.default_rng(65)
    n = 180
    Le = 9.0
    dist = rng.choice([1.6, 1.9, 2.2], n)
    sigi = rng.choice([-0.012, 0.006, 0.018], n)
    out.append(_case("eismclachlan180_damped", EISMCLACHLAN, DAMPED, 200, 0.005, [Le] * 3,
                     rng.uniform(0, Le, (n, 3)), rng.normal(0, 0.02, (n, 3)), np.ones(n),
                     np.stack([dist, sigi, np.zeros(n)], 1), 0.3, [1, 10, 100, 200], damping=0.5))
    # 18. RepulsionDragPair (soft repulsion with a drag on the relative normal velocity),
    #     per-atom exponent 2 or 2.5 and gamma, 3D Verlet from random positions and velocities;
    #     the constructor takes (eps, sigma, gamma, exponent), the fixture keeps the fields
    #     (eps, sigma, exponent, gamma)
    rng = np.random.default_rng(66)
    n = 160
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Lr = (np.sum(np.pi * sig ** 3 / 6) / 0.6) ** (1 / 3)
    expo = rng.choice([2.0, 2.5], n)
    gam = rng.choice([0.1, 0.3], n)
    eps = rng.choice([1.0, 2.0], n)
    out.append(_case("repulsiondrag160_verlet", REPULSIONDRAG, VERLET, 300, 0.01, [Lr] * 3,
                     rng.uniform(0, Lr, (n, 3)), rng.normal(0, 0.3, (n, 3)), np.ones(n),
                     np.stack([eps, sig, expo, gam], 1), 0.3, [1, 10, 100, 300],
                     deck_params=np.stack([eps, sig, gam, expo], 1)))
    # 19-24. indexed pair epsilons (and sigmas): three atom types, a symmetric table with one
    #        non-positive entry (the repulsion-only branch of the kinds that have one)
    L, x, v = lj_lattice_deck((6, 6, 6), 71)
    n = len(x)
    rng = np.random.default_rng(71)
    t = rng.integers(0, 3, n).astype(np.float64)
    teps = np.array([[1.0, 0.6, 0.3], [0.6, 1.3, -0.5], [0.3, -0.5, 0.8]])
    tsig = np.array([[1.0, 1.1, 1.05], [1.1, 1.2, 1.15], [1.05, 1.15, 0.95]])
    cutv = rng.choice([2.0, 2.5], n)
    # (an asymmetric table: a pair takes its first atom's row, the later one in the list)
    teps_a = np.array([[1.0, 0.7, 0.4], [0.5, 1.2, 0.9], [0.3, 0.8, 0.6]])
    tsig_a = np.array([[1.0, 1.1, 1.05], [1.08, 1.2, 1.12], [1.02, 1.17, 0.95]])
    out.append(_case("ljcut_iepsisig216_verlet", LJCUT_IEPSISIG, VERLET, 300, 0.002, L * 1.1, x * 1.1, v,
                     np.ones(n), np.stack([t, cutv, np.zeros(n)], 1), 0.3, [1, 10, 100, 300],
                     order=rng.permutation(n), pair_eps=teps_a, pair_sig=tsig_a))
    out.append(_case("ljattract_iepsisig216_verlet", LJATTRACT_IEPSISIG, VERLET, 300, 0.002, L * 1.1, x * 1.1,
                     v, np.ones(n), np.stack([t, cutv, np.zeros(n)], 1), 0.3, [1, 10, 100, 300],
                     pair_eps=np.abs(teps), pair_sig=tsig))
    sgv = rng.choice([1.0, 1.2], n)
    out.append(_case("ljattract_ieps216_verlet", LJATTRACT_IEPS, VERLET, 300, 0.002, L * 1.1, x * 1.1, v,
                     np.ones(n), np.stack([t, sgv, cutv], 1), 0.3, [1, 10, 100, 300], pair_eps=np.abs(teps)))
    out.append(_case("ljattractrepulse216_verlet", LJATTRACTREPULSE, VERLET, 300, 0.002, L * 1.1, x * 1.1, v,
                     np.ones(n), np.stack([t, sgv, cutv], 1), 0.3, [1, 10, 100, 300], pair_eps=teps))
    rep = rng.choice([0.5, 2.0], n)
    out.append(_case("ljattractfixedrepulse216_verlet", LJATTRACTFIXEDREPULSE, VERLET, 300, 0.002, L * 1.1,
                     x * 1.1, v, np.ones(n), np.stack([t, rep, sgv, cutv], 1), 0.3, [1, 10, 100, 300],
                     pair_eps=teps))
    nexp = rng.choice([8.0, 12.0], n)
    teps_b = teps.copy()
    teps_b[0, 2] = -0.2   # asymmetric, and not positive in one order only
    out.append(_case("ljish216_verlet", LJISH, VERLET, 300, 0.002, L * 1.1, x * 1.1, v, np.ones(n),
                     np.stack([t, rep, sgv, nexp, cutv], 1), 0.3, [1, 10, 100, 300], pair_eps=teps_b))
    # 25. RepulsionPair on IEpsISigExpAtom (pyparm's RepulsionII): indexed epsilon and sigma,
    #     per-atom exponent 2 or 2.5 (averaged), 3D soft spheres, damped
    rng = np.random.default_rng(72)
    n = 200
    t = rng.integers(0, 3, n).astype(np.float64)
    teps = np.array([[1.0, 0.8, 1.1], [0.8, 1.4, 0.9], [1.1, 0.9, 0.7]])
    tsig = np.array([[1.0, 1.2, 1.1], [1.2, 1.4, 1.3], [1.1, 1.3, 1.2]])
    Lr2 = (200 * np.pi * 1.2 ** 3 / 6 / 0.6) ** (1 / 3)
    out.append(_case("repulsion_iepsisig200_damped", REPULSION_IEPSISIG, DAMPED, 300, 0.01, [Lr2] * 3,
                     rng.uniform(0, Lr2, (n, 3)), np.zeros((n, 3)), np.ones(n),
                     np.stack([t, rng.choice([2.0, 2.5], n), np.zeros(n)], 1), 0.2, [1, 10, 100, 300],
                     damping=0.5, pair_eps=teps, pair_sig=tsig))
    # 26. LJAttractRepulseSigsPair (separate repulsive and attractive epsilons and lengths),
    #     per-atom values, cut-offs in both of the constructor's branches (sigcut < 1, >= 1)
    rng = np.random.default_rng(73)
    L, x, v = lj_lattice_deck((6, 6, 6), 73)
    n = len(x)
    out.append(_case("ljattractrepulsesigs216_verlet", LJATTRACTREPULSESIGS, VERLET, 300, 0.002, L * 1.1, x * 1.1,
                     v, np.ones(n), np.stack([rng.choice([1.0, 1.5], n), rng.choice([0.5, 0.8], n),
                                              rng.choice([1.0, 1.1], n), rng.choice([0.9, 1.2], n),
                                              rng.choice([0.95, 2.0, 2.5], n)], 1), 0.3, [1, 10, 100, 300]))
    # 27-28. LeesEdwardsBox: the minimum image across y shifts x by the shear; soft spheres
    #        (damped) and LJ (Verlet) at shears 0.3 and -0.75 (an image offset past half a box)
    rng = np.random.default_rng(74)
    n = 200
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    Lle = (np.sum(np.pi * sig ** 3 / 6) / 0.6) ** (1 / 3)
    out.append(_case("lees_spheres200_damped", REPULSION, DAMPED, 300, 0.01, [Lle] * 3, rng.uniform(0, Lle, (n, 3)),
                     np.zeros((n, 3)), np.ones(n), np.stack([np.ones(n), sig, np.full(n, 2.0)], 1), 0.2,
                     [1, 10, 100, 300], damping=0.5, le_gamma=0.3))
    L, x, v = lj_lattice_deck((8, 8, 8), 75)
    n = len(x)
    out.append(_case("lees_lj512_verlet", LJCUT, VERLET, 300, 0.002, L, x, v, np.ones(n),
                     np.tile([1.0, 1.0, cut], (n, 1)), 0.3, [1, 10, 100, 300], le_gamma=-0.75))
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default=os.environ.get("PARM_REFERENCE_SRC", "/root/reference/src"))
    ap.add_argument("--only", default=None)
    a = ap.parse_args(argv)
    subprocess.run(["make", "-C", str(REFBUILD), f"REF={a.ref_src}", f"OUT={REFOUT}", "-j2"], check=True)
    for c in cases():
        if a.only and c["name"] != a.only:
            continue
        nd = c["L"].shape[0]
        exe = REFOUT / f"ref_driver{nd}d"
        r = subprocess.run([str(exe)], input=_deck(c), capture_output=True, text=True, check=True)
        res = _parse(r.stdout, len(c["m"]), nd)
        arrays = {k: v for k, v in c.items() if k != "name"}
        arrays.update(res)
        arrays = {k: (np.asarray(v) if not isinstance(v, np.ndarray) else v) for k, v in arrays.items()}
        np.savez_compressed(HERE / f"{c['name']}.npz", **arrays)
        print(f"{c['name']}: n={len(c['m'])} pairs={len(res['pairs'])} E0={res['init'][0]!r} "
              f"which={res['which_steps'].tolist()}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
