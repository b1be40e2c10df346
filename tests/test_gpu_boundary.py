"""The reference's interaction / neighbour-list interface beyond the time steps, on the GPU.

* NeighborList::add(atom, diameter) through parm_set_list_diameters: members
  with their own list diameter and no pair parameters; pair list (order
  included), forces and energy bit-exact against the oracle's restatement;
* the host API's NListed(atoms, neighbours), list iteration, per-pair
  evaluation, set_forces_get_stress, the virtual stress and the rejection of
  interactions a Collection cannot step (tests/programs/host_api_extras.cpp);
* an LJ program written like the reference's src/bin/LJatoms.cpp
  (tests/programs/lj_verlet.cpp): 20000 CollectionVerlet time steps, one
  timestep() call at a time, with the total energy conserved.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from host_api import compile_program
from parm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

PROGRAMS = Path(__file__).resolve().parent / "programs"


@pytest.mark.parametrize("ndim", [3, 2])
def test_list_diameters_match_oracle(ndim):
    from oracle.oracle import Oracle
    from parm_gb300 import System
    w = W.small_random(n=400, ndim=ndim, kind=1, seed=60 + ndim, phi=0.5, skin=0.3)
    n, nm = w.n, 40
    params = w.params.copy()
    params[n - nm:] = 0.0                       # list members without pair parameters
    rng = np.random.default_rng(5)
    dia = np.full(n, np.nan)
    dia[n - nm:] = rng.uniform(0.8, 1.6, nm)
    order = np.concatenate([rng.permutation(n - nm), np.arange(n - nm, n)])
    rank = np.empty(n, dtype=np.uint32)
    rank[order] = np.arange(n, dtype=np.uint32)
    g = System(n, ndim=ndim, precision="fp64")
    g.set_boxes(w.L)
    g.set_atoms(x=w.x, v=w.v, a=np.zeros_like(w.x), f=np.zeros_like(w.x), m=w.m)
    g.set_list_diameters(dia)
    g.set_interaction(w.kind, params, w.skin, rank=rank)
    o = Oracle(n, ndim)
    o.set_box(w.L[0])
    o.set_state(x=w.x, v=w.v, m=w.m)
    o.set_interaction(w.kind, params, w.skin, order=[int(i) for i in order[: n - nm]])
    for i in order[n - nm:]:
        o.add_member(int(i), dia[i])
    g.nlist_update(True)
    o.nl_update(True)
    assert np.array_equal(g.pairs(), o.pairs())
    g.set_forces(True)
    o.set_forces(True)
    st, ref = g.get_atoms(), o.get_state()
    assert np.array_equal(st["f"], ref["f"])
    assert np.all(st["f"][n - nm:] == 0.0)
    assert g.energy()[0] == pytest.approx(o.energy(), rel=1e-12, abs=1e-14)
    g.close()


def _run(src, tmp_path, ndim=3, timeout=900):
    exe = tmp_path / src.stem
    r = compile_program(src, exe, ndim=ndim)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=timeout, cwd=tmp_path,
                       env={"PARM_PRECISION": "fp64", "PATH": "/usr/bin:/bin"})
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
    return r.stdout


@pytest.mark.parametrize("ndim", [3, 2])
def test_host_api_extras_program(tmp_path, built_lib, ndim):
    out = _run(PROGRAMS / "host_api_extras.cpp", tmp_path, ndim)
    checks = [line.split() for line in out.splitlines() if line.startswith("check")]
    assert len(checks) >= 12, out
    failed = [c[1] for c in checks if c[2] != "1"]
    assert not failed, out


def test_lj_program_conserves_energy(tmp_path, built_lib):
    out = _run(PROGRAMS / "lj_verlet.cpp", tmp_path)
    E = np.array([float(line.split()[3]) for line in out.splitlines() if line.startswith("block")])
    assert len(E) == 20
    # The program adds its interaction after the Collection's initialisation (as LJatoms.cpp
    # does), so the first step starts from zero accelerations and the energy moves once; from
    # then on the total energy stays within 1e-4 per atom over 19000 steps (the cut-off
    # potential's force jumps give a small random walk, no drift)
    assert np.abs(E - E[0]).max() <= 1e-4 * 200, E


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cell_scale_leaves_results_unchanged(precision):
    """Wider cells (parm_set_cell_scale) change how lists are built, not what they hold: the same
    pairs in the same order; FP64 forces and trajectories bit for bit, mixed forces within the mixed
    path's tolerance (a different cell grid can select another kernel variant)."""
    from helpers import force_error, make_gpu
    w = W.lj_lattice(shape=(14, 14, 14), skin_prime=0.3, seed=71)
    out = []
    for scale in (1.0, 1.7):
        g = make_gpu(w, precision)
        g.set_cell_scale(scale)
        g.nlist_update(True)
        g.set_forces(True)
        f0 = g.get_atoms(8)["f"]
        g.verlet(0.001, 30)
        out.append((g.pairs(), f0, g.get_atoms()))
        g.close()
    assert np.array_equal(out[0][0], out[1][0])
    if precision == "fp64":
        np.testing.assert_array_equal(out[0][1], out[1][1])
        for k in ("x", "v", "f"):
            np.testing.assert_array_equal(out[0][2][k], out[1][2][k])
    else:
        assert force_error(out[1][1], out[0][1]) <= 1e-5


@pytest.mark.parametrize("kind", [4, 5, 6, 7])
def test_lois_uniform_parameters_match_oracle(kind):
    """The Lois-O'Hern / Lois-Lin pairs with shared C (or f) and l, and with only l varying: pair list,
    forces and 50 Verlet steps bit-exact against the oracle (the uniform-parameter shortcuts of the FP64
    kernels and the list build)."""
    from oracle.oracle import Oracle
    from parm_gb300 import System
    rng = np.random.default_rng(70 + kind)
    n = 300
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    L = (np.sum(np.pi * sig ** 3 / 6) / 0.55) ** (1 / 3)
    x = rng.uniform(0, L, (n, 3))
    v = rng.normal(0, 0.05, (n, 3))
    third = 0.08 if kind < 6 else 0.04
    for lvals in (np.full(n, 0.05), rng.choice([0.03, 0.06], n)):
        params = np.stack([np.ones(n), sig, np.full(n, third), lvals], 1)
        g = System(n, ndim=3, precision="fp64")
        g.set_boxes(np.full((1, 3), L))
        g.set_atoms(x=x, v=v, a=np.zeros((n, 3)), f=np.zeros((n, 3)), m=np.ones(n))
        g.set_interaction(kind, params, 0.2)
        o = Oracle(n, 3)
        o.set_box(np.full(3, L))
        o.set_state(x=x, v=v, m=np.ones(n))
        o.set_interaction(kind, params, 0.2)
        g.nlist_update(True)
        o.nl_update(True)
        assert np.array_equal(g.pairs(), o.pairs())
        g.set_forces(True)
        o.set_forces(True)
        assert np.array_equal(g.get_atoms()["f"], o.get_state()["f"])
        g.verlet(0.005, 50)
        o.verlet(0.005, 50)
        st, ref = g.get_atoms(), o.get_state()
        for k in ("x", "v", "f"):
            assert np.array_equal(st[k], ref[k]), k
        assert g.energy()[0] == pytest.approx(o.energy(), rel=1e-12, abs=1e-13)
        g.close()


def test_lois_kinds_need_fp64_handles():
    from parm_gb300 import System
    w = W.small_random(n=64, ndim=3, kind=1, seed=3)
    g = System(w.n, ndim=3, precision="mixed")
    g.set_boxes(w.L)
    g.set_atoms(x=w.x, v=w.v, a=np.zeros_like(w.x), f=np.zeros_like(w.x), m=w.m)
    with pytest.raises(ValueError, match="FP64"):
        g.set_interaction(4, np.tile([1.0, 1.0, 0.1, 0.05], (w.n, 1)), 0.2)
    g.close()


def test_eismclachlan_uniform_dist_matches_oracle():
    """Eis-Mclachlan atoms sharing their dist (the uniform list-diameter path of the FP64 list build)
    with solvation parameters of either sign: pairs, forces and 50 damped steps bit-exact against the
    oracle."""
    from oracle.oracle import Oracle
    from parm_gb300 import System
    rng = np.random.default_rng(81)
    n, L = 250, 10.0
    x = rng.uniform(0, L, (n, 3))
    params = np.stack([np.full(n, 1.8), rng.choice([-0.01, 0.015], n), np.zeros(n)], 1)
    g = System(n, ndim=3, precision="fp64")
    g.set_boxes(np.full((1, 3), L))
    g.set_atoms(x=x, v=np.zeros((n, 3)), a=np.zeros((n, 3)), f=np.zeros((n, 3)), m=np.ones(n))
    g.set_interaction(8, params, 0.3)
    o = Oracle(n, 3)
    o.set_box(np.full(3, L))
    o.set_state(x=x, v=np.zeros((n, 3)), m=np.ones(n))
    o.set_interaction(8, params, 0.3)
    g.nlist_update(True)
    o.nl_update(True)
    assert np.array_equal(g.pairs(), o.pairs())
    g.set_forces(True)
    o.set_forces(True)
    assert np.array_equal(g.get_atoms()["f"], o.get_state()["f"])
    g.damped(0.002, 0.5, 50)
    o.damped(0.002, 0.5, 50)
    st, ref = g.get_atoms(), o.get_state()
    for k in ("x", "v", "f"):
        assert np.array_equal(st[k], ref[k]), k
    assert g.energy()[0] == pytest.approx(o.energy(), rel=1e-12, abs=1e-12)
    g.close()


@pytest.mark.parametrize("vary_gamma", [False, True])
def test_repulsion_drag_matches_oracle(vary_gamma):
    """RepulsionDragPair (velocity-dependent pair forces) with exponent 2: pairs, forces, virial and 100
    Verlet steps bit-exact against the oracle, with a shared drag coefficient (the uniform-parameter
    shortcut) and with per-atom ones."""
    from oracle.oracle import Oracle
    from parm_gb300 import System
    rng = np.random.default_rng(90 + vary_gamma)
    n = 240
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    L = (np.sum(np.pi * sig ** 3 / 6) / 0.6) ** (1 / 3)
    x = rng.uniform(0, L, (n, 3))
    v = rng.normal(0, 0.3, (n, 3))
    gam = rng.choice([0.1, 0.4], n) if vary_gamma else np.full(n, 0.2)
    params = np.stack([np.ones(n), sig, np.full(n, 2.0), gam], 1)
    g = System(n, ndim=3, precision="fp64")
    g.set_boxes(np.full((1, 3), L))
    g.set_atoms(x=x, v=v, a=np.zeros((n, 3)), f=np.zeros((n, 3)), m=np.ones(n))
    g.set_interaction(9, params, 0.3)
    o = Oracle(n, 3)
    o.set_box(np.full(3, L))
    o.set_state(x=x, v=v, m=np.ones(n))
    o.set_interaction(9, params, 0.3)
    g.nlist_update(True)
    o.nl_update(True)
    assert np.array_equal(g.pairs(), o.pairs())
    g.set_forces(True)
    o.set_forces(True)
    assert np.array_equal(g.get_atoms()["f"], o.get_state()["f"])
    g.verlet(0.01, 100)
    o.verlet(0.01, 100)
    st, ref = g.get_atoms(), o.get_state()
    for k in ("x", "v", "f"):
        assert np.array_equal(st[k], ref[k]), k
    assert g.virial()[0] == pytest.approx(o.pressure()[0], rel=1e-12, abs=1e-12)
    g.close()


@pytest.mark.parametrize("kind", [10, 12])
def test_indexed_asymmetric_table_matches_oracle(kind):
    """Indexed epsilons with an asymmetric table and a shuffled insertion order: each pair takes the row
    of its first atom (the later one in the neighbour list), as IEps*Atom::get_epsilon does.  Pairs,
    forces and 50 Verlet steps bit-exact against the oracle."""
    from oracle.oracle import Oracle
    from parm_gb300 import System
    L, x, v = None, None, None
    w = W.lj_lattice(shape=(6, 6, 6), skin_prime=0.3, seed=83)
    n = w.n
    x, v, L = w.x * 1.1, w.v, w.L[0] * 1.1
    rng = np.random.default_rng(83)
    t = rng.integers(0, 3, n).astype(np.float64)
    teps = np.array([[1.0, 0.7, 0.4], [0.5, 1.2, 0.9], [0.3, 0.8, 0.6]])
    tsig = np.array([[1.0, 1.1, 1.05], [1.08, 1.2, 1.12], [1.02, 1.17, 0.95]])
    cutv = rng.choice([2.0, 2.5], n)
    params = (np.stack([t, cutv, np.zeros(n)], 1) if kind == 10
              else np.stack([t, rng.choice([1.0, 1.2], n), cutv], 1))
    order = rng.permutation(n)
    rank = np.empty(n, dtype=np.uint32)
    rank[order] = np.arange(n, dtype=np.uint32)
    g = System(n, ndim=3, precision="fp64")
    g.set_boxes(L[None, :])
    g.set_atoms(x=x, v=v, a=np.zeros((n, 3)), f=np.zeros((n, 3)), m=np.ones(n))
    g.set_pair_table(teps, tsig)
    g.set_interaction(kind, params, w.skin, rank=rank)
    o = Oracle(n, 3)
    o.set_box(L)
    o.set_state(x=x, v=v, m=np.ones(n))
    o.set_pair_table(teps, tsig)
    o.set_interaction(kind, params, w.skin, order=[int(i) for i in order])
    g.nlist_update(True)
    o.nl_update(True)
    assert np.array_equal(g.pairs(), o.pairs())
    g.set_forces(True)
    o.set_forces(True)
    assert np.array_equal(g.get_atoms()["f"], o.get_state()["f"])
    g.verlet(0.002, 50)
    o.verlet(0.002, 50)
    st, ref = g.get_atoms(), o.get_state()
    for k in ("x", "v", "f"):
        assert np.array_equal(st[k], ref[k]), k
    assert g.energy()[0] == pytest.approx(o.energy(), rel=1e-12, abs=1e-12)
    g.close()


@pytest.mark.parametrize("ndim", [2, 3])
def test_lees_edwards_shear_matches_oracle(ndim):
    """A LeesEdwardsBox sheared between runs (x += y dgamma, gamma += dgamma, as
    LeesEdwardsBox::shear(dgamma, atoms) does): pairs, forces and damped steps bit-exact against the
    oracle before and after the shear, including a shear past half a box."""
    from oracle.oracle import Oracle
    from parm_gb300 import System
    rng = np.random.default_rng(95 + ndim)
    n = 240
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    vol = np.sum((np.pi * sig ** 2 / 4) if ndim == 2 else (np.pi * sig ** 3 / 6)) / 0.6
    L = vol ** (1 / ndim)
    x = rng.uniform(0, L, (n, ndim))
    params = np.stack([np.ones(n), sig, np.full(n, 2.0)], 1)
    g = System(n, ndim=ndim, precision="fp64")
    g.set_boxes(np.full((1, ndim), L))
    g.set_lees_edwards([0.2])
    g.set_atoms(x=x, v=np.zeros((n, ndim)), a=np.zeros((n, ndim)), f=np.zeros((n, ndim)), m=np.ones(n))
    g.set_interaction(1, params, 0.2)
    o = Oracle(n, ndim)
    o.set_box(np.full(ndim, L))
    o.set_lees_edwards(0.2)
    o.set_state(x=x, v=np.zeros((n, ndim)), m=np.ones(n))
    o.set_interaction(1, params, 0.2)
    for gamma_next in (0.35, 0.9):
        g.nlist_update(True)
        o.nl_update(True)
        assert np.array_equal(g.pairs(), o.pairs())
        g.set_forces(True)
        o.set_forces(True)
        assert np.array_equal(g.get_atoms()["f"], o.get_state()["f"])
        g.damped(0.01, 0.5, 40)
        o.damped(0.01, 0.5, 40)
        st, ref = g.get_atoms(), o.get_state()
        for k in ("x", "v", "f"):
            assert np.array_equal(st[k], ref[k]), k
        # shear the box and the atoms
        gam = 0.2 if gamma_next == 0.35 else 0.35
        xs = ref["x"].copy()
        xs[:, 0] += xs[:, 1] * (gamma_next - gam)
        g.set_atoms(x=xs)
        g.set_lees_edwards([gamma_next])
        o.set_state(x=xs, v=ref["v"], a=ref["a"], f=ref["f"], m=np.ones(n))
        o.set_lees_edwards(gamma_next)
    g.close()


def test_lees_edwards_needs_fp64():
    from parm_gb300 import System
    g = System(64, ndim=3, precision="mixed")
    with pytest.raises(ValueError, match="FP64"):
        g.set_lees_edwards([0.1])
    g.close()
