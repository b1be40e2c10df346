"""Mixed-precision path: force/energy error and NVE drift against FP64.

Tolerances (stated by the benchmark specification for the mixed path):
  max_i |F_i - F_i^FP64| / rms_i |F_i^FP64|  <= 1e-5
  relative potential-energy error             <= 1e-6
"""
import numpy as np
import pytest

from helpers import force_error, make_gpu, make_oracle
from parm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5
ENERGY_TOL = 1e-6


def _equilibrated_lj(shape, steps=300, seed=12345):
    """LJ lattice melted with the FP64 GPU path (dt 0.002)."""
    w = W.lj_lattice(shape=shape, skin_prime=0.3, seed=seed)
    g = make_gpu(w, "fp64")
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    g.verlet(0.002, steps)
    st = g.get_atoms()
    w.x, w.v = st["x"], st["v"]
    return w


@pytest.fixture(scope="module")
def lj32k():
    return _equilibrated_lj((32, 32, 32))


def test_mixed_forces_within_tolerance(lj32k):
    w = lj32k
    m = make_gpu(w, "mixed")
    o = make_oracle(w)
    m.nlist_update(True)
    o.build_fast()
    assert np.array_equal(m.pairs(), o.pairs())   # the list test stays FP64-exact
    m.set_forces(True)
    o.set_forces(True)
    F = m.get_atoms()["f"]
    Fref = o.get_state()["f"]
    err = force_error(F, Fref)
    assert err <= FORCE_TOL, err
    e, eref = m.energy()[0], o.energy()
    assert abs(e - eref) / abs(eref) <= ENERGY_TOL
    p, _ = o.pressure()
    assert abs(m.virial()[0] - p) / abs(p) <= 1e-5


@pytest.mark.parametrize("exponent", [2.0, 2.5])
def test_mixed_soft_spheres(exponent):
    """Random overlapping soft spheres (the packings' starting state)."""
    w = W.small_random(n=4000, ndim=3, kind=1, seed=31, phi=0.6, exponent=exponent, skin=0.2)
    m = make_gpu(w, "mixed")
    o = make_oracle(w)
    m.nlist_update(True)
    o.nl_update(True)
    m.set_forces(True)
    o.set_forces(True)
    err = force_error(m.get_atoms()["f"], o.get_state()["f"])
    assert err <= FORCE_TOL, err


def test_mixed_wca_fluid():
    """WCA fluid at the replicas' densities (lattice start, as in the Langevin workload)."""
    w = W.wca_replicas(nrep=1, nmin=8000, nmax=8000, rho_lo=0.9, rho_hi=0.9, seed=32)
    m = make_gpu(w, "mixed")
    o = make_oracle(w)
    m.nlist_update(True)
    o.nl_update(True)
    m.set_forces(True)
    o.set_forces(True)
    err = force_error(m.get_atoms()["f"], o.get_state()["f"])
    assert err <= FORCE_TOL, err


@pytest.mark.parametrize("ndim", [3, 2])
def test_mixed_attractive_lj(ndim):
    """LJAttractCutPair (per-atom epsilon and sigma) on the mixed path's per-atom kernels."""
    w = W.small_random(n=3000, ndim=ndim, kind=3, seed=33 + ndim, phi=0.35, skin=0.3)
    m = make_gpu(w, "mixed")
    o = make_oracle(w)
    m.nlist_update(True)
    o.nl_update(True)
    assert np.array_equal(m.pairs(), o.pairs())
    m.set_forces(True)
    o.set_forces(True)
    err = force_error(m.get_atoms()["f"], o.get_state()["f"])
    assert err <= FORCE_TOL, err
    assert abs(m.energy()[0] - o.energy()) <= ENERGY_TOL * abs(o.energy())


def test_mixed_2d_disks():
    w = W.soft_disks(n=4096, phi=0.84)
    m = make_gpu(w, "mixed")
    o = make_oracle(w)
    m.nlist_update(True)
    o.build_fast()
    m.set_forces(True)
    o.set_forces(True)
    err = force_error(m.get_atoms()["f"], o.get_state()["f"])
    assert err <= FORCE_TOL, err


def _lj_replicas(nrep, shape, steps=300):
    """nrep independent LJ lattices (own jitter and velocities) in one handle, melted with the FP64 path."""
    reps = [W.lj_lattice(shape=shape, skin_prime=0.3, seed=1000 + q) for q in range(nrep)]
    r0 = reps[0]
    w = W.Workload("lj_replicas", 3, [r.n for r in reps], np.concatenate([r.L for r in reps]),
                   np.concatenate([r.x for r in reps]), np.concatenate([r.v for r in reps]),
                   np.concatenate([r.m for r in reps]), r0.kind, np.concatenate([r.params for r in reps]), r0.skin)
    g = make_gpu(w, "fp64")
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    g.verlet(0.002, steps)
    st = g.get_atoms()
    g.close()
    w.x, w.v = st["x"], st["v"]
    return w


def _drift_slopes(g, steps, every):
    """Per-system least-squares slope of the total energy over `steps` steps (sampled every `every`),
    per 10^5 steps and relative to that system's |E(0)|."""
    E = [g.energy() + g.kinetic_energy()]
    for _ in range(steps // every):
        g.verlet(0.002, every)
        E.append(g.energy() + g.kinetic_energy())
    E = np.array(E)                      # (samples, nsys)
    t = np.arange(len(E), dtype=np.float64) * every
    tc = t - t.mean()
    slope = (tc[:, None] * (E - E.mean(0))).sum(0) / (tc ** 2).sum()
    return slope * 1e5 / np.abs(E[0])


def test_mixed_nve_drift_comparable():
    """NVE energy drift of the mixed path is the FP64 path's.  16 independent 4096-atom LJ replicas run
    20000 steps on each path from the same states; the mean fitted slope (per 10^5 steps, relative) of
    the two paths differs by less than four standard errors of the replica spread plus 1e-5, and the
    mixed path's mean slope is below 1e-4.  (A single trajectory's least-squares error understates the
    slope's spread: the energy error is correlated over many steps.)"""
    nrep = 16
    w = _lj_replicas(nrep, (16, 16, 16))
    out = {}
    for prec in ("fp64", "mixed"):
        g = make_gpu(w, prec)
        g.set_graph_steps(50)
        g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
        out[prec] = _drift_slopes(g, 20000, 100)
        g.close()
    m64, m32 = out["fp64"].mean(), out["mixed"].mean()
    se64, se32 = out["fp64"].std(ddof=1) / np.sqrt(nrep), out["mixed"].std(ddof=1) / np.sqrt(nrep)
    info = {"fp64": (m64, se64), "mixed": (m32, se32)}
    print("drift per 1e5 steps (mean, standard error):", info)
    assert abs(m32 - m64) <= 4 * np.hypot(se32, se64) + 1e-5, info
    assert abs(m32) <= 1e-4, info


@pytest.mark.parametrize("tpa", [200, 1, 2, 4, 101, 104, 108, 116, 132])
def test_mixed_threads_per_atom(lj32k, tpa):
    """Every threads-per-atom variant of the mixed kernel meets the force tolerance."""
    w = lj32k
    m = make_gpu(w, "mixed")
    m.set_threads_per_atom(tpa)
    o = make_oracle(w)
    m.nlist_update(True)
    o.build_fast()
    m.set_forces(True)
    o.set_forces(True)
    assert force_error(m.get_atoms()["f"], o.get_state()["f"]) <= FORCE_TOL


def test_autotune_leaves_state_unchanged(lj32k):
    m = make_gpu(lj32k, "mixed")
    m.nlist_update(False); m.set_forces(True); m.nlist_update(False)
    m.verlet(0.002, 5)
    before = m.get_atoms()
    tpa = m.autotune()
    assert tpa == 2000 or (tpa // 1000 in (0, 1) and (tpa % 1000) // 10 in (1, 2, 4, 8, 16, 32)
                           and tpa % 10 in (1, 2, 4))
    after = m.get_atoms()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
