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


def _drift(g, steps, every):
    """Least-squares slope of the total energy (per 10^5 steps, relative to |E(0)|) and its standard error."""
    E = [g.energy()[0] + g.kinetic_energy()[0]]
    for _ in range(steps // every):
        g.verlet(0.002, every)
        E.append(g.energy()[0] + g.kinetic_energy()[0])
    E = np.array(E)
    t = np.arange(len(E), dtype=np.float64) * every
    A = np.stack([t, np.ones_like(t)], 1)
    coef = np.linalg.lstsq(A, E, rcond=None)[0]
    resid = E - A @ coef
    se = np.sqrt((resid ** 2).sum() / (len(E) - 2) / ((t - t.mean()) ** 2).sum())
    scale = 1e5 / abs(E[0])
    return coef[0] * scale, se * scale


def test_mixed_nve_drift_comparable(lj32k):
    """NVE energy drift of the mixed path is the FP64 path's: over 20000 steps from the same state the
    fitted slopes (per 10^5 steps, relative) differ by less than three combined standard errors plus
    1e-5, and the mixed slope is below 1e-4."""
    w = lj32k
    out = {}
    for prec in ("fp64", "mixed"):
        g = make_gpu(w, prec)
        g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
        out[prec] = _drift(g, 20000, 100)
        g.close()
    (d64, se64), (d32, se32) = out["fp64"], out["mixed"]
    assert abs(d32 - d64) <= 3 * np.hypot(se32, se64) + 1e-5, out
    assert abs(d32) <= 1e-4, out


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
