"""Batched (ragged) systems in one handle: every system equals its own single-system run."""
import numpy as np
import pytest

from helpers import force_error, make_gpu, make_oracle
from parm_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_batched_packings_fp64_bit_exact():
    """Damped minimisation steps of 12 harmonic packings of uneven N, per-system boxes."""
    w = W.packings(nsys=12, nmin=64, nmax=700, exponent=2.0, seed=41, skin=0.15)
    g = make_gpu(w)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    g.damped(0.01, 1.0, 120)
    st = g.get_atoms()
    which = g.which()
    for s in range(len(w.sizes)):
        o = make_oracle(w, sys=s)
        o.initialize()
        o.damped(0.01, 1.0, 120)
        ref = o.get_state()
        off = int(sum(w.sizes[:s]))
        sl = slice(off, off + w.sizes[s])
        for k in ("x", "v", "a", "f"):
            assert np.array_equal(st[k][sl], ref[k]), (s, k)
        assert which[s] == o.which(), s
        assert np.array_equal(g.pairs(s) - off, o.pairs())


def test_batched_energies_and_counts():
    w = W.packings(nsys=7, nmin=100, nmax=400, exponent=2.5, seed=42, skin=0.1)
    g = make_gpu(w)
    g.nlist_update(True)
    E = g.energy()
    C = g.contacts()
    npairs = g.numpairs()
    for s in range(len(w.sizes)):
        o = make_oracle(w, sys=s)
        o.nl_update(True)
        assert E[s] == pytest.approx(o.energy(), rel=1e-12)
        assert C[s] == o.contacts()
        assert npairs[s] == len(o.pairs())


def test_batched_wca_sol_mixed():
    """Batched Langevin replicas, mixed precision: forces per replica within tolerance."""
    w = W.wca_replicas(nrep=6, nmin=256, nmax=3000, seed=43)
    m = make_gpu(w, "mixed")
    m.nlist_update(True)
    m.set_forces(True)
    F = m.get_atoms()["f"]
    for s in range(len(w.sizes)):
        o = make_oracle(w, sys=s)
        o.nl_update(True)
        o.set_forces(True)
        off = int(sum(w.sizes[:s]))
        err = force_error(F[off:off + w.sizes[s]], o.get_state()["f"])
        assert err <= 1e-5, (s, err)
    m.sol(0.001, 1.0, 1.0, 5, 50)
    st = m.get_atoms()
    assert np.all(np.isfinite(st["x"]))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_frozen_systems_keep_their_state(precision):
    """parm_set_active: frozen systems do not move; the others step as if alone."""
    w = W.packings(nsys=4, nmin=200, nmax=500, exponent=2.0, seed=44, skin=0.15)
    g = make_gpu(w, precision)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    g.damped(0.01, 1.0, 10)
    frozen = g.get_atoms()
    g.set_active([True, False, True, True])
    g.damped(0.01, 1.0, 25)
    st = g.get_atoms()
    off = np.cumsum([0] + w.sizes)
    sl = slice(off[1], off[2])
    for k in ("x", "v", "a", "f"):
        assert np.array_equal(st[k][sl], frozen[k][sl]), k
    g.set_active([True] * 4)
    if precision == "fp64":
        # the systems that kept stepping equal their own 35-step runs
        for s in (0, 2, 3):
            o = make_oracle(w, sys=s)
            o.initialize()
            o.damped(0.01, 1.0, 35)
            ref = o.get_state()
            for k in ("x", "v"):
                assert np.array_equal(st[k][off[s]:off[s + 1]], ref[k]), (s, k)


@pytest.mark.parametrize("tpa", [200, 1, 2, 4, 101, 104])
def test_batched_soft_spheres_every_kernel(tpa):
    """Small uneven systems (3 cells per axis at N = 64), exponent 2.5, every mixed kernel variant."""
    w = W.packings(nsys=24, nmin=64, nmax=1200, exponent=2.5, seed=45, skin=0.1)
    m = make_gpu(w, "mixed")
    m.set_threads_per_atom(tpa)
    m.nlist_update(True)
    m.set_forces(True)
    F = m.get_atoms()["f"]
    off = np.cumsum([0] + w.sizes)
    for s in range(len(w.sizes)):
        o = make_oracle(w, sys=s)
        o.nl_update(True)
        o.set_forces(True)
        err = force_error(F[off[s]:off[s + 1]], o.get_state()["f"])
        assert err <= 1e-5, (s, w.sizes[s], err)
    m.damped(0.01, 1.0, 300)
    st = m.get_atoms()
    assert np.isfinite(st["x"]).all() and np.isfinite(st["f"]).all()
