"""FP64 GPU path against the oracle: pair sets, forces and trajectories bit-exact."""
import math

import numpy as np
import pytest

from helpers import make_gpu, make_oracle
from parm_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_remainder_matches_ieee():
    """The device minimum image equals IEEE remainder, ties and signed zeros included."""
    from parm_gb300 import debug_remainder
    rng = np.random.default_rng(1)
    n = 20000
    L = rng.uniform(0.5, 200, n)
    d = rng.uniform(-5, 5, n) * L
    k = rng.integers(-7, 8, 2000)
    d[:2000] = L[:2000] * (k + 0.5)                                  # exact ties
    d[2000:4000] = np.nextafter(L[2000:4000] * 0.5, 0)               # just below half a box
    d[4000:6000] = np.nextafter(L[4000:6000] * (k + 0.5), np.inf)    # just above a tie
    d[6000:6100] = L[6000:6100] * rng.integers(-5, 6, 100)           # exact multiples (signed zeros)
    d[6100:6200] = -d[6000:6100]
    d = np.concatenate([[1.5, -1.5, 4.5, -4.5, 7.5, 0.0, -0.0, 1e10], d])
    L = np.concatenate([[3.0] * 7, [7.0], L])
    got = debug_remainder(d, L)
    want = np.array([math.remainder(a, b) for a, b in zip(d, L)])
    assert np.array_equal(got, want)
    assert np.array_equal(np.signbit(got), np.signbit(want))


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
@pytest.mark.parametrize("ndim", [2, 3])
def test_pairs_and_forces_bit_exact(kind, ndim):
    w = W.small_random(n=500, ndim=ndim, kind=kind, seed=3 * kind + ndim, phi=0.45)
    g = make_gpu(w)
    o = make_oracle(w)
    g.nlist_update(True)
    o.nl_update(True)
    assert np.array_equal(g.pairs(), o.pairs())
    assert g.which()[0] == o.which() == 1
    assert g.numpairs()[0] == len(o.pairs())
    g.set_forces(True)
    o.set_forces(True)
    st = g.get_atoms()
    ref = o.get_state()
    assert np.array_equal(st["f"], ref["f"])
    assert np.array_equal(st["a"], ref["a"])
    assert g.energy()[0] == pytest.approx(o.energy(), rel=1e-12, abs=1e-12)
    p, stress = o.pressure()
    assert g.virial()[0] == pytest.approx(p, rel=1e-12, abs=1e-12)
    np.testing.assert_allclose(g.stress()[0], stress, rtol=1e-12, atol=1e-12)
    assert g.contacts()[0] == o.contacts()
    assert g.overlaps()[0] == o.overlaps()


def test_insertion_order_exclusions_and_nonmembers():
    """NeighborList rank = insertion order fixes the pair order; ignore() and partial membership."""
    w = W.small_random(n=300, ndim=3, kind=1, seed=5, phi=0.5)
    rng = np.random.default_rng(9)
    order = [int(i) for i in rng.permutation(w.n)[:250]]       # 50 atoms never added
    rank = np.full(w.n, 0xFFFFFFFF, dtype=np.uint32)
    rank[order] = np.arange(len(order))
    g = make_gpu(w, rank=rank)
    o = make_oracle(w, order=order)
    excl = [(order[0], order[1]), (order[5], order[17]), (3, 4)]
    for a, b in excl:
        g.ignore(a, b)
        o.ignore(a, b)
    g.nlist_update(False)   # ignorechanged forces the rebuild
    o.nl_update(False)
    assert np.array_equal(g.pairs(), o.pairs())
    g.set_forces(True)
    o.set_forces(True)
    assert np.array_equal(g.get_atoms()["f"], o.get_state()["f"])


def test_verlet_lj_config0_bit_exact():
    """Config 0: 1000 LJ atoms, CollectionVerlet dt=0.001, 1000 steps."""
    w = W.lj_lattice()
    g = make_gpu(w)
    o = make_oracle(w)
    # Collection::initialize
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    o.initialize()
    for chunk in (1, 9, 90, 900):
        g.verlet(0.001, chunk)
        o.verlet(0.001, chunk)
        st, ref = g.get_atoms(), o.get_state()
        for k in ("x", "v", "a", "f"):
            assert np.array_equal(st[k], ref[k]), (chunk, k)
        assert g.which()[0] == o.which()
    assert g.energy()[0] == pytest.approx(o.energy(), rel=1e-12)
    assert g.kinetic_energy()[0] == pytest.approx(o.kinetic_energy(), rel=1e-12)
    assert o.which() > 5   # the run exercises rebuilds


@pytest.mark.parametrize("ndim", [2, 3])
def test_damped_harmonic_bit_exact(ndim):
    w = W.small_random(n=400, ndim=ndim, kind=1, seed=21, phi=0.8, exponent=2.0, skin=0.2)
    g = make_gpu(w)
    o = make_oracle(w)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    o.initialize()
    g.damped(0.01, 1.0, 200)
    o.damped(0.01, 1.0, 200)
    st, ref = g.get_atoms(), o.get_state()
    for k in ("x", "v", "a", "f"):
        assert np.array_equal(st[k], ref[k]), k
    assert g.which()[0] == o.which()


def test_hertz_exponent_2p5_close():
    w = W.small_random(n=400, ndim=3, kind=1, seed=22, phi=0.7, exponent=2.5, skin=0.2)
    g = make_gpu(w)
    o = make_oracle(w)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    o.initialize()
    g.damped(0.01, 1.0, 50)
    o.damped(0.01, 1.0, 50)
    st, ref = g.get_atoms(), o.get_state()
    np.testing.assert_allclose(st["x"], ref["x"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(st["f"], ref["f"], rtol=1e-9, atol=1e-10)


def test_sol_langevin_matches_oracle_generator():
    """CollectionSol with the counter-based noise: same draws in the oracle."""
    from oracle.oracle import splitmix64
    w = W.small_random(n=300, ndim=3, kind=2, seed=23, phi=0.4, bidisperse=False)
    w.params[:, 0] = 1.0
    g = make_gpu(w)
    o = make_oracle(w)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    o.initialize()
    step0 = g.step_counter() + 1
    g.sol(0.001, 1.0, 1.0, 77, 10)
    o.sol(0.001, 1.0, 1.0, splitmix64(77), step0, 10)
    st, ref = g.get_atoms(), o.get_state()
    np.testing.assert_allclose(st["x"], ref["x"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(st["v"], ref["v"], rtol=1e-10, atol=1e-11)
    assert g.which()[0] == o.which()


def test_kinetic_momentum():
    w = W.small_random(n=257, ndim=3, kind=0, seed=24)
    w.m[5] = 0.0
    w.m[7] = np.inf
    g = make_gpu(w)
    o = make_oracle(w)
    assert g.kinetic_energy()[0] == pytest.approx(o.kinetic_energy(), rel=1e-13)
    mom, mass = g.momentum()
    ref, rmass = o.momentum()
    np.testing.assert_allclose(mom[0], ref, rtol=1e-12, atol=1e-12)
    assert mass[0] == pytest.approx(rmass, rel=1e-14)
    org = np.array([[0.1, -0.2, 0.3]])
    assert g.kinetic_energy(org)[0] == pytest.approx(o.kinetic_energy(org[0]), rel=1e-13)


def test_immobile_atoms_verlet():
    w = W.small_random(n=200, ndim=3, kind=1, seed=25, phi=0.6)
    w.m[:10] = 0.0
    w.m[10:12] = np.inf
    w.m[12] = -1.0
    g = make_gpu(w)
    o = make_oracle(w)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    o.initialize()
    g.verlet(0.005, 30)
    o.verlet(0.005, 30)
    st, ref = g.get_atoms(), o.get_state()
    for k in ("x", "v", "a", "f"):
        assert np.array_equal(st[k], ref[k]), k


def test_large_lattice_pairs_and_forces():
    """Config-1 geometry at 64k atoms: the pair set and forces still match bit for bit."""
    w = W.lj_lattice(shape=(40, 40, 40), skin_prime=0.3, seed=7)
    g = make_gpu(w)
    o = make_oracle(w)
    g.nlist_update(True)
    o.build_fast()
    assert np.array_equal(g.pairs(), o.pairs())
    g.set_forces(True)
    o.set_forces(True)
    assert np.array_equal(g.get_atoms()["f"], o.get_state()["f"])


@pytest.mark.parametrize("graph_steps", [0, 1, 7])
def test_launch_modes_identical(graph_steps):
    """Direct launches (profiling mode) and any graph size give the reference trajectory."""
    w = W.lj_lattice(shape=(8, 8, 8), seed=99)
    g = make_gpu(w)
    g.set_graph_steps(graph_steps)
    o = make_oracle(w)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    o.initialize()
    g.verlet(0.002, 150)
    o.verlet(0.002, 150)
    st, ref = g.get_atoms(), o.get_state()
    for k in ("x", "v", "a", "f"):
        assert np.array_equal(st[k], ref[k]), k
    assert g.which()[0] == o.which() > 2


def test_partial_field_transfers_keep_other_fields():
    """parm_get_atoms writes only the requested fields of the caller's records."""
    from parm_gb300 import capi
    import ctypes as C
    w = W.small_random(n=100, ndim=3, kind=1, seed=50)
    g = make_gpu(w)
    rec = np.full((w.n, 13), 7.0)
    capi.check(g.lib.parm_get_atoms(g.h, rec.ctypes.data_as(C.POINTER(C.c_double)), 13, capi.X))
    assert np.array_equal(rec[:, 0:3], w.x) and np.all(rec[:, 3:] == 7.0)
    rec2 = np.full((w.n, 20), 5.0)
    capi.check(g.lib.parm_get_atoms(g.h, rec2.ctypes.data_as(C.POINTER(C.c_double)), 20, capi.V | capi.M))
    assert np.array_equal(rec2[:, 3:6], w.v) and np.array_equal(rec2[:, 12], w.m)
    assert np.all(rec2[:, 0:3] == 5.0) and np.all(rec2[:, 6:12] == 5.0) and np.all(rec2[:, 13:] == 5.0)
