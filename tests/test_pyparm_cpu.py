"""The host side of the pyparm-compatible layer (parm_gb300/pyparm.py): atoms and their pickled
state, the boxes' minimum images against the C library's round / remainder, shears, atom parameter
records in the C ABI's layout.  (The GPU side: tests/test_gpu_pyparm.py.)"""
import ctypes
import ctypes.util
import math
import pickle

import numpy as np
import pytest

from parm_gb300 import capi, pyparm

libm = ctypes.CDLL(ctypes.util.find_library("m"))
libm.round.restype = ctypes.c_double
libm.round.argtypes = [ctypes.c_double]


def test_round_half_away_matches_c():
    rng = np.random.default_rng(1)
    vals = list(rng.normal(0, 10, 2000)) + [0.5, -0.5, 1.5, -2.5, 0.49999999999999994, -0.49999999999999994,
                                            2.0 ** 52 + 0.5, 1e300, -0.0, 0.0, 4503599627370495.5]
    for v in vals:
        assert pyparm._round_half_away(v) == libm.round(v), v


@pytest.mark.parametrize("sim", [pyparm.d2, pyparm.d3])
def test_atoms_state_and_pickling(sim):
    nd = sim.NDIM
    atoms = sim.AtomVec([1.0, 2.0, np.inf])
    atoms[1].x = np.arange(nd) + 0.5
    atoms[2].v = np.ones(nd)
    assert atoms.version > 0 and len(atoms) == 3 and atoms.getmass(1) == 2.0
    assert [a.n() for a in atoms] == [0, 1, 2]
    again = pickle.loads(pickle.dumps(atoms))
    assert np.array_equal(again.rec, atoms.rec)
    # immobile atoms carry no kinetic energy
    assert atoms.kinetic_energy() == 0.0


@pytest.mark.parametrize("sim", [pyparm.d2, pyparm.d3])
def test_box_minimum_images(sim):
    nd = sim.NDIM
    rng = np.random.default_rng(2)
    box = sim.OriginBox(7.3)
    for _ in range(200):
        r1, r2 = rng.uniform(-20, 20, nd), rng.uniform(-20, 20, nd)
        d = box.diff(r1, r2)
        assert np.array_equal(d, [math.remainder(a - b, 7.3) for a, b in zip(r1, r2)])
    le = sim.LeesEdwardsBox(7.3, 0.35)
    for _ in range(200):
        r1, r2 = rng.uniform(-20, 20, nd), rng.uniform(-20, 20, nd)
        d = le.diff(r1, r2)
        dy = r1[1] - r2[1]
        im = int(libm.round(dy / 7.3))
        want_y = dy - im * 7.3
        dx = r1[0] - r2[0]
        want_x = dx - libm.round(dx / 7.3 - im * 0.35) * 7.3 - im * 0.35 * 7.3
        assert d[0] == want_x and d[1] == want_y
        assert np.array_equal(le.diff(r2, r1), -d)


def test_shear_moves_atoms():
    sim = pyparm.d3
    atoms = sim.AtomVec(2)
    atoms[0].x = [1.0, 2.0, 0.0]
    le = sim.LeesEdwardsBox(10.0)
    le.shear(0.25, atoms)
    assert atoms[0].x[0] == 1.0 + 2.0 * 0.25 and le.get_gamma() == 0.25
    le.shear_to(0.5, atoms)
    assert le.get_gamma() == 0.5


def test_atom_records_match_the_abi_layout():
    sim = pyparm.d3
    atoms = sim.AtomVec(3)
    assert sim.EpsSigExpAtom(atoms[0], 1.0, 1.4, 2.5).p == [1.0, 1.4, 2.5]
    assert sim.EpsSigExpDragAtom(atoms[0], 1.0, 1.4, 0.3).p == [1.0, 1.4, 2.5, 0.3]   # exponent default 2.5
    ll = sim.LoisLinAtom(atoms[0], 1.0, 1.2, 0.004, 0.08)
    assert ll.p == [1.0, 1.2, 0.004 / 0.08, 0.08] and len(ll.p) == capi.nparam(capi.LOISLIN)
    ie = sim.IEpsRepsSigExpCutAtom(atoms[1], [1.0, 0.5], 2.0, 1.1, 12.0, 1, 2.5)
    assert ie.p == [1, 2.0, 1.1, 12.0, 2.5] and ie.rows[0] == 1
    assert len(ie.p) == capi.nparam(capi.LJISH)
    with pytest.raises(TypeError):
        sim.Repulsion(sim.OriginBox(5.0), atoms, 0.3).add(sim.EpsSigAtom(atoms[0], 1.0, 1.0))


def test_records_are_read_back_only_when_the_host_reads_them():
    sim = pyparm.d3
    atoms = sim.AtomVec([1.0, 2.0, 3.0, 4.0])

    class DeviceStub:   # stands in for a NeighborList whose device holds newer records
        fetches = 0

        def _fetch(self):
            DeviceStub.fetches += 1
            atoms._rec[:, 0] = 7.0
            atoms.touch()

    atoms._dev = DeviceStub()
    assert len(atoms) == 4 and atoms.getmass(2) == 3.0 and atoms.mass() == 10.0
    assert DeviceStub.fetches == 0           # sizes and masses never change on the device
    assert atoms[1].x[0] == 7.0
    assert DeviceStub.fetches == 1
    atoms[2].x = [1.0, 2.0, 3.0]
    assert DeviceStub.fetches == 1 and atoms._dev is None


def test_atom_group_quantities():
    sim = pyparm.d3
    atoms = sim.AtomVec([1.0, 2.0, 0.0, float("inf")])
    xs = np.array([[1.0, 0, 0], [0, 3.0, 0], [5.0, 5.0, 5.0], [7.0, 7.0, 7.0]])
    for a, x in zip(atoms, xs):
        a.x = x
        a.v = [1.0, 2.0, 3.0]
    np.testing.assert_allclose(atoms.com(), [1 / 3, 2.0, 0.0])   # mobile atoms only
    np.random.seed(5)
    atoms.randomize_velocities(2.0)
    v = atoms.rec[:, 3:6]
    assert np.array_equal(v[2], [1.0, 2.0, 3.0]) and np.array_equal(v[3], [1.0, 2.0, 3.0])
    assert np.all(np.isfinite(v)) and not np.array_equal(v[0], [1.0, 2.0, 3.0])
    atoms.add_velocity([1.0, 0.0, 0.0])
    assert atoms.rec[2, 3] == 2.0
    assert atoms.gyradius() == pytest.approx(np.sqrt(np.sum((xs - xs.mean(axis=0)) ** 2) / 4))
    box = sim.OriginBox([2.0, 2.0, 4.0])
    box.resize_to_L(4.0)
    np.testing.assert_allclose(box.V(), 64.0)


def test_interaction_and_collection_checks():
    """The layer's checks that run before any device call (the C++ host API raises the same ones)."""
    sim = pyparm.d3
    box = sim.OriginBox(10.0)
    atoms = sim.AtomVec([1.0] * 4)
    rep = sim.Repulsion(box, atoms, 0.3)
    rep.add(sim.EpsSigExpAtom(atoms[0], 1.0, 1.0, 2.0))
    with pytest.raises(ValueError):        # an atom added twice
        rep.add(sim.EpsSigExpAtom(atoms[0], 1.0, 1.0, 2.0))
    with pytest.raises(TypeError):         # an atom type of another interaction
        rep.add(sim.EpsSigCutAtom(atoms[1], 1.0, 1.0, 2.5))
    with pytest.raises(ValueError):        # a second NListed on the same neighbour list
        other = sim.LJRepulse(atoms, rep.neighbor_list())
        other.add(sim.EpsSigAtom(atoms[2], 1.0, 1.0))
    with pytest.raises(ValueError):        # constraints are outside the GPU path
        sim.CollectionVerlet(box, atoms, 0.01, [rep], [rep.neighbor_list()], [object()])
    rep2 = sim.Repulsion(box, atoms, 0.3)
    with pytest.raises(ValueError):        # one neighbour list per Collection
        sim.CollectionVerlet(box, atoms, 0.01, [rep, rep2], [], [])
    with pytest.raises(ValueError):        # an interaction of another AtomVec
        sim.CollectionVerlet(box, sim.AtomVec([1.0] * 4), 0.01, [rep], [], [])
    ii = sim.LJIICut(box, sim.AtomVec([1.0] * 2), 0.3)
    a0, a1 = ii.nl.atoms[0], ii.nl.atoms[1]
    ii.add(sim.IEpsISigCutAtom(a0, [1.0, 0.5], [1.0, 1.1], 0, 2.5))
    with pytest.raises(ValueError):        # atoms of one type index share their rows
        ii.add(sim.IEpsISigCutAtom(a1, [0.9, 0.5], [1.0, 1.1], 0, 2.5))
    with pytest.raises(ValueError):
        sim.CollectionSol(box, atoms, 0.0, 1.0, 1.0, [rep], [], [])   # dt must be positive


def test_records_of_every_atom_type():
    """Each atom type's C ABI record holds the number of parameters its kind takes."""
    sim = pyparm.d3
    atoms = sim.AtomVec([1.0])
    a = atoms[0]
    cases = {
        sim.LJRepulse: sim.EpsSigAtom(a, 1.0, 1.1),
        sim.LJCut: sim.EpsSigCutAtom(a, 1.0, 1.1, 2.5),
        sim.Repulsion: sim.EpsSigExpAtom(a, 1.0, 1.1, 2.5),
        sim.HertzianDrag: sim.EpsSigExpDragAtom(a, 1.0, 1.1, 0.3),
        sim.LoisOhern: sim.LoisOhernAtom(a, 1.0, 1.1, 0.2, 0.1),
        sim.LoisLin: sim.LoisLinAtom(a, 1.0, 1.1, 0.2, 0.1),
        sim.EisMclachlan: sim.EisMclachlanAtom(a, 1.5, 0.2),
        sim.LJAttractRepulseSigs: sim.EpsEpsSigSigCutAtom(a, 1.0, 0.5, 1.0, 1.2, 2.5),
        sim.LJAttractICut: sim.IEpsSigCutAtom(a, [1.0, 0.5], 1, 1.1, 2.5),
        sim.LJAttractFixedRepulse: sim.IEpsRepsSigCutAtom(a, [1.0, 0.5], 0.7, 1.1, 1, 2.5),
        sim.LJish: sim.IEpsRepsSigExpCutAtom(a, [1.0, 0.5], 0.7, 1.1, 6.0, 1, 2.5),
        sim.RepulsionII: sim.IEpsISigExpAtom(a, [1.0, 0.5], [1.0, 1.2], 1, 2.0),
    }
    for cls, atom in cases.items():
        kind = next(iter(cls.kinds.values()))
        assert type(atom) in cls.kinds
        assert len(atom.p) >= capi.nparam(kind), (cls.__name__, atom.p)
        assert atom.max_size() > 0
    drag = cases[sim.HertzianDrag]
    assert drag.p == [1.0, 1.1, 2.5, 0.3]   # (eps, sigma, exponent, gamma): exponent defaults to 2.5
    lin = cases[sim.LoisLin]
    assert lin.p[2] == pytest.approx(2.0) and lin.p[3] == 0.1   # f = depth / width
