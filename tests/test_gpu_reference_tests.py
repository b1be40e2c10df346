"""The reference's own statistical tests of this path, on the GPU.

pyparm/tests.py:218-317 (PairedCollectionTest, RandomHertzianVerletTest):
12 bidisperse (1.0 / 1.4) soft spheres at phi = 0.3 in an OriginBox,
NListed<EpsSigExpAtom, RepulsionPair> with epsilon 1.2, exponent 2, skin 0.4,
masses sigma^3, positions and velocities from numpy's legacy generator seeded
131; CollectionVerlet with dt = 0.01.  reset(): 1000 steps, each followed by
scale_velocities_to_temp(1.0).  testEnergy: 10^4 steps with |dE/E| < 1e-2 per
step, <T> = 1 within 10 %, std(E) / <E> < 1e-2.  Same seeds and tolerances.
"""
import numpy as np
import pytest

from parm_gb300 import System

pytestmark = pytest.mark.gpu


def _fixture():
    N = 12
    sig = np.array([1.0] * (N // 2) + [1.4] * (N - N // 2))
    L = float((np.sum((sig / 2) ** 3) * 4 / 3 * np.pi / 0.3) ** (1 / 3))
    rs = np.random.RandomState(131)
    x, v = [], []
    for s in sig:
        x.append(rs.uniform(0.0, L, size=(3,)))
        v.append(rs.normal(size=(3,)) / s ** 3)
        rs.normal(size=(3,))
    m = sig ** 3
    params = np.stack([np.full(N, 1.2), sig, np.full(N, 2.0)], 1)
    return np.array(x), np.array(v), m, params, L


def _temp(v, m):
    """Collection::temp(minuscomv=True) (src/collection.cpp:116-142)."""
    com = (v * m[:, None]).sum(0) / m.sum()
    cv = v - com
    ke = float((m / 2 * (cv * cv).sum(1)).sum())
    ndof = 3 * len(m) - 3
    return ke * 2 / ndof


def test_random_hertzian_verlet_energy():
    x, v, m, params, L = _fixture()
    g = System([len(m)], ndim=3, precision="fp64")
    g.set_boxes(np.full((1, 3), L))
    g.set_atoms(x=x, v=v, a=np.zeros_like(x), f=np.zeros_like(x), m=m)
    g.set_interaction(1, params, 0.4)
    g.nlist_update(True)                                    # resetPositions: update_list(True)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)   # Collection::initialize
    dt = 0.01

    def rescale():
        st = g.get_atoms(2 | 16)
        vv = st["v"] * np.sqrt(1.0 / _temp(st["v"], m))
        g.set_atoms(v=vv)

    rescale()
    for _ in range(1000):                                   # reset()
        g.verlet(dt, 1)
        rescale()
    E = lambda: g.energy()[0] + g.kinetic_energy()[0]
    lastE = E()
    ekut = []
    for _ in range(1000):
        for _ in range(10):
            g.verlet(dt, 1)
            e = E()
            assert e == pytest.approx(lastE, rel=1e-2)
            lastE = e
        st = g.get_atoms(2 | 16)
        ekut.append((E(), _temp(st["v"], m)))
    ekut = np.array(ekut)
    assert np.mean(ekut[:, 1]) == pytest.approx(1.0, rel=1e-1)
    assert np.std(ekut[:, 0]) / np.mean(ekut[:, 0]) == pytest.approx(0.0, abs=1e-2)
