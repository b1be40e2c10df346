"""CPU checks of the oracle restatement itself (no GPU needed)."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from parm_gb300 import workloads as W


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("ndim", [2, 3])
def test_celllist_pairs_equal_reference_loop(kind, ndim):
    """The cell-list pair construction reproduces update_list(true)'s O(N^2) pair set and order."""
    w = W.small_random(n=400, ndim=ndim, kind=kind, seed=11 * kind + ndim)
    o = Oracle(w.n, ndim)
    o.set_box(w.L[0])
    o.set_state(x=w.x, v=w.v, m=w.m)
    o.set_interaction(w.kind, w.params, w.skin)
    o.nl_update(True)
    assert np.array_equal(o.pairs(), o.pairs_celllist())


def test_sqrt_of_square_is_identity():
    """sqrt(e*e) == e in binary64: uniform epsilons may skip the sqrt(e_i*e_j) of the pair ctor."""
    rng = np.random.default_rng(0)
    e = np.concatenate([rng.uniform(0, 10, 200000), np.exp(rng.uniform(-300, 300, 200000))])
    assert np.array_equal(np.sqrt(e * e), e)
    s = rng.uniform(0.1, 5, 100000)
    assert np.array_equal((s + s) / 2, s)


def test_unwrapped_min_image_and_tie_rule():
    """OriginBox::diff is IEEE remainder on unwrapped coordinates (ties to the even quotient)."""
    import math
    L = 3.0
    for d, want in [(1.5, 1.5), (-1.5, -1.5), (4.5, -1.5), (7.5, 1.5), (3.0, 0.0), (10.1, 10.1 - 3 * L)]:
        assert math.remainder(d, L) == pytest.approx(want, abs=1e-12)


def _scale_to_temp(o, T, ndim):
    st = o.get_state()
    v, m = st["v"], st["m"]
    mob = (m > 0) & np.isfinite(m)
    com = (v[mob] * m[mob, None]).sum(0) / m[mob].sum()
    ke = 0.5 * (m[mob, None] * (v[mob] - com) ** 2).sum()
    ndof = ndim * mob.sum() - ndim
    t = ke * 2 / ndof
    v[mob] *= np.sqrt(T / t)
    o.set_state(v=v)


def _temp(o, ndim):
    st = o.get_state()
    v, m = st["v"], st["m"]
    com = (v * m[:, None]).sum(0) / m.sum()
    return o.kinetic_energy(com) * 2 / (ndim * len(m) - ndim)


def hertzian_fixture(N=12, phi=0.3):
    """PairedCollectionTest set-up (pyparm/tests.py:218-281): bidisperse 1.0/1.4, Repulsion skin 0.4."""
    sig = np.array([1.0] * (N // 2) + [1.4] * (N - N // 2))
    masses = sig ** 3
    L = float((np.sum((sig / 2) ** 3) * 4 / 3 * np.pi / phi) ** (1 / 3))
    np.random.seed(131)
    x = np.zeros((N, 3)); v = np.zeros((N, 3)); f = np.zeros((N, 3))
    for i, m in enumerate(masses):
        x[i] = np.random.uniform(0.0, L, size=(3,))
        v[i] = np.random.normal(size=(3,)) / m
        f[i] = np.random.normal(size=(3,))
    params = np.stack([np.full(N, 1.2), sig, np.full(N, 2.0)], 1)
    return L, x, v, f, masses, params


def test_oracle_random_hertzian_verlet():
    """Port of RandomHertzianVerletTest (pyparm/tests.py:284-317) on the oracle (shortened 10x)."""
    L, x, v, f, m, params = hertzian_fixture()
    o = Oracle(12, 3)
    o.set_box([L] * 3)
    o.set_state(x=x, v=v, a=np.zeros_like(x), f=f, m=m)
    o.set_interaction(1, params, 0.4)
    o.nl_update(True)
    o.initialize()
    # reset(): positions again, T=1, 1000 steps rescaling each step
    o.set_state(x=x, v=v, f=f)
    o.nl_update(True)
    _scale_to_temp(o, 1.0, 3)
    for _ in range(1000):
        o.verlet(0.01, 1)
        _scale_to_temp(o, 1.0, 3)
    E = lambda: o.energy() + o.kinetic_energy()
    lastE = E()
    Es, Ts = [], []
    for _ in range(100):
        for _ in range(10):
            o.verlet(0.01, 1)
            assert E() == pytest.approx(lastE, rel=1e-2)
            lastE = E()
        Es.append(E())
        Ts.append(_temp(o, 3))
    assert np.mean(Ts) == pytest.approx(1.0, rel=0.1 * 3)  # 100 samples instead of 1000
    assert np.std(Es) / np.mean(Es) == pytest.approx(0.0, abs=1e-2)
