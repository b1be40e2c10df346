"""The mean-square-displacement oracle against the reference's own known answers.

The reference's RSQTest (pyparm/tests.py:504-569) moves 8 atoms by fixed
steps between tracker updates; after 128 updates every window of n updates
has seen the displacement n * dr exactly.  No GPU needed.
"""
import numpy as np

from oracle.rsq import RsqOracle

RSQ_NS = [1, 2, 4, 8, 16, 32]
RSQ_DXS = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0],
                    [0, 0, 1], [0, 0, -1], [0, 2, 1], [-2.1, 4, 1]], dtype=np.float64)


def rsq_kat_masses():
    rng = np.random.RandomState(13763)
    radii = rng.uniform(1.0, 2.0, size=(8,))
    return radii ** 3


def rsq_kat_positions():
    """Positions after each of the 128 moves (tests.py:533-540)."""
    x = np.zeros((8, 3))
    out = []
    for _ in range(RSQ_NS[-1] * 4):
        x = x + RSQ_DXS
        out.append(x.copy())
    return out


def test_oracle_matches_reference_rsqtest():
    m = rsq_kat_masses()
    o = RsqOracle(np.zeros((8, 3)), m, RSQ_NS, usecom=False)
    for x in rsq_kat_positions():
        o.update(x)
    for j, n in enumerate(RSQ_NS):
        d = RSQ_DXS * n
        np.testing.assert_allclose(o.r2()[j], np.sum(d ** 2, axis=-1), rtol=1e-12)
        np.testing.assert_allclose(o.xyz2()[j], d ** 2, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(o.r4()[j], np.sum(d ** 2, axis=-1) ** 2, rtol=1e-12)
        np.testing.assert_allclose(o.xyz4()[j], d ** 4, rtol=1e-12, atol=1e-12)
        assert o.counts()[j] == 128 // n


def test_oracle_centre_of_mass_removes_common_motion():
    """A uniform translation of every atom is invisible with usecom, fully seen without."""
    rng = np.random.RandomState(5)
    x0 = rng.uniform(-3, 3, size=(20, 3))
    m = rng.uniform(0.5, 2.0, size=20)
    with_com = RsqOracle(x0, m, [1, 2], usecom=True)
    without = RsqOracle(x0, m, [1, 2], usecom=False)
    for t in range(1, 7):
        x = x0 + np.array([0.25, -0.5, 1.0]) * t
        with_com.update(x)
        without.update(x)
    assert np.abs(with_com.r2()).max() < 1e-24
    np.testing.assert_allclose(without.r2()[0], 0.25 ** 2 + 0.5 ** 2 + 1.0, rtol=1e-14)
    np.testing.assert_allclose(without.r2()[1], 4 * (0.25 ** 2 + 0.5 ** 2 + 1.0), rtol=1e-14)
