"""The oracle's Langevin generator against Philox4x32-10 written from its
published definition, and the moments of the normals drawn from it."""
import math

import numpy as np

from philox_py import edge_rows, philox_rows, random_rows


def test_oracle_philox_matches_published_definition():
    from oracle.oracle import philox
    rows = np.concatenate([edge_rows(), random_rows(3000, 5)])
    assert np.array_equal(philox(rows), philox_rows(rows))


def test_oracle_normals_moments():
    """Box-Muller normals of counters (atom, step, block): mean 0, variance 1,
    uncorrelated components, Gaussian fourth moment (5 standard errors)."""
    from oracle.oracle import normals6
    n = 40000
    g = np.array([normals6(0x1234ABCD5678, 17, i) for i in range(n)])
    z = g.ravel()
    k = z.size
    assert abs(z.mean()) < 5 / math.sqrt(k)
    assert abs(z.var() - 1.0) < 5 * math.sqrt(2.0 / k)
    assert abs((z ** 4).mean() - 3.0) < 5 * math.sqrt(96.0 / k)
    c = np.corrcoef(g.T)
    off = c[~np.eye(6, dtype=bool)]
    assert np.abs(off).max() < 5 / math.sqrt(n)
