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
