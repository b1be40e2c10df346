"""The 1,048,576-atom LJ system of the headline measurement itself
(128 x 128 x 64 lattice at rho' = 0.8, cut 2.5 sigma', skin 0.3 sigma'):

* the FP64 GPU path's pair set, forces and accelerations equal the oracle's
  bit for bit at this size;
* the mixed path's pair set and order equal the FP64 path's;
* mixed forces are within max_i |dF_i| / rms |F| <= 1e-5 of the FP64 forces,
  the potential energy within 1e-6 and the virial within 1e-5 (relative).
The NVE energy drift of both paths at this size is measured by bench.py
(fitted slope over 10^4 steps).
"""
import numpy as np
import pytest

from helpers import force_error, make_gpu, make_oracle
from parm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5
ENERGY_TOL = 1e-6


@pytest.fixture(scope="module")
def lj1m():
    return W.lj_lattice(shape=(128, 128, 64), skin_prime=0.3, seed=12345)


def test_lj1m_fp64_bit_exact_with_oracle(lj1m):
    w = lj1m
    g = make_gpu(w, "fp64")
    g.nlist_update(True)
    g.set_forces(True)
    o = make_oracle(w)
    o.build_fast()
    o.set_forces(True)
    pg = g.pairs()
    assert len(pg) == int(g.numpairs()[0])
    assert np.array_equal(pg, o.pairs())
    st, ref = g.get_atoms(), o.get_state()
    assert np.array_equal(st["f"], ref["f"])
    assert np.array_equal(st["a"], ref["a"])
    assert g.energy()[0] == pytest.approx(o.energy(), rel=1e-12)
    g.close()


def test_lj1m_mixed_against_fp64(lj1m):
    w = lj1m
    g64 = make_gpu(w, "fp64")
    m = make_gpu(w, "mixed")
    for g in (g64, m):
        g.nlist_update(True)
        g.set_forces(True)
    assert m.threads_per_atom() == 200           # the cell-block kernels run at this size
    assert np.array_equal(m.pairs(), g64.pairs())
    F64, F32 = g64.get_atoms(8)["f"], m.get_atoms(8)["f"]
    err = force_error(F32, F64)
    assert err <= FORCE_TOL, err
    e64, e32 = g64.energy()[0], m.energy()[0]
    assert abs(e32 - e64) / abs(e64) <= ENERGY_TOL
    v64, v32 = g64.virial()[0], m.virial()[0]
    assert abs(v32 - v64) / abs(v64) <= 1e-5
    g64.close()
    m.close()
