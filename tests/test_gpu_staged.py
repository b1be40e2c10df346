"""Cell-block (staged) kernels of the mixed path.

The staged list build must give the reference's pair set exactly, its forces
must meet the mixed-precision tolerance against the oracle, and switching
between list formats (cell blocks <-> row-major lists) must keep the pairs
and their order, so that forces are bit-identical before and after.
"""
import numpy as np
import pytest

from helpers import force_error, make_gpu, make_oracle
from parm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5
STAGED = 200


def _lj_mix(n_side=16, seed=4):
    """Bidisperse LJ (epsilon, sigma and cut-off per atom): per-atom parameters."""
    w = W.lj_lattice(shape=(n_side,) * 3, skin_prime=0.3, seed=seed)
    rng = np.random.default_rng(seed)
    sg = rng.choice([1.0, 1.15], w.n)
    eps = rng.choice([0.9, 1.1], w.n)
    w.params = np.stack([eps, sg, np.full(w.n, W.LJ_SIGCUT)], 1)
    w.L = w.L * 1.1
    w.x = w.x * 1.1
    return w


CASES = {
    "lj_uniform": lambda: W.lj_lattice(shape=(20, 20, 20), skin_prime=0.3, seed=3),
    "lj_mixed_params": _lj_mix,
    "spheres_sigma": lambda: W.small_random(n=6000, ndim=3, kind=1, seed=31, phi=0.6, exponent=2.5, skin=0.2),
    "wca_uniform": lambda: W.wca_replicas(nrep=1, nmin=8000, nmax=8000, rho_lo=0.8, rho_hi=0.8, seed=32),
    "disks_2d": lambda: W.soft_disks(n=8192, phi=0.84),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_staged_pairs_and_forces(case):
    w = CASES[case]()
    m = make_gpu(w, "mixed")
    assert m.threads_per_atom() == STAGED          # the default where the grids allow
    o = make_oracle(w)
    m.nlist_update(True)
    o.build_fast()
    assert np.array_equal(m.pairs(), o.pairs())
    m.set_forces(True)
    o.set_forces(True)
    err = force_error(m.get_atoms()["f"], o.get_state()["f"])
    assert err <= FORCE_TOL, err
    assert m.energy()[0] == pytest.approx(o.energy(), rel=1e-6)


def test_staged_exclusions_order_nonmembers():
    w = W.small_random(n=5000, ndim=3, kind=1, seed=5, phi=0.55, skin=0.2)
    rng = np.random.default_rng(9)
    order = [int(i) for i in rng.permutation(w.n)[:4700]]
    rank = np.full(w.n, 0xFFFFFFFF, dtype=np.uint32)
    rank[order] = np.arange(len(order))
    m = make_gpu(w, "mixed", rank=rank)
    o = make_oracle(w, order=order)
    for a, b in [(order[0], order[1]), (order[5], order[17]), (3, 4)]:
        m.ignore(a, b)
        o.ignore(a, b)
    m.nlist_update(False)
    o.nl_update(False)
    assert m.threads_per_atom() == STAGED
    assert np.array_equal(m.pairs(), o.pairs())
    m.set_forces(True)
    o.set_forces(True)
    st = m.get_atoms()
    assert force_error(st["f"], o.get_state()["f"]) <= FORCE_TOL
    nonm = np.setdiff1d(np.arange(w.n), order)
    assert np.all(st["f"][nonm] == 0.0) and np.all(st["a"][nonm] == 0.0)


def test_format_switches_keep_forces_bitwise():
    w = CASES["lj_uniform"]()
    m = make_gpu(w, "mixed")
    m.nlist_update(True)
    m.set_forces(False)
    f_st = m.get_atoms()["f"]
    pairs = m.pairs()
    m.set_threads_per_atom(101)      # staged lists -> row-major
    m.set_forces(False)
    f_g = m.get_atoms()["f"]
    assert force_error(f_g, f_st) <= FORCE_TOL
    m.set_threads_per_atom(200)      # row-major -> staged (same order as before)
    m.set_forces(False)
    assert np.array_equal(m.get_atoms()["f"], f_st)
    assert np.array_equal(m.pairs(), pairs)
    m.set_capacity(m.capacity() + 64)  # re-pitched staged lists
    m.set_forces(False)
    assert np.array_equal(m.get_atoms()["f"], f_st)


@pytest.mark.parametrize("cap", [0, 96, 512])
def test_partial_staging_is_bitwise_identical(cap):
    """Neighbourhoods larger than the shared-memory stage read the rest from global memory."""
    w = CASES["spheres_sigma"]()
    m = make_gpu(w, "mixed")
    m.nlist_update(True)
    m.set_forces(False)
    ref = m.get_atoms()["f"]
    ref_pairs = m.pairs()
    m.debug_stage_cap(cap if cap else 32)
    m.nlist_update(True)          # build with the small stage
    assert np.array_equal(m.pairs(), ref_pairs)
    m.set_forces(False)
    assert np.array_equal(m.get_atoms()["f"], ref)
    m.debug_stage_cap(0)


def test_grid_change_falls_back_then_restages():
    """A box change that alters the cell grid keeps the lists (row-major) until every system rebuilds."""
    w = CASES["wca_uniform"]()
    m = make_gpu(w, "mixed")
    m.nlist_update(True)
    m.set_forces(False)
    f0 = m.get_atoms()["f"]
    assert m.threads_per_atom() == STAGED
    L2 = w.L * 1.2                   # more cells per axis; atoms unchanged
    m.set_boxes(L2)
    assert m.threads_per_atom() == 101
    w2 = W.Workload(w.name, w.ndim, w.sizes, L2, w.x, w.v, w.m, w.kind, w.params, w.skin)
    o = make_oracle(w2)
    o.build_fast()
    m.nlist_update(True)             # rebuild on the new grid -> cell blocks again
    assert m.threads_per_atom() == STAGED
    assert np.array_equal(m.pairs(), o.pairs())
    m.set_forces(False)
    o.set_forces(False)
    assert force_error(m.get_atoms()["f"], o.get_state()["f"]) <= FORCE_TOL
    assert not np.array_equal(m.get_atoms()["f"], f0)


def test_staged_nve_matches_gather_statistics():
    """Same trajectory statistics from both kernels over a short NVE run."""
    w = W.lj_lattice(shape=(16, 16, 16), skin_prime=0.3, seed=7)
    E = {}
    for tpa in (200, 101):
        g = make_gpu(w, "mixed")
        g.set_threads_per_atom(tpa)
        g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
        g.verlet(0.002, 200)
        E[tpa] = g.energy()[0] + g.kinetic_energy()[0]
        assert g.threads_per_atom() == tpa
    assert E[200] == pytest.approx(E[101], rel=1e-4)
