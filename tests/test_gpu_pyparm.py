"""The pyparm-compatible layer (parm_gb300/pyparm.py) on the GPU:

* the reference's own RandomHertzianVerletTest (pyparm/tests.py:218-317) written against it, with
  the reference's seeds and tolerances (fewer outer iterations);
* golden fixtures replayed through it: the Verlet and damped trajectories bit for bit, the
  conjugate-gradient minimiser to rounding, a Lees-Edwards box and indexed epsilons;
* a neighbour list iterated as the reference's Python layer iterates it (NeighborList.__iter__).
"""
import numpy as np
import pytest

from golden_cases import DAMPED, NLCG, NLCGV, VERLET, load
from parm_gb300 import capi, pyparm

pytestmark = pytest.mark.gpu


class _RandomHertzianVerlet:
    """PairedCollectionTest's set-up with RandomHertzianVerletTest's parameters."""
    N, phi, seed, dt = 12, 0.3, 131, 0.01

    def sigmas(self):
        return [1.0] * (self.N // 2) + [1.4] * (self.N - self.N // 2)

    def masses(self):
        return [s ** 3 for s in self.sigmas()]

    def __init__(self):
        sim = pyparm.d3
        np.random.seed(self.seed)
        V = np.sum((np.asarray(self.sigmas()) / 2.0) ** 3) * 4 / 3 * np.pi / self.phi
        self.L = float(V ** (1.0 / 3.0))
        self.box = sim.OriginBox(self.L)
        self.atoms = sim.AtomVec(self.masses())
        self.interaction = sim.Repulsion(self.box, self.atoms, 0.4)
        for a, sg in zip(self.atoms, self.sigmas()):
            self.interaction.add(sim.EpsSigExpAtom(a, 1.2, sg, 2.0))
        self.reset_positions()
        self.collec = sim.CollectionVerlet(self.box, self.atoms, self.dt, [self.interaction],
                                           [self.interaction.neighbor_list()], [])

    def reset_positions(self):
        np.random.seed(131)
        for a, m in zip(self.atoms, self.masses()):
            a.x = np.random.uniform(0.0, self.L, size=(3,))
            a.v = np.random.normal(size=(3,)) / m
            a.f = np.random.normal(size=(3,))
        self.interaction.neighbor_list().update_list(True)

    def reset(self):
        self.reset_positions()
        self.collec.scale_velocities_to_temp(1.0)
        for _ in range(1000):
            self.collec.timestep()
            self.collec.scale_velocities_to_temp(1.0)


def test_random_hertzian_verlet_energy():
    t = _RandomHertzianVerlet()
    t.reset()
    collec = t.collec
    EKUTs = []
    lastE = collec.energy()
    for _ in range(1000):
        for _ in range(10):
            collec.timestep()
            assert collec.energy() == pytest.approx(lastE, rel=1e-2)
            lastE = collec.energy()
        EKUTs.append((collec.energy(), collec.kinetic_energy(), collec.potential_energy(), collec.temp()))
    E, K, U, T = np.asarray(EKUTs).T
    assert np.mean(T) == pytest.approx(1.0, rel=1e-1)
    assert abs(np.std(E) / np.mean(E)) <= 1e-2


def test_random_hertzian_matches_the_c_abi():
    """The same run through the layer and through System directly: identical trajectories."""
    from parm_gb300 import System
    t = _RandomHertzianVerlet()
    x0, v0 = t.atoms.rec[:, 0:3].copy(), t.atoms.rec[:, 3:6].copy()
    t.collec.timesteps(500)
    s = System([t.N], ndim=3, precision="fp64")
    s.set_boxes(np.full((1, 3), t.L))
    s.set_atoms(x=x0, v=v0, a=np.zeros((t.N, 3)), f=np.zeros((t.N, 3)), m=t.masses())
    s.set_interaction(capi.REPULSION, np.array([[1.2, sg, 2.0] for sg in t.sigmas()]), 0.4)
    s.nlist_update(True)
    s.nlist_update(False)
    s.set_forces(True)
    s.verlet(t.dt, 500)
    st = s.get_atoms()
    np.testing.assert_array_equal(t.atoms.rec[:, 0:3], st["x"])
    np.testing.assert_array_equal(t.atoms.rec[:, 3:6], st["v"])
    s.close()


def test_records_stay_on_the_device_between_calls():
    t = _RandomHertzianVerlet()
    nl = t.interaction.neighbor_list()
    t.collec.timesteps(10)
    assert nl.resident()
    ke, T = t.collec.kinetic_energy(), t.collec.temp()
    assert np.isfinite(t.collec.energy())
    assert nl.resident()            # kinetic energy and momentum are summed on the device
    t.collec.timesteps(5)
    t.collec.timesteps(5)
    x = t.atoms[0].x                # a host read brings the records back
    assert not nl.resident()
    assert np.all(np.isfinite(x))
    t.collec.timesteps(0)
    ke_h = t.collec.kinetic_energy()
    t2 = _RandomHertzianVerlet()     # the same steps with the records read back after each call
    for _ in range(10):
        t2.collec.timestep()
        t2.atoms[0].x
    assert t2.collec.kinetic_energy() == pytest.approx(ke, rel=1e-13)
    assert t2.collec.temp() == pytest.approx(T, rel=1e-13)
    t2.collec.timesteps(10)
    np.testing.assert_array_equal(t2.atoms.rec, t.atoms.rec)
    assert ke_h == pytest.approx(t2.collec.kinetic_energy(), rel=1e-13)


def _build(d, sim):
    n, nd = d["n"], d["ndim"]
    if "le_gamma" in d:
        box = sim.LeesEdwardsBox(d["L"], float(d["le_gamma"]))
    else:
        box = sim.OriginBox(d["L"])
    atoms = sim.AtomVec(d["m"])
    for i in range(n):
        atoms[i].x = d["x"][i]
        atoms[i].v = d["v"][i]
    kind = d["kind"]
    p = d["params"]
    if kind == 0:
        inter = sim.LJCut(box, atoms, d["skin"])
        mk = lambda a, q: sim.EpsSigCutAtom(a, *q)
    elif kind == 1:
        inter = sim.Repulsion(box, atoms, d["skin"])
        mk = lambda a, q: sim.EpsSigExpAtom(a, *q)
    elif kind == 10:
        inter = sim.LJIICut(box, atoms, d["skin"])
        te, ts = d["pair_eps"], d["pair_sig"]
        mk = lambda a, q: sim.IEpsISigCutAtom(a, te[int(q[0])], ts[int(q[0])], int(q[0]), q[1])
    else:
        raise AssertionError(kind)
    for i in d["order"]:
        inter.add(mk(atoms[int(i)], p[int(i)]))
    for a, b in d["ignores"]:
        inter.neighbor_list().ignore(atoms[int(a)], atoms[int(b)])
    return box, atoms, inter


@pytest.mark.parametrize("name", ["lj1000_verlet", "hertz12_verlet", "disks256_damped", "lees_spheres200_damped",
                                  "ljcut_iepsisig216_verlet", "ljmix512_order_excl"])
def test_golden_trajectories(name):
    d = load(name)
    sim = pyparm.d3 if d["ndim"] == 3 else pyparm.d2
    box, atoms, inter = _build(d, sim)
    nl = inter.neighbor_list()
    nl.update_list(True)
    assert nl.numpairs() == len(d["pairs"])
    got = np.array([[p.first().n(), p.last().n()] for p in nl])
    np.testing.assert_array_equal(got, d["pairs"])
    if d["integ"] == VERLET:
        col = sim.CollectionVerlet(box, atoms, d["dt"], [inter], [nl], [])
    else:
        assert d["integ"] == DAMPED
        col = sim.CollectionDamped(box, atoms, d["dt"], d["damping"], [inter], [nl], [])
    nd = d["ndim"]
    # a non-integer exponent calls the device pow: within 1e-12 of the largest entry, else bit for bit
    exact = not (d["kind"] == capi.REPULSION and np.any(d["params"][:, 2] != np.rint(d["params"][:, 2])))

    def close(got, want, what):
        if exact:
            np.testing.assert_array_equal(got, want, err_msg=what)
        else:
            assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max(), what
    close(atoms.rec[:, 3 * nd:4 * nd], d["f0"], "initial forces")
    done = 0
    for i, step in enumerate(d["steps"]):
        col.timesteps(int(step) - done)
        done = int(step)
        close(atoms.rec[:, 0:nd], d["x_steps"][i], f"x at step {step}")
        close(atoms.rec[:, nd:2 * nd], d["v_steps"][i], f"v at step {step}")
        assert nl.which() == d["which_steps"][i]
        assert col.potential_energy() == pytest.approx(d["energy_steps"][i], rel=1e-12, abs=1e-13)


def test_nlcg_packing_matches_reference():
    d = load("nlcg64_pack")
    sim = pyparm.d3
    box, atoms, inter = _build(d, sim)
    nl = inter.neighbor_list()
    nl.update_list(True)
    cg = d["cg"]
    col = sim.CollectionNLCG(box, atoms, cg[0], cg[1], [inter], [nl], [], cg[2], cg[3], int(cg[4]), cg[5])
    col.set_max_alpha(cg[6])
    col.set_max_alpha_fraction(cg[7])
    col.set_max_dx(cg[8])
    col.set_max_step(cg[9])
    col.set_forces(True, True)
    done = 0
    for i, step in enumerate(d["steps"][:6]):   # the first ten steps: to 1e-12
        col.timesteps(int(step) - done)
        done = int(step)
        x = atoms.rec[:, 0:3]
        scale = np.abs(d["x_steps"][i]).max()
        assert np.abs(x - d["x_steps"][i]).max() <= 1e-12 * scale, step
        assert np.abs(box.box_shape() - d["box_steps"][i]).max() <= 1e-12 * d["box_steps"][i].max(), step


def test_rsq_tracker_reference_known_answers():
    """RSQTest (pyparm/tests.py:504-569) through the module: 8 atoms moved by fixed steps."""
    import itertools
    sim = pyparm.d3
    ns = [1, 2, 4, 8, 16, 32]
    dxs = [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [0, 2, 1], [-2.1, 4, 1]]
    np.random.seed(13763)
    radii = np.random.uniform(1.0, 2.0, size=(8,))
    atoms = sim.AtomVec(radii ** 3)
    box = sim.OriginBox(float((np.sum(radii ** 3) * 4 / 3 * np.pi / 0.3) ** (1 / 3)))
    rsqs = sim.RsqTracker(atoms, ns, False)
    drs = []
    for t in range(ns[-1] * 4):
        for i, (a, dr) in enumerate(zip(atoms, itertools.cycle(dxs))):
            a.x += dr
            if t == 0:
                drs.append(dr)
        rsqs.update(box)
    drs = np.asarray(drs, dtype=float)
    for n, r2n, xyz2n, r4n, xyz4n in zip(ns, rsqs.r2(), rsqs.xyz2(), rsqs.r4(), rsqs.xyz4()):
        d = drs * n
        np.testing.assert_allclose(r2n, np.sum(d ** 2, axis=-1), rtol=1e-12)
        np.testing.assert_allclose(xyz2n, d ** 2, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(r4n, np.sum(d ** 2, axis=-1) ** 2, rtol=1e-12)
        np.testing.assert_allclose(xyz4n, d ** 4, rtol=1e-12, atol=1e-12)


def test_rsq_tracker_bound_in_a_collection():
    """A tracker of the Collection's own atoms is updated inside the GPU steps (one call for twelve
    steps); the same tracker standing alone, updated by hand after every step, gives the same results."""
    def run(bound):
        t = _RandomHertzianVerlet()
        sim = pyparm.d3
        rsq = sim.RsqTracker(t.atoms, [1, 3], True)
        nl = t.interaction.neighbor_list()
        trackers = [nl, rsq] if bound else [nl]
        col = sim.CollectionVerlet(t.box, t.atoms, t.dt, [t.interaction], trackers, [])
        if bound:
            assert rsq.nl is nl
            col.timesteps(12)
        else:
            assert rsq.nl is None
            rsq.update(t.box)   # Collection::initialize updates its trackers twice
            rsq.update(t.box)
            for _ in range(12):
                col.timestep()
                rsq.update(t.box)
        return rsq, t.atoms.rec[:, 0:3].copy()
    a, xa = run(True)
    b, xb = run(False)
    np.testing.assert_array_equal(xa, xb)
    assert a.counts() == b.counts()
    for f in ("r2", "xyz2", "r4", "xyz4"):
        for u, v in zip(getattr(a, f)(), getattr(b, f)()):
            np.testing.assert_allclose(u, v, rtol=1e-12, atol=1e-300)


def test_xyz_frames_of_device_resident_atoms():
    """Frames written between device calls hold the positions of the last step (one read-back)."""
    import io
    from parm_gb300.xyzfile import XYZreader, XYZwriter
    t = _RandomHertzianVerlet()
    nl = t.interaction.neighbor_list()
    f = io.StringIO()
    w = XYZwriter(f)
    for k in range(3):
        t.collec.timesteps(10)
        assert nl.resident()
        w.writeframe(t.atoms, time=10 * (k + 1), E=t.collec.energy())
        assert not nl.resident()
    f.seek(0)
    frames = XYZreader(f).all()
    assert [fr.time for fr in frames] == [10.0, 20.0, 30.0]
    np.testing.assert_allclose(frames[-1].locs, t.atoms.rec[:, 0:3], atol=5e-5)
    np.testing.assert_allclose(frames[-1].vels, t.atoms.rec[:, 3:6], atol=5e-5)


def test_rsq_tracker_in_a_minimiser():
    """The conjugate-gradient steps update no tracker themselves: a bound tracker is updated from the
    host after every step, as the reference's update_trackers does."""
    d = load("nlcg64_pack")
    sim = pyparm.d3
    box, atoms, inter = _build(d, sim)
    nl = inter.neighbor_list()
    nl.update_list(True)
    rsq = sim.RsqTracker(atoms, [1, 2], False)
    cg = d["cg"]
    col = sim.CollectionNLCG(box, atoms, cg[0], cg[1], [inter], [nl, rsq], [], cg[2], cg[3], int(cg[4]), cg[5])
    assert rsq.nl is nl
    col.timesteps(6)
    assert rsq.counts() == [8.0, 4.0]   # two updates at construction and one per step, windows of 1 and 2
