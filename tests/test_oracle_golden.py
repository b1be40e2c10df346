"""The oracle against the reference's own outputs (CPU).

The fixtures were produced by the reference's sources compiled as they are
(``tests/golden/make_golden.py``); the oracle must reproduce every recorded
number bit for bit: the neighbour list (its order too), forces and
accelerations, energy, pressure, stress, contact and overlap counts, and the
trajectories of CollectionVerlet, CollectionDamped and CollectionSol (T = 0),
and the conjugate-gradient minimisers CollectionNLCG (box included) and
CollectionNLCGV with their scalar state.
"""
import numpy as np
import pytest

from golden_cases import DAMPED, NLCG, NLCGV, SOL, VERLET, load, names
from oracle.oracle import NLCG_STATE, Oracle, OracleNLCG

CASES = names()


def replay(d):
    o = Oracle(d["n"], d["ndim"])
    o.set_box(d["L"])
    if "le_gamma" in d:
        o.set_lees_edwards(float(d["le_gamma"]))
    o.set_state(x=d["x"], v=d["v"], m=d["m"])
    if "pair_eps" in d:
        o.set_pair_table(d["pair_eps"], d["pair_sig"])
    o.set_interaction(d["kind"], d["params"], d["skin"], order=[int(i) for i in d["order"]])
    for a, b in d["ignores"]:
        o.ignore(int(a), int(b))
    o.nl_update(True)
    return o


def minimiser(o, d):
    """Collection set-up of the conjugate-gradient cases, as the fixture driver does it."""
    if d["integ"] == NLCG:
        g = OracleNLCG(o, d["cg"], boxed=True)
        g.set_forces(True)
    else:
        g = OracleNLCG(o, d["cg"], boxed=False)
        g.reset()
    return g


def step_to(o, d, done, target, g=None):
    k = target - done
    if k <= 0:
        return
    if g is not None:
        g.timestep(k)
    elif d["integ"] == VERLET:
        o.verlet(d["dt"], k)
    elif d["integ"] == DAMPED:
        o.damped(d["dt"], d["damping"], k)
    else:
        assert d["T"] == 0.0
        o.sol(d["dt"], d["damping"], 0.0, seed=1, step0=done, nsteps=k)


def test_fixtures_present():
    assert len(CASES) >= 8, CASES


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    d = load(name)
    o = replay(d)
    np.testing.assert_array_equal(o.pairs(), d["pairs"])
    o.initialize()
    g = minimiser(o, d) if d["integ"] >= NLCG else None
    st = o.get_state()
    np.testing.assert_array_equal(st["f"], d["f0"])
    np.testing.assert_array_equal(st["a"], d["a0"])
    assert o.energy() == d["init"][0]
    p, stress = o.pressure()
    assert p == d["init"][1]
    np.testing.assert_array_equal(stress, d["stress"])
    assert o.contacts() == d["init_counts"][0]
    assert o.overlaps() == d["init_counts"][1]
    assert o.which() == d["init_counts"][2]
    done = 0
    for i, s in enumerate(d["steps"]):
        step_to(o, d, done, int(s), g)
        done = int(s)
        if g is not None:
            np.testing.assert_array_equal(g.box(), d["box_steps"][i], err_msg=f"box at step {s}")
            state = g.state()
            np.testing.assert_array_equal([state[k] for k in NLCG_STATE], d["cg_state_steps"][i],
                                          err_msg=f"minimiser state at step {s}")
        st = o.get_state()
        for key in ("x", "v", "a", "f"):
            np.testing.assert_array_equal(st[key], d[f"{key}_steps"][i], err_msg=f"{key} at step {s}")
        assert o.which() == d["which_steps"][i]
        assert o.energy() == d["energy_steps"][i]
        assert o.kinetic_energy() == d["ke_steps"][i]


def test_boundary_fixture_semantics():
    """Atoms at exactly +-L/2 pair through the boundary; |r| == cut + skin is excluded."""
    d = load("edges64_pairs")
    from golden_cases import pair_set
    P = pair_set(d["pairs"])
    assert (2, 3) not in P          # separated by exactly 2.5 = cut + skin
    assert (4, 5) in P              # 2.5 - 2**-40
    assert (0, 1) in P              # through the +-L/2 faces, unwrapped by 3 L
