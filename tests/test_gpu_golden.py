"""FP64 GPU path against the reference's own outputs (golden fixtures).

Same decks as tests/test_oracle_golden.py, run through the C ABI: the pair
list (order included), forces, accelerations and Verlet / damped / Langevin
(T = 0) trajectories must equal the reference's bit for bit.  Two documented
exceptions: pair laws with a non-integer exponent call the device ``pow``,
which may differ from the host's by an ulp, so those cases are held to
1e-12 relative (scaled by the largest entry of the array); and energies,
pressures and stresses are parallel sums, held to 1e-12 relative.
"""
import numpy as np
import pytest

from golden_cases import DAMPED, NLCG, VERLET, load, names

pytestmark = pytest.mark.gpu

CASES = [n for n in names() if load(n)["integ"] < NLCG]   # the minimiser cases: test_gpu_nlcg.py
RTOL = 1e-12
POW_KINDS = (13, 14, 15, 17)   # LJAttractRepulse, LJAttractFixedRepulse, LJish, LJAttractRepulseSigs


def step_tol(kind, step):
    """The laws that call pow at every pair: the device's pow and the host's differ by an ulp now and
    then, and the dynamics amplifies that (LJish: ~1e-11 after 300 steps); 1e-12 through step 100."""
    return 1e-9 if (kind in POW_KINDS and step > 100) else RTOL


def _close(got, want, exact, what, tol=RTOL):
    if exact:
        np.testing.assert_array_equal(got, want, err_msg=what)
    else:
        scale = max(float(np.abs(want).max()), 1e-300)
        err = float(np.abs(got - want).max()) / scale
        assert err <= tol, f"{what}: relative error {err:.3e}"


def _gpu(d):
    from parm_gb300 import System
    n, nd = d["n"], d["ndim"]
    s = System([n], ndim=nd, precision="fp64")
    s.set_boxes(d["L"][None, :])
    if "le_gamma" in d:
        s.set_lees_edwards([float(d["le_gamma"])])
    s.set_atoms(x=d["x"], v=d["v"], a=np.zeros((n, nd)), f=np.zeros((n, nd)), m=d["m"])
    if "pair_eps" in d:
        s.set_pair_table(d["pair_eps"], d["pair_sig"])
    rank = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
    rank[d["order"]] = np.arange(len(d["order"]), dtype=np.uint32)
    s.set_interaction(d["kind"], d["params"], d["skin"], rank=rank)
    for a, b in d["ignores"]:
        s.ignore(int(a), int(b))
    return s


@pytest.mark.parametrize("name", CASES)
def test_gpu_fp64_matches_reference(name):
    d = load(name)
    ecol = 1 if d["kind"] == 16 else 2   # the exponent's column
    exact = not ((d["kind"] in (1, 9, 16) and np.any(d["params"][:, ecol] != np.rint(d["params"][:, ecol])))
                 or d["kind"] in POW_KINDS)   # laws that call the device pow
    s = _gpu(d)
    s.nlist_update(True)
    np.testing.assert_array_equal(s.pairs(), d["pairs"])
    s.set_forces(True)
    st = s.get_atoms()
    _close(st["f"], d["f0"], exact, "initial forces")
    _close(st["a"], d["a0"], exact, "initial accelerations")
    assert s.energy()[0] == pytest.approx(d["init"][0], rel=RTOL, abs=1e-13)
    assert s.virial()[0] == pytest.approx(d["init"][1], rel=RTOL, abs=1e-13)
    np.testing.assert_allclose(s.stress()[0], d["stress"], rtol=RTOL, atol=1e-13 * np.abs(d["stress"]).max())
    assert s.contacts()[0] == d["init_counts"][0]
    assert s.overlaps()[0] == d["init_counts"][1]
    assert s.which()[0] == d["init_counts"][2]
    done = 0
    for i, step in enumerate(d["steps"]):
        k = int(step) - done
        if d["integ"] == VERLET:
            s.verlet(d["dt"], k)
        elif d["integ"] == DAMPED:
            s.damped(d["dt"], d["damping"], k)
        else:
            s.sol(d["dt"], d["damping"], 0.0, seed=1, nsteps=k)
        done = int(step)
        st = s.get_atoms()
        tol = step_tol(d["kind"], int(step))
        for key in ("x", "v", "a", "f"):
            _close(st[key], d[f"{key}_steps"][i], exact, f"{key} at step {step}", tol)
        assert s.which()[0] == d["which_steps"][i], f"rebuilds at step {step}"
        assert s.energy()[0] == pytest.approx(d["energy_steps"][i], rel=tol, abs=1e-13)
        assert s.kinetic_energy()[0] == pytest.approx(d["ke_steps"][i], rel=tol, abs=1e-13)
    s.close()
