"""The C++ host API on the GPU reproduces the reference's own outputs.

oracle/refbuild/ref_driver.cpp drives OriginBox, AtomVec, NListed,
NeighborList and CollectionVerlet / CollectionDamped / CollectionSol exactly
as a reference program does.  Built against the reference it produced the
golden fixtures; built unchanged against parm_gb300/host (FP64 GPU path) it
must print the same numbers: bit for bit, except that pair laws with a
non-integer exponent (device pow) are held to 1e-12 relative.
"""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from golden_cases import NLCG, load, names
from host_api import DECK_DRIVER, compile_program

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import make_golden as MG  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def drivers(tmp_path_factory, built_lib):
    d = tmp_path_factory.mktemp("host_api")
    out = {}
    for nd in (3, 2):
        r = compile_program(DECK_DRIVER, d / f"drv{nd}", ndim=nd)
        assert r.returncode == 0, r.stderr[-3000:]
        out[nd] = d / f"drv{nd}"
    return out


def _check_minimiser(got, d):
    """CollectionNLCG / CollectionNLCGV through the host API: the same bars as the C ABI test
    (tests/test_gpu_nlcg.py), the sums being parallel."""
    from test_gpu_nlcg import RTOL_EARLY, RTOL_LATE, EARLY, rel_err
    np.testing.assert_array_equal(got["pairs"], d["pairs"])
    np.testing.assert_allclose(got["init"], d["init"], rtol=1e-12, atol=1e-13)
    assert rel_err(got["f0"], d["f0"]) <= 1e-12
    np.testing.assert_array_equal(got["steps"], d["steps"])
    for i, s in enumerate(d["steps"]):
        tol = RTOL_EARLY if s <= EARLY else RTOL_LATE
        for key in ("x", "v", "f"):
            err = rel_err(got[f"{key}_steps"][i], d[f"{key}_steps"][i])
            assert err <= tol, f"{key} at step {s}: {err:.3e}"
        assert rel_err(got["box_steps"][i], d["box_steps"][i]) <= tol
        assert abs(got["energy_steps"][i] - d["energy_steps"][i]) <= tol * max(abs(d["energy_steps"][0]), 1e-300)


def _close(got, want, exact, what, tol=1e-12):
    if exact:
        np.testing.assert_array_equal(got, want, err_msg=what)
    else:
        scale = max(float(np.abs(want).max()), 1e-300)
        assert float(np.abs(got - want).max()) / scale <= tol, what


@pytest.mark.parametrize("name", names())
def test_host_api_matches_reference(drivers, name):
    d = load(name)
    case = {k: d[k] for k in ("kind", "integ", "nsteps", "dt", "damping", "T", "skin", "L", "x", "v", "m",
                              "params", "deck_params", "pair_eps", "pair_sig", "le_gamma", "order", "ignores", "out_steps",
                              "cg")
            if k in d}
    deck = MG._deck(case)
    r = subprocess.run([str(drivers[d["ndim"]])], input=deck, capture_output=True, text=True, timeout=600,
                       env={"PARM_PRECISION": "fp64", "PATH": "/usr/bin:/bin"})
    assert r.returncode == 0, r.stderr[-2000:]
    got = MG._parse(r.stdout, d["n"], d["ndim"])
    if d["integ"] >= NLCG:
        _check_minimiser(got, d)
        return
    ecol = 1 if d["kind"] == 16 else 2   # the exponent's column
    exact = not ((d["kind"] in (1, 9, 16) and np.any(d["params"][:, ecol] != np.rint(d["params"][:, ecol])))
                 or d["kind"] in (13, 14, 15, 17))   # laws that call the device pow
    np.testing.assert_array_equal(got["pairs"], d["pairs"])
    np.testing.assert_array_equal(got["init_counts"], d["init_counts"])
    np.testing.assert_allclose(got["init"], d["init"], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(got["stress"], d["stress"], rtol=1e-12, atol=1e-13 * np.abs(d["stress"]).max())
    _close(got["f0"], d["f0"], exact, "initial forces")
    _close(got["a0"], d["a0"], exact, "initial accelerations")
    np.testing.assert_array_equal(got["steps"], d["steps"])
    np.testing.assert_array_equal(got["which_steps"], d["which_steps"])
    from test_gpu_golden import step_tol
    for i, step in enumerate(d["steps"]):
        tol = step_tol(d["kind"], int(step))
        for key in ("x", "v", "a", "f"):
            _close(got[f"{key}_steps"][i], d[f"{key}_steps"][i], exact, f"{key} at step {step}", tol)
        np.testing.assert_allclose(got["energy_steps"][i], d["energy_steps"][i], rtol=tol, atol=1e-13)
        np.testing.assert_allclose(got["ke_steps"][i], d["ke_steps"][i], rtol=tol, atol=1e-13)
