"""Conjugate-gradient minimisers on the GPU (CollectionNLCG with the box,
CollectionNLCGV with a fixed box) against the reference's own outputs.

The fixtures (tests/golden/nlcg*.npz) hold the reference's trajectories,
boxes and minimiser scalars.  The GPU sums fdotv, vdotv, fdota and the virial
in parallel (fixed order, not the reference's sequential one), so results
agree to rounding: arrays within RTOL_EARLY of their largest entry over the
first EARLY steps and within RTOL_LATE after, where the secant searches of
two runs that differ by rounding may stop one iteration apart.  Every other
check is exact: batched systems equal the same systems run alone bit for
bit, graph-captured steps equal directly launched ones bit for bit.
"""
import subprocess

import numpy as np
import pytest

from golden_cases import NLCG, load, names
from parm_gb300 import capi

pytestmark = pytest.mark.gpu

CASES = [n for n in names() if load(n)["integ"] >= NLCG]
EARLY = 10
RTOL_EARLY = 1e-12
RTOL_LATE = 1e-6


def rel_err(got, want) -> float:
    scale = max(float(np.abs(want).max()), 1e-300)
    return float(np.abs(np.asarray(got) - np.asarray(want)).max()) / scale


def _setup(d, precision="fp64"):
    """The fixture driver's set-up through the C ABI: NListed + update_list(true), the Collection
    constructor's initialize(), then set_forces(true, true) (NLCG) or reset() (NLCGV)."""
    from parm_gb300 import System
    n, nd = d["n"], d["ndim"]
    s = System([n], ndim=nd, precision=precision)
    s.set_boxes(d["L"][None, :])
    s.set_atoms(x=d["x"], v=d["v"], a=np.zeros((n, nd)), f=np.zeros((n, nd)), m=d["m"])
    rank = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
    rank[d["order"]] = np.arange(len(d["order"]), dtype=np.uint32)
    s.set_interaction(d["kind"], d["params"], d["skin"], rank=rank)
    s.nlist_update(True)
    s.nlist_update(False)
    s.set_forces(True)
    s.nlist_update(False)
    boxed = d["integ"] == NLCG
    s.nlcg_init(d["cg"], boxed=boxed)
    if boxed:
        s.nlcg_set_forces(True)
    else:
        s.nlcg_reset()
    return s


@pytest.mark.parametrize("name", CASES)
def test_nlcg_matches_reference(name):
    d = load(name)
    s = _setup(d)
    np.testing.assert_array_equal(s.pairs(), d["pairs"])
    st = s.get_atoms()
    assert rel_err(st["f"], d["f0"]) <= 1e-12
    done = 0
    report = []
    for i, step in enumerate(d["steps"]):
        s.nlcg_timestep(int(step) - done)
        done = int(step)
        tol = RTOL_EARLY if step <= EARLY else RTOL_LATE
        st = s.get_atoms()
        errs = {k: rel_err(st[k], d[f"{k}_steps"][i]) for k in ("x", "v", "a", "f")}
        errs["box"] = rel_err(s.boxes()[0], d["box_steps"][i])
        errs["E"] = abs(s.energy()[0] - d["energy_steps"][i]) / abs(d["energy_steps"][0])
        state = s.nlcg_state()[0]
        ref = d["cg_state_steps"][i]
        for q in (capi.NLCG_STATE.index("vl"), capi.NLCG_STATE.index("fl"), capi.NLCG_STATE.index("dxsum")):
            errs[capi.NLCG_STATE[q]] = abs(state[q] - ref[q]) / max(abs(ref[q]), 1e-300)
        report.append((int(step), errs))
        for k, e in errs.items():
            if k in ("vl", "fl") and abs(ref[capi.NLCG_STATE.index(k)]) < 1e-12:
                continue   # a scalar that is zero to rounding
            assert e <= tol, f"{name}: {k} at step {step}: relative error {e:.3e}; all steps: {report}"
    print(name, report)
    s.close()


@pytest.mark.parametrize("name", CASES)
def test_graph_steps_equal_direct_launches(name):
    """The secant loop as a conditional WHILE node equals the same kernels launched one by one."""
    d = load(name)
    out = []
    for gk in (16, 0):
        s = _setup(d)
        s.set_graph_steps(gk)
        s.nlcg_timestep(40)
        out.append((s.get_atoms(), s.boxes(), s.nlcg_state(), s.which()))
        s.close()
    (a, b, c, w), (a2, b2, c2, w2) = out
    for k in a:
        np.testing.assert_array_equal(a[k], a2[k])
    np.testing.assert_array_equal(b, b2)
    np.testing.assert_array_equal(c, c2)
    np.testing.assert_array_equal(w, w2)


def test_batch_equals_systems_alone():
    """Systems minimised together in one handle equal each system minimised alone, bit for bit."""
    from parm_gb300 import System
    from parm_gb300 import workloads as W
    w = W.packings(nsys=5, nmin=40, nmax=300, phi_lo=0.45, phi_hi=0.7, exponent=2.0, seed=77, skin=0.3)
    cg = np.array([0.1, 1e-3, 10.0, 1000, 40, 1e-20, 2.0, 0.0, 100.0, 1e-3, 0.0])

    def run(lo, hi):
        o0, o1 = int(sum(w.sizes[:lo])), int(sum(w.sizes[:hi]))
        s = System(w.sizes[lo:hi], ndim=3, precision="fp64")
        s.set_boxes(w.L[lo:hi])
        n = o1 - o0
        s.set_atoms(x=w.x[o0:o1], v=np.zeros((n, 3)), a=np.zeros((n, 3)), f=np.zeros((n, 3)), m=w.m[o0:o1])
        s.set_interaction(w.kind, w.params[o0:o1], w.skin)
        s.nlist_update(False); s.set_forces(True); s.nlist_update(False)
        s.nlcg_init(cg, boxed=True)
        s.nlcg_set_forces(True)
        s.nlcg_timestep(60)
        r = (s.get_atoms(), s.boxes(), s.nlcg_state(), s.which())
        s.close()
        return r

    batch = run(0, 5)
    off = np.concatenate([[0], np.cumsum(w.sizes)])
    for q in range(5):
        one = run(q, q + 1)
        for k in one[0]:
            np.testing.assert_array_equal(batch[0][k][off[q]:off[q + 1]], one[0][k], err_msg=f"system {q} {k}")
        np.testing.assert_array_equal(batch[1][q], one[1][0])
        np.testing.assert_array_equal(batch[2][q], one[2][0])
        assert batch[3][q] == one[3][0]


def test_long_run_against_oracle():
    """400 time steps of a 3D packing: GPU and oracle reach the same box and energy."""
    from oracle.oracle import Oracle, OracleNLCG, nlcg_params
    from parm_gb300 import workloads as W
    from helpers import make_gpu
    w = W.small_random(n=200, ndim=3, kind=1, seed=91, phi=0.5, skin=0.3)
    w.params[:, 0] = 1.0
    w.v[:] = 0.0
    cg = nlcg_params(0.1, P0=1e-3)
    g = make_gpu(w)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    g.nlcg_init(cg, boxed=True)
    g.nlcg_set_forces(True)
    o = Oracle(w.n, 3)
    o.set_box(w.L[0])
    o.set_state(x=w.x, v=w.v, m=w.m)
    o.set_interaction(w.kind, w.params, w.skin)
    o.initialize()
    on = OracleNLCG(o, cg, boxed=True)
    on.set_forces(True)
    g.nlcg_timestep(400)
    on.timestep(400)
    assert rel_err(g.boxes()[0], on.box()) <= 1e-6
    e_g, e_o = g.energy()[0], o.energy()
    assert abs(e_g - e_o) <= 1e-6 * abs(e_o) + 1e-12, (e_g, e_o)
    g.close()


def test_mixed_precision_reaches_the_same_packing():
    """The mixed path minimises a packing to the FP64 path's box (relative 1e-4) and energy (1e-3:
    the two runs follow slightly different paths into the same basin)."""
    from parm_gb300 import workloads as W
    from helpers import make_gpu
    w = W.small_random(n=400, ndim=3, kind=1, seed=92, phi=0.6, skin=0.3)
    w.params[:, 0] = 1.0
    w.v[:] = 0.0
    cg = np.array([0.1, 1e-3, 10.0, 1000, 40, 1e-20, 2.0, 0.0, 100.0, 1e-3, 0.0])
    res = {}
    for prec in ("fp64", "mixed"):
        g = make_gpu(w, prec)
        g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
        g.nlcg_init(cg, boxed=True)
        g.nlcg_set_forces(True)
        g.nlcg_timestep(1500)
        res[prec] = (g.boxes()[0][0], g.energy()[0], np.sqrt(g.max_force_sq()[0]))
        g.close()
    (L64, E64, F64), (L32, E32, F32) = res["fp64"], res["mixed"]
    assert abs(L32 - L64) <= 1e-4 * L64, res
    assert abs(E32 - E64) <= 1e-3 * abs(E64) + 1e-9, res


def test_packing_program_runs(tmp_path, built_lib):
    """A packing program on the host API's CollectionNLCG (tests/programs/nlcg_packing.cpp, the calls
    the reference's src/bin/packer.cpp makes): 80 harmonic spheres compressed through five goal
    pressures (1e-4 .. 1e-8), each stage ending on |P/P0 - 1| < 1e-4 and max |F| < 1e-14, at a
    jammed density."""
    from pathlib import Path
    from host_api import compile_program
    src = Path(__file__).resolve().parent / "programs" / "nlcg_packing.cpp"
    exe = tmp_path / "packing"
    r = compile_program(src, exe)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900, cwd=tmp_path,
                       env={"PARM_PRECISION": "fp64", "PATH": "/usr/bin:/bin"})
    assert r.returncode == 0, r.stderr[-2000:]
    stages = [line.split() for line in r.stdout.splitlines() if line.startswith("stage")]
    assert len(stages) == 5, r.stdout[-3000:]
    for st in stages:
        assert abs(float(st[4])) < 1e-4 and float(st[5]) < 1e-14, st
    phi = float(stages[-1][6])
    assert 0.55 < phi < 0.75, stages
