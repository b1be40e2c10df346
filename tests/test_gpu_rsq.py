"""State trackers: the device mean-square-displacement tracker (parm_rsq_*) against the
reference, and the host API's trackers inside Collections.

* the reference's own known answers (RSQTest, pyparm/tests.py:504-569), with
  the tracker updated explicitly after each move;
* updates inside the time-step graphs: the tracker run along an FP64 Verlet
  trajectory equals the NumPy restatement of RsqTracker fed with the same
  trajectory step by step (bit for bit without the centre of mass; to
  rounding with it, whose sum runs in another order), for graph and direct
  launches, one system and a batch of three.
"""
import numpy as np
import pytest

from helpers import make_gpu
from oracle.rsq import RsqOracle
from parm_gb300 import capi
from parm_gb300 import workloads as W
from test_rsq_cpu import RSQ_DXS, RSQ_NS, rsq_kat_masses, rsq_kat_positions

pytestmark = pytest.mark.gpu

OUTS = [capi.RSQ_XYZ2, capi.RSQ_XYZ4, capi.RSQ_R2, capi.RSQ_R4, capi.RSQ_COUNTS]


def _oracle_out(o, what):
    return {capi.RSQ_XYZ2: o.xyz2, capi.RSQ_XYZ4: o.xyz4, capi.RSQ_R2: o.r2, capi.RSQ_R4: o.r4,
            capi.RSQ_COUNTS: o.counts}[what]()


def test_rsq_reference_known_answers():
    from parm_gb300 import System
    m = rsq_kat_masses()
    s = System(8)
    s.set_boxes(np.full(3, 20.0))
    z = np.zeros((8, 3))
    s.set_atoms(x=z, v=z, a=z, f=z, m=m)
    s.rsq_start(RSQ_NS, usecom=False)
    o = RsqOracle(z, m, RSQ_NS, usecom=False)
    for x in rsq_kat_positions():
        s.set_atoms(x=x)
        s.rsq_update()
        o.update(x)
    for j, n in enumerate(RSQ_NS):
        d = RSQ_DXS * n
        np.testing.assert_allclose(s.rsq_get(capi.RSQ_R2)[j], np.sum(d ** 2, axis=-1), rtol=1e-12)
        np.testing.assert_allclose(s.rsq_get(capi.RSQ_XYZ2)[j], d ** 2, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(s.rsq_get(capi.RSQ_R4)[j], np.sum(d ** 2, axis=-1) ** 2, rtol=1e-12)
        np.testing.assert_allclose(s.rsq_get(capi.RSQ_XYZ4)[j], d ** 4, rtol=1e-12, atol=1e-12)
    for what in OUTS:   # and bit for bit with the restatement
        assert np.array_equal(s.rsq_get(what), _oracle_out(o, what))
    s.close()


def _trajectory(w, steps, dt):
    """Positions after each FP64 Verlet step (one call per step)."""
    g = make_gpu(w, "fp64")
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    xs = []
    for _ in range(steps):
        g.verlet(dt, 1)
        xs.append(g.get_atoms()["x"])
    g.close()
    return xs


@pytest.mark.parametrize("usecom", [False, True])
@pytest.mark.parametrize("graph_steps", [16, 0])
def test_rsq_inside_time_steps(usecom, graph_steps):
    w = W.lj_lattice(shape=(6, 6, 6), skin_prime=0.3, seed=4)
    steps, dt, skips = 37, 0.002, [1, 3, 5, 16]
    xs = _trajectory(w, steps, dt)
    o = RsqOracle(w.x, w.m, skips, usecom=usecom)
    for x in xs:
        o.update(x)
    g = make_gpu(w, "fp64")
    g.set_graph_steps(graph_steps)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    g.rsq_start(skips, usecom=usecom)
    g.verlet(dt, steps)   # the tracker is updated at the end of every step
    assert np.array_equal(g.get_atoms()["x"], xs[-1])
    for what in OUTS:
        got, ref = g.rsq_get(what), _oracle_out(o, what)
        if usecom:
            np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-18)
        else:
            assert np.array_equal(got, ref), what
    g.rsq_stop()
    g.close()


def test_rsq_batch_and_mixed_precision():
    """Three systems of one handle, each with its own centre of mass; the mixed path runs the same tracker."""
    w = W.wca_replicas(nrep=3, nmin=200, nmax=600, seed=7)
    w.v = np.random.RandomState(8).normal(0.0, 1.0, size=w.x.shape)
    skips = [1, 4]
    for precision in ("fp64", "mixed"):
        g = make_gpu(w, precision)
        g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
        x0 = g.get_atoms()["x"]
        g.rsq_start(skips, usecom=True)
        o = RsqOracle(x0, w.m, skips, usecom=True, sizes=w.sizes)
        for _ in range(9):
            g.verlet(0.002, 1)
            g.rsq_update()   # explicit updates on top of the in-step ones
            x = g.get_atoms()["x"]
            o.update(x)
            o.update(x)
        assert np.array_equal(g.rsq_get(capi.RSQ_COUNTS), o.counts())
        for what in (capi.RSQ_XYZ2, capi.RSQ_R2, capi.RSQ_R4):
            np.testing.assert_allclose(g.rsq_get(what), _oracle_out(o, what), rtol=1e-9, atol=1e-18)
        g.close()


def _parse(text):
    """Tracker outputs and positions printed by tests/programs/rsq_tracker.cpp."""
    out, xs = {}, {}
    for line in text.splitlines():
        f = line.split()
        if f[0] == "X":
            s, i, d, v = int(f[1]), int(f[2]), int(f[3]), float(f[4])
            xs.setdefault(s, {})[(i, d)] = v
        else:
            out[(f[0], f[1]) + tuple(int(q) for q in f[2:-1])] = float(f[-1])
    pos = {}
    for s, vals in xs.items():
        n = max(i for i, _ in vals) + 1
        a = np.zeros((n, 3))
        for (i, d), v in vals.items():
            a[i, d] = v
        pos[s] = a
    return out, pos


def _check_program(out, tag, o, exact):
    for j, c in enumerate(o.counts()):
        assert out[(tag, "COUNT", j)] == c
    ref = {"R2": o.r2(), "R4": o.r4(), "XYZ2": o.xyz2(), "XYZ4": o.xyz4()}
    for key, val in out.items():
        if key[0] != tag or key[1] == "COUNT":
            continue
        r = ref[key[1]][key[2:]]
        if exact:
            assert val == r, key
        else:
            assert abs(val - r) <= 1e-9 * abs(r) + 1e-18, key


def test_host_api_rsq_tracker(tmp_path):
    """The C++ RsqTracker: standalone (the reference's known answers) and inside a CollectionVerlet."""
    import subprocess
    from pathlib import Path
    from host_api import compile_program
    src = Path(__file__).resolve().parent / "programs" / "rsq_tracker.cpp"
    exe = tmp_path / "rsq_tracker"
    r = compile_program(src, exe)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr
    out, pos = _parse(run.stdout)
    kat = RsqOracle(np.zeros((8, 3)), np.ones(8), RSQ_NS, usecom=False)
    for x in rsq_kat_positions():
        kat.update(x)
    _check_program(out, "KAT", kat, exact=True)
    n = len(pos[0])
    col = RsqOracle(pos[0], np.ones(n), [1, 3], usecom=True)
    col.update(pos[0])   # Collection::initialize updates the trackers twice
    col.update(pos[0])
    for s in range(1, 13):
        col.update(pos[s])
    _check_program(out, "COL", col, exact=False)
    # the tracker of the Collection's own atoms is bound to its handle, and
    # twelve steps in one call update it inside the GPU steps: the same results
    assert out[("BOUND", "COL")] == 1 and out[("BOUND", "ONE")] == 1
    ones = {key[1:]: v for key, v in out.items() if key[0] == "ONE"}
    cols = {key[1:]: v for key, v in out.items() if key[0] == "COL"}
    assert ones.keys() == cols.keys() and ones
    for key, v in ones.items():
        assert abs(v - cols[key]) <= 1e-12 * abs(cols[key]) + 1e-300, key
    for (name, step, i, d), v in ((k, v) for k, v in out.items() if k[0] == "Y"):
        assert v == pos[12][i, d]


def test_host_api_energy_tracker(tmp_path):
    """EnergyTracker and a caller-defined tracker inside a CollectionVerlet (updated after every step)."""
    import subprocess
    from pathlib import Path
    from host_api import compile_program
    src = Path(__file__).resolve().parent / "programs" / "energy_tracker.cpp"
    exe = tmp_path / "energy_tracker"
    r = compile_program(src, exe)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "UPDATES 12 SAMPLES 4 4" in run.stdout
    assert "ENERGY OK" in run.stdout
