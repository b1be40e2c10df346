"""XYZ frames (parm_gb300/xyzfile.py, the interface of pyparm/xyzfile.py) written from and read
into the Python module's AtomVec, on the host."""
import io

import numpy as np
import pytest

from parm_gb300 import pyparm
from parm_gb300.xyzfile import Frame, XYZError, XYZreader, XYZwriter


def _atoms(n=5, seed=3):
    rng = np.random.default_rng(seed)
    atoms = pyparm.d3.AtomVec(rng.uniform(1, 2, n))
    for a in atoms:
        a.x = rng.uniform(-7, 7, 3)
        a.v = rng.normal(size=3)
    return atoms


def test_frames_round_trip():
    atoms = _atoms()
    f = io.StringIO()
    w = XYZwriter(f)
    w.writeframe(atoms, time=0.5, E=-1.25)
    w.writeframe(atoms, time=1.0, elements="Ar", sigmas=[1.0, 1.4, 1.0, 1.4, 1.0])
    text = f.getvalue().splitlines()
    assert text[0] == "5" and text[1] == "time=0.5 E=-1.25"
    assert len(text[2].split()) == 7 and text[2].split()[0] == "C"
    f.seek(0)
    frames = XYZreader(f).all()
    assert len(frames) == 2
    a, b = frames
    assert a.time == 0.5 and a.values == {"E": "-1.25"} and b.time == 1.0
    np.testing.assert_allclose(a.locs, atoms.rec[:, 0:3], atol=5e-5)
    np.testing.assert_allclose(a.vels, atoms.rec[:, 3:6], atol=5e-5)
    assert a.sigmas is None and list(b.sigmas) == [1.0, 1.4, 1.0, 1.4, 1.0]
    assert set(b.elems) == {"Ar"} and b.indx == 1
    other = _atoms(seed=9)
    a.into(other)
    np.testing.assert_allclose(other.rec[:, 0:3], a.locs)
    np.testing.assert_allclose(other.rec[:, 3:6], a.vels)


def test_box_and_centre():
    atoms = _atoms()
    box = pyparm.d3.OriginBox(4.0)
    f = io.StringIO()
    com = np.array([0.5, -0.25, 1.0])
    XYZwriter(f, usevels=False).writeframe(atoms, com=com, box=box, time=2)
    f.seek(0)
    fr = XYZreader(f).readframe()
    assert fr.vels is None and fr.time == 2.0
    want = np.array([box.diff(x, com) for x in atoms.rec[:, 0:3]])
    np.testing.assert_allclose(fr.locs, want, atol=5e-5)
    assert np.all(np.abs(fr.locs) <= 2.0 + 1e-4)


def test_two_dimensional_atoms():
    atoms = pyparm.d2.AtomVec([1.0, 1.0])
    atoms[0].x, atoms[1].x = [1.5, -2.0], [0.25, 3.0]
    f = io.StringIO()
    XYZwriter(f).writeframe(atoms, time=0)
    f.seek(0)
    fr = XYZreader(f).readframe()
    np.testing.assert_allclose(fr.locs, [[1.5, -2.0, 0.0], [0.25, 3.0, 0.0]])


def test_errors():
    with pytest.raises(ValueError):
        XYZwriter(io.StringIO()).writeframe(_atoms(), E=1.0)
    with pytest.raises(XYZError):
        XYZreader(io.StringIO("x\ntime=0\n")).readframe()
    with pytest.raises(XYZError):
        XYZreader(io.StringIO("2\ntime=0\nC 1 2 3\n")).readframe()
    with pytest.raises(XYZError):
        XYZreader(io.StringIO("2\ntime=0\nC 1 2 3\nC 1 2\n")).readframe()
    assert XYZreader(io.StringIO("")).readframe() is None
    assert Frame([("C", (1.0, 2.0, 3.0), 1.5)]).sigmas[0] == 1.5
