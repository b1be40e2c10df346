"""XYZ trajectory frames for the atoms of ``parm_gb300.pyparm``.

This module provides the interface of pyparm's ``xyzfile`` module
(pyparm/xyzfile.py: ``XYZwriter`` 7-75, ``XYZreader`` 108-258, ``Frame`` and
``Frames`` 260-326).

Each frame has three parts:

* the atom count;
* a comment line of ``key=value`` pairs, which must include ``time``;
* one line per atom: element, x y z, then vx vy vz when velocities are
  written, then sigma when the atoms carry one.

Coordinates are written with 4 decimals and sigma with 6.

A pyparm ``AtomVec`` is written from its record array.  That is one read-back
from the device per frame when the device holds the newest records, not one
per atom.  Element names come from ``elements=`` (one name, or one per atom),
else from the atoms' ``element`` attributes, else ``C``.
"""
from __future__ import annotations

import re

import numpy as np

__all__ = ["XYZError", "XYZwriter", "XYZreader", "Frame", "Frames"]


class XYZError(Exception):
    """A line of an XYZ file that does not parse."""


def _records(atoms):
    """(positions, velocities, element attributes or None, sigmas or None) of an AtomVec or of a
    sequence of atom objects with .x / .v (and optionally .element / .sigma)."""
    rec = getattr(atoms, "rec", None)
    if rec is not None:
        nd = (rec.shape[1] - 1) // 4
        return rec[:, 0:nd], rec[:, nd:2 * nd], None, None
    items = list(atoms)
    x = np.array([np.asarray(a.x, dtype=np.float64) for a in items])
    v = np.array([np.asarray(a.v, dtype=np.float64) for a in items])
    elems = [a.element for a in items] if items and all(hasattr(a, "element") for a in items) else None
    sig = np.array([a.sigma for a in items]) if items and all(hasattr(a, "sigma") for a in items) else None
    return x, v, elems, sig


class XYZwriter:
    """Writes frames to an open text file."""

    def __init__(self, f, usevels=True):
        self.file = f
        self.usevels = usevels

    def writeframe(self, atoms, com=None, box=None, elements=None, sigmas=None, **kwargs):
        """One frame. ``com``: positions are written relative to it. ``box``: positions are
        written as their minimum image (relative to ``com`` or the origin). The keyword arguments
        form the comment line and must include ``time``."""
        if "time" not in kwargs:
            raise ValueError("Time must be in keyword arguments, or .xyz will not be readable")
        x, v, elems, sig = _records(atoms)
        n = len(x)
        pos = x - (0.0 if com is None else np.asarray(com, dtype=np.float64))
        if box is not None:
            L = np.asarray(box.box_shape(), dtype=np.float64)
            pos = pos - L * np.rint(pos / L)
        if elements is not None:
            elems = [elements] * n if isinstance(elements, str) else list(elements)
        if elems is None:
            elems = ["C"] * n
        if sigmas is not None:
            sig = np.asarray(sigmas, dtype=np.float64)
        if pos.shape[1] == 2:   # 2D atoms: z (and vz) written as 0, so the frame reads as any other
            pos = np.hstack([pos, np.zeros((n, 1))])
            v = np.hstack([v, np.zeros((n, 1))])
        num = np.hstack([pos, v] if self.usevels else [pos])
        lines = [str(n), " ".join(f"{k}={val}" for k, val in kwargs.items())]
        for i in range(n):
            fields = [elems[i]] + ["%.4f" % q for q in num[i]]
            if sig is not None:
                fields.append("%.6f" % sig[i])
            lines.append(" ".join(fields))
        self.file.write("\n".join(lines) + "\n")
        self.file.flush()

    def size(self):
        here = self.file.tell()
        self.file.seek(0, 2)
        end = self.file.tell()
        self.file.seek(here)
        return end

    def close(self):
        self.file.close()


class Frame:
    """One frame: element names ``elems``, positions ``locs`` (n, 3), velocities ``vels`` and
    sigmas ``sigmas`` (or None), time ``t``, the comment line and its other values."""

    dtype = np.float64

    def __init__(self, locs, t=None):
        cols = list(zip(*locs))
        self.t = t
        self.vels = self.sigmas = None
        if len(cols) == 2:
            self.elems, xs = cols
        elif len(cols) == 3:
            self.elems, xs, third = cols
            if np.ndim(third[0]) == 0:
                self.sigmas = np.array(third, dtype=self.dtype)
            else:
                self.vels = np.array(third, dtype=self.dtype)
        elif len(cols) == 4:
            self.elems, xs, vs, ss = cols
            self.vels = np.array(vs, dtype=self.dtype)
            self.sigmas = np.array(ss, dtype=self.dtype)
        else:
            raise ValueError("Resized wrong length (%d)" % len(cols))
        self.locs = np.array(xs, dtype=self.dtype)
        self.comment = ""
        self.values = {}

    @property
    def time(self):
        return self.t

    def __iter__(self):
        return iter(self.locs)

    def __len__(self):
        return len(self.locs)

    def into(self, atoms, check=True):
        """Set the atoms' positions (and velocities) from this frame."""
        for k, a in enumerate(atoms):
            if k >= len(self.locs):
                break
            if check and hasattr(a, "element") and a.element != self.elems[k]:
                raise TypeError("Element mismatch for atom %d: %s is not %s" % (k, a.element, self.elems[k]))
            a.x = tuple(float(q) for q in self.locs[k])
            if self.vels is not None:
                a.v = tuple(float(q) for q in self.vels[k])


class Frames(list):
    def into(self, atoms, check=True):
        for f in self:
            f.into(atoms, check)
            yield f.time, f.values


class XYZreader:
    """Reads frames from an open text file (iteration stops at its end)."""

    _count = re.compile(r"^\s*([0-9]+)\s*$")

    def __init__(self, f):
        self.file = f
        self.lineno = 1
        self._size = None

    def _line(self):
        line = self.file.readline()
        if line == "":
            return None
        self.lineno += 1
        return line.rstrip("\n")

    @staticmethod
    def _values(comment):
        c = comment.strip()
        if "=" in c:
            return dict(pair.split("=", 1) for pair in c.split())
        if " " in c:
            key, val = c.split(None, 1)
            return {key: val}
        if c:
            try:
                return {"time": float(c)}
            except ValueError:
                return {"comment": c}
        return {}

    def readframe(self):
        """The next frame, or None at the end of the file."""
        first = self._line()
        if first is None:
            return None
        m = self._count.match(first)
        if m is None:
            raise XYZError("Failed to parse first frame line at line %d: %r" % (self.lineno - 1, first))
        n = int(m.group(1))
        comment = self._line()
        if comment is None:
            raise XYZError("Comment line expected at end of file, line %d" % self.lineno)
        start = self.lineno - 2
        rows = []
        for k in range(n):
            line = self._line()
            if line is None:
                raise XYZError("Coordinate line expected at end of file, line %d (frame started at %d)"
                               % (self.lineno, start))
            rows.append(line.replace("\t", " ").split())
        width = len(rows[0]) if rows else 4
        for k, r in enumerate(rows):
            if len(r) not in (4, 5, 7, 8) or len(r) != width:
                raise XYZError("bad coordinate line %d (frame started at %d): %r" % (start + 2 + k, start, r))
        try:
            if width == 4:
                locs = [(r[0], tuple(map(float, r[1:4]))) for r in rows]
            elif width == 5:
                locs = [(r[0], tuple(map(float, r[1:4])), float(r[4])) for r in rows]
            elif width == 7:
                locs = [(r[0], tuple(map(float, r[1:4])), tuple(map(float, r[4:7]))) for r in rows]
            else:
                locs = [(r[0], tuple(map(float, r[1:4])), tuple(map(float, r[4:7])), float(r[7])) for r in rows]
        except ValueError as e:
            raise XYZError("bad number in the frame started at line %d: %s" % (start, e)) from None
        vals = self._values(comment)
        t = vals.pop("time", None)
        f = Frame(locs, None if t is None else float(t)) if locs else None
        if f is None:
            raise XYZError("empty frame at line %d" % start)
        f.comment = comment
        f.values = vals
        return f

    def __iter__(self):
        while True:
            f = self.readframe()
            if f is None:
                return
            yield f

    def into(self, atoms, check=True):
        for f in self:
            f.into(atoms, check)
            vals = f.values
            if f.sigmas is not None:
                if "sigmas" in f.values:
                    raise ValueError("sigmas already in f.values, don't know what to do")
                vals = dict(f.values, sigmas=f.sigmas)
            yield f.time, vals

    def all(self):
        frames = Frames(iter(self))
        for k, f in enumerate(frames):
            f.indx = k
        return frames

    def size(self):
        if self._size is None:
            here = self.file.tell()
            self.file.seek(0, 2)
            self._size = self.file.tell()
            self.file.seek(here)
        return self._size

    def close(self):
        self.file.close()
