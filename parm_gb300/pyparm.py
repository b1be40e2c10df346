"""The reference's Python module, on the GPU: the class names, constructors and
call patterns of pyparm's SWIG module ``sim`` (src/sim.i: its ``%template``
names, 621-643, and its Python extensions, 494-667), on this package's C ABI.

    from parm_gb300 import pyparm
    sim = pyparm.d3                      # pyparm's d3 (and d2) modules
    box = sim.OriginBox(L)
    atoms = sim.AtomVec(masses)
    rep = sim.Repulsion(box, atoms, 0.4)
    for a, s in zip(atoms, sigmas):
        rep.add(sim.EpsSigExpAtom(a, 1.0, s, 2.0))
    collec = sim.CollectionVerlet(box, atoms, 0.01, [rep], [rep.neighbor_list()], [])
    collec.timestep()

As in the C++ host API (parm_gb300/host), Python reads and writes the atoms
between calls (``atoms[i].x = ...``).  Every call that runs on the GPU first
uploads them when they changed.  After a device call the records stay on the
device and come back only when Python reads them.  One neighbour list
carries one GPU handle; an NListed interaction evaluates the pairs of its
list; a Collection steps the atoms of its (single) interaction.  An
RsqTracker of the Collection's own atoms is updated inside the GPU steps.
Precision: FP64 (the reference's numbers) unless PARM_PRECISION=mixed is set
when the list's handle is made.  Beyond the reference,
``Collection.timesteps(n)`` runs n steps in one call.
"""
from __future__ import annotations

import math
import os
import types

import numpy as np

from . import capi
from .system import System

_seed = [0x5EED5EED]


def seed(n=None):
    """The seed of CollectionSol's counter-based noise (pyparm's seed(), src/vecrand.cpp)."""
    _seed[0] = int(np.random.SeedSequence(n).generate_state(1, np.uint64)[0]) if n is None else int(n)


def _make(ndim: int):
    NDIM = ndim
    REC = 4 * ndim + 1   # the Atom record: x, v, a, f, m

    def Vec(*c):
        return np.array(c if c else [0.0] * NDIM, dtype=np.float64)

    # ------------------------------------------------------------------ atoms
    class AtomVec:
        """Atom records in host memory (src/box.hpp:441-479); AtomVec(masses) or AtomVec(N, mass)."""

        def __init__(self, masses, mass=1.0):
            m = np.full(int(masses), float(mass)) if np.isscalar(masses) else np.asarray(masses, np.float64)
            self._rec = np.zeros((len(m), REC))
            self._rec[:, 4 * NDIM] = m
            self.version = 0
            self._dev = None   # the NeighborList whose device handle holds newer records

        @property
        def rec(self):
            """The records (n, 4*NDIM + 1); read back from the device first when it holds newer ones."""
            if self._dev is not None:
                nl, self._dev = self._dev, None
                nl._fetch()
            return self._rec

        def touch(self):
            self.version += 1

        def size(self):
            return len(self._rec)

        N = size

        def __len__(self):
            return len(self._rec)

        def get_id(self, i):
            if not 0 <= int(i) < len(self._rec):
                raise IndexError("atom index out of range")
            return AtomID(self, int(i))

        get = get_id

        def __getitem__(self, i):
            return self.get_id(i)

        def __iter__(self):
            for i in range(len(self._rec)):
                yield AtomID(self, i)

        def getmass(self, i):
            return float(self._rec[i, 4 * NDIM])   # masses change only on the host

        def _mobile(self):
            m = self._rec[:, 4 * NDIM]
            return ~((m <= 0) | np.isinf(m))

        def kinetic_energy(self, v0=None):
            v = self.rec[:, NDIM:2 * NDIM] - (0.0 if v0 is None else np.asarray(v0))
            m = self.rec[:, 4 * NDIM]
            mob = self._mobile()
            return float(0.5 * np.sum(m[mob] * np.sum(v[mob] ** 2, axis=1)))

        def momentum(self):
            mob = self._mobile()
            return np.sum(self.rec[mob, 4 * NDIM, None] * self.rec[mob, NDIM:2 * NDIM], axis=0)

        def mass(self):
            return float(np.sum(self._rec[self._mobile(), 4 * NDIM]))

        def com_velocity(self):
            return self.momentum() / self.mass()

        def reset_com_velocity(self):
            # add_velocity(-com_velocity()) (src/box.hpp:426): every atom, immobile ones too
            self.add_velocity(-self.com_velocity())

        def com(self):
            """Centre of mass of the mobile atoms (src/box.cpp:228-237)."""
            mob = self._mobile()
            r = self.rec
            return np.sum(r[mob, 4 * NDIM, None] * r[mob, 0:NDIM], axis=0) / self.mass()

        def com_force(self):
            return np.sum(self.rec[:, 3 * NDIM:4 * NDIM], axis=0)

        def gyradius(self):
            x = self.rec[:, 0:NDIM]
            return float(np.sqrt(np.sum((x - x.mean(axis=0)) ** 2) / len(x)))

        def add_velocity(self, v):
            self.rec[:, NDIM:2 * NDIM] += np.asarray(v, np.float64)
            self.touch()

        def randomize_velocities(self, T):
            """Normal velocity components of variance T/m (src/box.cpp:419-425, numpy's global
            generator); atoms of zero or infinite mass keep theirs."""
            r = self.rec
            m = r[:, 4 * NDIM]
            sel = ~((m == 0) | np.isinf(m))
            r[sel, NDIM:2 * NDIM] = np.random.normal(size=(int(sel.sum()), NDIM)) * np.sqrt(T / m[sel])[:, None]
            self.touch()

        def reset_forces(self):
            self.rec[:, 3 * NDIM:4 * NDIM] = 0.0
            self.touch()

        def __getstate__(self):
            return ([self.getmass(i) for i in range(len(self))], [a.__getstate__() for a in self])

        def __setstate__(self, st):
            masses, atomstates = st
            self.__init__(masses)
            for a, s in zip(self, atomstates):
                a.__setstate__(s)

    def _field(k):
        def get(self):
            return self.vec.rec[self.i, k * NDIM:(k + 1) * NDIM].copy()

        def set(self, val):
            self.vec.rec[self.i, k * NDIM:(k + 1) * NDIM] = np.asarray(val, np.float64)
            self.vec.touch()
        return property(get, set)

    class AtomID:
        """An atom of an AtomVec (the reference's AtomID: n() and the Atom's fields)."""

        def __init__(self, vec, i):
            self.vec, self.i = vec, i

        x, v, a, f = _field(0), _field(1), _field(2), _field(3)

        @property
        def m(self):
            return float(self.vec.rec[self.i, 4 * NDIM])

        @m.setter
        def m(self, val):
            self.vec.rec[self.i, 4 * NDIM] = float(val)
            self.vec.touch()

        def n(self):
            return self.i

        def __eq__(self, o):
            return isinstance(o, AtomID) and o.vec is self.vec and o.i == self.i

        def __hash__(self):
            return hash((id(self.vec), self.i))

        def __getstate__(self):
            return (tuple(self.x), tuple(self.v), tuple(self.f), tuple(self.a))

        def __setstate__(self, st):
            self.x, self.v, self.f, self.a = [np.asarray(r, np.float64) for r in st]

        def __repr__(self):
            return "<AtomID %d at (%s)>" % (self.i, ",".join("%.2f" % q for q in self.x))

    class IDPair:
        def __init__(self, a, b):
            self._a, self._b = a, b

        def first(self):
            return self._a

        def last(self):
            return self._b

        def __iter__(self):
            return iter((self._a, self._b))

    # ------------------------------------------------------------------ boxes
    class OriginBox:
        """Periodic box with its origin at the centre (src/box.hpp:101-160)."""

        def __init__(self, L):
            self.boxsize = np.full(NDIM, float(L)) if np.isscalar(L) else np.asarray(L, np.float64).copy()

        def diff(self, r1, r2):
            # vec_mod (src/box.hpp:68-78): the IEEE remainder per axis
            return np.array([math.remainder(float(a) - float(b), float(L)) for a, b, L in zip(r1, r2, self.boxsize)])

        def V(self):
            return float(np.prod(self.boxsize))

        def L(self):
            return float(np.sum(self.boxsize) / NDIM)

        def box_shape(self):
            return self.boxsize.copy()

        def rand_loc(self):
            return self.diff(np.random.uniform(0, 1, NDIM) * self.boxsize, np.zeros(NDIM))

        def resize(self, factor, atoms=None):
            self.boxsize = self.boxsize * factor
            if atoms is not None:
                atoms.rec[:, 0:NDIM] *= factor
                atoms.touch()
            return self.V()

        def resize_to(self, newsize, atoms=None):
            newsize = np.asarray(newsize, np.float64)
            if atoms is not None:
                atoms.rec[:, 0:NDIM] *= newsize / self.boxsize
                atoms.touch()
            self.boxsize = newsize.copy()
            return self.V()

        def resize_to_V(self, newV, atoms=None):
            return self.resize((newV / self.V()) ** (1.0 / NDIM), atoms)

        def resize_to_L(self, newL, atoms=None):
            # the current length is V^(1/NDIM), as src/box.cpp:44-55 takes it
            return self.resize(newL / self.V() ** (1.0 / NDIM), atoms)

    class LeesEdwardsBox(OriginBox):
        """Sheared periodic box (src/box.hpp:165-196, box.cpp:72-135): FP64 handles."""

        def __init__(self, L, gamma=0.0):
            super().__init__(L)
            self.gamma = float(gamma)

        def diff(self, r1, r2):
            Ly, Lx = float(self.boxsize[1]), float(self.boxsize[0])
            dy = float(r1[1]) - float(r2[1])
            im = int(_round_half_away(dy / Ly))
            dy = dy - (im * Ly)
            dx = float(r1[0]) - float(r2[0])
            dx = dx - _round_half_away((dx / Lx) - im * self.gamma) * Lx - im * self.gamma * Lx
            out = [dx, dy]
            if NDIM == 3:
                out.append(math.remainder(float(r1[2]) - float(r2[2]), float(self.boxsize[2])))
            return np.array(out)

        def get_gamma(self):
            return self.gamma

        def shear(self, dgamma, atoms=None):
            if atoms is not None:
                atoms.rec[:, 0] += atoms.rec[:, 1] * dgamma
                atoms.touch()
            self.gamma += dgamma

        def shear_to(self, gamma, atoms=None):
            self.shear(gamma - self.gamma, atoms)

        def affine(self, v):
            v = np.array(v, np.float64)
            v[0] += self.gamma * v[1]
            return v

        def non_affine(self, v):
            v = np.array(v, np.float64)
            v[0] -= self.gamma * v[1]
            return v

    # -------------------------------------------------- atom parameter types
    class _AtomP:
        """An atom with its pair parameters; `p` is its C ABI record."""

        rows = None   # indexed atoms: (type, epsilons, sigmas or None)

        def __init__(self, atom, p):
            self.atom, self.p = atom, [float(q) for q in p]

        def n(self):
            return self.atom.n()

    def _atom_type(name, fields, record, max_size, defaults=()):
        """An atom type with constructor (atom, *fields); `defaults` fill the last fields."""
        def __init__(self, atom, *args):
            missing = len(fields) - len(args)
            if missing < 0 or missing > len(defaults):
                raise TypeError(f"{name}(atom, {', '.join(fields)})")
            vals = list(args) + list(defaults[len(defaults) - missing:])
            for k, v in zip(fields, vals):
                setattr(self, k, float(v))
            _AtomP.__init__(self, atom, record(self))
        cls = type(name, (_AtomP,), {"__init__": __init__, "max_size": lambda self: max_size(self)})
        return cls

    EpsSigAtom = _atom_type("EpsSigAtom", ("epsilon", "sigma"), lambda a: (a.epsilon, a.sigma, 0.0),
                            lambda a: a.sigma)
    EpsSigCutAtom = _atom_type("EpsSigCutAtom", ("epsilon", "sigma", "sigcut"),
                               lambda a: (a.epsilon, a.sigma, a.sigcut), lambda a: a.sigma * a.sigcut)
    EpsSigExpAtom = _atom_type("EpsSigExpAtom", ("eps", "sigma", "exponent"), lambda a: (a.eps, a.sigma, a.exponent),
                               lambda a: a.sigma)
    EpsSigExpDragAtom = _atom_type("EpsSigExpDragAtom", ("eps", "sigma", "gamma", "exponent"),
                                   lambda a: (a.eps, a.sigma, a.exponent, a.gamma), lambda a: a.sigma,
                                   defaults=(2.5,))
    LoisOhernAtom = _atom_type("LoisOhernAtom", ("eps", "sigma", "C", "l"), lambda a: (a.eps, a.sigma, a.C, a.l),
                               lambda a: a.sigma * (1 + a.C + a.l))

    class LoisLinAtom(_AtomP):
        def __init__(self, atom, eps, sigma, depth, width):
            self.eps, self.sigma = eps, sigma
            self.f = depth / width if width > 0 else 0.0
            self.l = width
            super().__init__(atom, (eps, sigma, self.f, self.l))

        def max_size(self):
            return self.sigma * (1 + self.l)

    EisMclachlanAtom = _atom_type("EisMclachlanAtom", ("dist", "sigmai"), lambda a: (a.dist, a.sigmai, 0.0),
                                  lambda a: a.dist)
    EpsEpsSigSigCutAtom = _atom_type("EpsEpsSigSigCutAtom", ("eps_r", "eps_a", "sig_r", "sig_a", "sigcut"),
                                     lambda a: (a.eps_r, a.eps_a, a.sig_r, a.sig_a, a.sigcut),
                                     lambda a: a.sig_r + a.sig_a * (a.sigcut - 1))

    class IEpsISigCutAtom(_AtomP):
        def __init__(self, atom, epsilons, sigmas, indx, cut):
            self.epsilons, self.sigmas, self.indx, self.sigcut = list(epsilons), list(sigmas), int(indx), cut
            self.rows = (self.indx, self.epsilons, self.sigmas)
            super().__init__(atom, (indx, cut, 0.0))

        def max_size(self):
            return max(self.sigmas) * self.sigcut

    class IEpsSigCutAtom(_AtomP):
        def __init__(self, atom, epsilons, indx, sigma, cut):
            self.epsilons, self.indx, self.sigma, self.sigcut = list(epsilons), int(indx), sigma, cut
            self.rows = (self.indx, self.epsilons, None)
            super().__init__(atom, (indx, sigma, cut))

        def max_size(self):
            return self.sigma * self.sigcut

    class IEpsRepsSigCutAtom(_AtomP):
        def __init__(self, atom, epsilons, repeps, sigma, indx, cut):
            self.epsilons, self.repeps, self.sig, self.indx, self.sigcut = list(epsilons), repeps, sigma, int(indx), cut
            self.rows = (self.indx, self.epsilons, None)
            super().__init__(atom, (indx, repeps, sigma, cut))

        def max_size(self):
            return self.sig * self.sigcut

    class IEpsRepsSigExpCutAtom(_AtomP):
        def __init__(self, atom, epsilons, repeps, sigma, n, indx, cut):
            self.epsilons, self.repeps, self.sigma, self.exponent = list(epsilons), repeps, sigma, n
            self.indx, self.sigcut = int(indx), cut
            self.rows = (self.indx, self.epsilons, None)
            super().__init__(atom, (indx, repeps, sigma, n, cut))

        def max_size(self):
            return self.sigma * self.sigcut

    class IEpsISigExpAtom(_AtomP):
        def __init__(self, atom, epsilons, sigmas, indx, exponent=2.5):
            self.epsilons, self.sigmas, self.indx, self.exponent = list(epsilons), list(sigmas), int(indx), exponent
            self.rows = (self.indx, self.epsilons, self.sigmas)
            super().__init__(atom, (indx, exponent, 0.0))

        def max_size(self):
            return max(self.sigmas)

    # ---------------------------------------------------- neighbour list
    class NeighborList:
        """The Verlet list (src/trackers.hpp:133-215), and the GPU handle it carries."""

        def __init__(self, box, atoms, skin):
            self.box, self.atoms, self.skin = box, atoms, float(skin)
            n = len(atoms)
            self.kind = -1
            self.params = np.zeros((n, 5))
            self.rank = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
            self.ldiam = np.full(n, np.nan)
            self.nmembers = 0
            self.ignores = []
            self.rows = {}
            self.owner = None
            self.sys = None
            self._rsq = None   # the RsqTracker bound to this handle
            self._dirty = True
            self._pushed = (-1, None, None)
            self._pairs = None

        # -- the reference's interface
        def add(self, atom, diameter):
            i = atom.n()
            if self.rank[i] != 0xFFFFFFFF:
                raise ValueError("NeighborList::add: atom added twice")
            self.rank[i] = self.nmembers
            self.nmembers += 1
            self.ldiam[i] = float(diameter)
            self._dirty = True

        def ignore(self, a, b):
            self.ignores.append((a.n(), b.n()))
            self._dirty = True

        def update_list(self, force=True):
            self.push()
            rebuilt = bool(self.sys.nlist_update(bool(force))[0])
            self._pairs = None
            return rebuilt

        update = update_list

        def numpairs(self):
            self.push()
            return int(self.sys.numpairs()[0])

        def which(self):
            self.push()
            return int(self.sys.which()[0])

        def size(self):
            return self.nmembers

        def _pair_list(self):
            if self._pairs is None:
                self.push()
                self._pairs = self.sys.pairs(0)
            return self._pairs

        def get(self, k):
            p = self._pair_list()
            return IDPair(self.atoms[int(p[k, 0])], self.atoms[int(p[k, 1])])

        def __getitem__(self, k):
            if not 0 <= k < len(self._pair_list()):
                raise IndexError("Index out of bounds")
            return self.get(k)

        def __iter__(self):
            for k in range(len(self._pair_list())):
                yield self.get(k)

        # -- the handle
        def _member(self, atom, kind, p, owner, rows):
            i = atom.n()
            if self.owner is not None and owner is not self.owner:
                raise ValueError("parm_gb300: one NListed interaction per NeighborList")
            if self.kind >= 0 and kind != self.kind:
                raise ValueError("NListed::add: one pair law per interaction")
            if self.rank[i] != 0xFFFFFFFF:
                raise ValueError("NListed::add: atom added twice")
            if rows is not None:
                t, e, s = rows
                old = self.rows.get(t)
                if old is not None and (old[0] != e or old[1] != s):
                    raise ValueError("parm_gb300: atoms of one type index must share their epsilons and sigmas")
                self.rows[t] = (list(e), None if s is None else list(s))
            self.owner, self.kind = owner, kind
            self.params[i, :len(p)] = p
            self.rank[i] = self.nmembers
            self.nmembers += 1
            self._dirty = True

        def push(self):
            """Upload what changed: the box, the interaction, the Atom records."""
            if self.sys is None:
                prec = os.environ.get("PARM_PRECISION", "fp64")
                self.sys = System(len(self.atoms), ndim=NDIM, precision=prec)
            s = self.sys
            L = tuple(self.box.boxsize)
            gamma = getattr(self.box, "gamma", None)
            if self._pushed[1] != L:
                s.set_boxes(np.asarray(L)[None, :])
            if isinstance(self.box, LeesEdwardsBox) and self._pushed[2] != gamma:
                s.set_lees_edwards([gamma])
            if self._dirty and self.nmembers:
                if self.rows:
                    nt = max(max(self.rows) + 1, max(len(e) for e, _ in self.rows.values()))
                    te, ts = np.zeros((nt, nt)), np.zeros((nt, nt))
                    for t, (e, sg) in self.rows.items():
                        te[t, :len(e)] = e
                        if sg is not None:
                            ts[t, :len(sg)] = sg
                    s.set_pair_table(te, ts)
                if np.any(np.isfinite(self.ldiam)):
                    s.set_list_diameters(self.ldiam)
                kind = self.kind if self.kind >= 0 else capi.REPULSION
                s.set_interaction(kind, self.params[:, :capi.nparam(kind)], self.skin, rank=self.rank)
                for a, b in self.ignores:
                    s.ignore(a, b)
                self._dirty = False
                self._pairs = None
            if self._pushed[0] != self.atoms.version and self.atoms._dev is not self:
                r = self.atoms.rec
                s.set_atoms(x=r[:, 0:NDIM], v=r[:, NDIM:2 * NDIM], a=r[:, 2 * NDIM:3 * NDIM],
                            f=r[:, 3 * NDIM:4 * NDIM], m=r[:, 4 * NDIM])
            self._pushed = (self.atoms.version, L, gamma)

        def pull(self):
            """After a device call: the device holds the newest records; the host reads them back on
            its next access to AtomVec.rec (so consecutive calls move no records)."""
            self.atoms._dev = self
            self._pairs = None

        def _fetch(self):
            st = self.sys.get_atoms()
            r = self.atoms._rec
            r[:, 0:NDIM], r[:, NDIM:2 * NDIM] = st["x"], st["v"]
            r[:, 2 * NDIM:3 * NDIM], r[:, 3 * NDIM:4 * NDIM] = st["a"], st["f"]
            self.atoms.touch()   # other handles on these atoms upload them again
            self._pushed = (self.atoms.version, self._pushed[1], self._pushed[2])

        def resident(self):
            """True while the device holds newer Atom records than the host."""
            return self.atoms._dev is self

    # ------------------------------------------------------------ NListed
    class _NListed:
        """A neighbour-listed pair interaction (src/interaction.hpp:1876-1945)."""

        kinds = {}   # atom type -> PARM_* kind

        def __init__(self, *args):
            if len(args) == 3:
                box, atoms, skin = args
                self.nl = NeighborList(box, atoms, skin)
            else:
                atoms, nl = args
                if nl.atoms is not atoms:
                    raise ValueError("NListed: the NeighborList tracks another AtomVec")
                self.nl = nl
            self.atoms = []

        def add(self, atm):
            kind = self.kinds.get(type(atm))
            if kind is None:
                raise TypeError(f"{type(self).__name__}.add: not an atom of this interaction: {type(atm).__name__}")
            self.nl._member(atm.atom, kind, atm.p, self, atm.rows)
            self.atoms.append(atm)

        def neighbor_list(self):
            return self.nl

        def size(self):
            return len(self.atoms)

        def _eval(self, what):
            self.nl.push()
            return self.nl.sys.evaluate(what)[0]

        def energy(self, box=None):
            return float(self._eval(capi.EVAL_ENERGY))

        def pressure(self, box=None):
            return float(self._eval(capi.EVAL_VIRIAL))

        def stress(self, box=None):
            self.nl.push()
            return self.nl.sys.stress()[0]

        def contacts(self, box=None):
            return int(self._eval(capi.EVAL_CONTACTS))

        def overlaps(self, box=None):
            return int(self._eval(capi.EVAL_OVERLAPS))

        def set_forces(self, box=None):
            """Add the pair forces to the atoms' current forces."""
            f0 = self.nl.atoms.rec[:, 3 * NDIM:4 * NDIM].copy()
            self.nl.push()
            self.nl.sys.set_forces(False)
            self.nl.pull()
            self.nl.atoms.rec[:, 3 * NDIM:4 * NDIM] += f0
            self.nl.atoms.touch()

    def _nlisted(name, mapping):
        return type(name, (_NListed,), {"kinds": mapping})

    mod = types.SimpleNamespace()
    mod.NDIM = NDIM
    mod.Vec = Vec
    mod.AtomVec, mod.AtomID, mod.IDPair = AtomVec, AtomID, IDPair
    mod.OriginBox, mod.LeesEdwardsBox = OriginBox, LeesEdwardsBox
    for c in (EpsSigAtom, EpsSigCutAtom, EpsSigExpAtom, EpsSigExpDragAtom, LoisOhernAtom, LoisLinAtom,
              EisMclachlanAtom, EpsEpsSigSigCutAtom, IEpsISigCutAtom, IEpsSigCutAtom, IEpsRepsSigCutAtom,
              IEpsRepsSigExpCutAtom, IEpsISigExpAtom):
        setattr(mod, c.__name__, c)
    mod.NeighborList = NeighborList
    # the %template names of src/sim.i:621-643 (and LJCut: NListed<EpsSigCutAtom, LennardJonesCutPair>)
    for name, mapping in {
        "LJRepulse": {EpsSigAtom: capi.LJREPULSE},
        "LJCut": {EpsSigCutAtom: capi.LJCUT},
        "LJAttractCut": {EpsSigCutAtom: capi.LJATTRACTCUT},
        "LJAttractICut": {IEpsSigCutAtom: capi.LJATTRACTCUT_IEPS},
        "LJAttractIICut": {IEpsISigCutAtom: capi.LJATTRACTCUT_IEPSISIG},
        "LJIICut": {IEpsISigCutAtom: capi.LJCUT_IEPSISIG},
        "LJAttractRepulse": {IEpsSigCutAtom: capi.LJATTRACTREPULSE},
        "LJAttractFixedRepulse": {IEpsRepsSigCutAtom: capi.LJATTRACTFIXEDREPULSE},
        "EisMclachlan": {EisMclachlanAtom: capi.EISMCLACHLAN},
        "LJish": {IEpsRepsSigExpCutAtom: capi.LJISH},
        "LJAttractRepulseSigs": {EpsEpsSigSigCutAtom: capi.LJATTRACTREPULSESIGS},
        "Repulsion": {EpsSigExpAtom: capi.REPULSION},
        "RepulsionII": {IEpsISigExpAtom: capi.REPULSION_IEPSISIG},
        "HertzianDrag": {EpsSigExpDragAtom: capi.REPULSIONDRAG},
        "LoisOhern": {LoisOhernAtom: capi.LOISOHERN},
        "LoisOhernMin": {LoisOhernAtom: capi.LOISOHERN_MIN},
        "LoisLin": {LoisLinAtom: capi.LOISLIN},
        "LoisLinMin": {LoisLinAtom: capi.LOISLIN_MIN},
    }.items():
        setattr(mod, name, _nlisted(name, mapping))

    # ------------------------------------------------------------ trackers
    class RsqTracker:
        """Mean-square displacement over windows of ns[j] updates (src/constraints.hpp:318-361,
        src/constraints.cpp:404-564) on the GPU.  Alone it holds its own handle and is sent the
        positions at each update; a Collection stepping the same AtomVec binds it to its own handle,
        whose time steps then update it on the device."""

        def __init__(self, atoms, ns, usecom=True):
            self.atoms, self.ns, self.usecom = atoms, [int(n) for n in ns], bool(usecom)
            self.nl = None
            self.sys = System(len(atoms), ndim=NDIM, precision="fp64")
            self.sys.set_boxes(np.ones((1, NDIM)))   # positions are unwrapped: the box is not used
            self.reset()

        def _h(self):
            return self.nl.sys if self.nl is not None else self.sys

        def _push(self):
            if self.nl is not None:
                self.nl.push()
            else:
                r = self.atoms.rec
                self.sys.set_atoms(x=r[:, 0:NDIM], m=r[:, 4 * NDIM])

        def reset(self):
            self._push()
            self._h().rsq_start(self.ns, self.usecom)
            self._start = self.atoms.rec[:, 0:NDIM].copy()
            self._updates = 0

        def update(self, box=None):
            self._push()
            self._h().rsq_update()
            self._updates += 1

        def bind(self, nl):
            """Move onto `nl`'s handle; only before the first update since the last reset and with
            the atoms where they were then (nothing is lost), and one tracker per handle."""
            if self.nl is not None:
                return self.nl is nl
            if nl.atoms is not self.atoms or self._updates or getattr(nl, "_rsq", None) is not None:
                return False
            if not np.array_equal(self.atoms.rec[:, 0:NDIM], self._start):
                return False
            nl.push()
            nl.sys.rsq_start(self.ns, self.usecom)
            nl._rsq, self.nl = self, nl
            self.sys.close()
            self.sys = None
            return True

        def xyz2(self):
            return list(self._h().rsq_get(capi.RSQ_XYZ2))

        def xyz4(self):
            return list(self._h().rsq_get(capi.RSQ_XYZ4))

        def r2(self):
            return list(self._h().rsq_get(capi.RSQ_R2))

        def r4(self):
            return list(self._h().rsq_get(capi.RSQ_R4))

        def counts(self):
            return list(self._h().rsq_get(capi.RSQ_COUNTS))

    # ---------------------------------------------------------- collections
    class Collection:
        """Integrators of the atoms of one NListed interaction (src/collection.hpp:23-131)."""

        def __init__(self, box, atoms, interactions=(), trackers=(), constraints=(), initialize=True):
            if len(constraints):
                raise ValueError("parm_gb300: constraints are not supported on the GPU path")
            self.box, self.atoms = box, atoms
            self.interactions, self.trackers = list(interactions), list(trackers)
            nls = {id(i.nl): i.nl for i in self.interactions}
            nls.update({id(t): t for t in self.trackers if isinstance(t, NeighborList)})
            if len(nls) > 1:
                raise ValueError("parm_gb300: one NListed interaction (one neighbour list) per Collection")
            self.nl = next(iter(nls.values())) if nls else None
            if self.nl is not None and self.nl.atoms is not atoms:
                raise ValueError("parm_gb300: the interaction was built on another AtomVec")
            if self.nl is not None:
                for t in self.trackers:
                    if isinstance(t, RsqTracker):
                        t.bind(self.nl)
            if initialize:
                self.initialize()

        def initialize(self):
            self.update_trackers()
            self.set_forces(True)
            self.update_trackers()

        def update_trackers(self):
            for t in self.trackers:
                if isinstance(t, NeighborList):
                    t.update_list(False)
                else:
                    t.update(self.box)

        def set_forces(self, seta=True):
            if self.nl is None or not self.interactions:
                self.atoms.rec[:, 3 * NDIM:4 * NDIM] = 0.0
                if seta:
                    self.atoms.rec[:, 2 * NDIM:3 * NDIM] = 0.0
                self.atoms.touch()
                return
            self.nl.push()
            self.nl.sys.set_forces(bool(seta))
            self.nl.pull()

        def _steps(self, n):
            raise NotImplementedError

        def _host_trackers(self):
            # the GPU steps update the neighbour list and the trackers bound to its handle
            return [t for t in self.trackers
                    if not isinstance(t, NeighborList) and not (isinstance(t, RsqTracker) and t.nl is self.nl)]

        def timesteps(self, n):
            if n <= 0:
                return
            self.nl.push()
            host = self._host_trackers()
            if host:
                for _ in range(n):   # trackers of the host see every step
                    self._steps(1)
                    self.nl.pull()
                    for t in host:
                        t.update(self.box)
                    self.nl.push()
                return
            self._steps(n)
            self.nl.pull()

        def timestep(self):
            self.timesteps(1)

        def potential_energy(self):
            return float(sum(i.energy(self.box) for i in self.interactions))

        def _resident(self):
            return self.nl is not None and self.nl.resident()

        def _ke(self, v0=None):
            # on the device while it holds the newest velocities (no records move)
            if self._resident():
                return float(self.nl.sys.kinetic_energy(None if v0 is None else np.asarray(v0)[None, :])[0])
            return self.atoms.kinetic_energy(v0)

        def kinetic_energy(self):
            return self._ke()

        def energy(self):
            return self.potential_energy() + self.kinetic_energy()

        def degrees_of_freedom(self):
            return NDIM * int(np.sum(self.atoms._mobile()))

        def com(self):
            return self.atoms.com()

        def com_velocity(self):
            if self._resident():
                mom, mass = self.nl.sys.momentum()
                return mom[0] / mass[0]
            return self.atoms.com_velocity()

        def reset_com_velocity(self):
            self.atoms.reset_com_velocity()

        def temp(self, minuscomv=True):
            v = self.com_velocity() if minuscomv else None
            ndof = self.degrees_of_freedom() - (NDIM if minuscomv else 0)
            return self._ke(v) * 2 / ndof

        def pressure(self):
            E = 2.0 * self.kinetic_energy() + sum(i.pressure(self.box) for i in self.interactions)
            return E / self.box.V() / NDIM

        def scale_velocities(self, by):
            mob = self.atoms._mobile()
            self.atoms.rec[mob, NDIM:2 * NDIM] *= by
            self.atoms.touch()

        def scale_velocities_to_temp(self, T, minuscomv=True):
            self.scale_velocities(math.sqrt(T / self.temp(minuscomv)))

        def scale_velocities_to_energy(self, E):
            E0, k0 = self.energy(), self.kinetic_energy()
            self.scale_velocities(math.sqrt((k0 + (E - E0)) / k0))

    class CollectionVerlet(Collection):
        def __init__(self, box, atoms, dt, interactions=(), trackers=(), constraints=()):
            self.dt = float(dt)
            super().__init__(box, atoms, interactions, trackers, constraints)

        def _steps(self, n):
            self.nl.sys.verlet(self.dt, n)

    class CollectionDamped(Collection):
        def __init__(self, box, atoms, dt, damping, interactions=(), trackers=(), constraints=()):
            self.dt, self.damping = float(dt), float(damping)
            super().__init__(box, atoms, interactions, trackers, constraints)

        def _steps(self, n):
            self.nl.sys.damped(self.dt, self.damping, n)

    class CollectionSol(Collection):
        """Langevin dynamics (src/collection.cpp:230-322) with counter-based per-atom noise."""

        def __init__(self, box, atoms, dt, damping, desired_temperature, interactions=(), trackers=(),
                     constraints=()):
            if dt <= 0:
                raise ValueError("Collection::CollectionSol: dt >= 0")
            self.dt, self.damping, self.desT = float(dt), float(damping), float(desired_temperature)
            self.key = _seed[0]
            _seed[0] = (_seed[0] * 6364136223846793005 + 1442695040888963407) % 2 ** 64
            super().__init__(box, atoms, interactions, trackers, constraints)

        def _steps(self, n):
            self.nl.sys.sol(self.dt, self.damping, self.desT, self.key, n)

    _STATE = capi.NLCG_STATE

    class CollectionNLCG(Collection):
        """Conjugate-gradient minimiser of positions and box (src/collection.hpp:400-475)."""

        boxed = True
        _limits = (2.0, 0.0, 100.0, 1e-3)   # alphamax, afrac, dxmax, stepmax

        def __init__(self, box, atoms, dt, P0, interactions=(), trackers=(), constraints=(), kappa=10.0,
                     kmax=1000, secmax=40, seceps=1e-20):
            self.dt, self.P0, self.kappa, self.kmax = float(dt), float(P0), float(kappa), float(kmax)
            self.secmax, self.seceps = int(secmax), float(seceps)
            self.alphamax, self.afrac, self.dxmax, self.stepmax = self._limits
            self.maxdV = 0.0
            for k in _STATE:
                setattr(self, k, 0.0)
            self.sec = 0
            self._inited = None
            super().__init__(box, atoms, interactions, trackers, constraints, initialize=False)
            # the C++ constructor's Collection::initialize runs in the base class, so its set_forces
            # is Collection::set_forces (src/collection.cpp:494-501, 13-19)
            self.update_trackers()
            Collection.set_forces(self, True)
            self.update_trackers()

        def _params(self):
            return [self.dt, self.P0, self.kappa, self.kmax, float(self.secmax), self.seceps, self.alphamax,
                    self.afrac, self.dxmax, self.stepmax, self.maxdV]

        def _push(self):
            self.nl.push()
            s = self.nl.sys
            if self._inited is not s:
                s.nlcg_init(self._params(), boxed=self.boxed)
                self._inited = s
            else:
                s.nlcg_set_params(self._params())
            s.nlcg_set_state([float(getattr(self, k)) for k in _STATE])
            return s

        def _pull(self, s):
            st = s.nlcg_state()[0]
            for k, v in zip(_STATE, st):
                setattr(self, k, float(v))
            self.sec = int(self.sec)
            self.nl.pull()
            if self.boxed:
                self.box.boxsize = s.boxes()[0].copy()
                self.nl._pushed = (self.nl._pushed[0], tuple(self.box.boxsize), self.nl._pushed[2])

        def set_forces(self, seta=True, setV=True):
            if self.nl is None or not self.interactions:
                return Collection.set_forces(self, seta)
            if not self.boxed:
                return Collection.set_forces(self, seta)
            s = self._push()
            s.nlcg_set_forces(bool(seta))
            self._pull(s)

        def reset(self):
            s = self._push()
            s.nlcg_reset()
            self._pull(s)

        def descend(self):
            s = self._push()
            s.nlcg_descend()
            self._pull(s)

        def timesteps(self, n):
            if n <= 0:
                return
            # the minimiser's steps update no tracker but the neighbour list
            host = [t for t in self.trackers if not isinstance(t, NeighborList)]
            if not host:
                s = self._push()
                s.nlcg_timestep(n)
                self._pull(s)
                return
            for _ in range(n):
                s = self._push()
                s.nlcg_timestep(1)
                self._pull(s)
                for t in host:
                    t.update(self.box)

        def set_dt(self, dt):
            self.dt = float(dt)
            self.reset()

        def set_pressure_goal(self, P0):
            self.P0 = float(P0)
            self.reset()

        def set_kappa(self, kappa):
            self.kappa = float(kappa)
            self.reset()

        def set_max_alpha(self, a):
            self.alphamax = float(a)

        def set_max_alpha_fraction(self, a):
            self.afrac = float(a)

        def set_max_dx(self, d):
            self.dxmax = float(d)

        def set_max_step(self, d):
            self.stepmax = float(d)

        def hamiltonian(self):
            return self.potential_energy() + self.P0 * self.box.V()

        def kinetic_energy(self):
            # CollectionNLCG::kinetic_energy (src/collection.cpp:572-587): masses ignored
            r = self.atoms.rec
            mob = self.atoms._mobile()
            Lfac = math.exp(self.vl / (self.kappa * NDIM))
            v = r[mob, NDIM:2 * NDIM] + r[mob, 0:NDIM] * Lfac
            return float(np.sum(v * v) / 2.0)

        def pressure(self):
            return sum(i.pressure(self.box) for i in self.interactions) / self.box.V() / NDIM

    class CollectionNLCGV(CollectionNLCG):
        """Conjugate-gradient minimiser of the positions in a fixed box (src/collection.hpp:490-566)."""

        boxed = False
        _limits = (0.0, 0.0, 0.0, 0.0)

        def __init__(self, box, atoms, dt, interactions=(), trackers=(), constraints=(), kmax=1000, secmax=10,
                     seceps=1e-4):
            super().__init__(box, atoms, dt, 0.0, interactions, trackers, constraints, 10.0, kmax, secmax, seceps)

        def kinetic_energy(self):
            return self.atoms.kinetic_energy()

    for c in (Collection, CollectionVerlet, CollectionDamped, CollectionSol, CollectionNLCG, CollectionNLCGV,
              RsqTracker):
        setattr(mod, c.__name__, c)
    mod.seed = seed
    # picklable by name: pyparm.d3.AtomVec and so on
    for name, obj in vars(mod).items():
        if isinstance(obj, type):
            obj.__qualname__ = f"d{NDIM}.{name}"
            obj.__module__ = __name__
    return mod


def _round_half_away(x: float) -> float:
    """C's round(): halves away from zero (abs(x) - floor(abs(x)) is exact below 2^52)."""
    a = abs(x)
    if a >= 2 ** 52:
        return x
    t = math.floor(a)
    return math.copysign(t + 1.0 if a - t >= 0.5 else t, x)


d3 = _make(3)
d2 = _make(2)
