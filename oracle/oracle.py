"""ctypes wrapper of the CPU oracle (oracle.cpp) — test infrastructure only.

The class mirrors the reference objects one simulation at a time: an
AtomVec + OriginBox, one NListed<A,P> interaction with its NeighborList, and
the Collection time steps.  Arrays are (natoms, ndim) float64 in atom order.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from .build import build

_dp = C.POINTER(C.c_double)
_u32p = C.POINTER(C.c_uint32)
_lib = None

LJCUT, REPULSION, LJREPULSE = 0, 1, 2


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        sig = {
            "orc_create": (C.c_void_p, [C.c_int, C.c_uint32]),
            "orc_destroy": (None, [C.c_void_p]),
            "orc_set_box": (None, [C.c_void_p, _dp]),
            "orc_set_state": (None, [C.c_void_p, _dp, _dp, _dp, _dp, _dp]),
            "orc_get_state": (None, [C.c_void_p, _dp, _dp, _dp, _dp, _dp]),
            "orc_set_interaction": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
            "orc_add_atom": (C.c_int, [C.c_void_p, C.c_uint32, _dp]),
            "orc_ignore": (None, [C.c_void_p, C.c_uint32, C.c_uint32]),
            "orc_add_member": (C.c_int, [C.c_void_p, C.c_uint32, C.c_double]),
            "orc_set_lees": (None, [C.c_void_p, C.c_int, C.c_double]),
            "orc_set_pair_table": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_double),
                                             C.POINTER(C.c_double)]),
            "orc_nl_update": (C.c_int, [C.c_void_p, C.c_int]),
            "orc_nl_which": (C.c_uint32, [C.c_void_p]),
            "orc_nl_numpairs": (C.c_uint64, [C.c_void_p]),
            "orc_nl_get_pairs": (None, [C.c_void_p, _u32p]),
            "orc_energy": (C.c_double, [C.c_void_p]),
            "orc_pressure": (C.c_double, [C.c_void_p, _dp]),
            "orc_contacts": (C.c_uint64, [C.c_void_p]),
            "orc_overlaps": (C.c_uint64, [C.c_void_p]),
            "orc_set_forces": (None, [C.c_void_p, C.c_int, _dp, _dp]),
            "orc_initialize": (None, [C.c_void_p]),
            "orc_update_trackers": (None, [C.c_void_p]),
            "orc_verlet": (None, [C.c_void_p, C.c_double, C.c_uint32]),
            "orc_damped": (None, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_uint32]),
            "orc_sol": (None, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                               C.c_double, C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_uint64,
                               C.c_uint32]),
            "orc_normals6": (None, [C.c_uint64, C.c_uint64, C.c_uint32, _dp]),
            "orc_philox": (None, [_u32p, _u32p, C.c_uint64]),
            "orc_nlcg_create": (C.c_void_p, [C.c_int, _dp]),
            "orc_nlcg_destroy": (None, [C.c_void_p]),
            "orc_nlcg_set_params": (None, [C.c_void_p, _dp]),
            "orc_nlcg_get_state": (None, [C.c_void_p, _dp]),
            "orc_nlcg_set_state": (None, [C.c_void_p, _dp]),
            "orc_nlcg_set_forces": (None, [C.c_void_p, C.c_void_p, C.c_int]),
            "orc_nlcg_reset": (None, [C.c_void_p, C.c_void_p]),
            "orc_nlcg_descend": (None, [C.c_void_p, C.c_void_p]),
            "orc_nlcg_timestep": (None, [C.c_void_p, C.c_void_p, C.c_uint32]),
            "orc_get_box": (None, [C.c_void_p, _dp]),
            "orc_kinetic_energy": (C.c_double, [C.c_void_p, _dp]),
            "orc_momentum": (C.c_double, [C.c_void_p, _dp]),
            "orc_pairs_celllist": (C.c_uint64, [C.c_void_p, _u32p, C.c_uint64]),
            "orc_nl_install": (None, [C.c_void_p, _u32p, C.c_uint64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def splitmix64(x: int) -> int:
    m = (1 << 64) - 1
    x = (x + 0x9E3779B97F4A7C15) & m
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & m
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & m
    return x ^ (x >> 31)


def damped_constants(dt: float, damping: float):
    """CollectionDamped::set_constants (src/collection.cpp:339-354)."""
    if damping <= 0.0:
        return 1.0, 1.0, 0.5
    dampdt = damping * dt
    c0 = math.exp(-dampdt)
    c1 = (-math.expm1(-dampdt)) / dampdt
    c2 = (1 - c1) / dampdt
    return c0, c1, c2


def sol_constants(dt: float, damping: float):
    """CollectionSol::set_constants (src/collection.cpp:230-263) + BivariateGauss::set."""
    if damping <= 0.0:
        c0, c1, c2, sr, sv, corr = 1.0, 1.0, 0.5, 0.0, 0.0, 1.0
    else:
        dampdt = damping * dt
        c0 = math.exp(-dampdt)
        c1 = (-math.expm1(-dampdt)) / dampdt
        c2 = (1 - c1) / dampdt
        if dampdt > 1e-4:
            sr = math.sqrt((1 / dampdt) * (2 - (-4 * math.expm1(-dampdt) + math.expm1(-2 * dampdt)) / dampdt))
        else:
            sr = math.sqrt(2 * dampdt / 3 - dampdt * dampdt / 2 + 7 * dampdt * dampdt * dampdt / 30)
        sv = math.sqrt(-math.expm1(-2 * dampdt))
        ex = -math.expm1(-dampdt)
        corr = ex * ex / dampdt / sr / sv
    return c0, c1, c2, sr, sv * corr, sv * math.sqrt(1 - corr * corr)



def nparam(kind: int) -> int:
    """Doubles per atom of a pair kind's parameters (the C ABI's PARM_NPARAM)."""
    if 4 <= kind <= 7 or kind in (9, 14):
        return 4
    if kind in (15, 17):
        return 5
    return 3

class Oracle:
    def __init__(self, n: int, ndim: int = 3):
        self.L_ = lib()
        self.n, self.ndim = n, ndim
        self.h = self.L_.orc_create(ndim, n)

    def __del__(self):
        if getattr(self, "h", None):
            self.L_.orc_destroy(self.h)
            self.h = None

    def set_box(self, L):
        arr = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (self.ndim,)))
        self.L_.orc_set_box(self.h, _d(arr))

    def set_state(self, x=None, v=None, a=None, f=None, m=None):
        sh = (self.n, self.ndim)
        cv = lambda q, s: None if q is None else np.ascontiguousarray(np.broadcast_to(np.asarray(q, np.float64), s))
        x, v, a, f, m = cv(x, sh), cv(v, sh), cv(a, sh), cv(f, sh), cv(m, (self.n,))
        self.L_.orc_set_state(self.h, _d(x), _d(v), _d(a), _d(f), _d(m))

    def get_state(self):
        sh = (self.n, self.ndim)
        x, v, a, f = (np.zeros(sh) for _ in range(4))
        m = np.zeros(self.n)
        self.L_.orc_get_state(self.h, _d(x), _d(v), _d(a), _d(f), _d(m))
        return {"x": x, "v": v, "a": a, "f": f, "m": m}

    def set_interaction(self, kind, params, skin, order=None):
        """NListed(box, atoms, skin) and add() of every atom in `order`."""
        assert self.L_.orc_set_interaction(self.h, kind, float(skin)) == 0
        params = np.asarray(params, dtype=np.float64).reshape(self.n, nparam(kind))
        order = range(self.n) if order is None else order
        for i in order:
            p = np.ascontiguousarray(params[i])
            assert self.L_.orc_add_atom(self.h, int(i), _d(p)) == 0

    def set_lees_edwards(self, gamma):
        """A LeesEdwardsBox of shear gamma (None: the OriginBox)."""
        self.L_.orc_set_lees(self.h, 0 if gamma is None else 1, 0.0 if gamma is None else float(gamma))

    def set_pair_table(self, eps, sig=None):
        """Pair tables of the indexed kinds (10-15): eps[a, b] = first atom's epsilons[b] for a
        first atom of type a."""
        eps = np.ascontiguousarray(np.asarray(eps, dtype=np.float64))
        nt = eps.shape[0]
        sp = None
        if sig is not None:
            sig = np.ascontiguousarray(np.asarray(sig, dtype=np.float64).reshape(nt, nt))
            sp = _d(sig)
        assert self.L_.orc_set_pair_table(self.h, nt, _d(eps), sp) == 0

    def add_member(self, i, diameter):
        """NeighborList::add(atom, diameter): a list member without pair parameters."""
        assert self.L_.orc_add_member(self.h, int(i), float(diameter)) == 0

    def ignore(self, a, b):
        self.L_.orc_ignore(self.h, int(a), int(b))

    def nl_update(self, force=True) -> bool:
        return bool(self.L_.orc_nl_update(self.h, 1 if force else 0))

    def which(self) -> int:
        return int(self.L_.orc_nl_which(self.h))

    def pairs(self) -> np.ndarray:
        k = int(self.L_.orc_nl_numpairs(self.h))
        out = np.zeros((k, 2), dtype=np.uint32)
        if k:
            self.L_.orc_nl_get_pairs(self.h, out.ctypes.data_as(_u32p))
        return out

    def pairs_celllist(self) -> np.ndarray:
        k = int(self.L_.orc_pairs_celllist(self.h, None, 0))
        out = np.zeros((k, 2), dtype=np.uint32)
        if k:
            self.L_.orc_pairs_celllist(self.h, out.ctypes.data_as(_u32p), k)
        return out

    def install_pairs(self, pairs: np.ndarray):
        p = np.ascontiguousarray(pairs, dtype=np.uint32)
        self.L_.orc_nl_install(self.h, p.ctypes.data_as(_u32p), len(p))

    def build_fast(self):
        """update_list(true) through the cell-list construction of the same pair set."""
        self.install_pairs(self.pairs_celllist())

    def energy(self) -> float:
        return float(self.L_.orc_energy(self.h))

    def pressure(self):
        st = np.zeros(self.ndim * self.ndim)
        p = float(self.L_.orc_pressure(self.h, _d(st)))
        return p, st.reshape(self.ndim, self.ndim)

    def contacts(self) -> int:
        return int(self.L_.orc_contacts(self.h))

    def overlaps(self) -> int:
        return int(self.L_.orc_overlaps(self.h))

    def set_forces(self, constraints_and_a=True, with_pressure=False):
        if with_pressure:
            p = np.zeros(1)
            st = np.zeros(self.ndim * self.ndim)
            self.L_.orc_set_forces(self.h, 1 if constraints_and_a else 0, _d(p), _d(st))
            return float(p[0]), st.reshape(self.ndim, self.ndim)
        self.L_.orc_set_forces(self.h, 1 if constraints_and_a else 0, None, None)
        return None

    def initialize(self):
        self.L_.orc_initialize(self.h)

    def update_trackers(self):
        self.L_.orc_update_trackers(self.h)

    def verlet(self, dt, nsteps=1):
        self.L_.orc_verlet(self.h, float(dt), int(nsteps))

    def damped(self, dt, damping, nsteps=1):
        c0, c1, c2 = damped_constants(dt, damping)
        self.L_.orc_damped(self.h, float(dt), c0, c1, c2, int(nsteps))

    def sol(self, dt, damping, T, seed, step0, nsteps=1):
        """step0: the generator counter of the first step (GPU: counter after its advance)."""
        c0, c1, c2, x11, x21, x22 = sol_constants(dt, damping)
        self.L_.orc_sol(self.h, float(dt), float(damping), float(T), c0, c1, c2, x11, x21, x22,
                        int(seed), int(step0), int(nsteps))

    def kinetic_energy(self, origin=None) -> float:
        o = None if origin is None else np.ascontiguousarray(np.asarray(origin, np.float64))
        return float(self.L_.orc_kinetic_energy(self.h, _d(o)))

    def momentum(self):
        out = np.zeros(self.ndim)
        mass = float(self.L_.orc_momentum(self.h, _d(out)))
        return out, mass


def normals6(seed: int, step: int, atom: int) -> np.ndarray:
    out = np.zeros(6)
    lib().orc_normals6(int(seed), int(step), int(atom), out.ctypes.data_as(_dp))
    return out


def philox(ctr_key) -> np.ndarray:
    """Philox4x32-10 of the oracle on rows (c0, c1, c2, c3, k0, k1); returns (n, 4) uint32."""
    a = np.ascontiguousarray(np.asarray(ctr_key, dtype=np.uint32).reshape(-1, 6))
    out = np.zeros((a.shape[0], 4), dtype=np.uint32)
    lib().orc_philox(a.ctypes.data_as(_u32p), out.ctypes.data_as(_u32p), a.shape[0])
    return out


NLCG_PARAMS = ("dt", "P0", "kappa", "kmax", "secmax", "seceps", "alphamax", "afrac", "dxmax", "stepmax", "maxdV")
NLCG_STATE = ("Knew", "k", "vl", "fl", "al", "alpha", "beta", "betaused", "dxsum", "alphavmax", "sec")


def nlcg_params(dt, P0=0.0, kappa=10.0, kmax=1000, secmax=40, seceps=1e-20, alphamax=2.0, afrac=0.0,
                dxmax=100.0, stepmax=1e-3, maxdV=0.0) -> np.ndarray:
    """CollectionNLCG's parameter vector, defaults of its constructor (collection.cpp:494-523)."""
    return np.array([dt, P0, kappa, kmax, secmax, seceps, alphamax, afrac, dxmax, stepmax, maxdV],
                    dtype=np.float64)


def nlcgv_params(dt, kmax=1000, secmax=10, seceps=1e-4, alphamax=0.0, afrac=0.0, dxmax=0.0,
                 stepmax=0.0) -> np.ndarray:
    """CollectionNLCGV's parameter vector, defaults of its constructor (collection.cpp:877-898);
    P0, kappa and maxdV do not apply."""
    return np.array([dt, 0.0, 1.0, kmax, secmax, seceps, alphamax, afrac, dxmax, stepmax, 0.0],
                    dtype=np.float64)


class OracleNLCG:
    """CollectionNLCG (boxed) / CollectionNLCGV on an Oracle system."""

    def __init__(self, orc: "Oracle", params, boxed=True):
        self.o = orc
        self.L_ = lib()
        p = np.ascontiguousarray(params, dtype=np.float64)
        self.g = self.L_.orc_nlcg_create(1 if boxed else 0, _d(p))

    def __del__(self):
        if getattr(self, "g", None):
            self.L_.orc_nlcg_destroy(self.g)
            self.g = None

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float64)
        self.L_.orc_nlcg_set_params(self.g, _d(p))

    def state(self) -> dict:
        out = np.zeros(len(NLCG_STATE))
        self.L_.orc_nlcg_get_state(self.g, _d(out))
        return dict(zip(NLCG_STATE, out))

    def set_forces(self, constraints_and_a=True):
        self.L_.orc_nlcg_set_forces(self.g, self.o.h, 1 if constraints_and_a else 0)

    def reset(self):
        self.L_.orc_nlcg_reset(self.g, self.o.h)

    def descend(self):
        self.L_.orc_nlcg_descend(self.g, self.o.h)

    def timestep(self, n=1):
        self.L_.orc_nlcg_timestep(self.g, self.o.h, int(n))

    def box(self) -> np.ndarray:
        out = np.zeros(self.o.ndim)
        self.L_.orc_get_box(self.o.h, _d(out))
        return out
