"""Python view of one parm_gb300 handle (a batch of periodic systems on the GPU).

Arrays crossing this boundary use the reference's per-atom vectors as
``(natoms, ndim)`` float64 arrays in the caller's atom order; the library
converts to and from its internal cell-ordered layout on the GPU.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import capi
from .capi import check, dptr, u32ptr, u64ptr


def _as_f64(a, shape) -> np.ndarray:
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if arr.shape != shape:
        arr = np.ascontiguousarray(np.broadcast_to(arr, shape))
    return arr


class System:
    """A GPU handle for ``nsys`` independent periodic systems.

    ``natoms`` is an int (one system) or a sequence of per-system sizes.
    ``precision`` is ``"fp64"`` (bit-exact with the reference) or ``"mixed"``.
    """

    def __init__(self, natoms: int | Sequence[int], ndim: int = 3, precision: str = "fp64"):
        self.lib = capi.load()
        sizes = [int(natoms)] if np.isscalar(natoms) else [int(s) for s in natoms]
        self.sizes = np.asarray(sizes, dtype=np.uint32)
        self.nsys = len(sizes)
        self.n = int(self.sizes.sum())
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)[:-1]]).astype(np.int64)
        self.ndim = ndim
        self.precision = precision
        prec = {"fp64": capi.FP64, "mixed": capi.MIXED}[precision]
        h = C.c_void_p()
        check(self.lib.parm_create(C.byref(h), ndim, self.nsys, u32ptr(self.sizes), prec))
        self.h = h
        self.stride = 4 * ndim + 1
        self._rsq_n = 0

    # -- lifetime --
    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.parm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- box / atoms --
    def set_boxes(self, L) -> None:
        arr = _as_f64(L, (self.nsys, self.ndim))
        check(self.lib.parm_set_boxes(self.h, dptr(arr)))

    def set_atoms(self, x=None, v=None, a=None, f=None, m=None) -> None:
        nd = self.ndim
        buf = np.zeros((self.n, self.stride))
        fields = 0
        for bit, off, val in ((capi.X, 0, x), (capi.V, nd, v), (capi.A, 2 * nd, a), (capi.F, 3 * nd, f)):
            if val is not None:
                buf[:, off:off + nd] = _as_f64(val, (self.n, nd))
                fields |= bit
        if m is not None:
            buf[:, 4 * nd] = _as_f64(m, (self.n,))
            fields |= capi.M
        check(self.lib.parm_set_atoms(self.h, dptr(buf), self.stride, fields))

    def get_atoms(self, fields: int = 31) -> dict:
        buf = np.zeros((self.n, self.stride))
        check(self.lib.parm_get_atoms(self.h, dptr(buf), self.stride, fields))
        nd = self.ndim
        out = {}
        for name, bit, off in (("x", capi.X, 0), ("v", capi.V, nd), ("a", capi.A, 2 * nd), ("f", capi.F, 3 * nd)):
            if fields & bit:
                out[name] = buf[:, off:off + nd].copy()
        if fields & capi.M:
            out["m"] = buf[:, 4 * nd].copy()
        return out

    # -- interaction / neighbour list --
    def set_interaction(self, kind: int, params, skin: float, rank=None) -> None:
        p = _as_f64(params, (self.n, capi.nparam(kind)))
        rk = None
        if rank is not None:
            rk = np.ascontiguousarray(np.asarray(rank, dtype=np.uint32))
        check(self.lib.parm_set_interaction(self.h, kind, dptr(p), u32ptr(rk) if rk is not None else None,
                                            float(skin)))

    def set_lees_edwards(self, gamma) -> None:
        """LeesEdwardsBox shears, one per system (None: OriginBoxes again); FP64 handles."""
        if gamma is None:
            check(self.lib.parm_set_lees_edwards(self.h, None))
            return
        g = _as_f64(gamma, (self.nsys,))
        check(self.lib.parm_set_lees_edwards(self.h, dptr(g)))

    def set_pair_table(self, eps, sig=None) -> None:
        """Pair tables of the indexed kinds: eps[a, b] = epsilons[b] of the atoms of type a
        (IEps*Atom), sig likewise (IEpsISigCutAtom::sigmas)."""
        e = np.ascontiguousarray(np.asarray(eps, dtype=np.float64))
        nt = e.shape[0]
        e = _as_f64(e, (nt, nt))
        sg = _as_f64(sig, (nt, nt)) if sig is not None else None
        check(self.lib.parm_set_pair_table(self.h, nt, dptr(e), dptr(sg) if sg is not None else None))

    def set_list_diameters(self, diam) -> None:
        """NeighborList::add(atom, diameter): explicit list diameters (NaN: from the parameters); None clears."""
        if diam is None:
            check(self.lib.parm_set_list_diameters(self.h, None))
            return
        d = _as_f64(diam, (self.n,))
        check(self.lib.parm_set_list_diameters(self.h, dptr(d)))

    def ignore(self, a: int, b: int) -> None:
        check(self.lib.parm_nlist_ignore(self.h, int(a), int(b)))

    def nlist_update(self, force: bool = True) -> np.ndarray:
        out = np.zeros(self.nsys, dtype=np.uint8)
        check(self.lib.parm_nlist_update(self.h, 1 if force else 0, out.ctypes.data_as(C.POINTER(C.c_uint8))))
        return out.astype(bool)

    def which(self) -> np.ndarray:
        out = np.zeros(self.nsys, dtype=np.uint32)
        check(self.lib.parm_nlist_which(self.h, u32ptr(out)))
        return out

    def numpairs(self) -> np.ndarray:
        out = np.zeros(self.nsys, dtype=np.uint64)
        check(self.lib.parm_nlist_numpairs(self.h, u64ptr(out)))
        return out

    def pairs(self, sys: int = 0) -> np.ndarray:
        n = np.zeros(1, dtype=np.uint64)
        check(self.lib.parm_nlist_pairs(self.h, sys, None, 0, u64ptr(n)))
        out = np.zeros((int(n[0]), 2), dtype=np.uint32)
        check(self.lib.parm_nlist_pairs(self.h, sys, u32ptr(out), int(n[0]), u64ptr(n)))
        return out

    def set_capacity(self, maxnb: int) -> None:
        check(self.lib.parm_set_nlist_capacity(self.h, int(maxnb)))

    def capacity(self) -> int:
        v = C.c_uint32()
        check(self.lib.parm_get_nlist_capacity(self.h, C.byref(v)))
        return v.value

    # -- forces / quantities --
    def set_forces(self, constraints_and_a: bool = True) -> None:
        check(self.lib.parm_set_forces(self.h, 1 if constraints_and_a else 0))

    def evaluate(self, what: int) -> np.ndarray:
        ncomp = self.ndim * self.ndim if what == capi.EVAL_STRESS else 1
        out = np.zeros(self.nsys * ncomp)
        check(self.lib.parm_evaluate(self.h, what, dptr(out)))
        if what == capi.EVAL_STRESS:
            return out.reshape(self.nsys, self.ndim, self.ndim)
        return out

    def energy(self) -> np.ndarray:
        return self.evaluate(capi.EVAL_ENERGY)

    def virial(self) -> np.ndarray:
        return self.evaluate(capi.EVAL_VIRIAL)

    def stress(self) -> np.ndarray:
        return self.evaluate(capi.EVAL_STRESS)

    def contacts(self) -> np.ndarray:
        return self.evaluate(capi.EVAL_CONTACTS)

    def overlaps(self) -> np.ndarray:
        return self.evaluate(capi.EVAL_OVERLAPS)

    def kinetic_energy(self, origin=None) -> np.ndarray:
        out = np.zeros(self.nsys)
        o = None if origin is None else _as_f64(origin, (self.nsys, self.ndim))
        check(self.lib.parm_kinetic_energy(self.h, dptr(o) if o is not None else None, dptr(out)))
        return out

    def momentum(self):
        mom = np.zeros((self.nsys, self.ndim))
        mass = np.zeros(self.nsys)
        check(self.lib.parm_momentum(self.h, dptr(mom), dptr(mass)))
        return mom, mass

    def max_force_sq(self) -> np.ndarray:
        out = np.zeros(self.nsys)
        check(self.lib.parm_max_force_sq(self.h, dptr(out)))
        return out

    # -- mean-square-displacement tracker (RsqTracker) --
    def rsq_start(self, skips, usecom: bool = True) -> None:
        """(Re)start the device tracker at the current positions; windows of `skips` updates."""
        sk = np.ascontiguousarray(np.asarray(skips, dtype=np.uint64).ravel())
        self._rsq_n = len(sk)
        check(self.lib.parm_rsq_start(self.h, sk.ctypes.data_as(C.POINTER(C.c_uint64)), len(sk), int(bool(usecom))))

    def rsq_update(self) -> None:
        check(self.lib.parm_rsq_update(self.h))

    def rsq_get(self, what: int) -> np.ndarray:
        """Means as RsqTracker returns them: xyz2/xyz4 (nwin, n, ndim), r2/r4 (nwin, n), counts (nwin,)."""
        nw = max(self._rsq_n, 1)   # without a tracker the call reports the error
        shape = {capi.RSQ_XYZ2: (nw, self.n, self.ndim), capi.RSQ_XYZ4: (nw, self.n, self.ndim),
                 capi.RSQ_R2: (nw, self.n), capi.RSQ_R4: (nw, self.n), capi.RSQ_COUNTS: (nw,)}[what]
        out = np.zeros(shape)
        check(self.lib.parm_rsq_get(self.h, int(what), dptr(out)))
        return out

    def rsq_stop(self) -> None:
        check(self.lib.parm_rsq_stop(self.h))
        self._rsq_n = 0

    # -- integrators --
    def verlet(self, dt: float, nsteps: int = 1) -> None:
        check(self.lib.parm_verlet(self.h, float(dt), int(nsteps)))

    def damped(self, dt: float, damping: float, nsteps: int = 1) -> None:
        check(self.lib.parm_damped(self.h, float(dt), float(damping), int(nsteps)))

    def sol(self, dt: float, damping: float, T: float, seed: int, nsteps: int = 1) -> None:
        check(self.lib.parm_sol(self.h, float(dt), float(damping), float(T), int(seed), int(nsteps)))

    # -- conjugate-gradient minimisers (CollectionNLCG / CollectionNLCGV) --
    def nlcg_init(self, params, boxed: bool = True) -> None:
        """Start a minimiser per system; params: (11,) or (nsys, 11) in the order of capi.NLCG_PARAMS."""
        p = _as_f64(params, (self.nsys, len(capi.NLCG_PARAMS)))
        check(self.lib.parm_nlcg_init(self.h, 1 if boxed else 0, dptr(p)))

    def nlcg_set_params(self, params) -> None:
        p = _as_f64(params, (self.nsys, len(capi.NLCG_PARAMS)))
        check(self.lib.parm_nlcg_set_params(self.h, dptr(p)))

    def nlcg_state(self) -> np.ndarray:
        """(nsys, 11) state in the order of capi.NLCG_STATE."""
        out = np.zeros((self.nsys, len(capi.NLCG_STATE)))
        check(self.lib.parm_nlcg_get_state(self.h, dptr(out)))
        return out

    def nlcg_set_state(self, state) -> None:
        st = _as_f64(state, (self.nsys, len(capi.NLCG_STATE)))
        check(self.lib.parm_nlcg_set_state(self.h, dptr(st)))

    def nlcg_set_forces(self, constraints_and_a: bool = True) -> None:
        check(self.lib.parm_nlcg_set_forces(self.h, 1 if constraints_and_a else 0))

    def nlcg_reset(self) -> None:
        check(self.lib.parm_nlcg_reset(self.h))

    def nlcg_descend(self) -> None:
        check(self.lib.parm_nlcg_descend(self.h))

    def nlcg_timestep(self, nsteps: int = 1) -> None:
        check(self.lib.parm_nlcg_timestep(self.h, int(nsteps)))

    def boxes(self) -> np.ndarray:
        out = np.zeros((self.nsys, self.ndim))
        check(self.lib.parm_get_boxes(self.h, dptr(out)))
        return out

    def step_counter(self) -> int:
        v = C.c_uint64()
        check(self.lib.parm_get_step(self.h, C.byref(v)))
        return v.value

    def set_step_counter(self, step: int) -> None:
        check(self.lib.parm_set_step(self.h, int(step)))

    def set_cell_scale(self, scale: float) -> None:
        """Cells no narrower than `scale` times the list radius (results do not depend on it)."""
        check(self.lib.parm_set_cell_scale(self.h, float(scale)))

    def set_graph_steps(self, k: int) -> None:
        check(self.lib.parm_set_graph_steps(self.h, int(k)))

    def set_threads_per_atom(self, tpa: int) -> None:
        check(self.lib.parm_set_threads_per_atom(self.h, int(tpa)))

    def set_active(self, active) -> None:
        """Freeze (False) or step (True) each system of the batch."""
        a = np.ascontiguousarray(np.asarray(active, dtype=np.uint8).reshape(self.nsys))
        check(self.lib.parm_set_active(self.h, a.ctypes.data_as(C.POINTER(C.c_uint8))))

    def threads_per_atom(self) -> int:
        v = C.c_uint32(0)
        check(self.lib.parm_get_threads_per_atom(self.h, C.byref(v)))
        return int(v.value)

    def debug_stage_cap(self, cap: int) -> None:
        check(self.lib.parm_debug_stage_cap(self.h, int(cap)))

    def autotune(self) -> int:
        v = C.c_uint32()
        check(self.lib.parm_autotune(self.h, C.byref(v)))
        return v.value

    def timing(self, enable: bool) -> None:
        check(self.lib.parm_timing(self.h, 1 if enable else 0))

    def timing_read(self) -> dict:
        fm, dm = C.c_double(), C.c_double()
        fl, rb = C.c_uint64(), C.c_uint64()
        check(self.lib.parm_timing_read(self.h, C.byref(fm), C.byref(fl), C.byref(dm), C.byref(rb)))
        return {"force_ms": fm.value, "force_launches": fl.value, "drift_ms": dm.value, "rebuilds": rb.value}

    def last_launches(self) -> int:
        v = C.c_uint64()
        check(self.lib.parm_last_launches(self.h, C.byref(v)))
        return v.value

    def sync(self) -> None:
        check(self.lib.parm_sync(self.h))

    def stream(self) -> int:
        return self.lib.parm_stream(self.h) or 0


def debug_remainder(d, L) -> np.ndarray:
    lib = capi.load()
    d = np.ascontiguousarray(np.asarray(d, dtype=np.float64))
    L = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), d.shape))
    out = np.zeros_like(d)
    check(lib.parm_debug_remainder(dptr(d), dptr(L), dptr(out), d.size))
    return out


def debug_philox(ctr_key) -> np.ndarray:
    """The library's Philox4x32-10 on rows (c0, c1, c2, c3, k0, k1); returns (n, 4) uint32."""
    lib = capi.load()
    a = np.ascontiguousarray(np.asarray(ctr_key, dtype=np.uint32).reshape(-1, 6))
    out = np.zeros((a.shape[0], 4), dtype=np.uint32)
    check(lib.parm_debug_philox(capi.u32ptr(a), capi.u32ptr(out), a.shape[0]))
    return out


def debug_fpbits(d, f):
    """The per-atom update's bit-pattern conversions on the GPU: ((float)d, (double)f)."""
    import ctypes as C
    lib = capi.load()
    d = np.ascontiguousarray(np.asarray(d, dtype=np.float64).ravel())
    f = np.ascontiguousarray(np.asarray(f, dtype=np.float32).ravel())
    n = min(d.size, f.size)
    d2f = np.zeros(n, dtype=np.float32)
    f2d = np.zeros(n)
    fp = C.POINTER(C.c_float)
    check(lib.parm_debug_fpbits(dptr(d), f.ctypes.data_as(fp), n, d2f.ctypes.data_as(fp), dptr(f2d)))
    return d2f, f2d


def debug_normals(seed: int, sys: int, step: int, natoms: int) -> np.ndarray:
    """The (natoms, 6) standard normals parm_sol draws for system `sys` at counter `step`."""
    lib = capi.load()
    out = np.zeros((natoms, 6))
    check(lib.parm_debug_normals(int(seed), int(sys), int(step), int(natoms), dptr(out)))
    return out
