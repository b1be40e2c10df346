"""Shared set-up for parity tests: the same workload on the GPU and in the oracle."""
import numpy as np

from oracle.oracle import Oracle


def make_gpu(w, precision="fp64", rank=None, sys_slices=None):
    from parm_gb300 import System
    s = System(w.sizes, ndim=w.ndim, precision=precision)
    s.set_boxes(w.L)
    s.set_atoms(x=w.x, v=w.v, a=np.zeros_like(w.x), f=np.zeros_like(w.x), m=w.m)
    s.set_interaction(w.kind, w.params, w.skin, rank=rank)
    return s


def make_oracle(w, sys=0, order=None):
    off = int(sum(w.sizes[:sys]))
    n = int(w.sizes[sys])
    o = Oracle(n, w.ndim)
    o.set_box(w.L[sys])
    sl = slice(off, off + n)
    o.set_state(x=w.x[sl], v=w.v[sl], a=np.zeros((n, w.ndim)), f=np.zeros((n, w.ndim)), m=w.m[sl])
    o.set_interaction(w.kind, w.params[sl], w.skin, order=order)
    return o


def force_error(F, Fref):
    """max_i |dF_i| / rms_i |F_i| (the mixed-precision force metric)."""
    err = np.sqrt(((F - Fref) ** 2).sum(1))
    rms = np.sqrt((Fref ** 2).sum(1).mean())
    return float(err.max() / rms)
