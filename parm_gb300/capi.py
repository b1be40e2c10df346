"""ctypes binding of the C ABI in ``include/parm_gb300.h``.

The shared library is built in-tree (``parm_gb300/build.py``) and there is no
other implementation: importing this module on a machine where the library is
missing or cannot be loaded raises, so nothing silently falls back to CPU code.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIBDIR = Path(__file__).resolve().parent / "_lib"
LIBPATH = LIBDIR / "libparm_gb300.so"

PARM_OK = 0
PARM_ERR_ARG = -1
PARM_ERR_RUNTIME = -2
PARM_ERR_CUDA = -3
PARM_ERR_CAPACITY = -4

FP64 = 0
MIXED = 1

LJCUT = 0
REPULSION = 1
LJREPULSE = 2
LJATTRACTCUT = 3
LOISOHERN = 4       # params (eps, sigma, C, l); FP64 handles
LOISOHERN_MIN = 5
LOISLIN = 6         # params (eps, sigma, f, l); FP64 handles
LOISLIN_MIN = 7
EISMCLACHLAN = 8    # params (dist, sigmai, unused); FP64 handles
REPULSIONDRAG = 9   # params (eps, sigma, exponent, gamma); FP64 handles
# indexed epsilons (parm_set_pair_table first); params begin with the type index; FP64 handles
LJCUT_IEPSISIG = 10             # (indx, sigcut, unused)
LJATTRACTCUT_IEPSISIG = 11      # (indx, sigcut, unused)
LJATTRACTCUT_IEPS = 12          # (indx, sigma, sigcut)
LJATTRACTREPULSE = 13           # (indx, sigma, sigcut)
LJATTRACTFIXEDREPULSE = 14      # (indx, repeps, sigma, sigcut)
LJISH = 15                      # (indx, repeps, sigma, n, sigcut)
REPULSION_IEPSISIG = 16         # (indx, exponent, unused)
LJATTRACTREPULSESIGS = 17       # (eps_r, eps_a, sig_r, sig_a, sigcut); FP64 handles


def nparam(kind: int) -> int:
    """Doubles per atom in parm_set_interaction's params (PARM_NPARAM)."""
    if LOISOHERN <= kind <= LOISLIN_MIN or kind in (REPULSIONDRAG, LJATTRACTFIXEDREPULSE):
        return 4
    return 5 if kind in (LJISH, LJATTRACTREPULSESIGS) else 3

X, V, A, F, M = 1, 2, 4, 8, 16

EVAL_ENERGY, EVAL_VIRIAL, EVAL_STRESS, EVAL_CONTACTS, EVAL_OVERLAPS = range(5)

RSQ_XYZ2, RSQ_XYZ4, RSQ_R2, RSQ_R4, RSQ_COUNTS = range(5)

NOT_MEMBER = 0xFFFFFFFF

# conjugate-gradient minimisers: parameter and state vectors (PARM_NLCG_P_* / PARM_NLCG_S_*)
NLCG_PARAMS = ("dt", "P0", "kappa", "kmax", "secmax", "seceps", "alphamax", "afrac", "dxmax", "stepmax", "maxdV")
NLCG_STATE = ("Knew", "k", "vl", "fl", "al", "alpha", "beta", "betaused", "dxsum", "alphavmax", "sec")

_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)
_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_h = C.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "parm_last_error": (C.c_char_p, []),
    "parm_version": (C.c_int, []),
    "parm_use_device": (C.c_int, [C.c_int]),
    "parm_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_uint32, _u32p, C.c_int]),
    "parm_destroy": (C.c_int, [_h]),
    "parm_set_boxes": (C.c_int, [_h, _dp]),
    "parm_set_atoms": (C.c_int, [_h, _dp, C.c_uint64, C.c_uint32]),
    "parm_get_atoms": (C.c_int, [_h, _dp, C.c_uint64, C.c_uint32]),
    "parm_set_interaction": (C.c_int, [_h, C.c_int, _dp, _u32p, C.c_double]),
    "parm_set_pair_table": (C.c_int, [_h, C.c_uint32, _dp, _dp]),
    "parm_set_lees_edwards": (C.c_int, [_h, _dp]),
    "parm_nlist_ignore": (C.c_int, [_h, C.c_uint32, C.c_uint32]),
    "parm_set_list_diameters": (C.c_int, [_h, _dp]),
    "parm_nlist_update": (C.c_int, [_h, C.c_int, _u8p]),
    "parm_nlist_which": (C.c_int, [_h, _u32p]),
    "parm_nlist_numpairs": (C.c_int, [_h, _u64p]),
    "parm_nlist_pairs": (C.c_int, [_h, C.c_uint32, _u32p, C.c_uint64, _u64p]),
    "parm_set_forces": (C.c_int, [_h, C.c_int]),
    "parm_evaluate": (C.c_int, [_h, C.c_int, _dp]),
    "parm_verlet": (C.c_int, [_h, C.c_double, C.c_uint32]),
    "parm_damped": (C.c_int, [_h, C.c_double, C.c_double, C.c_uint32]),
    "parm_sol": (C.c_int, [_h, C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_uint32]),
    "parm_kinetic_energy": (C.c_int, [_h, _dp, _dp]),
    "parm_momentum": (C.c_int, [_h, _dp, _dp]),
    "parm_max_force_sq": (C.c_int, [_h, _dp]),
    "parm_rsq_start": (C.c_int, [_h, _u64p, C.c_uint32, C.c_int]),
    "parm_rsq_update": (C.c_int, [_h]),
    "parm_rsq_get": (C.c_int, [_h, C.c_int, _dp]),
    "parm_rsq_stop": (C.c_int, [_h]),
    "parm_get_step": (C.c_int, [_h, _u64p]),
    "parm_set_step": (C.c_int, [_h, C.c_uint64]),
    "parm_set_nlist_capacity": (C.c_int, [_h, C.c_uint32]),
    "parm_get_nlist_capacity": (C.c_int, [_h, _u32p]),
    "parm_set_graph_steps": (C.c_int, [_h, C.c_uint32]),
    "parm_set_cell_scale": (C.c_int, [_h, C.c_double]),
    "parm_set_threads_per_atom": (C.c_int, [_h, C.c_uint32]),
    "parm_autotune": (C.c_int, [_h, _u32p]),
    "parm_get_threads_per_atom": (C.c_int, [_h, _u32p]),
    "parm_set_active": (C.c_int, [_h, C.POINTER(C.c_uint8)]),
    "parm_debug_stage_cap": (C.c_int, [_h, C.c_uint32]),
    "parm_timing": (C.c_int, [_h, C.c_int]),
    "parm_timing_read": (C.c_int, [_h, _dp, _u64p, _dp, _u64p]),
    "parm_last_launches": (C.c_int, [_h, _u64p]),
    "parm_sync": (C.c_int, [_h]),
    "parm_stream": (C.c_void_p, [_h]),
    "parm_host_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_uint64]),
    "parm_host_free": (C.c_int, [C.c_void_p]),
    "parm_debug_remainder": (C.c_int, [_dp, _dp, _dp, C.c_uint32]),
    "parm_debug_philox": (C.c_int, [_u32p, _u32p, C.c_uint32]),
    "parm_debug_fpbits": (C.c_int, [_dp, C.POINTER(C.c_float), C.c_uint32, C.POINTER(C.c_float), _dp]),
    "parm_nlcg_init": (C.c_int, [_h, C.c_int, _dp]),
    "parm_nlcg_set_params": (C.c_int, [_h, _dp]),
    "parm_nlcg_get_state": (C.c_int, [_h, _dp]),
    "parm_nlcg_set_state": (C.c_int, [_h, _dp]),
    "parm_nlcg_set_forces": (C.c_int, [_h, C.c_int]),
    "parm_nlcg_reset": (C.c_int, [_h]),
    "parm_nlcg_descend": (C.c_int, [_h]),
    "parm_nlcg_timestep": (C.c_int, [_h, C.c_uint32]),
    "parm_get_boxes": (C.c_int, [_h, _dp]),
    "parm_debug_normals": (C.c_int, [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint32, _dp]),
    "parm_kinetic_energy_noalloc": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, C.c_int, _dp, C.c_void_p,
                                              C.c_void_p]),
}

_lib = None


def load() -> C.CDLL:
    """Load (once) the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIBPATH.exists():
        raise ImportError(
            f"{LIBPATH} is missing: build it with `python -m parm_gb300.build` "
            "(the CUDA library is required; there is no CPU implementation)")
    lib = C.CDLL(str(LIBPATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class ParmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class CapacityError(ParmError):
    pass


def check(code: int) -> None:
    if code != PARM_OK:
        msg = load().parm_last_error().decode(errors="replace")
        if code == PARM_ERR_ARG:
            raise ValueError(msg)
        if code == PARM_ERR_CAPACITY:
            raise CapacityError(code, msg)
        raise ParmError(code, msg)


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def u32ptr(a: np.ndarray):
    return a.ctypes.data_as(_u32p)


def u64ptr(a: np.ndarray):
    return a.ctypes.data_as(_u64p)
