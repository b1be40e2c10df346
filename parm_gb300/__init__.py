"""parm_gb300 — GB300 (sm_103a) implementation of ParM's molecular-dynamics step.

The compute path is the CUDA library ``_lib/libparm_gb300.so`` (C ABI in
``include/parm_gb300.h``); :class:`System` is its Python view and
``host/`` holds the C++ API that mirrors the reference's classes.
"""
from .capi import (FP64, LJCUT, LJREPULSE, MIXED, REPULSION, CapacityError, ParmError, load)  # noqa: F401
from .system import System, debug_remainder  # noqa: F401

__all__ = ["System", "debug_remainder", "load", "FP64", "MIXED", "LJCUT", "REPULSION", "LJREPULSE",
           "ParmError", "CapacityError"]
