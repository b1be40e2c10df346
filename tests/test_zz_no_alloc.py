"""parm_kinetic_energy_noalloc: the entry point for callers that cannot allocate.

Such callers (frameworks whose memory pool owns every device buffer, loops
that must never enter the allocator, processes under a fixed device-memory
budget) pass Atom records they already hold in device memory and a device
location for the result.  The entry point keeps its scratch in a static device array,
so its result must equal the handle-based parm_kinetic_energy on the same
atoms, call after call.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import make_gpu
from parm_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu

RTOL = 1e-12   # the two entry points sum the same terms in different orders


def _records(w):
    nd = w.ndim
    rec = np.zeros((w.n, 4 * nd + 1))
    rec[:, 0:nd] = w.x
    rec[:, nd:2 * nd] = w.v
    rec[:, 4 * nd] = w.m
    return rec


@pytest.mark.parametrize("ndim", [3, 2])
def test_noalloc_matches_handle_twice(ndim):
    torch = pytest.importorskip("torch")
    w = W.small_random(n=20000, ndim=ndim, kind=1, seed=71)
    w.m[3] = 0.0
    w.m[4] = np.inf
    w.m[5] = -2.0
    g = make_gpu(w)
    origin = np.array([0.3, -0.1, 0.2][:ndim])
    ref = g.kinetic_energy()[0]
    ref_o = g.kinetic_energy(origin[None, :])[0]
    lib = capi.load()
    rec = torch.from_numpy(_records(w)).cuda()
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    stride = 4 * ndim + 1
    for _ in range(2):   # the static scratch keeps the last call's contents
        rc = lib.parm_kinetic_energy_noalloc(C.c_void_p(rec.data_ptr()), stride, w.n, ndim, None,
                                             C.c_void_p(out.data_ptr()), stream)
        assert rc == capi.PARM_OK, lib.parm_last_error()
        torch.cuda.synchronize()
        assert out.item() == pytest.approx(ref, rel=RTOL)
        o = np.ascontiguousarray(origin)
        rc = lib.parm_kinetic_energy_noalloc(C.c_void_p(rec.data_ptr()), stride, w.n, ndim, capi.dptr(o),
                                             C.c_void_p(out.data_ptr()), stream)
        assert rc == capi.PARM_OK, lib.parm_last_error()
        torch.cuda.synchronize()
        assert out.item() == pytest.approx(ref_o, rel=RTOL)


def test_noalloc_rejects_oversized_input():
    torch = pytest.importorskip("torch")
    lib = capi.load()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = lib.parm_kinetic_energy_noalloc(C.c_void_p(buf.data_ptr()), 13, (1 << 18) + 1, 3, None,
                                         C.c_void_p(buf.data_ptr()), None)
    assert rc == capi.PARM_ERR_ARG
    assert b"262144" in lib.parm_last_error()


def test_noalloc_leaves_free_device_memory_unchanged():
    """After the first call (which looks up the static scratch), repeated calls take no device memory."""
    torch = pytest.importorskip("torch")
    w = W.small_random(n=50000, ndim=3, kind=1, seed=72)
    lib = capi.load()
    rec = torch.from_numpy(_records(w)).cuda()
    out = torch.zeros((1,), dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = (C.c_void_p(rec.data_ptr()), 13, w.n, 3, None, C.c_void_p(out.data_ptr()), stream)
    assert lib.parm_kinetic_energy_noalloc(*args) == capi.PARM_OK
    torch.cuda.synchronize()
    first = out.item()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(200):
        assert lib.parm_kinetic_energy_noalloc(*args) == capi.PARM_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert out.item() == first   # same terms, same order: the same sum
