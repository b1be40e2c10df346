"""Langevin noise of CollectionSol on the GPU, pinned against published and
statistical references (the reference's own Boost stream cannot be
reproduced, so parity of the noise is established here):

* the device Philox4x32-10 block function equals cuRAND's
  curand_Philox4x32_10 (an independent implementation of Salmon et al.,
  SC'11) and the definition written out in tests/philox_py.py;
* the normals have mean 0, variance 1, Gaussian fourth moment and no
  correlation between components, atoms or steps;
* one step from rest of non-interacting atoms gives position and velocity
  increments with the variances and correlation that
  CollectionSol::set_constants (src/collection.cpp:230-263) and
  BivariateGauss::set (src/vecrand.cpp:48-62) prescribe, on both branches of
  sigma_r (damping * dt above and below 1e-4);
* the kinetic temperature relaxes as T (1 - c0^(2n)) from rest and stays at T,
  free Brownian motion has the Ornstein-Uhlenbeck mean-square displacement,
  and a WCA fluid thermostatted at T = 1 has <T> = 1 within 1 %.

Statistical bounds are 5 standard errors of the estimator at the sample size.
"""
import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

from philox_py import edge_rows, philox_rows, random_rows

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def curand_lib():
    import ctypes as C
    from parm_gb300.build import nvcc
    out = HERE / "_build" / "libcurand_philox.so"
    src = HERE / "csrc" / "curand_philox.cu"
    out.parent.mkdir(exist_ok=True)
    if not out.exists() or out.stat().st_mtime < src.stat().st_mtime:
        subprocess.run([nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-Xcompiler", "-fPIC",
                        "-shared", str(src), "-o", str(out)], check=True)
    lib = C.CDLL(str(out))
    lib.curand_philox_rows.restype = C.c_int
    lib.curand_philox_rows.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint32]
    return lib


def _curand(lib, rows):
    import ctypes as C
    rows = np.ascontiguousarray(rows, dtype=np.uint32)
    out = np.zeros((rows.shape[0], 4), dtype=np.uint32)
    p = C.POINTER(C.c_uint32)
    assert lib.curand_philox_rows(rows.ctypes.data_as(p), out.ctypes.data_as(p), rows.shape[0]) == 0
    return out


def test_philox_matches_curand_and_definition(curand_lib):
    from oracle.oracle import philox as oracle_philox
    from parm_gb300.system import debug_philox
    rows = np.concatenate([edge_rows(), random_rows(1 << 16, 11)])
    dev = debug_philox(rows)
    assert np.array_equal(dev, _curand(curand_lib, rows))
    assert np.array_equal(dev[:2000], philox_rows(rows[:2000]))
    assert np.array_equal(dev, oracle_philox(rows))


def test_normals_match_oracle_and_moments():
    from oracle.oracle import normals6, splitmix64
    from parm_gb300.system import debug_normals
    seed, sysid, step, n = 99, 3, 123456789012, 200000
    g = debug_normals(seed, sysid, step, n)
    key = splitmix64(seed + sysid)
    ref = np.array([normals6(key, step, i) for i in range(0, n, 97)])
    np.testing.assert_allclose(g[::97], ref, rtol=1e-14, atol=1e-14)
    z = g.ravel()
    k = z.size
    assert abs(z.mean()) < 5 / math.sqrt(k)
    assert abs(z.var() - 1.0) < 5 * math.sqrt(2.0 / k)
    assert abs((z ** 4).mean() - 3.0) < 5 * math.sqrt(96.0 / k)
    assert abs(np.mean(np.abs(z) < 1.0) - 0.6826894921370859) < 5 * math.sqrt(0.2173 / k)
    c = np.corrcoef(g.T)
    assert np.abs(c[~np.eye(6, dtype=bool)]).max() < 5 / math.sqrt(n)
    # neighbouring atoms, the next step counter and the next system are independent draws
    nxt = debug_normals(seed, sysid, step + 1, n)
    oth = debug_normals(seed, sysid + 1, step, n)
    for other in (g[1:], nxt, oth):
        m = min(len(other), n)
        r = np.corrcoef(g[:m].ravel(), other[:m].ravel())[0, 1]
        assert abs(r) < 5 / math.sqrt(m * 6)


def _free_atoms(n, precision, v=None, L=2000.0):
    """n atoms on a sparse lattice with a WCA interaction of tiny diameter: no pairs, zero forces."""
    from parm_gb300 import System
    k = int(math.ceil(n ** (1 / 3)))
    g = np.stack(np.meshgrid(np.arange(k), np.arange(k), np.arange(k), indexing="ij"), -1).reshape(-1, 3)[:n]
    x = (g + 0.5) * (L / k)
    s = System(n, ndim=3, precision=precision)
    s.set_boxes([L, L, L])
    z = np.zeros((n, 3))
    s.set_atoms(x=x, v=z if v is None else v, a=z, f=z, m=np.ones(n))
    s.set_interaction(2, np.tile([1.0, 1e-3, 0.0], (n, 1)), 0.0)
    s.nlist_update(True)
    s.set_forces(True)
    assert int(s.numpairs()[0]) == 0
    return s, x


def _sol_constants(dt, damping):
    from oracle.oracle import sol_constants
    c0, c1, c2, x11, x21, x22 = sol_constants(dt, damping)
    sv = math.hypot(x21, x22)
    return c0, x11, sv, x21 / sv


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dt,damping", [(0.001, 1.0), (0.001, 0.05)])   # damping*dt 1e-3 and 5e-5
def test_one_step_from_rest_has_prescribed_moments(precision, dt, damping):
    T, n = 1.7, 200000
    s, x0 = _free_atoms(n, precision)
    s.sol(dt, damping, T, 4242, 1)
    st = s.get_atoms()
    c0, sr, sv, corr = _sol_constants(dt, damping)
    if damping * dt <= 1e-4:
        # the series branch of sigma_r (collection.cpp:252-254)
        q = damping * dt
        assert sr == math.sqrt(2 * q / 3 - q * q / 2 + 7 * q * q * q / 30)
    dx = ((st["x"] - x0) / (dt * math.sqrt(T))).ravel()
    vv = (st["v"] / math.sqrt(T)).ravel()
    k = dx.size
    assert abs(dx.mean()) < 5 * sr / math.sqrt(k)
    assert abs(vv.mean()) < 5 * sv / math.sqrt(k)
    assert abs(dx.var() / sr ** 2 - 1) < 5 * math.sqrt(2.0 / k)
    assert abs(vv.var() / sv ** 2 - 1) < 5 * math.sqrt(2.0 / k)
    r = np.corrcoef(dx, vv)[0, 1]
    assert abs(r - corr) < 5 * (1 - corr * corr) / math.sqrt(k)
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_temperature_relaxes_from_rest(precision):
    """Free atoms from v = 0: <v^2>/(T/m) = 1 - c0^(2n) after n steps (exact for this update)."""
    T, n, dt, damping = 1.0, 100000, 0.01, 1.0
    s, _ = _free_atoms(n, precision)
    c0 = math.exp(-damping * dt)
    done = 0
    for steps in (50, 450):
        s.sol(dt, damping, T, 7, steps)
        done += steps
        v = s.get_atoms(2)["v"].ravel()
        want = T * (1 - c0 ** (2 * done))
        assert abs((v * v).mean() / want - 1) < 5 * math.sqrt(2.0 / v.size)
    s.close()


def test_free_brownian_msd():
    """Free atoms with Maxwell velocities at T: MSD(t) = 2 d (T/m/g) (t - (1 - exp(-g t))/g)."""
    T, n, dt, damping, steps = 1.0, 100000, 0.001, 2.0, 1000
    rng = np.random.default_rng(8)
    v0 = rng.normal(0.0, math.sqrt(T), size=(n, 3))
    s, x0 = _free_atoms(n, "fp64", v=v0)
    s.sol(dt, damping, T, 31, steps)
    x = s.get_atoms(1)["x"]
    msd = ((x - x0) ** 2).sum(1)
    t = steps * dt
    want = 2 * 3 * T / damping * (t - (1 - math.exp(-damping * t)) / damping)
    # per-atom squared displacement: 3-dof chi-square, relative spread sqrt(2/3)
    assert abs(msd.mean() / want - 1) < 5 * math.sqrt(2.0 / 3.0) / math.sqrt(n)
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_wca_fluid_temperature(precision):
    """WCA fluid (rho' = 0.7) under CollectionSol at T = 1: time-averaged kinetic temperature 1 within 1 %."""
    from parm_gb300 import workloads as W
    from helpers import make_gpu
    w = W.wca_replicas(nrep=1, nmin=32768, nmax=32768, rho_lo=0.7, rho_hi=0.7, seed=12)
    g = make_gpu(w, precision)
    g.nlist_update(False); g.set_forces(True); g.nlist_update(False)
    g.sol(0.001, 1.0, 1.0, 5, 3000)          # equilibrate (1/damping = 1000 steps)
    temps = []
    for _ in range(20):
        g.sol(0.001, 1.0, 1.0, 5, 100)
        ke = g.kinetic_energy()[0]
        temps.append(2 * ke / (3 * w.n))
    assert abs(np.mean(temps) - 1.0) < 0.01
    g.close()
