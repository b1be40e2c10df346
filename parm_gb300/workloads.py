"""Seeded synthetic inputs for the benchmark configurations.

Units are the reference's: sigma = position of the LJ minimum
(src/interaction.hpp:11 "ε(σ⁶/r⁶ - 1)², minimum at r = σ"), and
sigma' = sigma / 2**(1/6) is the conventional LJ length.

* lj_lattice   — simple-cubic lattice at number density 0.8 sigma'^-3 with a
                 uniform +-0.05 sigma' jitter, Gaussian velocities at T with
                 the centre-of-mass velocity removed (LJ NVE configurations).
* soft_disks   — 2D bidisperse harmonic disks (1.0 / 1.4) at a given area
                 fraction, uniform random positions.
* packings     — batches of 3D bidisperse soft spheres with per-system N and
                 volume fraction.
* wca_replicas — batches of WCA fluids with per-replica N and density.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

SIG_PRIME = 2.0 ** (-1.0 / 6.0)   # sigma' in sigma units
LJ_SIGCUT = 2.5 * SIG_PRIME       # cutoff 2.5 sigma' in sigma units


@dataclass
class Workload:
    name: str
    ndim: int
    sizes: list
    L: np.ndarray          # (nsys, ndim)
    x: np.ndarray          # (n, ndim)
    v: np.ndarray
    m: np.ndarray
    kind: int
    params: np.ndarray     # (n, 3)
    skin: float
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(sum(self.sizes))


def lj_lattice(shape=(10, 10, 10), rho_prime=0.8, jitter_prime=0.05, T=1.0, seed=12345,
               skin_prime=0.4) -> Workload:
    """LJ (LennardJonesCut, eps = 1, sigma = 1, cut 2.5 sigma') on a jittered cubic lattice."""
    rng = np.random.default_rng(seed)
    rho = rho_prime / SIG_PRIME ** 3
    a = (1.0 / rho) ** (1.0 / 3.0)
    nx, ny, nz = shape
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    x = (g + 0.5) * a + rng.uniform(-jitter_prime * SIG_PRIME, jitter_prime * SIG_PRIME, size=g.shape)
    n = len(x)
    v = rng.normal(0.0, np.sqrt(T), size=(n, 3))
    v -= v.mean(axis=0)
    L = np.array([[nx * a, ny * a, nz * a]])
    params = np.tile([1.0, 1.0, LJ_SIGCUT], (n, 1))
    return Workload(f"lj{n}", 3, [n], L, x, v, np.ones(n), 0, params, skin_prime * SIG_PRIME,
                    {"rho_prime": rho_prime, "lattice": shape})


def soft_disks(n=65536, phi=0.84, exponent=2.0, seed=2, skin=0.1) -> Workload:
    """2D bidisperse (1.0 / 1.4, 50:50) RepulsionPair disks at area fraction phi."""
    rng = np.random.default_rng(seed)
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4)
    area = np.sum(np.pi * sig ** 2 / 4)
    Lside = np.sqrt(area / phi)
    x = rng.uniform(0, Lside, size=(n, 2))
    params = np.stack([np.ones(n), sig, np.full(n, exponent)], 1)
    return Workload(f"disks{n}", 2, [n], np.array([[Lside, Lside]]), x, np.zeros((n, 2)), np.ones(n),
                    1, params, skin, {"phi": phi})


def packings(nsys=4096, nmin=64, nmax=4096, phi_lo=0.62, phi_hi=0.66, exponent=2.5, seed=3,
             skin=0.1) -> Workload:
    """Batch of 3D bidisperse soft-sphere systems (RepulsionPair) with random N and phi."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, size=nsys).tolist()
    xs, ps, Ls = [], [], []
    for N in sizes:
        sig = np.where(np.arange(N) < N // 2, 1.0, 1.4)
        phi = rng.uniform(phi_lo, phi_hi)
        V = np.sum(np.pi * sig ** 3 / 6) / phi
        Lside = V ** (1 / 3)
        xs.append(rng.uniform(0, Lside, size=(N, 3)))
        ps.append(np.stack([np.ones(N), sig, np.full(N, exponent)], 1))
        Ls.append([Lside] * 3)
    x = np.concatenate(xs)
    n = len(x)
    return Workload(f"packings{nsys}", 3, sizes, np.array(Ls), x, np.zeros((n, 3)), np.ones(n), 1,
                    np.concatenate(ps), skin, {})


def wca_replicas(nrep=512, nmin=256, nmax=32768, rho_lo=0.5, rho_hi=0.9, seed=4, skin_prime=0.3) -> Workload:
    """Batch of WCA fluids (LJRepulsePair, cut at sigma) with log-uniform N and uniform density."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=nrep)).astype(int).tolist()
    xs, Ls = [], []
    for N in sizes:
        rho = rng.uniform(rho_lo, rho_hi) / SIG_PRIME ** 3
        Lside = (N / rho) ** (1 / 3)
        # jittered lattice start avoids the huge overlaps of uniform positions
        k = int(np.ceil(N ** (1 / 3)))
        g = np.stack(np.meshgrid(np.arange(k), np.arange(k), np.arange(k), indexing="ij"), -1).reshape(-1, 3)[:N]
        a = Lside / k
        xs.append((g + 0.5) * a + rng.uniform(-0.05, 0.05, size=(N, 3)) * a)
        Ls.append([Lside] * 3)
    x = np.concatenate(xs)
    n = len(x)
    params = np.tile([1.0, 1.0, 0.0], (n, 1))
    return Workload(f"wca{nrep}", 3, sizes, np.array(Ls), x, np.zeros((n, 3)), np.ones(n), 2, params,
                    skin_prime * SIG_PRIME, {})


def small_random(n=64, ndim=3, kind=0, phi=0.3, bidisperse=True, seed=0, skin=0.4, exponent=2.0):
    """Small random configurations for parity tests (positions uniform in the box)."""
    rng = np.random.default_rng(seed)
    sig = np.where(np.arange(n) < n // 2, 1.0, 1.4) if bidisperse else np.ones(n)
    if ndim == 3:
        Lside = (np.sum(np.pi * sig ** 3 / 6) / phi) ** (1 / 3)
    else:
        Lside = np.sqrt(np.sum(np.pi * sig ** 2 / 4) / phi)
    x = rng.uniform(0, Lside, size=(n, ndim))
    v = rng.normal(size=(n, ndim))
    third = {0: LJ_SIGCUT, 1: exponent, 2: 0.0, 3: LJ_SIGCUT}[kind]
    params = np.stack([np.full(n, 1.2), sig, np.full(n, third)], 1)
    return Workload(f"small{n}", ndim, [n], np.full((1, ndim), Lside), x, v, sig ** ndim, kind, params, skin, {})
