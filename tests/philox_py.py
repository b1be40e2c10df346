"""Philox4x32-10 written directly from its published definition (Salmon,
Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11,
section 4.2): ten rounds of two 32x32->64-bit multiplications by the
constants M0 = 0xD2511F53 and M1 = 0xCD9E8D57 with the Weyl key schedule
W0 = 0x9E3779B9, W1 = 0xBB67AE85 added to the key between rounds.

A round maps (c0, c1, c2, c3) with key (k0, k1) to
    (hi(M1*c2) ^ c1 ^ k0,  lo(M1*c2),  hi(M0*c0) ^ c3 ^ k1,  lo(M0*c0)).
Test infrastructure: Python integers, independent of the C and CUDA code.
"""
import numpy as np

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    c0, c1, c2, c3 = (int(v) & MASK for v in ctr)
    k0, k1 = (int(v) & MASK for v in key)
    for r in range(10):
        if r:
            k0 = (k0 + W0) & MASK
            k1 = (k1 + W1) & MASK
        p0 = M0 * c0
        p1 = M1 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & MASK, p1 & MASK, ((p0 >> 32) ^ c3 ^ k1) & MASK, p0 & MASK
    return c0, c1, c2, c3


def philox_rows(rows) -> np.ndarray:
    rows = np.asarray(rows, dtype=np.uint64).reshape(-1, 6)
    return np.array([philox4x32_10(r[:4], r[4:]) for r in rows], dtype=np.uint32).reshape(-1, 4)


def edge_rows() -> np.ndarray:
    """Counters and keys at the ends of their ranges and single-bit patterns."""
    F = MASK
    rows = [[0, 0, 0, 0, 0, 0], [F, F, F, F, F, F], [F, F, F, F, 0, 0], [0, 0, 0, 0, F, F],
            [1, 0, 0, 0, 0, 0], [0, 1, 0, 0, 0, 0], [0, 0, 1, 0, 0, 0], [0, 0, 0, 1, 0, 0],
            [0, 0, 0, 0, 1, 0], [0, 0, 0, 0, 0, 1], [F, 0, F, 0, F, 0], [0x80000000] * 6]
    for b in range(32):
        rows.append([1 << b, 0, 1 << b, 0, 1 << b, 0])
    return np.array(rows, dtype=np.uint32)


def random_rows(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.integers(0, 1 << 32, size=(n, 6), dtype=np.uint64).astype(np.uint32)
