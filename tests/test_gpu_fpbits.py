"""The per-atom update's float <-> double conversions on bit patterns equal
the IEEE conversions on the GPU itself (numpy's casts as the reference):
random bit patterns, values of the magnitudes positions, fine parts and
forces take, exact rounding ties, carries into the exponent and both ends of
the float range."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _doubles(rng, n):
    bits = rng.integers(0, 2 ** 64, size=n, dtype=np.uint64)
    e = rng.integers(-60, 60, size=n)
    mod = np.ldexp(rng.random(n), e) * np.where(rng.random(n) < 0.5, -1.0, 1.0)
    exp = ((1023 + e).astype(np.uint64) << np.uint64(52))
    frac = rng.integers(0, 2 ** 52, size=n, dtype=np.uint64) & np.uint64(0xFFFFFFFFE0000000)
    ties = [(exp | frac | np.uint64(t)).view(np.float64) for t in (0x10000000, 0x0FFFFFFF, 0x10000001)]
    ones = (exp | np.uint64(0xFFFFFFFFFFFFF)).view(np.float64)
    ends = [((np.uint64(k) << np.uint64(52)) | (bits & np.uint64(0xFFFFFFFFFFFFF))).view(np.float64)
            for k in (895, 896, 897, 1149, 1150, 1151)]
    return np.concatenate([bits.view(np.float64), mod] + ties + [ones] + ends)


def test_fpbits_match_ieee_on_gpu():
    from parm_gb300.system import debug_fpbits
    rng = np.random.default_rng(2026)
    d = _doubles(rng, 200000)
    f = np.concatenate([rng.integers(0, 2 ** 32, size=d.size // 2, dtype=np.uint64).astype(np.uint32).view(np.float32),
                        (rng.standard_normal(d.size - d.size // 2) * 10.0).astype(np.float32)])
    with np.errstate(over="ignore", invalid="ignore"):
        want_f = d.astype(np.float32)
        want_d = f.astype(np.float64)
    got_f, got_d = debug_fpbits(d, f)
    nan_f = np.isnan(want_f)
    assert np.array_equal(np.isnan(got_f), nan_f)
    assert np.array_equal(got_f[~nan_f].view(np.uint32), want_f[~nan_f].view(np.uint32))
    nan_d = np.isnan(want_d)
    assert np.array_equal(np.isnan(got_d), nan_d)
    assert np.array_equal(got_d[~nan_d].view(np.uint64), want_d[~nan_d].view(np.uint64))
