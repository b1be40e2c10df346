"""Mean-square-displacement tracker restated in NumPy.

Test infrastructure only: the oracle the device tracker (parm_rsq_*) is
checked against.  It follows the reference's RsqTracker1 / RsqTracker
(wackywendell/parm src/constraints.hpp:318-361, src/constraints.cpp:404-564)
operation for operation, so that with ``usecom=False`` the device results are
bit-identical to it:

* constructor / reset (constraints.cpp:404-428): pastlocs = x - com, sums 0;
* update (constraints.cpp:429-455, 494-503): t += 1; for every window whose
  length divides t: d = r - past, d *= d, d4 = d * d, dist4 = ((0 + d_x) +
  d_y) + d_z, dist4 *= dist4; the sums grow by d, d4 and dist4; past = r;
* means (constraints.cpp:457-481, 510-564): sums / count; r2 is the row sum
  of the xyz2 means, (m_x + m_y) + m_z.

The centre of mass (AtomGroup::com, src/box.cpp:228-247) is summed here in
atom order; the device sums it in a fixed chunked order, so with
``usecom=True`` the two agree to rounding, not bit for bit.  ``sizes`` splits
the atoms into independent systems, each with its own centre of mass.
"""
import numpy as np


def _com(x, m):
    ok = (m > 0) & np.isfinite(m)
    v = np.zeros(x.shape[1])
    mass = 0.0
    for i in np.nonzero(ok)[0]:
        v = v + x[i] * m[i]
        mass += m[i]
    return v / mass


class RsqOracle:
    def __init__(self, x, m, skips, usecom=True, sizes=None):
        x = np.asarray(x, dtype=np.float64)
        self.m = np.asarray(m, dtype=np.float64)
        self.skips = [int(s) for s in skips]
        self.usecom = bool(usecom)
        self.sizes = [len(x)] if sizes is None else [int(s) for s in sizes]
        self.t = 0
        n, nd = x.shape
        r = self._r(x)
        self.past = [r.copy() for _ in self.skips]
        self.s_x2 = [np.zeros((n, nd)) for _ in self.skips]
        self.s_x4 = [np.zeros((n, nd)) for _ in self.skips]
        self.s_r4 = [np.zeros(n) for _ in self.skips]
        self.count = [0 for _ in self.skips]

    def _r(self, x):
        if not self.usecom:
            return x - 0.0
        r = np.empty_like(x)
        off = 0
        for n in self.sizes:
            sl = slice(off, off + n)
            r[sl] = x[sl] - _com(x[sl], self.m[sl])
            off += n
        return r

    def update(self, x):
        x = np.asarray(x, dtype=np.float64)
        self.t += 1
        r = self._r(x)
        for j, skip in enumerate(self.skips):
            if self.t % skip:
                continue
            d = r - self.past[j]
            d = d * d
            d4 = d * d
            dist4 = np.zeros(len(x))
            for k in range(x.shape[1]):
                dist4 = dist4 + d[:, k]
            dist4 = dist4 * dist4
            self.s_x2[j] = self.s_x2[j] + d
            self.s_x4[j] = self.s_x4[j] + d4
            self.s_r4[j] = self.s_r4[j] + dist4
            self.past[j] = r.copy()
            self.count[j] += 1

    def xyz2(self):
        return np.array([s / float(c) for s, c in zip(self.s_x2, self.count)])

    def xyz4(self):
        return np.array([s / float(c) for s, c in zip(self.s_x4, self.count)])

    def r2(self):
        out = []
        for m in self.xyz2():
            acc = m[:, 0]
            for k in range(1, m.shape[1]):
                acc = acc + m[:, k]
            out.append(acc)
        return np.array(out)

    def r4(self):
        return np.array([s / float(c) for s, c in zip(self.s_r4, self.count)])

    def counts(self):
        return np.array(self.count, dtype=np.float64)
