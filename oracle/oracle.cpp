// ORACLE — test infrastructure only, never part of the product path.
//
// A scalar CPU restatement of ParM's MD hot path (wackywendell/parm), written
// to reproduce the reference's floating-point evaluation order exactly so that
// the CUDA FP64 path can be checked bit-for-bit.  Only the test-suite, the
// smoke check and bench.py's CPU-baseline leg load this library.
//
// Parity status: pinned.  The fixtures under tests/golden/ are produced by the
// reference's own sources (src/vecrand.cpp, src/box.cpp, src/trackers.cpp,
// src/collection.cpp and the NListed templates of src/interaction.hpp)
// compiled as they are against a restatement of the Eigen/Boost subset they
// use (oracle/refbuild/shim, recipe oracle/refbuild/Makefile, generator
// tests/golden/make_golden.py), and tests/test_oracle_golden.py checks this
// file against them bit for bit: pair lists, forces, energies, stresses and
// Verlet / damped / Langevin (T = 0) trajectories up to 1000 steps.
// Not pinned: Eigen's own arithmetic (the restatement fixes its reduction
// order) and the Langevin noise stream (the reference draws from Boost's
// mt19937; here a counter-based generator), whose parity is statistical.
//
// Evaluation-order facts taken from the reference (all FP64, no FMA; build
// with -ffp-contract=off):
//   * OriginBox::diff = remainder(r1 - r2, L) per component (box.hpp:68-78,103)
//   * Eigen fixed-size 3-vector squaredNorm/dot reduce as ((v0 + v1) + v2)
//     (2-wide packet pre-reduction followed by the tail element)
//   * norm = sqrt(squaredNorm)
//   * coefficient-wise expressions evaluate left to right per component.
//
// Build:  g++ -O2 -ffp-contract=off -fPIC -shared -std=c++17 oracle.cpp

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <set>
#include <vector>
#include <utility>

namespace {

enum PairKind {
    LJCUT = 0, REPULSION = 1, LJREPULSE = 2, LJATTRACT = 3,
    LOISOHERN = 4, LOISOHERN_MIN = 5, LOISLIN = 6, LOISLIN_MIN = 7, EISMCLACHLAN = 8, REPULSIONDRAG = 9,
    // indexed pair epsilons (and sigmas): the pair's values come from a table by the two atoms'
    // type indices, first atom's row (IEps*Atom::get_epsilon)
    LJCUT_IEPSISIG = 10, LJATTRACT_IEPSISIG = 11, LJATTRACT_IEPS = 12, LJATTRACTREPULSE = 13,
    LJATTRACTFIXEDREPULSE = 14, LJISH = 15, REPULSION_IEPSISIG = 16,
    LJATTRACTREPULSESIGS = 17   // EpsEpsSigSigCutAtom: (eps_r, eps_a, sig_r, sig_a, sigcut)
};

inline bool indexed_kind(int kind) { return kind >= LJCUT_IEPSISIG && kind <= REPULSION_IEPSISIG; }

// kinds whose atoms carry four parameters
inline bool four_params(int kind) { return (kind >= LOISOHERN && kind <= LOISLIN_MIN) || kind == REPULSIONDRAG; }

struct V3 {
    double c[3] = {0, 0, 0};
};

// Eigen squaredNorm / dot order for NDIM=3: ((a0*b0 + a1*b1) + a2*b2);
// for NDIM=2: a0*b0 + a1*b1.
inline double dotv(const double* a, const double* b, int nd) {
    double s = a[0] * b[0] + a[1] * b[1];
    if (nd == 3) s = s + a[2] * b[2];
    return s;
}

struct AtomParams {
    // kind-dependent: (eps, sigma, sigcut|exponent) or, for the Lois kinds,
    // (eps, sigma, C, l) / (eps, sigma, f, l); the indexed kinds: type t and
    // (repeps, sigma, sigcut, exponent)
    double p0 = 0, p1 = 0, p2 = 0, p3 = 0, p4 = 0;
    uint32_t t = 0;
};

struct PairConst {
    // the pair constructors' outputs; for the Lois kinds third = C (or f),
    // fourth = l and cut = sigcut
    double eps, sig, third, cut_energy, fourth = 0, cut = 0;
};

struct System {
    int nd;
    uint32_t n;
    double L[3] = {1, 1, 1};
    bool lees = false;   // LeesEdwardsBox (box.hpp:165-196) with shear gamma
    double gamma = 0;
    std::vector<double> x, v, a, f, m;  // n*nd each (AoS of Vec)

    // NListed<A,P> + NeighborList state (interaction.hpp:1876-1945, trackers.hpp:157-214)
    int kind = -1;
    double skin = 0;
    std::vector<uint32_t> members;      // SubGroup order (insertion order)
    std::vector<double> diameters;      // A::max_size() per member
    std::vector<double> lastlocs;       // per member
    std::vector<AtomParams> params;     // indexed by AtomVec index
    uint32_t ntypes = 0;
    std::vector<double> teps, tsig;     // ntypes x ntypes: row = first atom's type
    std::vector<uint8_t> has_params;
    std::vector<std::pair<uint32_t, uint32_t>> curpairs;  // (first.n, last.n)
    std::set<std::pair<uint32_t, uint32_t>> ignored;      // (max, min) by AtomVec index
    uint32_t updatenum = 0;
    bool ignorechanged = true;

    System(int nd_, uint32_t n_) : nd(nd_), n(n_), x(n_ * nd_), v(n_ * nd_), a(n_ * nd_),
                                   f(n_ * nd_), m(n_, 1.0), params(n_), has_params(n_, 0) {}

    // OriginBox::diff (box.hpp:103) with vec_mod (box.hpp:68-78)
    inline void diff(const double* r1, const double* r2, double* out) const {
        if (lees) {
            // LeesEdwardsBox::diff (box.cpp:72-91): the y image shifts x by im * gamma * Lx
            const double Ly = L[1];
            double dy = r1[1] - r2[1];
            const int im = (int)std::round(dy / Ly);
            dy = dy - (im * Ly);
            const double Lx = L[0];
            double dx = r1[0] - r2[0];
            dx = dx - std::round((dx / Lx) - im * gamma) * Lx - im * gamma * Lx;
            out[0] = dx;
            out[1] = dy;
            if (nd == 3) out[2] = std::remainder(r1[2] - r2[2], L[2]);
            return;
        }
        for (int d = 0; d < nd; d++) out[d] = std::remainder(r1[d] - r2[d], L[d]);
    }

    PairConst pair_const(uint32_t i, uint32_t j) const {
        // P(atoms[first], atoms[last]) with first = i (interaction.hpp:2109-2113)
        const AtomParams& A = params[i];
        const AtomParams& B = params[j];
        PairConst pc{};
        if (kind == LJCUT) {
            // LennardJonesCutPair(EpsSigCutAtom, EpsSigCutAtom) (interaction.hpp:967-976)
            // and LennardJonesCut ctor (interaction.hpp:250-255)
            pc.eps = std::sqrt(A.p0 * B.p0);
            pc.sig = (A.p1 + B.p1) / 2;
            pc.third = std::max(A.p2, B.p2);
            double rsix = std::pow(pc.third, 6);
            double mid = (1 - 1 / rsix);
            pc.cut_energy = pc.eps * (mid * mid - 1);
        } else if (kind == LJATTRACT) {
            // LJAttractCutPair(EpsSigCutAtom, EpsSigCutAtom) (interaction.hpp:1020-1027)
            // and LJAttractCut ctor (interaction.hpp:203-208): cut_energy = LJAttract::energy(cut) * eps
            pc.eps = std::sqrt(A.p0 * B.p0);
            pc.sig = (A.p1 + B.p1) / 2;
            pc.third = std::max(A.p2, B.p2);
            double e;   // LJAttract::energy(rsig) (interaction.hpp:170-177)
            if (pc.third < 1) {
                e = -1;
            } else {
                double rsq = pc.third * pc.third;
                double rsix = rsq * rsq * rsq;
                double mid = (1 - 1 / rsix);
                e = mid * mid - 1;
            }
            pc.cut_energy = e * pc.eps;
        } else if (kind == REPULSION) {
            // RepulsionPair(EpsSigExpAtom, EpsSigExpAtom) (interaction.hpp:1532-1537)
            pc.eps = std::sqrt(A.p0 * B.p0);
            pc.sig = (A.p1 + B.p1) / 2.0;
            pc.third = (A.p2 + B.p2) / 2.0;
            pc.cut_energy = 0;
        } else if (kind == LOISOHERN || kind == LOISOHERN_MIN) {
            // LoisOhernPair(LoisOhernAtom, LoisOhernAtom) (interaction.hpp:1693-1703) and
            // LoisOhernPairMinCLs (1746-1751): averages, or the smaller C and l
            pc.eps = std::sqrt(A.p0 * B.p0);
            pc.sig = (A.p1 + B.p1) / 2.0;
            if (kind == LOISOHERN) {
                pc.third = (A.p2 + B.p2) / 2.0;
                pc.fourth = (A.p3 + B.p3) / 2.0;
            } else {
                pc.third = A.p2 < B.p2 ? A.p2 : B.p2;
                pc.fourth = A.p3 < B.p3 ? A.p3 : B.p3;
            }
            pc.cut = pc.sig * (1 + pc.third + pc.fourth);
            pc.cut_energy = 0;
        } else if (kind == LOISLIN || kind == LOISLIN_MIN) {
            // LoisLinPair(LoisLinAtom, LoisLinAtom) (interaction.hpp:1782-1800) and
            // LoisLinPairMin (1831-1836)
            pc.eps = std::sqrt(A.p0 * B.p0);
            pc.sig = (A.p1 + B.p1) / 2.0;
            if (kind == LOISLIN) {
                pc.third = (A.p2 + B.p2) / 2.0;
                pc.fourth = (A.p3 + B.p3) / 2.0;
            } else {
                pc.third = A.p2 < B.p2 ? A.p2 : B.p2;
                pc.fourth = A.p3 < B.p3 ? A.p3 : B.p3;
            }
            pc.cut = pc.sig + pc.fourth;
            pc.cut_energy = 0;
        } else if (indexed_kind(kind)) {
            const double te = teps[A.t * ntypes + B.t];   // a1.get_epsilon(a2)
            pc.cut = 0;
            if (kind == REPULSION_IEPSISIG) {
                // RepulsionPair(IEpsISigExpAtom, IEpsISigExpAtom) (interaction.hpp:1538-1543)
                pc.eps = te;
                pc.sig = tsig[A.t * ntypes + B.t];
                pc.third = (A.p2 + B.p2) / 2.0;
                pc.cut_energy = 0;
            } else if (kind == LJCUT_IEPSISIG) {
                // LennardJonesCutPair(IEpsISigCutAtom, IEpsISigCutAtom) (interaction.hpp:977-982)
                pc.eps = te;
                pc.sig = tsig[A.t * ntypes + B.t];
                pc.third = std::max(A.p2, B.p2);
                double rsix = std::pow(pc.third, 6);
                double mid = (1 - 1 / rsix);
                pc.cut_energy = pc.eps * (mid * mid - 1);
            } else if (kind == LJATTRACT_IEPSISIG || kind == LJATTRACT_IEPS) {
                // LJAttractCutPair(IEpsISigCutAtom...) / (IEpsSigCutAtom...) (interaction.hpp:1028-1037)
                pc.eps = te;
                pc.sig = (kind == LJATTRACT_IEPSISIG) ? tsig[A.t * ntypes + B.t] : (A.p1 + B.p1) / 2;
                pc.third = std::max(A.p2, B.p2);
                double e;
                if (pc.third < 1) {
                    e = -1;
                } else {
                    double rsq = pc.third * pc.third;
                    double rsix = rsq * rsq * rsq;
                    double mid = (1 - 1 / rsix);
                    e = mid * mid - 1;
                }
                pc.cut_energy = e * pc.eps;
            } else if (kind == LJATTRACTREPULSE) {
                // LJAttractRepulsePair(IEpsSigCutAtom, IEpsSigCutAtom) (interaction.hpp:1255-1268)
                pc.eps = te;
                pc.sig = (A.p1 + B.p1) / 2.0;
                pc.third = std::max(A.p2, B.p2);
                if (pc.eps <= 0) {
                    pc.third = 1;
                    pc.cut_energy = 0;
                    pc.eps = std::abs(pc.eps);
                } else {
                    double mid = (1 - std::pow(pc.third, -6));
                    pc.cut_energy = pc.eps * (mid * mid);
                }
            } else if (kind == LJATTRACTFIXEDREPULSE) {
                // LJAttractFixedRepulsePair(IEpsRepsSigCutAtom...) (interaction.hpp:1349-1365); fourth = repeps
                pc.eps = std::abs(te);
                pc.fourth = std::sqrt(A.p0 * B.p0);
                pc.sig = (A.p1 + B.p1) / 2.0;
                pc.third = std::max(A.p2, B.p2);
                bool attract = te > 0;
                if (!attract || pc.eps == 0) {
                    pc.third = 1;
                    pc.cut_energy = 0;
                    pc.eps = 0;
                } else {
                    double mid = (1 - std::pow(pc.third, -6.0));
                    pc.cut_energy = pc.eps * (mid * mid);
                }
            } else {
                // LJishPair(IEpsRepsSigExpCutAtom...) (interaction.hpp:1098-1114); fourth = repeps,
                // cut = the exponent n
                pc.eps = te;
                pc.fourth = std::sqrt(A.p0 * B.p0);
                pc.sig = (A.p1 + B.p1) / 2.0;
                pc.cut = (A.p3 + B.p3) / 2;
                pc.third = std::max(A.p2, B.p2);
                if (pc.eps <= 0) {
                    pc.third = 1;
                    pc.cut_energy = 0;
                    pc.eps = 0;
                } else {
                    double mid = (1 - std::pow(pc.third, -pc.cut));
                    pc.cut_energy = pc.eps * (mid * mid);
                }
            }
        } else if (kind == LJATTRACTREPULSESIGS) {
            // LJAttractRepulseSigsPair(a1, a2) (interaction.hpp:1171-1190): eps = eps_r, fourth = eps_a,
            // sig = sig_r, cut = sig_a, third = the cut in sigma units, cut_energy as constructed
            pc.eps = std::sqrt(A.p0 * B.p0);
            pc.fourth = std::sqrt(A.p1 * B.p1);
            pc.sig = (A.p2 + B.p2) / 2.0;
            pc.cut = (A.p3 + B.p3) / 2.0;
            pc.third = std::max(A.p4, B.p4);
            const double cu = pc.sig + pc.cut * (pc.third - 1);
            pc.cut_energy = (pc.third >= 1) ? sigs_attract_energy(pc, cu) : sigs_repulse_energy(pc, cu);
        } else if (kind == REPULSIONDRAG) {
            // RepulsionDragPair(EpsSigExpDragAtom, EpsSigExpDragAtom) (interaction.hpp:1613-1621):
            // atom fields (eps, sigma, exponent, gamma)
            pc.eps = std::sqrt(A.p0 * B.p0);
            pc.sig = (A.p1 + B.p1) / 2.0;
            pc.third = (A.p2 + B.p2) / 2.0;
            pc.fourth = (A.p3 + B.p3) / 2;
            pc.cut_energy = 0;
        } else if (kind == EISMCLACHLAN) {
            // EisMclachlanPair(EisMclachlanAtom, EisMclachlanAtom) (interaction.hpp:1425-1438):
            // E = c0/R + c1 + c2 R out to dist1 + dist2 (atom fields p0 = dist, p1 = sigmai)
            pc.eps = -M_PI * (A.p1 * B.p0 - B.p1 * A.p0) * (A.p0 * A.p0 - B.p0 * B.p0);      // c0
            pc.sig = -2 * M_PI * (A.p1 * B.p0 * B.p0 + B.p1 * A.p0 * A.p0);                // c1
            pc.third = M_PI * (A.p1 * B.p0 + B.p1 * A.p0);                                 // c2
            pc.cut = A.p0 + B.p0;
            pc.cut_energy = 0;
        } else {
            // LJRepulsePair(EpsSigAtom, EpsSigAtom) (interaction.hpp:875-880)
            pc.eps = std::sqrt(A.p0 * B.p0);
            pc.sig = (A.p1 + B.p1) / 2;
            pc.third = 0;
            pc.cut_energy = 0;
        }
        return pc;
    }

    // LJAttractRepulseSigsPair::attract_energy / repulse_energy (interaction.hpp:1192-1202)
    static double sigs_attract_energy(const PairConst& pc, double r) {
        double r_over_sig = (r - pc.sig + pc.cut) / pc.cut;
        double mid = (1 - std::pow(r_over_sig, -6));
        return pc.fourth * (mid * mid) - pc.fourth;
    }
    static double sigs_repulse_energy(const PairConst& pc, double r) {
        double r_over_sig = r / pc.sig;
        double mid = (1 - std::pow(r_over_sig, -6));
        return pc.eps * (mid * mid) - pc.fourth;
    }

    // P::energy(box) for the three pair kinds
    double pair_energy(const PairConst& pc, const double* rij) const {
        double dsq = dotv(rij, rij, nd);
        if (kind == LJCUT) {
            // LennardJonesCut::energy (interaction.hpp:256-262)
            double rsq = dsq / (pc.sig * pc.sig);
            if (rsq > (pc.third * pc.third)) return 0;
            double rsix = rsq * rsq * rsq;
            double mid = (1 - 1 / rsix);
            return pc.eps * (mid * mid - 1) - pc.cut_energy;
        } else if (kind == LJATTRACT) {
            // LJAttractCut::energy (interaction.hpp:211-216), LJAttract::energy (162-169)
            if (pc.eps == 0) return 0;
            if (dsq > (pc.third * pc.third * pc.sig * pc.sig)) return 0;
            double rsq = dsq / (pc.sig * pc.sig);
            double e;
            if (rsq < 1) {
                e = -pc.eps;
            } else {
                double rsix = rsq * rsq * rsq;
                double mid = (1 - 1 / rsix);
                e = pc.eps * (mid * mid - 1);
            }
            return e - pc.cut_energy;
        } else if (kind == REPULSION || kind == REPULSION_IEPSISIG) {
            // RepulsionPair::energy (interaction.hpp:1544-1550)
            if (dsq > pc.sig * pc.sig) return 0.0;
            double R = std::sqrt(dsq);
            return pc.eps * std::pow(1.0 - (R / pc.sig), pc.third) / pc.third;
        } else if (kind == LOISOHERN || kind == LOISOHERN_MIN) {
            // LoisOhernPair::energy (interaction.hpp:1713-1727)
            const double C = pc.third, l = pc.fourth;
            if (dsq >= pc.cut * pc.cut) return 0.0;
            double R = std::sqrt(dsq) / pc.sig;
            if (R <= 1 + C) {
                double dR = R - 1;
                return -pc.eps * pc.sig / 2 * (C * (C + l) - dR * dR);
            }
            double dR2 = C + l + 1 - R;
            return -C * pc.eps * pc.sig / 2 / l * dR2 * dR2;
        } else if (kind == LOISLIN || kind == LOISLIN_MIN) {
            // LoisLinPair::energy (interaction.hpp:1802-1815)
            const double f = pc.third, l = pc.fourth;
            if (dsq >= pc.cut * pc.cut) return 0.0;
            double R = std::sqrt(dsq);
            if (R <= pc.sig) {
                double dR = 1.0 - (R / pc.sig);
                return pc.eps / 2 * dR * dR - f * l;
            }
            return -f * (pc.sig + l - R);
        } else if (kind == LJATTRACTREPULSESIGS) {
            // LJAttractRepulseSigsPair::energy (interaction.hpp:1204-1216)
            double dist = std::sqrt(dsq);
            double cu = pc.sig + pc.cut * (pc.third - 1);
            if (pc.third > 0 && dist > cu) return 0;
            if (dist <= pc.sig) return sigs_repulse_energy(pc, dist) - pc.cut_energy;
            return sigs_attract_energy(pc, dist) - pc.cut_energy;
        } else if (kind == LJCUT_IEPSISIG) {
            double rsq = dsq / (pc.sig * pc.sig);
            if (rsq > (pc.third * pc.third)) return 0;
            double rsix = rsq * rsq * rsq;
            double mid = (1 - 1 / rsix);
            return pc.eps * (mid * mid - 1) - pc.cut_energy;
        } else if (kind == LJATTRACT_IEPSISIG || kind == LJATTRACT_IEPS) {
            if (pc.eps == 0) return 0;
            if (dsq > (pc.third * pc.third * pc.sig * pc.sig)) return 0;
            double rsq = dsq / (pc.sig * pc.sig);
            double e;
            if (rsq < 1) {
                e = -pc.eps;
            } else {
                double rsix = rsq * rsq * rsq;
                double mid = (1 - 1 / rsix);
                e = pc.eps * (mid * mid - 1);
            }
            return e - pc.cut_energy;
        } else if (kind == LJATTRACTREPULSE) {
            // LJAttractRepulsePair::energy (interaction.hpp:1269-1286)
            double rsq = dsq / (pc.sig * pc.sig);
            if (rsq > pc.third * pc.third) return 0;
            double mid = (1 - std::pow(rsq, -3));
            return pc.eps * (mid * mid) - pc.cut_energy;
        } else if (kind == LJATTRACTFIXEDREPULSE) {
            // LJAttractFixedRepulsePair::energy (interaction.hpp:1366-1389)
            double rsq = dsq / (pc.sig * pc.sig);
            if (rsq > pc.third * pc.third) return 0;
            double mid = (1 - std::pow(rsq, -3));
            if (rsq > 1) return pc.eps * (mid * mid) - pc.cut_energy;
            return pc.fourth * (mid * mid) - pc.cut_energy;
        } else if (kind == LJISH) {
            // LJishPair::energy (interaction.hpp:1115-1129)
            double rsq = dsq / (pc.sig * pc.sig);
            if (rsq > pc.third * pc.third) return 0;
            double mid = (1 - std::pow(rsq, -pc.cut / 2));
            if (rsq > 1) return pc.eps * (mid * mid) - pc.cut_energy;
            return pc.fourth * (mid * mid) - pc.cut_energy;
        } else if (kind == REPULSIONDRAG) {
            // RepulsionDragPair::energy (interaction.hpp:1622-1628)
            if (dsq > pc.sig * pc.sig) return 0.0;
            double R = std::sqrt(dsq);
            return pc.eps * std::pow(1.0 - (R / pc.sig), pc.third) / pc.third;
        } else if (kind == EISMCLACHLAN) {
            // EisMclachlanPair::energy (interaction.hpp:1439-1444)
            double R = std::sqrt(dsq);
            if (R > pc.cut) return 0;
            return pc.eps / R + pc.sig + pc.third * R;
        } else {
            // LJRepulsive::energy (interaction.hpp:127-134)
            double rsq = dsq / (pc.sig * pc.sig);
            if (rsq > 1) return 0;
            double rsix = rsq * rsq * rsq;
            double mid = (1 - 1 / rsix);
            return pc.eps * (mid * mid);
        }
    }

    // P::forces(box) of the pair (i, j); returns false when the pair is beyond its cutoff (force = 0)
    bool pair_force(const PairConst& pc, const double* rij, double* fo, uint32_t i, uint32_t j) const {
        double dsq = dotv(rij, rij, nd);
        double s;
        if (kind == LJCUT_IEPSISIG || kind == LJATTRACT_IEPSISIG || kind == LJATTRACT_IEPS) {
            // LennardJonesCut::forces (263-271), LJAttractCut::forces (219-229)
            const bool attr = kind != LJCUT_IEPSISIG;
            double rsq = dsq / (pc.sig * pc.sig);
            if ((attr && (pc.eps == 0 || rsq < 1)) || rsq > (pc.third * pc.third)) {
                for (int d = 0; d < nd; d++) fo[d] = 0;
                return false;
            }
            double rsix = rsq * rsq * rsq;
            double fmagTimesR = 12 * pc.eps / rsix * (1 / rsix - 1);
            s = fmagTimesR / dsq;
            for (int d = 0; d < nd; d++) fo[d] = rij[d] * s;
            return true;
        }
        if (kind == LJATTRACTREPULSESIGS) {
            // LJAttractRepulseSigsPair::forces (interaction.hpp:1218-1238)
            double cu = pc.sig + pc.cut * (pc.third - 1);
            if (pc.third > 0 && dsq > cu * cu) { for (int d = 0; d < nd; d++) fo[d] = 0; return false; }
            if (dsq > pc.sig * pc.sig) {
                double dist = std::sqrt(dsq);
                double rminus = dist - pc.sig + pc.cut;
                double r_over_sig = rminus / pc.cut;
                double rsix = std::pow(r_over_sig, -6);
                double fmag_over_r = 12 * rsix * (rsix - 1) / (dist * rminus);
                s = pc.fourth * fmag_over_r;
            } else {
                double r_over_sigsq = dsq / (pc.sig * pc.sig);
                double rsix = std::pow(r_over_sigsq, -3);
                double fmagTimesR = 12 * rsix * (rsix - 1);
                s = pc.eps * fmagTimesR / dsq;
            }
            for (int d = 0; d < nd; d++) fo[d] = rij[d] * s;
            return true;
        }
        if (kind == LJATTRACTREPULSE || kind == LJATTRACTFIXEDREPULSE || kind == LJISH) {
            // LJAttractRepulsePair::forces (1287-1297), LJAttractFixedRepulsePair::forces (1390-1398),
            // LJishPair::forces (1130-1140)
            if (kind == LJATTRACTREPULSE && pc.eps == 0) { for (int d = 0; d < nd; d++) fo[d] = 0; return false; }
            double rsq = dsq / (pc.sig * pc.sig);
            if (rsq > (pc.third * pc.third)) { for (int d = 0; d < nd; d++) fo[d] = 0; return false; }
            if (kind == LJATTRACTREPULSE) {
                double rsix = std::pow(rsq, -3);
                double fmagTimesR = 12 * pc.eps * rsix * (rsix - 1);
                s = fmagTimesR / dsq;
            } else if (kind == LJATTRACTFIXEDREPULSE) {
                double rsix = std::pow(rsq, -3);
                double fmagTimesR = 12 * rsix * (rsix - 1);
                s = (rsq < 1) ? pc.fourth * fmagTimesR / dsq : pc.eps * fmagTimesR / dsq;
            } else {
                double n = pc.cut;
                double rmid = std::pow(rsq, -n / 2);
                double fmagTimesR = 2 * n * rmid * (rmid - 1);
                s = (rsq < 1) ? pc.fourth * fmagTimesR / dsq : pc.eps * fmagTimesR / dsq;
            }
            for (int d = 0; d < nd; d++) fo[d] = rij[d] * s;
            return true;
        }
        if (kind == REPULSIONDRAG) {
            // RepulsionDragPair::forces (interaction.hpp:1629-1639): the repulsion minus gamma
            // times the relative velocity's component along rij
            double vij[3];
            for (int d = 0; d < nd; d++) vij[d] = v[i * nd + d] - v[j * nd + d];
            if (dsq > pc.sig * pc.sig) { for (int d = 0; d < nd; d++) fo[d] = 0; return false; }
            double R = std::sqrt(dsq);
            double vdot = dotv(vij, rij, nd);
            double sr = pc.eps * std::pow(1.0 - (R / pc.sig), pc.third - 1) / pc.sig / R;
            for (int d = 0; d < nd; d++) {
                double vperp = rij[d] * vdot / dsq;
                fo[d] = rij[d] * sr - vperp * pc.fourth;
            }
            return true;
        }
        if (kind == LJCUT) {
            // LennardJonesCut::forces (interaction.hpp:263-271)
            double rsq = dsq / (pc.sig * pc.sig);
            if (rsq > (pc.third * pc.third)) { for (int d = 0; d < nd; d++) fo[d] = 0; return false; }
            double rsix = rsq * rsq * rsq;
            double fmagTimesR = 12 * pc.eps / rsix * (1 / rsix - 1);
            s = fmagTimesR / dsq;
        } else if (kind == LJATTRACT) {
            // LJAttractCut::forces (interaction.hpp:219-229)
            double rsq = dsq / (pc.sig * pc.sig);
            if (pc.eps == 0 || rsq < 1 || rsq > (pc.third * pc.third)) {
                for (int d = 0; d < nd; d++) fo[d] = 0;
                return false;
            }
            double rsix = rsq * rsq * rsq;
            double fmagTimesR = 12 * pc.eps / rsix * (1 / rsix - 1);
            s = fmagTimesR / dsq;
        } else if (kind == REPULSION || kind == REPULSION_IEPSISIG) {
            // RepulsionPair::forces (interaction.hpp:1551-1556)
            if (dsq > pc.sig * pc.sig) { for (int d = 0; d < nd; d++) fo[d] = 0; return false; }
            double R = std::sqrt(dsq);
            s = pc.eps * std::pow(1.0 - (R / pc.sig), pc.third - 1) / pc.sig / R;
        } else if (kind == LOISOHERN || kind == LOISOHERN_MIN) {
            // LoisOhernPair::forces (interaction.hpp:1729-1743)
            const double C = pc.third, l = pc.fourth;
            if (dsq >= pc.cut * pc.cut) { for (int d = 0; d < nd; d++) fo[d] = 0; return false; }
            double R = std::sqrt(dsq);
            double rsig = R / pc.sig;
            if (rsig <= 1 + C) {
                double dR = rsig - 1;
                s = -pc.eps * dR / R;
            } else {
                double dR2 = rsig - (C + l + 1);
                s = C * pc.eps / l * dR2 / R;
            }
        } else if (kind == LOISLIN || kind == LOISLIN_MIN) {
            // LoisLinPair::forces (interaction.hpp:1817-1828); -rij * (f / R) is rij * -(f / R)
            const double f = pc.third;
            if (dsq >= pc.cut * pc.cut) { for (int d = 0; d < nd; d++) fo[d] = 0; return false; }
            double R = std::sqrt(dsq);
            if (R <= pc.sig) {
                double dR = 1.0 - (R / pc.sig);
                s = pc.eps * dR / pc.sig / R;
            } else {
                s = -(f / R);
            }
        } else if (kind == EISMCLACHLAN) {
            // EisMclachlanPair::forces (interaction.hpp:1445-1451)
            if (dsq > (pc.cut * pc.cut)) { for (int d = 0; d < nd; d++) fo[d] = 0; return false; }
            double R = std::sqrt(dsq);
            s = (pc.eps / dsq - pc.third) / R;
        } else {
            // LJRepulsive::forces (interaction.hpp:136-150)
            double rsq = dsq / (pc.sig * pc.sig);
            if (rsq > 1) { for (int d = 0; d < nd; d++) fo[d] = 0; return false; }
            double rsix = rsq * rsq * rsq;
            double fmagTimesR = 12 * pc.eps / rsix * (1 / rsix - 1);
            s = fmagTimesR / dsq;
        }
        for (int d = 0; d < nd; d++) fo[d] = rij[d] * s;
        return true;
    }

    double max_size(uint32_t i) const {
        // EpsSigCutAtom::max_size (interaction.hpp:904), EpsSigExpAtom (1464), EpsSigAtom (864)
        if (kind == LJCUT || kind == LJATTRACT) return params[i].p1 * params[i].p2;
        // LoisOhernAtom::max_size (interaction.hpp:1691), LoisLinAtom::max_size (1780)
        if (kind == LOISOHERN || kind == LOISOHERN_MIN) return params[i].p1 * (1 + params[i].p2 + params[i].p3);
        if (kind == LOISLIN || kind == LOISLIN_MIN) return params[i].p1 * (1 + params[i].p3);
        if (kind == EISMCLACHLAN) return params[i].p0;   // EisMclachlanAtom::max_size (1423)
        // EpsEpsSigSigCutAtom::max_size (1169): sig_r + sig_a (sigcut - 1)
        if (kind == LJATTRACTREPULSESIGS) return params[i].p2 + params[i].p3 * (params[i].p4 - 1);
        if (kind == LJCUT_IEPSISIG || kind == LJATTRACT_IEPSISIG || kind == REPULSION_IEPSISIG) {
            // IEpsISigCutAtom::max_size (947-953): the largest sigma of the atom's row times sigcut;
            // IEpsISigExpAtom::max_size (1505-1511): the largest sigma
            const double* row = &tsig[params[i].t * ntypes];
            double sg = row[0];
            for (uint32_t k = 1; k < ntypes; ++k)
                if (sg < row[k]) sg = row[k];
            return kind == REPULSION_IEPSISIG ? sg : sg * params[i].p2;
        }
        // IEpsSigCutAtom (1017), IEpsRepsSigCutAtom (1335), IEpsRepsSigExpCutAtom (1091): sigma * sigcut
        if (indexed_kind(kind)) return params[i].p1 * params[i].p2;
        // EpsSigExpDragAtom::max_size (1611) is sigma, as below
        return params[i].p1;
    }

    bool is_ignored(uint32_t i, uint32_t j) const {
        uint32_t hi = std::max(i, j), lo = std::min(i, j);
        return ignored.count({hi, lo}) > 0;
    }

    // NeighborList::update_list (trackers.cpp:19-85)
    bool update_list(bool force) {
        const size_t M = members.size();
        if (!force && !ignorechanged) {
            double bigdist = 0, biggestdist = 0;
            for (size_t k = 0; k < M; k++) {
                const double* xi = &x[members[k] * nd];
                double dd[3];
                for (int d = 0; d < nd; d++) dd[d] = xi[d] - lastlocs[k * nd + d];
                double curdist = std::sqrt(dotv(dd, dd, nd));
                if (curdist > biggestdist) {
                    bigdist = biggestdist;
                    biggestdist = curdist;
                } else if (curdist > bigdist) {
                    bigdist = curdist;
                } else
                    continue;
                if (bigdist + biggestdist >= skin) {
                    force = true;
                    break;
                }
            }
            if (!force) return false;
        }
        updatenum++;
        ignorechanged = false;
        curpairs.clear();
        for (size_t i = 0; i < M; i++) {
            uint32_t ai = members[i];
            const double* xi = &x[ai * nd];
            for (int d = 0; d < nd; d++) lastlocs[i * nd + d] = xi[d];
            for (size_t j = 0; j < i; j++) {
                uint32_t aj = members[j];
                if (is_ignored(ai, aj)) continue;
                double diam = (diameters[i] + diameters[j]) / 2;
                double r[3];
                diff(xi, &x[aj * nd], r);
                if (std::sqrt(dotv(r, r, nd)) < (diam + skin)) curpairs.push_back({ai, aj});
            }
        }
        return true;
    }

    // NListed::set_forces (interaction.hpp:2165-2175); adds into f
    void nlisted_set_forces(bool want_p, double* p_out, double* stress_out) {
        double p = 0;
        double st[9] = {0};
        for (auto& pr : curpairs) {
            PairConst pc = pair_const(pr.first, pr.second);
            double r[3], fo[3];
            diff(&x[pr.first * nd], &x[pr.second * nd], r);
            pair_force(pc, r, fo, pr.first, pr.second);
            for (int d = 0; d < nd; d++) {
                f[pr.first * nd + d] += fo[d];
                f[pr.second * nd + d] -= fo[d];
            }
            if (want_p) {
                // set_forces_get_pressure (2231-2245) / set_forces_get_stress (2262-2276)
                p += dotv(r, fo, nd);
                for (int aa = 0; aa < nd; aa++)
                    for (int bb = 0; bb < nd; bb++) st[aa * nd + bb] += r[aa] * fo[bb];
            }
        }
        if (p_out) *p_out = p;
        if (stress_out) std::memcpy(stress_out, st, sizeof(double) * nd * nd);
    }

    // NListed::energy (2152-2163)
    double nlisted_energy() const {
        double E = 0;
        for (auto& pr : curpairs) {
            PairConst pc = pair_const(pr.first, pr.second);
            double r[3];
            diff(&x[pr.first * nd], &x[pr.second * nd], r);
            E += pair_energy(pc, r);
        }
        return E;
    }

    // NListed::pressure (2247-2260) and stress (2278-2291)
    double nlisted_pressure(double* stress_out) const {
        double p = 0;
        double st[9] = {0};
        for (auto& pr : curpairs) {
            PairConst pc = pair_const(pr.first, pr.second);
            double r[3], fo[3];
            diff(&x[pr.first * nd], &x[pr.second * nd], r);
            pair_force(pc, r, fo, pr.first, pr.second);
            p += dotv(r, fo, nd);
            for (int aa = 0; aa < nd; aa++)
                for (int bb = 0; bb < nd; bb++) st[aa * nd + bb] += r[aa] * fo[bb];
        }
        if (stress_out) std::memcpy(stress_out, st, sizeof(double) * nd * nd);
        return p;
    }

    // NListed::contacts / overlaps (2124-2150)
    uint64_t nlisted_count(bool overlaps) const {
        uint64_t c = 0;
        for (auto& pr : curpairs) {
            PairConst pc = pair_const(pr.first, pr.second);
            double r[3];
            diff(&x[pr.first * nd], &x[pr.second * nd], r);
            double E = pair_energy(pc, r);
            if (overlaps ? (E > 0.0) : (E != 0.0)) c++;
        }
        return c;
    }

    static bool mobile(double mm) { return !(mm <= 0 || std::isinf(mm)); }

    // AtomGroup::reset_forces (box.cpp:427-431) + Collection::set_forces (collection.cpp:159-179)
    void collection_set_forces(bool constraints_and_a) {
        std::fill(f.begin(), f.end(), 0.0);
        if (kind >= 0) nlisted_set_forces(false, nullptr, nullptr);
        if (!constraints_and_a) return;
        for (uint32_t i = 0; i < n; i++) {
            if (!mobile(m[i])) {
                for (int d = 0; d < nd; d++) a[i * nd + d] = 0;
                continue;
            }
            for (int d = 0; d < nd; d++) a[i * nd + d] = f[i * nd + d] / m[i];
        }
    }

    void update_trackers() {
        if (kind >= 0) update_list(false);
    }

    // CollectionVerlet::timestep (collection.cpp:442-469)
    void verlet(double dt) {
        for (uint32_t i = 0; i < n; i++) {
            if (!mobile(m[i])) {
                for (int d = 0; d < nd; d++) v[i * nd + d] = 0;
                continue;
            }
            for (int d = 0; d < nd; d++) {
                x[i * nd + d] += v[i * nd + d] * dt + a[i * nd + d] * (dt * dt / 2);
                v[i * nd + d] += a[i * nd + d] * (dt / 2);
            }
        }
        collection_set_forces(false);
        for (uint32_t i = 0; i < n; i++) {
            if (!mobile(m[i])) {
                for (int d = 0; d < nd; d++) a[i * nd + d] = 0;
                continue;
            }
            for (int d = 0; d < nd; d++) {
                a[i * nd + d] = f[i * nd + d] / m[i];
                v[i * nd + d] += a[i * nd + d] * (dt / 2);
            }
        }
        update_trackers();
    }

    // CollectionDamped::timestep (collection.cpp:356-381); c0,c1,c2 from set_constants (339-354)
    void damped(double dt, double c0, double c1, double c2) {
        for (uint32_t i = 0; i < n; i++) {
            if (!mobile(m[i])) {
                for (int d = 0; d < nd; d++) v[i * nd + d] = 0;
                continue;
            }
            for (int d = 0; d < nd; d++) {
                x[i * nd + d] += v[i * nd + d] * (c1 * dt) + a[i * nd + d] * (c2 * dt * dt);
                v[i * nd + d] = v[i * nd + d] * c0 + a[i * nd + d] * (dt * (c1 - c2));
            }
        }
        collection_set_forces(true);
        for (uint32_t i = 0; i < n; i++) {
            if (!mobile(m[i])) continue;
            for (int d = 0; d < nd; d++) v[i * nd + d] += a[i * nd + d] * (dt * c2);
        }
        update_trackers();
    }

    // CollectionSol::timestep (collection.cpp:265-322) with the counter-based
    // Gaussian pair generator standing in for BivariateGauss::gen_vecs.
    void sol(double dt, double damping, double T, double c0, double c1, double c2,
             double x11, double x21, double x22, uint64_t seed, uint64_t step);
};

// ---- counter-based normal generator (Philox4x32-10, Salmon et al. SC'11) ----
inline void philox_round(uint32_t c[4], const uint32_t k[2]) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k[0];
    uint32_t n2 = hi0 ^ c[3] ^ k[1];
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
}

inline void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    uint32_t k[2] = {k0, k1};
    for (int r = 0; r < 10; r++) {
        philox_round(c, k);
        k[0] += 0x9E3779B9u;
        k[1] += 0xBB67AE85u;
    }
}

inline double u53(uint32_t a, uint32_t b) {
    uint64_t v = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
    return ((double)v + 0.5) * (1.0 / 9007199254740992.0);
}

// Six standard normals for (seed, step, atom): Philox blocks 0..2, Box-Muller.
void normals6(uint64_t seed, uint64_t step, uint32_t atom, double out[6]) {
    for (uint32_t blk = 0; blk < 3; blk++) {
        uint32_t c[4] = {atom, (uint32_t)step, (uint32_t)(step >> 32), blk};
        philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        double u1 = u53(c[0], c[1]);
        double u2 = u53(c[2], c[3]);
        double r = std::sqrt(-2.0 * std::log(u1));
        double th = 6.283185307179586 * u2;
        out[2 * blk] = r * std::cos(th);
        out[2 * blk + 1] = r * std::sin(th);
    }
}

void System::sol(double dt, double damping, double T, double c0, double c1, double c2,
                 double x11, double x21, double x22, uint64_t seed, uint64_t step) {
    for (uint32_t i = 0; i < n; i++) {
        if (m[i] <= 0 || std::isinf(m[i])) {
            for (int d = 0; d < nd; d++) v[i * nd + d] = 0;
            continue;
        }
        double v0 = std::sqrt(T / m[i]);
        double r0 = dt * v0;
        double g[6] = {0, 0, 0, 0, 0, 0};
        double drG[3] = {0, 0, 0}, dvG[3] = {0, 0, 0};
        if (damping > 0) {
            normals6(seed, step, i, g);
            // BivariateGauss::gen_vecs (vecrand.cpp:73-85): x1 = g[0..nd), x2 = g[nd..2nd)
            for (int d = 0; d < nd; d++) {
                drG[d] = g[d] * x11;
                dvG[d] = g[d] * x21 + g[nd + d] * x22;
            }
        }
        for (int d = 0; d < nd; d++) {
            x[i * nd + d] += v[i * nd + d] * (c1 * dt) + a[i * nd + d] * (c2 * dt * dt) + drG[d] * r0;
            v[i * nd + d] = v[i * nd + d] * c0 + a[i * nd + d] * (dt * (c1 - c2)) + dvG[d] * v0;
        }
    }
    collection_set_forces(false);
    for (uint32_t i = 0; i < n; i++) {
        if (m[i] == 0 || std::isinf(m[i])) {
            for (int d = 0; d < nd; d++) a[i * nd + d] = 0;
            continue;
        }
        for (int d = 0; d < nd; d++) a[i * nd + d] = f[i * nd + d] / m[i];
    }
    for (uint32_t i = 0; i < n; i++) {
        if (m[i] == 0 || std::isinf(m[i])) {
            for (int d = 0; d < nd; d++) v[i * nd + d] = 0;
            continue;
        }
        for (int d = 0; d < nd; d++) v[i * nd + d] += a[i * nd + d] * (dt * c2);
    }
    update_trackers();
}


// ---------------------------------------------------------------------------
// Conjugate-gradient minimisers: CollectionNLCG (positions and the box's
// log-volume, collection.hpp:400-475, collection.cpp:494-829) and
// CollectionNLCGV (positions only, collection.hpp:490-566,
// collection.cpp:894-1168), restated on one System with the reference's
// sequential sums.
// ---------------------------------------------------------------------------
struct Nlcg {
    bool boxed = true;   // CollectionNLCG (true) or CollectionNLCGV (false)
    // parameters (collection.hpp:407-425)
    double dt = 0, seceps = 1e-20, kappa = 10, alphamax = 2, afrac = 0, dxmax = 100, stepmax = 1e-3,
           kmax = 1000, P0 = 0, maxdV = 0;
    uint32_t secmax = 40;
    // state kept between time steps
    double Knew = 0, k = 0, vl = 0, fl = 0, al = 0;
    double alpha = 0, beta = 0, betaused = 0, dxsum = 0, alphavmax = 0;
    uint32_t sec = 0;

    // OriginBox::V (box.hpp:112): the product of the side lengths
    static double volume(const System& S) {
        double V = S.L[0] * S.L[1];
        if (S.nd == 3) V = V * S.L[2];
        return V;
    }
    // CollectionNLCG::get_length_squared (collection.cpp:641-649)
    static double lensq(const System& S) { return S.nd == 3 ? std::pow(volume(S), 2.0 / 3.0) : volume(S); }

    // fdota / fdotf / fdotv / vdotv (collection.cpp:651-705, 910-975)
    double dot_sum(const System& S, const std::vector<double>& p, const std::vector<double>& q) const {
        double r = 0;
        for (uint32_t i = 0; i < S.n; i++) {
            if (!System::mobile(S.m[i])) continue;
            r += dotv(&p[i * S.nd], &q[i * S.nd], S.nd);
        }
        return r;
    }
    double fdota(const System& S) const {
        double r = dot_sum(S, S.f, S.a);
        return boxed ? r / lensq(S) + fl * al : r;
    }
    double fdotv(const System& S) const {
        double r = dot_sum(S, S.f, S.v);
        return boxed ? r / lensq(S) + fl * vl : r;
    }
    double vdotv(const System& S) const {
        double r = dot_sum(S, S.v, S.v);
        return boxed ? r / lensq(S) + vl * vl : r;
    }

    // CollectionNLCG::stepx (collection.cpp:621-639) / CollectionNLCGV::stepx (900-908)
    void stepx(System& S, double dx) const {
        if (boxed) {
            const double Lfac = std::exp(dx * vl / (kappa * S.nd));
            for (uint32_t i = 0; i < S.n; i++)
                for (int d = 0; d < S.nd; d++) {
                    double& x = S.x[i * S.nd + d];
                    x *= Lfac;
                    x += S.v[i * S.nd + d] * dx;
                }
            for (int d = 0; d < S.nd; d++) S.L[d] *= Lfac;   // OriginBox::resize (box.hpp:125-128)
        } else {
            for (uint32_t i = 0; i < S.n; i++) {
                if (!System::mobile(S.m[i])) continue;
                for (int d = 0; d < S.nd; d++) S.x[i * S.nd + d] += S.v[i * S.nd + d] * dx;
            }
        }
    }

    // Collection::set_forces_get_pressure(false) (collection.cpp:181-208)
    static double forces_pressure(System& S) {
        std::fill(S.f.begin(), S.f.end(), 0.0);
        double p = 0;
        if (S.kind >= 0) S.nlisted_set_forces(true, &p, nullptr);
        for (uint32_t i = 0; i < S.n; i++)
            if (!System::mobile(S.m[i]))
                for (int d = 0; d < S.nd; d++) S.a[i * S.nd + d] = 0;
        return p;
    }

    // CollectionNLCG::set_forces(constraints_and_a, setV) (collection.cpp:534-566);
    // CollectionNLCGV has Collection::set_forces (collection.cpp:159-179)
    void set_forces(System& S, bool constraints_and_a, bool setV = true) {
        if (!boxed) {
            S.collection_set_forces(constraints_and_a);
            return;
        }
        const double V = volume(S);
        if (setV) {
            const double interacP = forces_pressure(S);
            fl = ((interacP / S.nd) - (P0 * V)) / kappa;
            if (constraints_and_a) {
                al = fl;
                vl = fl;
            }
        } else {
            S.collection_set_forces(false);
        }
        if (constraints_and_a) {
            for (uint32_t i = 0; i < S.n; i++) {
                if (!System::mobile(S.m[i])) {
                    for (int d = 0; d < S.nd; d++) S.v[i * S.nd + d] = S.a[i * S.nd + d] = 0;
                    continue;
                }
                for (int d = 0; d < S.nd; d++) S.a[i * S.nd + d] = S.v[i * S.nd + d] = S.f[i * S.nd + d];
            }
            Knew = fdota(S);
        }
    }

    // CollectionNLCG::reset (collection.cpp:525-532) / CollectionNLCGV::reset (977-988)
    void reset(System& S) {
        k = 0;
        if (boxed) {
            set_forces(S, true, true);
            for (size_t q = 0; q < S.v.size(); q++) S.v[q] = S.a[q];
            vl = al;
        } else {
            S.collection_set_forces(false);
            for (uint32_t i = 0; i < S.n; i++) {
                if (!System::mobile(S.m[i])) continue;
                for (int d = 0; d < S.nd; d++) S.v[i * S.nd + d] = S.a[i * S.nd + d] = S.f[i * S.nd + d];
            }
        }
    }

    // CollectionNLCG::descend (collection.cpp:811-829) / CollectionNLCGV::descend (990-1005)
    void descend(System& S) {
        set_forces(S, false, true);
        for (uint32_t i = 0; i < S.n; i++) {
            if (!System::mobile(S.m[i])) continue;
            for (int d = 0; d < S.nd; d++) S.v[i * S.nd + d] = S.a[i * S.nd + d] = S.f[i * S.nd + d];
        }
        if (boxed) {
            al = fl;
            vl = fl;
        }
        stepx(S, dt);
        S.update_trackers();
    }

    // CollectionNLCG::timestep (collection.cpp:682-809) / CollectionNLCGV::timestep (1019-1168)
    void timestep(System& S) {
        stepx(S, dt);
        set_forces(S, false, true);
        double eta0 = -fdotv(S);
        double eta;
        stepx(S, -dt);
        S.update_trackers();
        alpha = -dt;
        set_forces(S, false, true);
        dxsum = 0;
        const double vdv = vdotv(S);
        for (sec = 0; sec < secmax; sec++) {
            eta = -fdotv(S);
            double alphafac = -eta / std::abs(eta0 - eta);
            if (std::abs(eta0 - eta) <= 1e-12 * std::abs(eta)) {
                alphafac = alphamax > 0 ? alphamax : 1.1;
                sec = sec > 0 ? sec * 2 - 1 : 1;
            }
            if (alphamax > 0 && alphafac > alphamax) alphafac = alphamax;
            if (alphamax > 0 && alphafac < -alphamax) alphafac = -alphamax;
            alpha = std::abs(alpha) * alphafac;
            const double newdxsum = std::abs(dxsum + alpha);
            if (dxmax > 0 && newdxsum > dxmax) {
                k = 0;
                break;
            }
            if (boxed) {
                const double dVoverV = std::expm1(std::abs(dxsum + alpha) * vl / (kappa * S.nd));
                if (maxdV > 0 && dVoverV > maxdV) {
                    k = 0;
                    break;
                }
            }
            dxsum += alpha;
            stepx(S, alpha);
            if (!boxed) S.update_trackers();
            set_forces(S, false, true);
            eta0 = eta;
            if (alpha * alpha * vdv < seceps * seceps) break;
            if ((sec > 1) && (afrac > 0) && (std::abs(alpha) < std::abs(dxsum)) &&
                (std::abs(alpha) / std::abs(dxsum) < afrac))
                break;
            if (stepmax > 0 && dxsum * dxsum * vdv > stepmax * stepmax) {
                k = 0;
                break;
            }
        }
        alphavmax = std::sqrt(alpha * alpha * vdv);
        const double Kold = Knew;
        const double Kmid = fdota(S);
        for (uint32_t i = 0; i < S.n; i++) {
            if (boxed && !System::mobile(S.m[i])) {
                for (int d = 0; d < S.nd; d++) S.a[i * S.nd + d] = 0;
                continue;
            }
            for (int d = 0; d < S.nd; d++) S.a[i * S.nd + d] = S.f[i * S.nd + d];
        }
        al = fl;
        Knew = fdota(S);
        beta = (Knew - Kmid) / Kold;
        betaused = beta;
        k++;
        if (k >= kmax || std::isinf(betaused) || std::isnan(betaused) || betaused <= 0) {
            k = 0;
            betaused = 0;
        } else if (betaused > 1) {
            betaused = 1;
        }
        for (uint32_t i = 0; i < S.n; i++) {
            if (boxed && !System::mobile(S.m[i])) {
                for (int d = 0; d < S.nd; d++) S.v[i * S.nd + d] = 0;
                continue;
            }
            for (int d = 0; d < S.nd; d++) S.v[i * S.nd + d] = S.a[i * S.nd + d] + S.v[i * S.nd + d] * betaused;
        }
        if (boxed) vl = al + betaused * vl;
    }
};

// the parameter / state vectors of the C ABI (PARM_NLCG_P_*, PARM_NLCG_S_*)
void nlcg_set(Nlcg& G, const double* p) {
    G.dt = p[0]; G.P0 = p[1]; G.kappa = p[2]; G.kmax = p[3]; G.secmax = (uint32_t)p[4]; G.seceps = p[5];
    G.alphamax = p[6]; G.afrac = p[7]; G.dxmax = p[8]; G.stepmax = p[9]; G.maxdV = p[10];
}
void nlcg_get_state(const Nlcg& G, double* o) {
    const double v[11] = {G.Knew, G.k, G.vl, G.fl, G.al, G.alpha, G.beta, G.betaused, G.dxsum, G.alphavmax,
                          (double)G.sec};
    for (int q = 0; q < 11; q++) o[q] = v[q];
}
void nlcg_set_state(Nlcg& G, const double* o) {
    G.Knew = o[0]; G.k = o[1]; G.vl = o[2]; G.fl = o[3]; G.al = o[4]; G.alpha = o[5]; G.beta = o[6];
    G.betaused = o[7]; G.dxsum = o[8]; G.alphavmax = o[9]; G.sec = (uint32_t)o[10];
}

}  // namespace

extern "C" {

void* orc_create(int ndim, uint32_t n) {
    if (ndim != 2 && ndim != 3) return nullptr;
    return new System(ndim, n);
}
void orc_destroy(void* s) { delete static_cast<System*>(s); }

void orc_set_box(void* s, const double* L) {
    System* S = static_cast<System*>(s);
    for (int d = 0; d < S->nd; d++) S->L[d] = L[d];
}

// a LeesEdwardsBox of shear gamma (lees != 0) or the OriginBox
void orc_set_lees(void* s, int lees, double gamma) {
    System* S = static_cast<System*>(s);
    S->lees = lees != 0;
    S->gamma = gamma;
}

// arrays are (n, ndim) row-major (an AtomVec's x/v/a/f fields), m is (n,)
void orc_set_state(void* s, const double* x, const double* v, const double* a, const double* f,
                   const double* m) {
    System* S = static_cast<System*>(s);
    size_t k = (size_t)S->n * S->nd;
    if (x) std::memcpy(S->x.data(), x, k * 8);
    if (v) std::memcpy(S->v.data(), v, k * 8);
    if (a) std::memcpy(S->a.data(), a, k * 8);
    if (f) std::memcpy(S->f.data(), f, k * 8);
    if (m) std::memcpy(S->m.data(), m, (size_t)S->n * 8);
}

void orc_get_state(void* s, double* x, double* v, double* a, double* f, double* m) {
    System* S = static_cast<System*>(s);
    size_t k = (size_t)S->n * S->nd;
    if (x) std::memcpy(x, S->x.data(), k * 8);
    if (v) std::memcpy(v, S->v.data(), k * 8);
    if (a) std::memcpy(a, S->a.data(), k * 8);
    if (f) std::memcpy(f, S->f.data(), k * 8);
    if (m) std::memcpy(m, S->m.data(), (size_t)S->n * 8);
}

// NListed(box, atoms, skin) (interaction.hpp:1911-1914)
int orc_set_interaction(void* s, int kind, double skin) {
    System* S = static_cast<System*>(s);
    if (kind < 0 || kind > 17) return -1;
    S->kind = kind;
    S->skin = skin;
    return 0;
}

// NListed::add(A) -> NeighborList::add(atm, atm.max_size()) (interaction.hpp:1906-1910,
// trackers.hpp:194-201)
int orc_add_atom(void* s, uint32_t i, const double* p) {
    System* S = static_cast<System*>(s);
    if (i >= S->n || S->has_params[i]) return -1;
    if (indexed_kind(S->kind)) {
        // params: (indx, sigcut) for IEpsISigCutAtom, (indx, sigma, sigcut) for IEpsSigCutAtom,
        // (indx, repeps, sigma, sigcut) for IEpsRepsSigCutAtom, (indx, repeps, sigma, n, sigcut)
        // for IEpsRepsSigExpCutAtom
        AtomParams& a = S->params[i];
        a.t = (uint32_t)p[0];
        if (a.t >= S->ntypes) return -1;
        const int k = S->kind;
        if (k == LJCUT_IEPSISIG || k == LJATTRACT_IEPSISIG || k == REPULSION_IEPSISIG) a.p2 = p[1];
        else if (k == LJATTRACT_IEPS || k == LJATTRACTREPULSE) { a.p1 = p[1]; a.p2 = p[2]; }
        else if (k == LJATTRACTFIXEDREPULSE) { a.p0 = p[1]; a.p1 = p[2]; a.p2 = p[3]; }
        else { a.p0 = p[1]; a.p1 = p[2]; a.p3 = p[3]; a.p2 = p[4]; }
    } else if (S->kind == LJATTRACTREPULSESIGS) {
        AtomParams& a = S->params[i];
        a.p0 = p[0]; a.p1 = p[1]; a.p2 = p[2]; a.p3 = p[3]; a.p4 = p[4];
    } else {
        S->params[i].p0 = p[0];
        S->params[i].p1 = p[1];
        S->params[i].p2 = (S->kind == LJREPULSE) ? 0.0 : p[2];
        S->params[i].p3 = four_params(S->kind) ? p[3] : 0.0;
    }
    S->has_params[i] = 1;
    S->members.push_back(i);
    S->diameters.push_back(S->max_size(i));
    for (int d = 0; d < S->nd; d++) S->lastlocs.push_back(S->x[i * S->nd + d]);
    S->ignorechanged = true;
    return 0;
}

// the pair tables of the indexed kinds: eps[a * ntypes + b] = the epsilon of
// a pair whose first atom has type a and second type b (first.epsilons[b]);
// sig likewise (IEpsISigCutAtom), may be NULL
int orc_set_pair_table(void* s, uint32_t ntypes, const double* eps, const double* sig) {
    System* S = static_cast<System*>(s);
    S->ntypes = ntypes;
    S->teps.assign(eps, eps + (size_t)ntypes * ntypes);
    if (sig) S->tsig.assign(sig, sig + (size_t)ntypes * ntypes);
    else S->tsig.assign((size_t)ntypes * ntypes, 0.0);
    return 0;
}

// NeighborList::add(atom, diameter) (trackers.hpp:194-201): a member without
// pair parameters (an NListed on the list sees its default-constructed atom)
int orc_add_member(void* s, uint32_t i, double diameter) {
    System* S = static_cast<System*>(s);
    if (i >= S->n || S->has_params[i]) return -1;
    S->has_params[i] = 1;
    S->members.push_back(i);
    S->diameters.push_back(diameter);
    for (int d = 0; d < S->nd; d++) S->lastlocs.push_back(S->x[i * S->nd + d]);
    S->ignorechanged = true;
    return 0;
}

// NeighborList::ignore (trackers.hpp:190-193)
void orc_ignore(void* s, uint32_t i, uint32_t j) {
    System* S = static_cast<System*>(s);
    S->ignored.insert({std::max(i, j), std::min(i, j)});
    S->ignorechanged = true;
}

int orc_nl_update(void* s, int force) { return static_cast<System*>(s)->update_list(force != 0) ? 1 : 0; }
uint32_t orc_nl_which(void* s) { return static_cast<System*>(s)->updatenum; }
uint64_t orc_nl_numpairs(void* s) { return static_cast<System*>(s)->curpairs.size(); }
void orc_nl_get_pairs(void* s, uint32_t* out) {
    System* S = static_cast<System*>(s);
    for (size_t k = 0; k < S->curpairs.size(); k++) {
        out[2 * k] = S->curpairs[k].first;
        out[2 * k + 1] = S->curpairs[k].second;
    }
}

double orc_energy(void* s) { return static_cast<System*>(s)->nlisted_energy(); }
double orc_pressure(void* s, double* stress) { return static_cast<System*>(s)->nlisted_pressure(stress); }
uint64_t orc_contacts(void* s) { return static_cast<System*>(s)->nlisted_count(false); }
uint64_t orc_overlaps(void* s) { return static_cast<System*>(s)->nlisted_count(true); }

// Collection::set_forces(constraints_and_a); when p/stress given, the
// NListed::set_forces_get_pressure / set_forces_get_stress accumulations too.
void orc_set_forces(void* s, int constraints_and_a, double* p, double* stress) {
    System* S = static_cast<System*>(s);
    std::fill(S->f.begin(), S->f.end(), 0.0);
    S->nlisted_set_forces(p || stress, p, stress);
    if (!constraints_and_a) return;
    for (uint32_t i = 0; i < S->n; i++) {
        for (int d = 0; d < S->nd; d++)
            S->a[i * S->nd + d] = System::mobile(S->m[i]) ? S->f[i * S->nd + d] / S->m[i] : 0.0;
    }
}

// Collection::initialize (collection.cpp:13-19)
void orc_initialize(void* s) {
    System* S = static_cast<System*>(s);
    S->update_trackers();
    S->collection_set_forces(true);
    S->update_trackers();
}

void orc_update_trackers(void* s) { static_cast<System*>(s)->update_trackers(); }

void orc_verlet(void* s, double dt, uint32_t nsteps) {
    System* S = static_cast<System*>(s);
    for (uint32_t k = 0; k < nsteps; k++) S->verlet(dt);
}

void orc_damped(void* s, double dt, double c0, double c1, double c2, uint32_t nsteps) {
    System* S = static_cast<System*>(s);
    for (uint32_t k = 0; k < nsteps; k++) S->damped(dt, c0, c1, c2);
}

void orc_sol(void* s, double dt, double damping, double T, double c0, double c1, double c2,
             double x11, double x21, double x22, uint64_t seed, uint64_t step0, uint32_t nsteps) {
    System* S = static_cast<System*>(s);
    for (uint32_t k = 0; k < nsteps; k++)
        S->sol(dt, damping, T, c0, c1, c2, x11, x21, x22, seed, step0 + k);
}

// CollectionNLCG / CollectionNLCGV on the oracle system: create with the
// parameter vector (dt, P0, kappa, kmax, secmax, seceps, alphamax, afrac,
// dxmax, stepmax, maxdV); the state vector is (Knew, k, vl, fl, al, alpha,
// beta, betaused, dxsum, alphavmax, sec)
void* orc_nlcg_create(int boxed, const double* params) {
    Nlcg* G = new Nlcg();
    G->boxed = boxed != 0;
    nlcg_set(*G, params);
    return G;
}
void orc_nlcg_destroy(void* g) { delete static_cast<Nlcg*>(g); }
void orc_nlcg_set_params(void* g, const double* params) { nlcg_set(*static_cast<Nlcg*>(g), params); }
void orc_nlcg_get_state(void* g, double* out) { nlcg_get_state(*static_cast<Nlcg*>(g), out); }
void orc_nlcg_set_state(void* g, const double* in) { nlcg_set_state(*static_cast<Nlcg*>(g), in); }
void orc_nlcg_set_forces(void* g, void* s, int constraints_and_a) {
    static_cast<Nlcg*>(g)->set_forces(*static_cast<System*>(s), constraints_and_a != 0, true);
}
void orc_nlcg_reset(void* g, void* s) { static_cast<Nlcg*>(g)->reset(*static_cast<System*>(s)); }
void orc_nlcg_descend(void* g, void* s) { static_cast<Nlcg*>(g)->descend(*static_cast<System*>(s)); }
void orc_nlcg_timestep(void* g, void* s, uint32_t nsteps) {
    for (uint32_t q = 0; q < nsteps; q++) static_cast<Nlcg*>(g)->timestep(*static_cast<System*>(s));
}
void orc_get_box(void* s, double* L) {
    System* S = static_cast<System*>(s);
    for (int d = 0; d < S->nd; d++) L[d] = S->L[d];
}

void orc_normals6(uint64_t seed, uint64_t step, uint32_t atom, double* out) {
    normals6(seed, step, atom, out);
}

// raw Philox4x32-10 on rows (c0, c1, c2, c3, k0, k1) -> 4 words each
void orc_philox(const uint32_t* in, uint32_t* out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) {
        uint32_t c[4] = {in[6 * i], in[6 * i + 1], in[6 * i + 2], in[6 * i + 3]};
        philox10(c, in[6 * i + 4], in[6 * i + 5]);
        for (int q = 0; q < 4; q++) out[4 * i + q] = c[q];
    }
}

// AtomGroup::kinetic_energy(originvelocity) (box.cpp:401-411)
double orc_kinetic_energy(void* s, const double* origin) {
    System* S = static_cast<System*>(s);
    double totE = 0;
    for (uint32_t i = 0; i < S->n; i++) {
        double mm = S->m[i];
        if (mm == 0 || std::isinf(mm)) continue;
        double cv[3] = {0, 0, 0};
        for (int d = 0; d < S->nd; d++) cv[d] = S->v[i * S->nd + d] - (origin ? origin[d] : 0.0);
        totE += mm / 2 * dotv(cv, cv, S->nd);
    }
    return totE;
}

// AtomGroup::momentum (box.cpp:249-258) and mass (237-245)
double orc_momentum(void* s, double* out) {
    System* S = static_cast<System*>(s);
    double tot[3] = {0, 0, 0};
    double mass = 0;
    for (uint32_t i = 0; i < S->n; i++) {
        double mm = S->m[i];
        if (mm <= 0 || std::isinf(mm)) continue;
        for (int d = 0; d < S->nd; d++) tot[d] += S->v[i * S->nd + d] * mm;
        mass += mm;
    }
    for (int d = 0; d < S->nd; d++) out[d] = tot[d];
    return mass;
}

// A cell-list construction of the same pair set as update_list(true), for
// sizes where the reference's O(N^2) loop is too slow to use as a checker.
// Output order matches curpairs: i ascending over members, j ascending < i.
// Returns the number of pairs written (or required, when cap is too small).
uint64_t orc_pairs_celllist(void* s, uint32_t* out, uint64_t cap) {
    System* S = static_cast<System*>(s);
    const int nd = S->nd;
    const size_t M = S->members.size();
    double dmax = 0;
    for (double d : S->diameters) dmax = std::max(dmax, d);
    const double rl = dmax + S->skin;
    int nc[3] = {1, 1, 1};
    for (int d = 0; d < nd; d++) {
        int c = (int)std::floor(S->L[d] / rl);
        nc[d] = c >= 3 ? c : 1;
    }
    size_t ncell = (size_t)nc[0] * nc[1] * nc[2];
    std::vector<std::vector<uint32_t>> cells(ncell);
    std::vector<int> cellof(M * 3);
    for (size_t k = 0; k < M; k++) {
        const double* xi = &S->x[S->members[k] * nd];
        int ci[3] = {0, 0, 0};
        for (int d = 0; d < nd; d++) {
            double w = xi[d] - std::floor(xi[d] / S->L[d]) * S->L[d];
            int c = (int)std::floor(w / S->L[d] * nc[d]);
            if (c < 0) c = 0;
            if (c >= nc[d]) c = nc[d] - 1;
            ci[d] = c;
            cellof[k * 3 + d] = c;
        }
        cells[(size_t)(ci[2] * nc[1] + ci[1]) * nc[0] + ci[0]].push_back((uint32_t)k);
    }
    uint64_t cnt = 0;
    std::vector<uint32_t> nb;
    for (size_t i = 0; i < M; i++) {
        nb.clear();
        int r[3] = {nc[0] >= 3 ? 1 : 0, nc[1] >= 3 ? 1 : 0, (nd == 3 && nc[2] >= 3) ? 1 : 0};
        for (int dz = -r[2]; dz <= r[2]; dz++)
            for (int dy = -r[1]; dy <= r[1]; dy++)
                for (int dx = -r[0]; dx <= r[0]; dx++) {
                    int c0 = (cellof[i * 3] + dx + nc[0]) % nc[0];
                    int c1 = (cellof[i * 3 + 1] + dy + nc[1]) % nc[1];
                    int c2 = (cellof[i * 3 + 2] + dz + nc[2]) % nc[2];
                    for (uint32_t j : cells[(size_t)(c2 * nc[1] + c1) * nc[0] + c0])
                        if (j < i) nb.push_back(j);
                }
        std::sort(nb.begin(), nb.end());
        uint32_t ai = S->members[i];
        for (uint32_t j : nb) {
            uint32_t aj = S->members[j];
            if (S->is_ignored(ai, aj)) continue;
            double diam = (S->diameters[i] + S->diameters[j]) / 2;
            double rr[3];
            S->diff(&S->x[ai * nd], &S->x[aj * nd], rr);
            if (std::sqrt(dotv(rr, rr, nd)) < (diam + S->skin)) {
                if (cnt < cap) {
                    out[2 * cnt] = ai;
                    out[2 * cnt + 1] = aj;
                }
                cnt++;
            }
        }
    }
    return cnt;
}

// Install a pair list directly (used with orc_pairs_celllist for large N):
// equivalent to the state after update_list(true) at the current positions.
void orc_nl_install(void* s, const uint32_t* pairs, uint64_t npairs) {
    System* S = static_cast<System*>(s);
    S->curpairs.resize(npairs);
    for (uint64_t k = 0; k < npairs; k++) S->curpairs[k] = {pairs[2 * k], pairs[2 * k + 1]};
    for (size_t k = 0; k < S->members.size(); k++)
        for (int d = 0; d < S->nd; d++) S->lastlocs[k * S->nd + d] = S->x[S->members[k] * S->nd + d];
    S->updatenum++;
    S->ignorechanged = false;
}

}  // extern "C"
