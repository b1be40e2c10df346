// FP64 pair forces, energies, virials and stresses — the drop-in path whose
// results match the reference CPU code bit for bit.
//
// Reference (wackywendell/parm src/interaction.hpp):
//   NListed<A,P>::set_forces               2165-2175  f_first += F, f_last -= F
//   NListed<A,P>::energy / pressure / stress 2152-2163, 2247-2291
//   LennardJonesCut + LennardJonesCutPair   238-281, 967-987
//   RepulsionPair                           1528-1590
//   LJRepulsive + LJRepulsePair             119-152, 875-891
//   LJAttractCut + LJAttractCutPair         154-236, 1020-1050
//   LoisOhernPair, LoisOhernPairMinCLs      1679-1751
//   LoisLinPair, LoisLinPairMin             1764-1836
//   EisMclachlanPair                        1415-1452
//   RepulsionDragPair                       1598-1640
//   LJAttractRepulseSigsPair                1149-1239
//   indexed epsilons: LennardJonesCutPair / LJAttractCutPair on IEps*Atoms
//   977-982, 1028-1037; LJAttractRepulsePair 1251-1298; LJishPair 1095-1141;
//   LJAttractFixedRepulsePair 1343-1399
//
// Summation order: the reference visits pairs (i, j<i) in ascending (i, j) and
// scatters +F to i and -F to j.  For atom k this is: neighbours j<k in
// ascending j (adding F(k,j)), then neighbours i>k in ascending i
// (subtracting F(i,k)).  Because the minimum image is an exact odd function
// and every pair law scales the displacement by a function of |r|^2,
// -F(i,k) == F(k,i) bit for bit, so gathering F(k, j) over the rank-sorted
// full list reproduces the reference sums exactly.  Pairs beyond the cut-off
// (the reference adds Vec::Zero()) are skipped after an FP32 screen.
//
// Compiled with -fmad=false.
#include "parm_check.cuh"

namespace parm {

__device__ __forceinline__ bool mobile64(double m) { return !(m <= 0.0 || isinf(m)); }

struct PairC {
    double eps, sig, third, m6;   // the Lois kinds: third = C (or f), m6 = l; LJish: m6 = n
    double cut;                   // the Lois kinds: sigcut; LJAttractRepulse, LJAttractFixedRepulse,
                                  // LJish: the cut energy
    double rep;                   // LJAttractFixedRepulse, LJish: the repulsive epsilon;
                                  // LJAttractRepulseSigs: the attractive one (eps_r in eps,
                                  // sig_a in m6)
};

// Pair constants of the indexed kinds, A the pair's first atom (the later one
// in the neighbour list: its row of the table is used, IEps*Atom::get_epsilon).
// Atom records: (repeps, sigma, sigcut, p3) with p3 = 1 - 1/sigcut^6
// (LennardJonesCut), LJAttract::energy(sigcut), 1 - sigcut^-6 (the attractive-
// repulsive pairs) or the exponent n (LJish).
template <int KIND>
__device__ __forceinline__ PairC combine_idx(const DevCtx& c, const AtomPrm& A, const AtomPrm& B, uint32_t ta,
                                             uint32_t tb, uint32_t uni) {
    PairC p;
    const uint32_t n = c.ptab_n;
    const double te = c.ptab[(size_t)ta * n + tb];
    p.sig = (uni & IDX_SIG) ? c.ptab[(size_t)n * n + (size_t)ta * n + tb] : (A.p1 + B.p1) / 2.0;
    const bool b_larger = B.p2 > A.p2;
    p.third = b_larger ? B.p2 : A.p2;            // max(a1.sigcut, a2.sigcut)
    const double pc3 = b_larger ? B.p3 : A.p3;   // its per-atom cut term
    p.rep = sqrt(A.p0 * B.p0);
    p.cut = 0.0;
    p.m6 = pc3;
    p.eps = te;
    if constexpr (KIND == KIND_REPULSION_IDX) {
        // RepulsionPair(IEpsISigExpAtom...) (interaction.hpp:1538-1543): the exponent averaged
        p.third = (A.p2 + B.p2) / 2.0;
        p.m6 = 0.0;
    } else if constexpr (KIND == KIND_LJATTRACTREPULSE) {
        if (te <= 0) {
            p.third = 1;
            p.eps = fabs(te);
        } else {
            p.cut = te * (pc3 * pc3);
        }
    } else if constexpr (KIND == KIND_LJFIXEDREPULSE) {
        p.eps = fabs(te);
        if (!(te > 0) || p.eps == 0) {
            p.third = 1;
            p.eps = 0;
        } else {
            p.cut = p.eps * (pc3 * pc3);
        }
    } else if constexpr (KIND == KIND_LJISH) {
        p.m6 = (A.p3 + B.p3) / 2;
        if (te <= 0) {
            p.third = 1;
            p.eps = 0;
        } else {
            const double mid = (1 - pow(p.third, -p.m6));
            p.cut = te * (mid * mid);
        }
    }
    return p;
}

// LJAttractRepulseSigsPair::attract_energy / repulse_energy (interaction.hpp:1192-1202)
__device__ __forceinline__ double sigs_attract(const PairC& p, double r) {
    double r_over_sig = (r - p.sig + p.m6) / p.m6;
    double mid = (1 - pow(r_over_sig, -6.0));
    return p.rep * (mid * mid) - p.rep;
}
__device__ __forceinline__ double sigs_repulse(const PairC& p, double r) {
    double r_over_sig = r / p.sig;
    double mid = (1 - pow(r_over_sig, -6.0));
    return p.eps * (mid * mid) - p.rep;
}

template <int KIND>
__device__ __forceinline__ PairC combine(const AtomPrm& A, const AtomPrm& B, uint32_t uni) {
    PairC p;
    // eps = sqrt(e1*e2) (sqrt(e*e) == e exactly, so uniform epsilon skips it)
    p.eps = (uni & UNI_EPS) ? A.p0 : sqrt(A.p0 * B.p0);
    p.sig = (uni & UNI_SIG) ? A.p1 : (A.p1 + B.p1) / 2;
    if constexpr (cut_kind<KIND>()) {
        // cut = max(a1.sigcut, a2.sigcut); its cut-energy term travels with it
        bool b_larger = B.p2 > A.p2;
        p.third = b_larger ? B.p2 : A.p2;
        p.m6 = b_larger ? B.p3 : A.p3;
    } else if constexpr (KIND == KIND_REPULSION) {
        p.third = (uni & UNI_THIRD) ? A.p2 : (A.p2 + B.p2) / 2.0;
        p.m6 = 0.0;
    } else if constexpr (KIND == KIND_REPULSIONDRAG) {
        // RepulsionDragPair(a1, a2) (interaction.hpp:1613-1621): exponent and gamma averaged
        p.third = (uni & UNI_THIRD) ? A.p2 : (A.p2 + B.p2) / 2.0;
        p.m6 = (uni & UNI_FOURTH) ? A.p3 : (A.p3 + B.p3) / 2;
    } else if constexpr (lois_kind<KIND>()) {
        // LoisOhernPair (interaction.hpp:1693-1703) / LoisLinPair (1782-1800): averages;
        // LoisOhernPairMinCLs (1746-1751) / LoisLinPairMin (1831-1836): the smaller values
        if (uni & COMB_MIN) {
            p.third = A.p2 < B.p2 ? A.p2 : B.p2;
            p.m6 = A.p3 < B.p3 ? A.p3 : B.p3;
        } else {
            p.third = (uni & UNI_THIRD) ? A.p2 : (A.p2 + B.p2) / 2.0;
            p.m6 = (uni & UNI_FOURTH) ? A.p3 : (A.p3 + B.p3) / 2.0;
        }
        // sigcut: sig * (1 + C + l) (LoisOhern), sig + l (LoisLin)
        p.cut = (KIND == KIND_LOISOHERN) ? p.sig * (1 + p.third + p.m6) : p.sig + p.m6;
        return p;
    } else if constexpr (KIND == KIND_LJATTREPSIGS) {
        // LJAttractRepulseSigsPair(a1, a2) (interaction.hpp:1171-1190), atoms (eps_r, eps_a,
        // sig_r, sig_a, sigcut): eps = eps_r, rep = eps_a, sig = sig_r, m6 = sig_a, third =
        // sigcut (max), cut = the cut energy
        p.eps = sqrt(A.p0 * B.p0);
        p.rep = sqrt(A.p1 * B.p1);
        p.sig = (A.p2 + B.p2) / 2.0;
        p.m6 = (A.p3 + B.p3) / 2.0;
        p.third = B.p4 > A.p4 ? B.p4 : A.p4;
        const double cu = p.sig + p.m6 * (p.third - 1);
        p.cut = (p.third >= 1) ? sigs_attract(p, cu) : sigs_repulse(p, cu);
        return p;
    } else if constexpr (KIND == KIND_EISMCLACHLAN) {
        // EisMclachlanPair(a1, a2) (interaction.hpp:1425-1438), atoms (dist, sigmai) =
        // (p0, p1): E = c0/R + c1 + c2 R with c0, c1, c2 in eps, sig, third; cut-off d1 + d2
        p.eps = -M_PI * (A.p1 * B.p0 - B.p1 * A.p0) * (A.p0 * A.p0 - B.p0 * B.p0);
        p.sig = -2 * M_PI * (A.p1 * B.p0 * B.p0 + B.p1 * A.p0 * A.p0);
        p.third = M_PI * (A.p1 * B.p0 + B.p1 * A.p0);
        p.m6 = 0.0;
        p.cut = A.p0 + B.p0;
        return p;
    } else {
        p.third = 0.0;
        p.m6 = 0.0;
    }
    p.cut = 0.0;
    return p;
}

// pair force scale s (F = r * s); returns false beyond the cut-off
template <int KIND>
__device__ __forceinline__ bool force_scale(const PairC& p, double dsq, uint32_t uni, double& s) {
    if constexpr (KIND == KIND_LJATTREPSIGS) {
        // LJAttractRepulseSigsPair::forces (interaction.hpp:1218-1238)
        double cu = p.sig + p.m6 * (p.third - 1);
        if (p.third > 0 && dsq > cu * cu) return false;
        if (dsq > p.sig * p.sig) {
            double dist = sqrt(dsq);
            double rminus = dist - p.sig + p.m6;
            double r_over_sig = rminus / p.m6;
            double rsix = pow(r_over_sig, -6.0);
            double fmag_over_r = 12 * rsix * (rsix - 1) / (dist * rminus);
            s = p.rep * fmag_over_r;
        } else {
            double r_over_sigsq = dsq / (p.sig * p.sig);
            double rsix = pow(r_over_sigsq, -3.0);
            double fmagTimesR = 12 * rsix * (rsix - 1);
            s = p.eps * fmagTimesR / dsq;
        }
        return true;
    } else if constexpr (KIND == KIND_LJATTRACTREPULSE) {
        // LJAttractRepulsePair::forces (interaction.hpp:1287-1297)
        if (p.eps == 0) return false;
        double rsq = dsq / (p.sig * p.sig);
        if (rsq > (p.third * p.third)) return false;
        double rsix = pow(rsq, -3.0);
        double fmagTimesR = 12 * p.eps * rsix * (rsix - 1);
        s = fmagTimesR / dsq;
        return true;
    } else if constexpr (KIND == KIND_LJFIXEDREPULSE || KIND == KIND_LJISH) {
        // LJAttractFixedRepulsePair::forces (1390-1398), LJishPair::forces (1130-1140)
        double rsq = dsq / (p.sig * p.sig);
        if (rsq > (p.third * p.third)) return false;
        double fmagTimesR;
        if constexpr (KIND == KIND_LJFIXEDREPULSE) {
            double rsix = pow(rsq, -3.0);
            fmagTimesR = 12 * rsix * (rsix - 1);
        } else {
            double n = p.m6;
            double rmid = pow(rsq, -n / 2);
            fmagTimesR = 2 * n * rmid * (rmid - 1);
        }
        s = (rsq < 1) ? p.rep * fmagTimesR / dsq : p.eps * fmagTimesR / dsq;
        return true;
    } else if constexpr (KIND == KIND_LJCUT || KIND == KIND_LJCUT_IDX) {
        double rsq = (uni & UNI_SIG_ONE) ? dsq : dsq / (p.sig * p.sig);
        if (rsq > (p.third * p.third)) return false;
        double rsix = rsq * rsq * rsq;
        double fmagTimesR = 12 * p.eps / rsix * (1 / rsix - 1);
        s = fmagTimesR / dsq;
        return true;
    } else if constexpr (KIND == KIND_REPULSION || KIND == KIND_REPULSION_IDX) {
        if (dsq > p.sig * p.sig) return false;
        double R = sqrt(dsq);
        double b = 1.0 - (R / p.sig);
        double pw = (p.third == 2.0) ? b : pow(b, p.third - 1);   // pow(b, 1) == b exactly
        s = p.eps * pw / p.sig / R;
        return true;
    } else if constexpr (KIND == KIND_LJATTRACT || KIND == KIND_LJATTRACT_IDX) {
        // LJAttractCut::forces (interaction.hpp:219-229)
        if (p.eps == 0) return false;
        double rsq = (uni & UNI_SIG_ONE) ? dsq : dsq / (p.sig * p.sig);
        if (rsq < 1 || rsq > (p.third * p.third)) return false;
        double rsix = rsq * rsq * rsq;
        double fmagTimesR = 12 * p.eps / rsix * (1 / rsix - 1);
        s = fmagTimesR / dsq;
        return true;
    } else if constexpr (KIND == KIND_LOISOHERN) {
        // LoisOhernPair::forces (interaction.hpp:1729-1743): harmonic to (1 + C) sigma,
        // then a linear return to zero at sigcut
        const double C = p.third, l = p.m6;
        if (dsq >= p.cut * p.cut) return false;
        double R = sqrt(dsq);
        double rsig = R / p.sig;
        if (rsig <= 1 + C) {
            double dR = rsig - 1;
            s = -p.eps * dR / R;
        } else {
            double dR2 = rsig - (C + l + 1);
            s = C * p.eps / l * dR2 / R;
        }
        return true;
    } else if constexpr (KIND == KIND_EISMCLACHLAN) {
        // EisMclachlanPair::forces (interaction.hpp:1445-1451)
        if (dsq > (p.cut * p.cut)) return false;
        double R = sqrt(dsq);
        s = (p.eps / dsq - p.third) / R;
        return true;
    } else if constexpr (KIND == KIND_LOISLIN) {
        // LoisLinPair::forces (interaction.hpp:1817-1828); -rij * (f / R) == rij * -(f / R)
        if (dsq >= p.cut * p.cut) return false;
        double R = sqrt(dsq);
        if (R <= p.sig) {
            double dR = 1.0 - (R / p.sig);
            s = p.eps * dR / p.sig / R;
        } else {
            s = -(p.third / R);
        }
        return true;
    } else {
        double rsq = (uni & UNI_SIG_ONE) ? dsq : dsq / (p.sig * p.sig);
        if (rsq > 1) return false;
        double rsix = rsq * rsq * rsq;
        double fmagTimesR = 12 * p.eps / rsix * (1 / rsix - 1);
        s = fmagTimesR / dsq;
        return true;
    }
}

template <int KIND>
__device__ __forceinline__ double pair_energy(const PairC& p, double dsq, uint32_t uni) {
    if constexpr (KIND == KIND_LJATTREPSIGS) {
        // LJAttractRepulseSigsPair::energy (interaction.hpp:1204-1216)
        double dist = sqrt(dsq);
        double cu = p.sig + p.m6 * (p.third - 1);
        if (p.third > 0 && dist > cu) return 0.0;
        if (dist <= p.sig) return sigs_repulse(p, dist) - p.cut;
        return sigs_attract(p, dist) - p.cut;
    } else if constexpr (KIND == KIND_LJATTRACTREPULSE || KIND == KIND_LJFIXEDREPULSE || KIND == KIND_LJISH) {
        // LJAttractRepulsePair::energy (1269-1286), LJAttractFixedRepulsePair::energy (1366-1389),
        // LJishPair::energy (1115-1129)
        double rsq = dsq / (p.sig * p.sig);
        if (rsq > p.third * p.third) return 0.0;
        double mid = (KIND == KIND_LJISH) ? (1 - pow(rsq, -p.m6 / 2)) : (1 - pow(rsq, -3.0));
        if constexpr (KIND == KIND_LJATTRACTREPULSE) return p.eps * (mid * mid) - p.cut;
        if (rsq > 1) return p.eps * (mid * mid) - p.cut;
        return p.rep * (mid * mid) - p.cut;
    } else if constexpr (KIND == KIND_LJCUT || KIND == KIND_LJCUT_IDX) {
        double rsq = (uni & UNI_SIG_ONE) ? dsq : dsq / (p.sig * p.sig);
        if (rsq > (p.third * p.third)) return 0.0;
        double rsix = rsq * rsq * rsq;
        double mid = (1 - 1 / rsix);
        double cut_energy = p.eps * (p.m6 * p.m6 - 1);
        return p.eps * (mid * mid - 1) - cut_energy;
    } else if constexpr (KIND == KIND_REPULSION || KIND == KIND_REPULSIONDRAG || KIND == KIND_REPULSION_IDX) {
        // RepulsionPair::energy (1544-1550), RepulsionDragPair::energy (1622-1628)
        if (dsq > p.sig * p.sig) return 0.0;
        double R = sqrt(dsq);
        double b = 1.0 - (R / p.sig);
        double pw = (p.third == 2.0) ? b * b : pow(b, p.third);   // pow(b, 2) == b*b exactly
        return p.eps * pw / p.third;
    } else if constexpr (KIND == KIND_LJATTRACT || KIND == KIND_LJATTRACT_IDX) {
        // LJAttractCut::energy (interaction.hpp:211-216) with LJAttract::energy (162-169)
        if (p.eps == 0) return 0.0;
        if (dsq > (p.third * p.third * p.sig * p.sig)) return 0.0;
        double rsq = dsq / (p.sig * p.sig);
        double e;
        if (rsq < 1) {
            e = -p.eps;
        } else {
            double rsix = rsq * rsq * rsq;
            double mid = (1 - 1 / rsix);
            e = p.eps * (mid * mid - 1);
        }
        return e - p.m6 * p.eps;
    } else if constexpr (KIND == KIND_LOISOHERN) {
        // LoisOhernPair::energy (interaction.hpp:1713-1727)
        const double C = p.third, l = p.m6;
        if (dsq >= p.cut * p.cut) return 0.0;
        double R = sqrt(dsq) / p.sig;
        if (R <= 1 + C) {
            double dR = R - 1;
            return -p.eps * p.sig / 2 * (C * (C + l) - dR * dR);
        }
        double dR2 = C + l + 1 - R;
        return -C * p.eps * p.sig / 2 / l * dR2 * dR2;
    } else if constexpr (KIND == KIND_EISMCLACHLAN) {
        // EisMclachlanPair::energy (interaction.hpp:1439-1444)
        double R = sqrt(dsq);
        if (R > p.cut) return 0.0;
        return p.eps / R + p.sig + p.third * R;
    } else if constexpr (KIND == KIND_LOISLIN) {
        // LoisLinPair::energy (interaction.hpp:1802-1815)
        const double f = p.third, l = p.m6;
        if (dsq >= p.cut * p.cut) return 0.0;
        double R = sqrt(dsq);
        if (R <= p.sig) {
            double dR = 1.0 - (R / p.sig);
            return p.eps / 2 * dR * dR - f * l;
        }
        return -f * (p.sig + l - R);
    } else {
        double rsq = (uni & UNI_SIG_ONE) ? dsq : dsq / (p.sig * p.sig);
        if (rsq > 1) return 0.0;
        double rsix = rsq * rsq * rsq;
        double mid = (1 - 1 / rsix);
        return p.eps * (mid * mid);
    }
}

// RepulsionDragPair::forces (interaction.hpp:1629-1639): the soft repulsion
// minus gamma times the relative velocity's component along r; false beyond
// the cut-off.  F(i, j) == -F(j, i) bit for bit (r and v_i - v_j both flip).
template <int ND>
__device__ __forceinline__ bool drag_force(const PairC& p, const double* r, double dsq, const double* vi,
                                           const double* vj, double* fo) {
    if (dsq > p.sig * p.sig) return false;
    double R = sqrt(dsq);
    double vij[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < ND; d++) vij[d] = vi[d] - vj[d];
    double vdot = vij[0] * r[0] + vij[1] * r[1];
    if constexpr (ND == 3) vdot = vdot + vij[2] * r[2];
    double b = 1.0 - (R / p.sig);
    double pw = (p.third == 2.0) ? b : pow(b, p.third - 1);   // pow(b, 1) == b exactly
    double sr = p.eps * pw / p.sig / R;
#pragma unroll
    for (int d = 0; d < ND; d++) {
        double vperp = r[d] * vdot / dsq;
        fo[d] = r[d] * sr - vperp * p.m6;
    }
    return true;
}

// FP32 screen: true when the pair is certainly beyond the cut-off
// (Q = (sqrt(eps), sigma, third, fourth) in FP32)
template <int KIND>
__device__ __forceinline__ bool beyond32(float d2, const float4& Qi, const float4& Qj, uint32_t uni) {
    if constexpr (idx_kind<KIND>() || KIND == KIND_LJATTREPSIGS) return false;   // every pair takes the exact test
    float sg = (uni & UNI_SIG) ? Qi.y : 0.5f * (Qi.y + Qj.y);
    float rc;
    if constexpr (cut_kind<KIND>()) {
        rc = sg * fmaxf(Qi.z, Qj.z);
    } else if constexpr (lois_kind<KIND>()) {
        const bool mn = uni & COMB_MIN;
        const float th = mn ? fminf(Qi.z, Qj.z) : 0.5f * (Qi.z + Qj.z);
        const float l = mn ? fminf(Qi.w, Qj.w) : 0.5f * (Qi.w + Qj.w);
        rc = (KIND == KIND_LOISOHERN) ? sg * (1.0f + th + l) : sg + l;
    } else if constexpr (KIND == KIND_EISMCLACHLAN) {
        rc = Qi.x + Qj.x;   // dist_i + dist_j
    } else {
        rc = sg;
    }
    return d2 > rc * rc * 1.0002f;
}

template <int ND>
__device__ __forceinline__ void load3(const void* p, uint32_t i, double* o) {
    using V = typename DVec<ND>::T;
    V t = static_cast<const V*>(p)[i];
    const double* q = reinterpret_cast<const double*>(&t);
#pragma unroll
    for (int d = 0; d < ND; d++) o[d] = q[d];
}

template <int ND>
__device__ __forceinline__ void store3(void* p, uint32_t i, const double* o) {
    using V = typename DVec<ND>::T;
    V t;
    double* q = reinterpret_cast<double*>(&t);
#pragma unroll
    for (int d = 0; d < (int)(sizeof(V) / 8); d++) q[d] = d < ND ? o[d] : 0.0;
    static_cast<V*>(p)[i] = t;
}

template <int ND>
__device__ __forceinline__ float d2_32(const SysConst& S, const float4& Ai, const float4& Bi,
                                       const float4& Aj, const float4& Bj) {
    float dx = disp32(Ai.x, Aj.x, Bi.x, Bj.x, S.Lhi[0], S.Llo[0], S.invLf[0]);
    float dy = disp32(Ai.y, Aj.y, Bi.y, Bj.y, S.Lhi[1], S.Llo[1], S.invLf[1]);
    float d2 = dx * dx + dy * dy;
    if constexpr (ND == 3) {
        float dz = disp32(Ai.z, Aj.z, Bi.z, Bj.z, S.Lhi[2], S.Llo[2], S.invLf[2]);
        d2 += dz * dz;
    }
    return d2;
}

template <int ND, int KIND, int MODE>
__global__ void __launch_bounds__(BLOCK) k_force64(DevCtx c) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < c.n && c.active[c.atom_sys[i]];
    const uint32_t uni = c.uniform;
    double f[3] = {0.0, 0.0, 0.0};
    uint32_t s = 0;
    bool member = false;
    if (active) {
        s = c.atom_sys[i];
        member = c.rank[i] != NOT_MEMBER;
    }
    if (member) {
        const SysConst& S = c.sys[s];
        double xi[3] = {0, 0, 0}, vi[3] = {0, 0, 0};
        load3<ND>(c.x, i, xi);
        if constexpr (KIND == KIND_REPULSIONDRAG) load3<ND>(c.v, i, vi);
        const float4 Ai = c.pos[2 * (size_t)(i)], Bi = c.pos[2 * (size_t)(i) + 1];
        const AtomPrm Pi = c.prm[i];
        const float4 Qi = c.prm32[i];
        const uint32_t nn = c.nnb[i];
        const uint32_t* nb = c.nbr + (size_t)i * c.maxnb;
        for (uint32_t k = 0; k < nn; k++) {
            const uint32_t j = __ldg(nb + k);
            float4 Aj, Bj;
            ld_pos(c.pos, j, Aj, Bj);
            float4 Qj = Qi;
            if ((uni & UNI_ALL) != UNI_ALL) Qj = c.prm32[j];
            // (the FP32 screen is per-axis periodic: not for a sheared box)
            if (!S.lees && beyond32<KIND>(d2_32<ND>(S, Ai, Bi, Aj, Bj), Qi, Qj, uni)) continue;
            double xj[3] = {0, 0, 0};
            load3<ND>(c.x, j, xj);
            double r[3] = {0, 0, 0};
            if (S.lees) {
                lees_diff<ND>(S, xi, xj, r);
            } else {
#pragma unroll
                for (int d = 0; d < ND; d++) r[d] = remainder_exact(xi[d] - xj[d], S.L[d], S.invL[d], S.halfL[d]);
            }
            double dsq = r[0] * r[0] + r[1] * r[1];
            if constexpr (ND == 3) dsq = dsq + r[2] * r[2];
            AtomPrm Pj = Pi;
            if ((uni & UNI_ALL) != UNI_ALL) Pj = c.prm[j];
            PairC pc;
            if constexpr (idx_kind<KIND>()) {
                // the pair's first atom is the one of higher neighbour-list rank
                const uint32_t ti = __float_as_uint(Qi.x), tj = __float_as_uint(Qj.x);
                pc = (c.rank[i] > c.rank[j]) ? combine_idx<KIND>(c, Pi, Pj, ti, tj, uni)
                                             : combine_idx<KIND>(c, Pj, Pi, tj, ti, uni);
            } else {
                pc = combine<KIND>(Pi, Pj, uni);
            }
            if constexpr (KIND == KIND_REPULSIONDRAG) {
                double vj[3] = {0, 0, 0}, fo[3];
                load3<ND>(c.v, j, vj);
                if (!drag_force<ND>(pc, r, dsq, vi, vj, fo)) continue;
#pragma unroll
                for (int d = 0; d < ND; d++) f[d] = f[d] + fo[d];
            } else {
                double sc;
                if (!force_scale<KIND>(pc, dsq, uni, sc)) continue;
#pragma unroll
                for (int d = 0; d < ND; d++) f[d] = f[d] + r[d] * sc;
            }
        }
    }
    if (active) {
        store3<ND>(c.f, i, f);
        if constexpr (MODE == FM_FORCES_A) {
            // Collection::set_forces(true): a = f/m, zero for m <= 0 or inf
            const double m = c.m[i];
            double a[3] = {0, 0, 0};
            if (mobile64(m)) {
#pragma unroll
                for (int d = 0; d < ND; d++) a[d] = f[d] / m;
            }
            store3<ND>(c.a, i, a);
        }
    }
}

// per-atom partial sums over the half list (neighbours of smaller rank), i.e.
// each reference pair (first = higher rank) exactly once
template <int ND, int KIND>
__global__ void __launch_bounds__(BLOCK) k_eval64(DevCtx c, int what) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const uint32_t uni = c.uniform;
    const int ncomp = (what == EV_STRESS) ? ND * ND : 1;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const uint32_t ri = c.rank[i];
    if (ri != NOT_MEMBER) {
        const uint32_t s = c.atom_sys[i];
        const SysConst& S = c.sys[s];
        double xi[3] = {0, 0, 0};
        load3<ND>(c.x, i, xi);
        const AtomPrm Pi = c.prm[i];
        const uint32_t nn = c.nnb[i];
        for (uint32_t k = 0; k < nn; k++) {
            const uint32_t j = c.nbr[(size_t)i * c.maxnb + k];
            if (c.rank[j] > ri) continue;
            double xj[3] = {0, 0, 0};
            load3<ND>(c.x, j, xj);
            double r[3] = {0, 0, 0};
            if (S.lees) {
                lees_diff<ND>(S, xi, xj, r);
            } else {
#pragma unroll
                for (int d = 0; d < ND; d++) r[d] = remainder_exact(xi[d] - xj[d], S.L[d], S.invL[d], S.halfL[d]);
            }
            double dsq = r[0] * r[0] + r[1] * r[1];
            if constexpr (ND == 3) dsq = dsq + r[2] * r[2];
            PairC pc;
            if constexpr (idx_kind<KIND>())   // i is the pair's first atom (higher rank)
                pc = combine_idx<KIND>(c, Pi, c.prm[j], __float_as_uint(c.prm32[i].x),
                                       __float_as_uint(c.prm32[j].x), uni);
            else
                pc = combine<KIND>(Pi, c.prm[j], uni);
            if (what == EV_ENERGY || what == EV_CONTACTS || what == EV_OVERLAPS) {
                double e = pair_energy<KIND>(pc, dsq, uni);
                if (what == EV_ENERGY) acc[0] = acc[0] + e;
                else if (what == EV_CONTACTS) acc[0] += (e != 0.0) ? 1.0 : 0.0;
                else acc[0] += (e > 0.0) ? 1.0 : 0.0;
            } else {
                double sc;
                double fo[3] = {0, 0, 0};
                if constexpr (KIND == KIND_REPULSIONDRAG) {
                    double vi[3] = {0, 0, 0}, vj[3] = {0, 0, 0};
                    load3<ND>(c.v, i, vi);
                    load3<ND>(c.v, j, vj);
                    if (!drag_force<ND>(pc, r, dsq, vi, vj, fo))
                        for (int d = 0; d < 3; d++) fo[d] = 0.0;
                } else if (force_scale<KIND>(pc, dsq, uni, sc)) {
#pragma unroll
                    for (int d = 0; d < ND; d++) fo[d] = r[d] * sc;
                }
                if (what == EV_VIRIAL) {
                    double p = r[0] * fo[0] + r[1] * fo[1];
                    if constexpr (ND == 3) p = p + r[2] * fo[2];
                    acc[0] = acc[0] + p;
                } else {
#pragma unroll
                    for (int aa = 0; aa < ND; aa++)
#pragma unroll
                        for (int bb = 0; bb < ND; bb++) acc[aa * ND + bb] = acc[aa * ND + bb] + r[aa] * fo[bb];
                }
            }
        }
    }
    for (int q = 0; q < ncomp; q++) c.red[(size_t)q * c.n + i] = acc[q];
}

template <int ND, int KIND>
static void force64_nd_kind(const DevCtx& c, cudaStream_t s, int mode) {
    unsigned g = grid_for(c.n);
    if (mode == FM_FORCES_A) k_force64<ND, KIND, FM_FORCES_A><<<g, BLOCK, 0, s>>>(c);
    else k_force64<ND, KIND, FM_FORCES><<<g, BLOCK, 0, s>>>(c);
}

template <int ND>
static void force64_nd(const DevCtx& c, cudaStream_t s, int mode) {
    if (c.kind == KIND_LJCUT) force64_nd_kind<ND, KIND_LJCUT>(c, s, mode);
    else if (c.kind == KIND_LJATTRACT) force64_nd_kind<ND, KIND_LJATTRACT>(c, s, mode);
    else if (c.kind == KIND_LOISOHERN) force64_nd_kind<ND, KIND_LOISOHERN>(c, s, mode);
    else if (c.kind == KIND_LOISLIN) force64_nd_kind<ND, KIND_LOISLIN>(c, s, mode);
    else if (c.kind == KIND_EISMCLACHLAN) force64_nd_kind<ND, KIND_EISMCLACHLAN>(c, s, mode);
    else if (c.kind == KIND_REPULSIONDRAG) force64_nd_kind<ND, KIND_REPULSIONDRAG>(c, s, mode);
    else if (c.kind == KIND_LJCUT_IDX) force64_nd_kind<ND, KIND_LJCUT_IDX>(c, s, mode);
    else if (c.kind == KIND_LJATTRACT_IDX) force64_nd_kind<ND, KIND_LJATTRACT_IDX>(c, s, mode);
    else if (c.kind == KIND_LJATTRACTREPULSE) force64_nd_kind<ND, KIND_LJATTRACTREPULSE>(c, s, mode);
    else if (c.kind == KIND_LJFIXEDREPULSE) force64_nd_kind<ND, KIND_LJFIXEDREPULSE>(c, s, mode);
    else if (c.kind == KIND_LJISH) force64_nd_kind<ND, KIND_LJISH>(c, s, mode);
    else if (c.kind == KIND_REPULSION_IDX) force64_nd_kind<ND, KIND_REPULSION_IDX>(c, s, mode);
    else if (c.kind == KIND_LJATTREPSIGS) force64_nd_kind<ND, KIND_LJATTREPSIGS>(c, s, mode);
    else if (c.kind == KIND_REPULSION) force64_nd_kind<ND, KIND_REPULSION>(c, s, mode);
    else force64_nd_kind<ND, KIND_LJREPULSE>(c, s, mode);
}

void launch_force64(const DevCtx& c, cudaStream_t s, int mode) {
    if (c.nd == 3) force64_nd<3>(c, s, mode); else force64_nd<2>(c, s, mode);
}

template <int ND>
static void eval64_nd(const DevCtx& c, cudaStream_t s, int what) {
    unsigned g = grid_for(c.n);
    if (c.kind == KIND_LJCUT) k_eval64<ND, KIND_LJCUT><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_LJATTRACT) k_eval64<ND, KIND_LJATTRACT><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_LOISOHERN) k_eval64<ND, KIND_LOISOHERN><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_LOISLIN) k_eval64<ND, KIND_LOISLIN><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_EISMCLACHLAN) k_eval64<ND, KIND_EISMCLACHLAN><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_REPULSIONDRAG) k_eval64<ND, KIND_REPULSIONDRAG><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_LJCUT_IDX) k_eval64<ND, KIND_LJCUT_IDX><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_LJATTRACT_IDX) k_eval64<ND, KIND_LJATTRACT_IDX><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_LJATTRACTREPULSE) k_eval64<ND, KIND_LJATTRACTREPULSE><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_LJFIXEDREPULSE) k_eval64<ND, KIND_LJFIXEDREPULSE><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_LJISH) k_eval64<ND, KIND_LJISH><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_REPULSION_IDX) k_eval64<ND, KIND_REPULSION_IDX><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_LJATTREPSIGS) k_eval64<ND, KIND_LJATTREPSIGS><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_REPULSION) k_eval64<ND, KIND_REPULSION><<<g, BLOCK, 0, s>>>(c, what);
    else k_eval64<ND, KIND_LJREPULSE><<<g, BLOCK, 0, s>>>(c, what);
}

void launch_eval64(const DevCtx& c, cudaStream_t s, int what) {
    if (c.nd == 3) eval64_nd<3>(c, s, what); else eval64_nd<2>(c, s, what);
}

}  // namespace parm
