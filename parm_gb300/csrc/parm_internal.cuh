// Internal definitions shared by the parm_gb300 CUDA translation units.
//
// Device data layout (one context = a batch of `nsys` independent periodic
// systems; a single simulation is nsys == 1):
//   * atoms of all systems are concatenated; system s owns the contiguous
//     range [atom_off[s], atom_off[s] + natoms[s]).
//   * inside a system the atoms are kept in "cell order": at every
//     neighbour-list rebuild they are counting-sorted by cell and, inside a
//     cell, by their original index.  `orig[k]` maps the internal slot k back
//     to the caller's atom index; `slot[orig]` is the inverse.
//   * positions, velocities, accelerations, forces and the last-build
//     positions are FP64 vectors stored as double4 (3D) / double2 (2D), so a
//     neighbour gather is one aligned 32-byte sector.
//   * `posq` is the FP32 view of the positions used by the mixed-precision
//     pair kernel and by the FP32 pre-filters of the FP64 path: a coarse part
//     X = trunc(x * 8) / 8 (exact in FP32) and a fine part xf = x - X.
//   * the neighbour list is a full list stored row-major:
//     nbr[i * maxnb + k] is the k-th neighbour of internal atom i.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace parm {

enum PairKind : int {
    KIND_LJCUT = 0, KIND_REPULSION = 1, KIND_LJREPULSE = 2, KIND_LJATTRACT = 3,
    // four-parameter atoms (eps, sigma, C, l) / (eps, sigma, f, l); FP64 path only
    KIND_LOISOHERN = 4, KIND_LOISLIN = 5,
    // (dist, sigmai) atoms, E = c0/R + c1 + c2 R; FP64 path only
    KIND_EISMCLACHLAN = 6,
    // (eps, sigma, exponent, gamma) atoms: soft repulsion with a drag on the
    // relative normal velocity; FP64 path only
    KIND_REPULSIONDRAG = 7,
    // indexed pair epsilons (IEps* atoms; FP64 path only): the pair's epsilon
    // (and sigma, flag IDX_SIG) from a table by the two atoms' types
    KIND_LJCUT_IDX = 8,          // LennardJonesCutPair(IEpsISigCutAtom)
    KIND_LJATTRACT_IDX = 9,      // LJAttractCutPair(IEpsISigCutAtom / IEpsSigCutAtom)
    KIND_LJATTRACTREPULSE = 10,  // LJAttractRepulsePair(IEpsSigCutAtom)
    KIND_LJFIXEDREPULSE = 11,    // LJAttractFixedRepulsePair(IEpsRepsSigCutAtom)
    KIND_LJISH = 12,             // LJishPair(IEpsRepsSigExpCutAtom)
    KIND_REPULSION_IDX = 13,     // RepulsionPair(IEpsISigExpAtom)
    // (eps_r, eps_a, sig_r, sig_a, sigcut) atoms; FP64 path only
    KIND_LJATTREPSIGS = 14       // LJAttractRepulseSigsPair(EpsEpsSigSigCutAtom)
};
template <int KIND>
__host__ __device__ constexpr bool idx_kind() { return KIND >= KIND_LJCUT_IDX && KIND <= KIND_REPULSION_IDX; }
template <int KIND>
__host__ __device__ constexpr bool lois_kind() { return KIND == KIND_LOISOHERN || KIND == KIND_LOISLIN; }
// kinds whose pair cut-off is max(sigcut_i, sigcut_j) sigma_ij, with a force
// that jumps there (LJ truncated without shift)
template <int KIND>
__host__ __device__ constexpr bool cut_kind() { return KIND == KIND_LJCUT || KIND == KIND_LJATTRACT; }
enum Precision : int { PREC_FP64 = 0, PREC_MIXED = 1 };

// status bits (device word, read back by the host after synchronising calls)
enum StatusBits : uint32_t {
    ST_NBR_OVERFLOW = 1u << 0,   // an atom had more neighbours than the list capacity
    ST_NONFINITE = 1u << 1,      // a non-finite position was binned
    ST_CELL_RANGE = 1u << 2,     // a cell index fell outside its system's grid (bug guard)
    ST_SORT_CAP = 1u << 3,       // FP64 path: a neighbour list longer than the in-thread sort buffer
    ST_TILE_OVERFLOW = 1u << 4,  // a tile had more distinct neighbours than its capacity
    ST_IMAGE_RANGE = 1u << 5,    // an atom is more than 7 box lengths from its tile frame
    ST_STAGE_TIMEOUT = 1u << 6,  // a cell block's bulk copies did not complete within the wait limit
};

constexpr uint32_t NOT_MEMBER = 0xFFFFFFFFu;

struct SysConst {
    double L[3];
    double invL[3];
    double halfL[3];
    float Lhi[3], Llo[3], invLf[3];
    float L8[3], Lr8[3];   // L rounded to the 1/8 grid (exact in FP32) and L - L8
    double skin;
    double rlist_max;   // largest (d_i + d_j)/2 + skin
    double cellmin;     // narrowest allowed cell (the list radius times the cell scale, with a margin)
    double rec_lim2;    // (2 skin + 1/2)^2: displacement limit of the cell-block records
    int nc[3];          // cells per axis (1 or >= 3)
    float cellw_inv[3]; // nc / L
    double cellw[3];    // L / nc
    float cellw32[3];   // L / nc in FP32
    uint32_t cell_off;  // first cell of this system in the global cell array
    uint32_t ncell;
    uint32_t atom_off;
    uint32_t natoms;
    int lees;           // a LeesEdwardsBox (FP64 path): the y image shifts x by gamma Lx
    double gamma;
};

// per-atom FP64 parameters of the pair interaction (kind dependent)
//   LJCUT:     p0 = epsilon, p1 = sigma, p2 = sigcut, p3 = 1 - 1/pow(sigcut, 6)
//   LJATTRACT: p0 = epsilon, p1 = sigma, p2 = sigcut, p3 = LJAttract::energy(sigcut)
//   REPULSION: p0 = eps,     p1 = sigma, p2 = exponent
//   LJREPULSE: p0 = epsilon, p1 = sigma
struct AtomPrm {
    double p0, p1, p2, p3;
    double p4;   // the fifth parameter (LJAttractRepulseSigs' sigcut), else 0
};

// flags that let the FP64 kernel skip combinations that are exact identities
enum UniformFlags : uint32_t {
    UNI_EPS = 1u << 0,     // all members share epsilon -> eps_ij = eps (sqrt(e*e) == e)
    UNI_SIG = 1u << 1,     // all members share sigma   -> sig_ij = sig
    UNI_THIRD = 1u << 2,   // all members share sigcut / exponent
    UNI_SIG_ONE = 1u << 3, // sigma == 1 exactly -> dsq / (sig*sig) == dsq
    UNI_FOURTH = 1u << 4,  // all members share the fourth parameter (p3)
    UNI_ALL = UNI_EPS | UNI_SIG | UNI_THIRD | UNI_FOURTH,
    // not a uniformity flag: the Lois pairs combine C (or f) and l as the
    // smaller of the two atoms' values (LoisOhernPairMinCLs, LoisLinPairMin)
    // instead of their average
    COMB_MIN = 1u << 5,
    UNI_DIAM = 1u << 6,    // all members share their list diameter
    IDX_SIG = 1u << 7,     // indexed kinds: the pair sigma comes from the table too
};

template <int ND> struct DVec;
template <> struct DVec<3> { using T = double4; };
template <> struct DVec<2> { using T = double2; };

// ---------------------------------------------------------------------------
// Exact IEEE-754 remainder(d, L) (the reference's OriginBox::diff applies
// remainder() per component on unwrapped coordinates).  The common case is
// one multiply, one rint and one fma: when n is the true quotient the fma
// result d - n*L is exactly representable and therefore exact.  A wrong
// candidate quotient always leaves |r| >= L/2, so the rare branch tries the
// three candidates and, for a genuine tie, picks the even quotient.  Valid
// for |d / L| < 2^50 (the candidate quotient is then off by at most one).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double remainder_exact(double d, double L, double invL, double halfL) {
    double n = rint(d * invL);
    double r = fma(-n, L, d);
    if (fabs(r) >= halfL) {
        double best = r;
        bool found = false;
        double tie_n = n;
#pragma unroll
        for (int k = -1; k <= 1; k++) {
            double nk = n + (double)k;
            double rk = fma(-nk, L, d);
            if (fabs(rk) < halfL) {
                best = rk;
                found = true;
            } else if (fabs(rk) == halfL) {
                long long ni = (long long)nk;
                if ((ni & 1LL) == 0) tie_n = nk;
            }
        }
        if (!found) best = fma(-tie_n, L, d);
        r = best;
    }
    if (r == 0.0) r = copysign(0.0, d);
    return r;
}

// LeesEdwardsBox::diff (reference src/box.cpp:72-91) in its own arithmetic:
// the y image im = round(dy / Ly) shifts x by im * gamma * Lx, z takes the
// periodic remainder.  Used by the FP64 units only (compiled with
// -fmad=false, so no operation is contracted).  diff(b, a) == -diff(a, b)
// bit for bit (round is odd, and so is every operation on negated inputs).
template <int ND>
__device__ __forceinline__ void lees_diff(const SysConst& S, const double* a, const double* b, double* r) {
    const double Ly = S.L[1];
    double dy = a[1] - b[1];
    const int im = (int)round(dy / Ly);
    dy = dy - (im * Ly);
    const double Lx = S.L[0];
    double dx = a[0] - b[0];
    dx = dx - round((dx / Lx) - im * S.gamma) * Lx - im * S.gamma * Lx;
    r[0] = dx;
    r[1] = dy;
    if constexpr (ND == 3) r[2] = remainder_exact(a[2] - b[2], S.L[2], S.invL[2], S.halfL[2]);
}

// FP32 minimum-image displacement from the coarse/fine position split.
// Xd = Xi - Xj is exact (multiples of 1/8); c = Xd - n*Lhi is exact; the fine
// parts carry the remaining bits, so the result is within ~1 ulp of the
// correctly rounded FP64 displacement.  n = round(Xd / L) uses the 1.5*2^23
// shift (exact round-to-nearest for |Xd/L| < 2^22) instead of a rounding
// instruction, keeping the whole routine on the FMA pipe.
__device__ __forceinline__ float disp32(float Xi, float Xj, float fi, float fj, float Lhi, float Llo,
                                       float invL) {
    const float kShift = 12582912.0f;   // 1.5 * 2^23
    float Xd = Xi - Xj;
    float n = __fsub_rn(__fmaf_rn(Xd, invL, kShift), kShift);
    float c = __fmaf_rn(-n, Lhi, Xd);
    float fd = __fmaf_rn(-n, Llo, fi - fj);
    return c + fd;
}

// One neighbour's FP32 position record (coarse X, fine xf: 32 bytes, 32-byte
// aligned) in a single 256-bit read-only load, so a gather touches its sector
// once instead of twice.
__device__ __forceinline__ void ld_pos(const float4* pos, uint32_t j, float4& A, float4& B) {
    const float* q = reinterpret_cast<const float*>(pos) + 8 * (size_t)j;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(A.x), "=f"(A.y), "=f"(A.z), "=f"(A.w), "=f"(B.x), "=f"(B.y), "=f"(B.z), "=f"(B.w)
        : "l"(q));
}

}  // namespace parm
