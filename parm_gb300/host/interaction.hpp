// parm_gb300 host API: pair interactions with the interface of the
// reference's src/interaction.hpp (wackywendell/parm), evaluated on the GPU.
//
// NListed<A, P> is the reference's neighbour-listed pair interaction
// (src/interaction.hpp:1876-1945); the atom types carry the per-atom
// parameters and the pair types select the pair law:
//   NListed<EpsSigCutAtom, LennardJonesCutPair>  LJ cut at sigcut * sigma
//   NListed<EpsSigExpAtom, RepulsionPair>         soft repulsion, exponent n
//   NListed<EpsSigAtom,    LJRepulsePair>         WCA (repulsive LJ)
//   NListed<EpsSigCutAtom, LJAttractCutPair>     attractive LJ cut at sigcut * sigma
// Sums over the pair list (forces, energies, virials, stresses) run on the
// GPU.  A pair object (get_pair, pair_iter) also evaluates its own energy and
// force on the host, with the reference's formulas, for code that inspects
// single pairs.
#ifndef PARM_GB300_INTERACTION_HPP
#define PARM_GB300_INTERACTION_HPP

#include <algorithm>
#include <stdexcept>
#include <string>
#include <typeinfo>
#include <vector>

#include "trackers.hpp"

//! Interface of everything a Collection sums (src/interaction.hpp:59-104).
class Interaction {
   public:
    virtual flt energy(Box& box) = 0;
    virtual void set_forces(Box& box) = 0;
    virtual flt set_forces_get_pressure(Box& box) {
        throw std::runtime_error(std::string("set_forces_get_pressure not defined for class ") +
                                 typeid(*this).name());
    }
    virtual flt pressure(Box& box) = 0;
    virtual Matrix stress(Box& box) {
        throw std::runtime_error(std::string("stress not defined for class ") + typeid(*this).name());
    }
    virtual ~Interaction() {}
};

//! An interaction evaluated on the GPU: the handle behind it.  Collections
//! step the atoms of the GPU interaction they hold.
class GpuInteraction {
   public:
    virtual sptr<GpuLink> gpu() = 0;
    virtual ~GpuInteraction() {}
};

//! (epsilon, sigma) per atom (src/interaction.hpp:857-865).
struct EpsSigAtom : public AtomID {
    flt epsilon, sigma;
    EpsSigAtom() : epsilon(0), sigma(0) {}
    EpsSigAtom(AtomID a, flt epsilon, flt sigma) : AtomID(a), epsilon(epsilon), sigma(sigma) {}
    EpsSigAtom(AtomID a, EpsSigAtom other) : AtomID(a), epsilon(other.epsilon), sigma(other.sigma) {}
    flt max_size() { return sigma; }
};

//! (epsilon, sigma, cut-off in units of sigma) per atom (src/interaction.hpp:896-905).
struct EpsSigCutAtom : public EpsSigAtom {
    flt sigcut;
    EpsSigCutAtom() : sigcut(0) {}
    EpsSigCutAtom(AtomID a, flt epsilon, flt sigma, flt cut) : EpsSigAtom(a, epsilon, sigma), sigcut(cut) {}
    EpsSigCutAtom(AtomID a, EpsSigCutAtom other) : EpsSigAtom(a, other), sigcut(other.sigcut) {}
    flt max_size() { return sigma * sigcut; }
};

//! (epsilon, sigma, exponent) per atom (src/interaction.hpp:1512-1526).
struct EpsSigExpAtom : public AtomID {
    flt eps, sigma, exponent;
    EpsSigExpAtom() : eps(0), sigma(0), exponent(2) {}
    EpsSigExpAtom(AtomID a, flt eps, flt sigma, flt exponent = 2.0)
        : AtomID(a), eps(eps), sigma(sigma), exponent(exponent) {}
    EpsSigExpAtom(AtomID a, EpsSigExpAtom other)
        : AtomID(a), eps(other.eps), sigma(other.sigma), exponent(other.exponent) {}
    flt max_size() { return sigma; }
};

//! Indexed epsilons and sigmas (src/interaction.hpp:911-954): the pair's
//! values are a1.epsilons[a2.indx], a1.sigmas[a2.indx].
struct IEpsISigCutAtom : public AtomID {
    std::vector<flt> epsilons, sigmas;
    uint indx;
    flt sigcut;
    IEpsISigCutAtom() : indx(0), sigcut(0) {}
    IEpsISigCutAtom(AtomID a, std::vector<flt> epsilons, std::vector<flt> sigmas, uint indx, flt cut)
        : AtomID(a), epsilons(epsilons), sigmas(sigmas), indx(indx), sigcut(cut) {}
    IEpsISigCutAtom(AtomID a, IEpsISigCutAtom other)
        : AtomID(a), epsilons(other.epsilons), sigmas(other.sigmas), indx(other.indx), sigcut(other.sigcut) {}
    flt get_epsilon(IEpsISigCutAtom& other) { return epsilons.at(other.indx); }
    flt get_sigma(IEpsISigCutAtom& other) { return sigmas.at(other.indx); }
    flt max_size() {
        flt sg = sigmas.at(0);
        for (uint i = 1; i < sigmas.size(); ++i)
            if (sg < sigmas[i]) sg = sigmas[i];
        return sg * sigcut;
    }
};

//! Indexed epsilons, own sigma (src/interaction.hpp:989-1018).
struct IEpsSigCutAtom : public AtomID {
    std::vector<flt> epsilons;
    uint indx;
    flt sigma, sigcut;
    IEpsSigCutAtom() : indx(0), sigma(0), sigcut(0) {}
    IEpsSigCutAtom(AtomID a, std::vector<flt> epsilons, uint indx, flt sigma, flt cut)
        : AtomID(a), epsilons(epsilons), indx(indx), sigma(sigma), sigcut(cut) {}
    IEpsSigCutAtom(AtomID a, IEpsSigCutAtom other)
        : AtomID(a), epsilons(other.epsilons), indx(other.indx), sigma(other.sigma), sigcut(other.sigcut) {}
    flt get_epsilon(IEpsSigCutAtom& other) { return epsilons.at(other.indx); }
    flt max_size() { return sigma * sigcut; }
};

//! Indexed attractive epsilons with a repulsive epsilon (src/interaction.hpp:1307-1336).
struct IEpsRepsSigCutAtom : public AtomID {
    std::vector<flt> epsilons;
    flt repeps, sig;
    uint indx;
    flt sigcut;
    IEpsRepsSigCutAtom() : repeps(0), sig(0), indx(0), sigcut(0) {}
    IEpsRepsSigCutAtom(AtomID a, std::vector<flt> epsilons, flt repeps, flt sigma, uint indx, flt cut)
        : AtomID(a), epsilons(epsilons), repeps(repeps), sig(sigma), indx(indx), sigcut(cut) {}
    IEpsRepsSigCutAtom(AtomID a, IEpsRepsSigCutAtom other)
        : AtomID(a), epsilons(other.epsilons), repeps(other.repeps), sig(other.sig), indx(other.indx),
          sigcut(other.sigcut) {}
    flt get_epsilon(IEpsRepsSigCutAtom& other) { return epsilons.at(other.indx); }
    flt max_size() { return sig * sigcut; }
};

//! Indexed epsilons, repulsive epsilon and exponent (src/interaction.hpp:1051-1092).
struct IEpsRepsSigExpCutAtom : public AtomID {
    std::vector<flt> epsilons;
    flt repeps, sigma, exponent;
    uint indx;
    flt sigcut;
    IEpsRepsSigExpCutAtom() : repeps(0), sigma(0), exponent(0), indx(0), sigcut(0) {}
    IEpsRepsSigExpCutAtom(AtomID a, std::vector<flt> epsilons, flt repeps, flt sigma, flt n, uint indx, flt cut)
        : AtomID(a), epsilons(epsilons), repeps(repeps), sigma(sigma), exponent(n), indx(indx), sigcut(cut) {}
    IEpsRepsSigExpCutAtom(AtomID a, IEpsRepsSigExpCutAtom other)
        : AtomID(a), epsilons(other.epsilons), repeps(other.repeps), sigma(other.sigma), exponent(other.exponent),
          indx(other.indx), sigcut(other.sigcut) {}
    flt get_epsilon(IEpsRepsSigExpCutAtom& other) { return epsilons.at(other.indx); }
    flt get_sigma(IEpsRepsSigExpCutAtom& other) { return (sigma + other.sigma) / 2.0; }
    flt max_size() { return sigma * sigcut; }
};

//! Indexed epsilons and sigmas with an exponent (src/interaction.hpp:1477-1511).
struct IEpsISigExpAtom : public AtomID {
    std::vector<flt> epsilons, sigmas;
    flt exponent;
    uint indx;
    IEpsISigExpAtom() : exponent(2.5), indx(0) {}
    IEpsISigExpAtom(AtomID a, std::vector<flt> epsilons, std::vector<flt> sigmas, uint indx, flt exponent = 2.5)
        : AtomID(a), epsilons(epsilons), sigmas(sigmas), exponent(exponent), indx(indx) {}
    IEpsISigExpAtom(AtomID a, IEpsISigExpAtom other)
        : AtomID(a), epsilons(other.epsilons), sigmas(other.sigmas), exponent(other.exponent), indx(other.indx) {}
    flt get_epsilon(IEpsISigExpAtom& other) { return epsilons.at(other.indx); }
    flt get_sigma(IEpsISigExpAtom& other) { return sigmas.at(other.indx); }
    flt max_size() {
        flt sg = sigmas.at(0);
        for (uint i = 1; i < sigmas.size(); ++i)
            if (sg < sigmas[i]) sg = sigmas[i];
        return sg;
    }
};

// the table rows an indexed atom brings to its neighbour list's GPU handle
inline void register_types(GpuLink&, const AtomID&) {}
inline void register_types(GpuLink& l, const IEpsISigCutAtom& a) { l.set_type_row(a.indx, a.epsilons, &a.sigmas); }
inline void register_types(GpuLink& l, const IEpsSigCutAtom& a) { l.set_type_row(a.indx, a.epsilons, nullptr); }
inline void register_types(GpuLink& l, const IEpsISigExpAtom& a) { l.set_type_row(a.indx, a.epsilons, &a.sigmas); }
inline void register_types(GpuLink& l, const IEpsRepsSigCutAtom& a) { l.set_type_row(a.indx, a.epsilons, nullptr); }
inline void register_types(GpuLink& l, const IEpsRepsSigExpCutAtom& a) {
    l.set_type_row(a.indx, a.epsilons, nullptr);
}

//! A pair's force and energy (src/interaction.hpp:1467-1472).
struct EnergyForce {
    Vec f;
    flt E;
    EnergyForce(Vec f, flt E) : f(f), E(E) {}
};

//! A pair, its force and its stiffness term, handed to an FPairXFunct
//! (src/interaction.hpp:822-836).
struct ForcePairX {
    AtomID a1, a2;
    flt xij;
    Vec fij;
};
class FPairXFunct {
   public:
    virtual void run(ForcePairX*) = 0;
    virtual ~FPairXFunct() {}
};

// Pair laws.  Each pair type holds its pair's constants (combined from the
// two atoms as the reference combines them) and its two atoms; `kind` and
// `params` tell the GPU which law and which per-atom numbers to use.

//! Truncated LJ, V = eps((1 - sigma^6/r^6)^2 - 1) - V(cut)
//! (src/interaction.hpp:238-281, 967-987).
struct LennardJonesCutPair {
    static const int kind = PARM_LJCUT;
    static void params(const EpsSigCutAtom& a, double p[3]) {
        p[0] = a.epsilon;
        p[1] = a.sigma;
        p[2] = a.sigcut;
    }
    static int kind_of(const EpsSigCutAtom&) { return PARM_LJCUT; }
    static int kind_of(const IEpsISigCutAtom&) { return PARM_LJCUT_IEPSISIG; }
    static void params(const IEpsISigCutAtom& a, double p[3]) {
        p[0] = a.indx;
        p[1] = a.sigcut;
        p[2] = 0.0;
    }
    flt epsilon, sigma, cut_distance, cut_energy;
    AtomID atom1, atom2;
    LennardJonesCutPair(EpsSigCutAtom a1, EpsSigCutAtom a2)
        : epsilon(std::sqrt(a1.epsilon * a2.epsilon)),
          sigma((a1.sigma + a2.sigma) / 2),
          cut_distance(std::max(a1.sigcut, a2.sigcut)),
          atom1(a1),
          atom2(a2) {
        set_cut_energy();
    }
    //! indexed epsilon and sigma (src/interaction.hpp:977-982)
    LennardJonesCutPair(IEpsISigCutAtom a1, IEpsISigCutAtom a2)
        : epsilon(a1.get_epsilon(a2)),
          sigma(a1.get_sigma(a2)),
          cut_distance(std::max(a1.sigcut, a2.sigcut)),
          atom1(a1),
          atom2(a2) {
        set_cut_energy();
    }
    void set_cut_energy() {
        const flt rsix = std::pow(cut_distance, 6);
        const flt mid = (1 - 1 / rsix);
        cut_energy = epsilon * (mid * mid - 1);
    }
    flt energy(Box& box) {
        const flt rsq = box.diff(atom1->x, atom2->x).squaredNorm() / (sigma * sigma);
        if (rsq > (cut_distance * cut_distance)) return 0;
        const flt rsix = rsq * rsq * rsq;
        const flt mid = (1 - 1 / rsix);
        return epsilon * (mid * mid - 1) - cut_energy;
    }
    Vec forces(Box& box) {
        const Vec diff = box.diff(atom1->x, atom2->x);
        const flt dsq = diff.squaredNorm();
        const flt rsq = dsq / (sigma * sigma);
        if (rsq > (cut_distance * cut_distance)) return Vec::Zero();
        const flt rsix = rsq * rsq * rsq;
        const flt fmagTimesR = 12 * epsilon / rsix * (1 / rsix - 1);
        return diff * (fmagTimesR / dsq);
    }
};

//! Soft repulsion, V = eps/n (1 - r/sigma)^n for r < sigma
//! (src/interaction.hpp:1528-1590).
struct RepulsionPair {
    static const int kind = PARM_REPULSION;
    static void params(const EpsSigExpAtom& a, double p[3]) {
        p[0] = a.eps;
        p[1] = a.sigma;
        p[2] = a.exponent;
    }
    static int kind_of(const EpsSigExpAtom&) { return PARM_REPULSION; }
    static int kind_of(const IEpsISigExpAtom&) { return PARM_REPULSION_IEPSISIG; }
    static void params(const IEpsISigExpAtom& a, double p[3]) {
        p[0] = a.indx;
        p[1] = a.exponent;
        p[2] = 0.0;
    }
    flt eps, sig, exponent;
    AtomID atom1, atom2;
    RepulsionPair(EpsSigExpAtom a1, EpsSigExpAtom a2)
        : eps(std::sqrt(a1.eps * a2.eps)),
          sig((a1.sigma + a2.sigma) / 2.0),
          exponent((a1.exponent + a2.exponent) / 2.0),
          atom1(a1),
          atom2(a2) {}
    //! indexed epsilon and sigma (src/interaction.hpp:1538-1543)
    RepulsionPair(IEpsISigExpAtom a1, IEpsISigExpAtom a2)
        : eps(a1.get_epsilon(a2)),
          sig(a1.get_sigma(a2)),
          exponent((a1.exponent + a2.exponent) / 2.0),
          atom1(a1),
          atom2(a2) {}
    //! the pair force and energy together (src/interaction.hpp:1557-1567)
    EnergyForce get_energy_forces(Box& box) {
        const Vec rij = box.diff(atom1->x, atom2->x);
        const flt dsq = rij.squaredNorm();
        if (dsq > sig * sig) return EnergyForce(Vec::Zero(), 0);
        const flt R = std::sqrt(dsq);
        return EnergyForce(rij * (eps * std::pow(1.0 - (R / sig), exponent - 1) / sig / R),
                           eps * std::pow(1.0 - (R / sig), exponent) / exponent);
    }
    //! the pair force and its pair stiffness term for NListedVirial's callback (1574-1589)
    void fill(Box& box, ForcePairX& fpair) {
        fpair.a1 = atom1;
        fpair.a2 = atom2;
        const Vec rij = box.diff(atom1->x, atom2->x);
        const flt dsq = rij.squaredNorm();
        if (dsq > sig * sig) {
            fpair.fij = Vec::Zero();
            fpair.xij = 0.0;
            return;
        }
        const flt R = std::sqrt(dsq);
        fpair.fij = rij * (eps * std::pow(1.0 - (R / sig), exponent - 1) / sig / R);
        const flt Rs = R / sig;
        fpair.xij = -Rs * eps * std::pow(1.0 - (R / sig), exponent - 2) * (1 - exponent * Rs);
    }
    flt energy(Box& box) {
        const flt dsq = box.diff(atom1->x, atom2->x).squaredNorm();
        if (dsq > sig * sig) return 0.0;
        const flt R = std::sqrt(dsq);
        return eps * std::pow(1.0 - (R / sig), exponent) / exponent;
    }
    Vec forces(Box& box) {
        const Vec rij = box.diff(atom1->x, atom2->x);
        const flt dsq = rij.squaredNorm();
        if (dsq > sig * sig) return Vec::Zero();
        const flt R = std::sqrt(dsq);
        return rij * (eps * std::pow(1.0 - (R / sig), exponent - 1) / sig / R);
    }
};

//! WCA, V = eps (1 - sigma^6/r^6)^2 for r < sigma (src/interaction.hpp:119-152, 875-891).
struct LJRepulsePair {
    static const int kind = PARM_LJREPULSE;
    static void params(const EpsSigAtom& a, double p[3]) {
        p[0] = a.epsilon;
        p[1] = a.sigma;
        p[2] = 0.0;
    }
    flt epsilon, sigma;
    AtomID atom1, atom2;
    LJRepulsePair(EpsSigAtom a1, EpsSigAtom a2)
        : epsilon(std::sqrt(a1.epsilon * a2.epsilon)), sigma((a1.sigma + a2.sigma) / 2), atom1(a1), atom2(a2) {}
    flt energy(Box& box) {
        const flt rsq = box.diff(atom1->x, atom2->x).squaredNorm() / (sigma * sigma);
        if (rsq > 1) return 0;
        const flt rsix = rsq * rsq * rsq;
        const flt mid = (1 - 1 / rsix);
        return epsilon * (mid * mid);
    }
    Vec forces(Box& box) {
        const Vec diff = box.diff(atom1->x, atom2->x);
        const flt dsq = diff.squaredNorm();
        const flt rsq = dsq / (sigma * sigma);
        if (rsq > 1) return Vec::Zero();
        const flt rsix = rsq * rsq * rsq;
        const flt fmagTimesR = 12 * epsilon / rsix * (1 / rsix - 1);
        return diff * (fmagTimesR / dsq);
    }
};

//! Attractive LJ (pyparm's LJAttractCut): V = eps((1 - sigma^6/r^6)^2 - 1) for
//! sigma <= r <= cut, -eps inside sigma, shifted by V(cut)
//! (src/interaction.hpp:154-236, 1020-1050).
struct LJAttractCutPair {
    static const int kind = PARM_LJATTRACTCUT;
    static void params(const EpsSigCutAtom& a, double p[3]) {
        p[0] = a.epsilon;
        p[1] = a.sigma;
        p[2] = a.sigcut;
    }
    static int kind_of(const EpsSigCutAtom&) { return PARM_LJATTRACTCUT; }
    static int kind_of(const IEpsISigCutAtom&) { return PARM_LJATTRACTCUT_IEPSISIG; }
    static int kind_of(const IEpsSigCutAtom&) { return PARM_LJATTRACTCUT_IEPS; }
    static void params(const IEpsISigCutAtom& a, double p[3]) {
        p[0] = a.indx;
        p[1] = a.sigcut;
        p[2] = 0.0;
    }
    static void params(const IEpsSigCutAtom& a, double p[3]) {
        p[0] = a.indx;
        p[1] = a.sigma;
        p[2] = a.sigcut;
    }
    flt epsilon, sigma, cut_distance, cut_energy;
    AtomID atom1, atom2;
    LJAttractCutPair(EpsSigCutAtom a1, EpsSigCutAtom a2)
        : LJAttractCutPair(a1, a2, std::sqrt(a1.epsilon * a2.epsilon), (a1.sigma + a2.sigma) / 2,
                           std::max(a1.sigcut, a2.sigcut)) {}
    //! indexed epsilon and sigma (src/interaction.hpp:1028-1032)
    LJAttractCutPair(IEpsISigCutAtom a1, IEpsISigCutAtom a2)
        : LJAttractCutPair(a1, a2, a1.get_epsilon(a2), a1.get_sigma(a2), std::max(a1.sigcut, a2.sigcut)) {}
    //! indexed epsilon (src/interaction.hpp:1033-1037)
    LJAttractCutPair(IEpsSigCutAtom a1, IEpsSigCutAtom a2)
        : LJAttractCutPair(a1, a2, a1.get_epsilon(a2), (a1.sigma + a2.sigma) / 2, std::max(a1.sigcut, a2.sigcut)) {}
    LJAttractCutPair(AtomID a1, AtomID a2, flt eps, flt sig, flt cut)
        : epsilon(eps), sigma(sig), cut_distance(cut), atom1(a1), atom2(a2) {
        flt e = -1;   // the unit-epsilon attraction at the cut
        if (cut_distance >= 1) {
            const flt rsq = cut_distance * cut_distance;
            const flt rsix = rsq * rsq * rsq;
            const flt mid = (1 - 1 / rsix);
            e = mid * mid - 1;
        }
        cut_energy = e * epsilon;
    }
    flt energy(Box& box) {
        if (epsilon == 0) return 0;
        const flt dsq = box.diff(atom1->x, atom2->x).squaredNorm();
        if (dsq > (cut_distance * cut_distance * sigma * sigma)) return 0;
        const flt rsq = dsq / (sigma * sigma);
        if (rsq < 1) return -epsilon - cut_energy;
        const flt rsix = rsq * rsq * rsq;
        const flt mid = (1 - 1 / rsix);
        return epsilon * (mid * mid - 1) - cut_energy;
    }
    Vec forces(Box& box) {
        if (epsilon == 0) return Vec::Zero();
        const Vec diff = box.diff(atom1->x, atom2->x);
        const flt dsq = diff.squaredNorm();
        const flt rsq = dsq / (sigma * sigma);
        if (rsq < 1 || rsq > (cut_distance * cut_distance)) return Vec::Zero();
        const flt rsix = rsq * rsq * rsq;
        const flt fmagTimesR = 12 * epsilon / rsix * (1 / rsix - 1);
        return diff * (fmagTimesR / dsq);
    }
};

//! Sticky spheres (src/interaction.hpp:1679-1691): repulsive epsilon, sigma,
//! and the widths C and l of the two halves of the attractive well.
struct LoisOhernAtom : public AtomID {
    flt eps, sigma, C, l;
    LoisOhernAtom() : eps(0), sigma(0), C(0), l(0) {}
    LoisOhernAtom(AtomID a, flt eps, flt sigma, flt C, flt l) : AtomID(a), eps(eps), sigma(sigma), C(C), l(l) {}
    LoisOhernAtom(AtomID a, LoisOhernAtom other)
        : AtomID(a), eps(other.eps), sigma(other.sigma), C(other.C), l(other.l) {}
    flt max_size() { return sigma * (1 + C + l); }
};

//! Lois-O'Hern pair (src/interaction.hpp:1693-1744): harmonic about sigma out
//! to (1 + C) sigma, then a linear return to zero force at sigcut =
//! sigma (1 + C + l); epsilon geometric mean, the rest averaged.
struct LoisOhernPair {
    static const int kind = PARM_LOISOHERN;
    static void params(const LoisOhernAtom& a, double p[4]) {
        p[0] = a.eps;
        p[1] = a.sigma;
        p[2] = a.C;
        p[3] = a.l;
    }
    flt eps, sig, C, l, sigcut;
    AtomID atom1, atom2;
    LoisOhernPair(LoisOhernAtom a1, LoisOhernAtom a2)
        : LoisOhernPair(a1, a2, std::sqrt(a1.eps * a2.eps), (a1.sigma + a2.sigma) / 2.0, (a1.C + a2.C) / 2.0,
                        (a1.l + a2.l) / 2.0) {}
    LoisOhernPair(LoisOhernAtom a1, LoisOhernAtom a2, flt eps, flt sig, flt C, flt l)
        : eps(eps), sig(sig), C(C), l(l), sigcut(sig * (1 + C + l)), atom1(a1), atom2(a2) {}
    flt energy(Box& box) {
        const flt dsq = box.diff(atom1->x, atom2->x).squaredNorm();
        if (dsq >= sigcut * sigcut) return 0.0;
        const flt R = std::sqrt(dsq) / sig;
        if (R <= 1 + C) {
            const flt dR = R - 1;
            return -eps * sig / 2 * (C * (C + l) - dR * dR);
        }
        const flt dR2 = C + l + 1 - R;
        return -C * eps * sig / 2 / l * dR2 * dR2;
    }
    Vec forces(Box& box) {
        const Vec rij = box.diff(atom1->x, atom2->x);
        const flt dsq = rij.squaredNorm();
        if (dsq >= sigcut * sigcut) return Vec::Zero();
        const flt R = std::sqrt(dsq);
        const flt rsig = R / sig;
        if (rsig <= 1 + C) return rij * (-eps * (rsig - 1) / R);
        return rij * (C * eps / l * (rsig - (C + l + 1)) / R);
    }
};

//! Lois-O'Hern pair with the smaller C and l of the two atoms
//! (src/interaction.hpp:1746-1751).
struct LoisOhernPairMinCLs : public LoisOhernPair {
    static const int kind = PARM_LOISOHERN_MIN;
    LoisOhernPairMinCLs(LoisOhernAtom a1, LoisOhernAtom a2)
        : LoisOhernPair(a1, a2, std::sqrt(a1.eps * a2.eps), (a1.sigma + a2.sigma) / 2.0, (a1.C < a2.C ? a1.C : a2.C),
                        (a1.l < a2.l ? a1.l : a2.l)) {}
};

//! Harmonic repulsion with a fixed attractive force (src/interaction.hpp:
//! 1764-1780): the constructor takes the well's depth and width and keeps
//! f = depth / width (0 for width 0) and l = width.
struct LoisLinAtom : public AtomID {
    flt eps, sigma, f, l;
    LoisLinAtom() : eps(0), sigma(0), f(0), l(0) {}
    LoisLinAtom(AtomID a, flt eps, flt sigma, flt depth, flt width)
        : AtomID(a), eps(eps), sigma(sigma), f(width > 0 ? depth / width : 0), l(width) {}
    LoisLinAtom(AtomID a, LoisLinAtom other) : AtomID(a), eps(other.eps), sigma(other.sigma), f(other.f), l(other.l) {}
    flt max_size() { return sigma * (1 + l); }
};

//! Lois-Lin pair (src/interaction.hpp:1782-1829): harmonic inside sigma, a
//! constant attractive force f out to sigcut = sigma + l.
struct LoisLinPair {
    static const int kind = PARM_LOISLIN;
    static void params(const LoisLinAtom& a, double p[4]) {
        p[0] = a.eps;
        p[1] = a.sigma;
        p[2] = a.f;
        p[3] = a.l;
    }
    flt eps, sig, f, l, sigcut;
    AtomID atom1, atom2;
    LoisLinPair(LoisLinAtom a1, LoisLinAtom a2)
        : LoisLinPair(a1, a2, std::sqrt(a1.eps * a2.eps), (a1.sigma + a2.sigma) / 2.0, (a1.f + a2.f) / 2.0,
                      (a1.l + a2.l) / 2.0) {}
    LoisLinPair(LoisLinAtom a1, LoisLinAtom a2, flt eps, flt sig, flt f, flt l)
        : eps(eps), sig(sig), f(f), l(l), sigcut(sig + l), atom1(a1), atom2(a2) {}
    flt energy(Box& box) {
        const flt dsq = box.diff(atom1->x, atom2->x).squaredNorm();
        if (dsq >= sigcut * sigcut) return 0.0;
        const flt R = std::sqrt(dsq);
        if (R <= sig) {
            const flt dR = 1.0 - (R / sig);
            return eps / 2 * dR * dR - f * l;
        }
        return -f * (sig + l - R);
    }
    Vec forces(Box& box) {
        const Vec rij = box.diff(atom1->x, atom2->x);
        const flt dsq = rij.squaredNorm();
        if (dsq >= sigcut * sigcut) return Vec::Zero();
        const flt R = std::sqrt(dsq);
        if (R <= sig) return rij * (eps * (1.0 - (R / sig)) / sig / R);
        return rij * -(f / R);
    }
};

//! Lois-Lin pair with the smaller f and l of the two atoms
//! (src/interaction.hpp:1831-1836).
struct LoisLinPairMin : public LoisLinPair {
    static const int kind = PARM_LOISLIN_MIN;
    LoisLinPairMin(LoisLinAtom a1, LoisLinAtom a2)
        : LoisLinPair(a1, a2, std::sqrt(a1.eps * a2.eps), (a1.sigma + a2.sigma) / 2.0, (a1.f < a2.f ? a1.f : a2.f),
                      (a1.l < a2.l ? a1.l : a2.l)) {}
};

//! (epsilon, sigma, exponent, drag coefficient gamma) per atom
//! (src/interaction.hpp:1598-1611); the constructor takes gamma before the
//! exponent.
struct EpsSigExpDragAtom : public AtomID {
    flt eps, sigma, exponent, gamma;
    EpsSigExpDragAtom() : eps(0), sigma(0), exponent(2.5), gamma(0) {}
    EpsSigExpDragAtom(AtomID a, flt eps, flt sigma, flt gamma, flt exponent = 2.5)
        : AtomID(a), eps(eps), sigma(sigma), exponent(exponent), gamma(gamma) {}
    EpsSigExpDragAtom(AtomID a, EpsSigExpDragAtom other)
        : AtomID(a), eps(other.eps), sigma(other.sigma), exponent(other.exponent), gamma(other.gamma) {}
    flt max_size() { return sigma; }
};

//! Soft repulsion with a drag on the relative normal velocity
//! (src/interaction.hpp:1613-1640): F = r eps (1 - r/sigma)^(n-1) / (sigma r)
//! - gamma v_perp, v_perp = r ((v1 - v2) . r) / r^2.
struct RepulsionDragPair {
    static const int kind = PARM_REPULSIONDRAG;
    static void params(const EpsSigExpDragAtom& a, double p[4]) {
        p[0] = a.eps;
        p[1] = a.sigma;
        p[2] = a.exponent;
        p[3] = a.gamma;
    }
    flt eps, sig, exponent, gamma;
    AtomID atom1, atom2;
    RepulsionDragPair(EpsSigExpDragAtom a1, EpsSigExpDragAtom a2)
        : eps(std::sqrt(a1.eps * a2.eps)),
          sig((a1.sigma + a2.sigma) / 2.0),
          exponent((a1.exponent + a2.exponent) / 2.0),
          gamma((a1.gamma + a2.gamma) / 2),
          atom1(a1),
          atom2(a2) {}
    flt energy(Box& box) {
        const flt dsq = box.diff(atom1->x, atom2->x).squaredNorm();
        if (dsq > sig * sig) return 0.0;
        const flt R = std::sqrt(dsq);
        return eps * std::pow(1.0 - (R / sig), exponent) / exponent;
    }
    Vec forces(Box& box) {
        const Vec rij = box.diff(atom1->x, atom2->x);
        const Vec vij = atom1->v - atom2->v;
        const flt dsq = rij.squaredNorm();
        if (dsq > sig * sig) return Vec::Zero();
        const flt R = std::sqrt(dsq);
        const Vec v_perp = rij * (vij.dot(rij)) / dsq;
        return rij * (eps * std::pow(1.0 - (R / sig), exponent - 1) / sig / R) - (v_perp * gamma);
    }
};

//! Separate repulsive and attractive epsilons and lengths
//! (src/interaction.hpp:1149-1169).
struct EpsEpsSigSigCutAtom : public AtomID {
    flt eps_r, eps_a, sig_r, sig_a, sigcut;
    EpsEpsSigSigCutAtom() : eps_r(0), eps_a(0), sig_r(0), sig_a(0), sigcut(0) {}
    EpsEpsSigSigCutAtom(AtomID a, flt eps_r, flt eps_a, flt sigma_r, flt sigma_a, flt cut)
        : AtomID(a), eps_r(eps_r), eps_a(eps_a), sig_r(sigma_r), sig_a(sigma_a), sigcut(cut) {}
    EpsEpsSigSigCutAtom(AtomID a, EpsEpsSigSigCutAtom other)
        : AtomID(a), eps_r(other.eps_r), eps_a(other.eps_a), sig_r(other.sig_r), sig_a(other.sig_a),
          sigcut(other.sigcut) {}
    flt max_size() { return sig_r + sig_a * (sigcut - 1); }
};

//! LJ repulsion eps_r (1 - (sig_r/r)^6)^2 inside sig_r and an LJ attraction
//! of depth eps_a and width sig_a beyond it, cut at sig_r + sig_a (sigcut - 1)
//! (src/interaction.hpp:1171-1239).
struct LJAttractRepulseSigsPair {
    static const int kind = PARM_LJATTRACTREPULSESIGS;
    static void params(const EpsEpsSigSigCutAtom& a, double p[5]) {
        p[0] = a.eps_r;
        p[1] = a.eps_a;
        p[2] = a.sig_r;
        p[3] = a.sig_a;
        p[4] = a.sigcut;
    }
    flt eps_r, eps_a, sig_r, sig_a, cut_distance, cut_energy;
    AtomID atom1, atom2;
    LJAttractRepulseSigsPair(EpsEpsSigSigCutAtom a1, EpsEpsSigSigCutAtom a2)
        : eps_r(std::sqrt(a1.eps_r * a2.eps_r)), eps_a(std::sqrt(a1.eps_a * a2.eps_a)),
          sig_r((a1.sig_r + a2.sig_r) / 2.0), sig_a((a1.sig_a + a2.sig_a) / 2.0),
          cut_distance(std::max(a1.sigcut, a2.sigcut)), cut_energy(0), atom1(a1), atom2(a2) {
        if (cut_distance <= 0) return;
        const flt cu = sig_r + sig_a * (cut_distance - 1);
        cut_energy = (cut_distance >= 1) ? attract_energy(cu) : repulse_energy(cu);
    }
    flt attract_energy(flt r) {
        const flt mid = (1 - std::pow((r - sig_r + sig_a) / sig_a, -6));
        return eps_a * (mid * mid) - eps_a;
    }
    flt repulse_energy(flt r) {
        const flt mid = (1 - std::pow(r / sig_r, -6));
        return eps_r * (mid * mid) - eps_a;
    }
    flt energy(Box& box) {
        const flt dist = box.diff(atom1->x, atom2->x).norm();
        const flt cu = sig_r + sig_a * (cut_distance - 1);
        if (cut_distance > 0 && dist > cu) return 0;
        if (dist <= sig_r) return repulse_energy(dist) - cut_energy;
        return attract_energy(dist) - cut_energy;
    }
    Vec forces(Box& box) {
        const Vec rij = box.diff(atom1->x, atom2->x);
        const flt rsq = rij.squaredNorm();
        const flt cu = sig_r + sig_a * (cut_distance - 1);
        if (cut_distance > 0 && rsq > cu * cu) return Vec::Zero();
        if (rsq > sig_r * sig_r) {
            const flt dist = std::sqrt(rsq);
            const flt rminus = dist - sig_r + sig_a;
            const flt rsix = std::pow(rminus / sig_a, -6);
            return rij * (eps_a * (12 * rsix * (rsix - 1) / (dist * rminus)));
        }
        const flt rsix = std::pow(rsq / (sig_r * sig_r), -3);
        return rij * (eps_r * (12 * rsix * (rsix - 1)) / rsq);
    }
};

//! Implicit-solvation atom (src/interaction.hpp:1415-1423): dist = the
//! atom's radius plus the water radius, sigmai its solvation parameter.
struct EisMclachlanAtom : public AtomID {
    flt dist, sigmai;
    EisMclachlanAtom() : dist(0), sigmai(0) {}
    EisMclachlanAtom(AtomID a, flt dist, flt sigmai) : AtomID(a), dist(dist), sigmai(sigmai) {}
    EisMclachlanAtom(AtomID a, EisMclachlanAtom other) : AtomID(a), dist(other.dist), sigmai(other.sigmai) {}
    flt max_size() { return dist; }
};

//! Eisenberg-McLachlan pair (src/interaction.hpp:1425-1452): E = c0/R + c1 +
//! c2 R out to dist_1 + dist_2.
struct EisMclachlanPair {
    static const int kind = PARM_EISMCLACHLAN;
    static void params(const EisMclachlanAtom& a, double p[4]) {
        p[0] = a.dist;
        p[1] = a.sigmai;
        p[2] = 0.0;
    }
    flt c0, c1, c2, cutoff;
    AtomID atom1, atom2;
    EisMclachlanPair(EisMclachlanAtom a1, EisMclachlanAtom a2)
        : c0(-M_PI * (a1.sigmai * a2.dist - a2.sigmai * a1.dist) * (a1.dist * a1.dist - a2.dist * a2.dist)),
          c1(-2 * M_PI * (a1.sigmai * a2.dist * a2.dist + a2.sigmai * a1.dist * a1.dist)),
          c2(M_PI * (a1.sigmai * a2.dist + a2.sigmai * a1.dist)),
          cutoff(a1.dist + a2.dist),
          atom1(a1),
          atom2(a2) {}
    flt energy(Box& box) {
        const flt R = box.diff(atom1->x, atom2->x).norm();
        if (R > cutoff) return 0;
        return c0 / R + c1 + c2 * R;
    }
    Vec forces(Box& box) {
        const Vec rij = box.diff(atom1->x, atom2->x);
        const flt dsq = rij.squaredNorm();
        if (dsq > (cutoff * cutoff)) return Vec::Zero();
        const flt R = std::sqrt(dsq);
        return rij * ((c0 / dsq - c2) / R);
    }
};

//! LJ with an indexed epsilon; repulsion only (|eps|, cut at sigma) when
//! the table's entry is not positive (src/interaction.hpp:1251-1298).
struct LJAttractRepulsePair {
    static const int kind = PARM_LJATTRACTREPULSE;
    static void params(const IEpsSigCutAtom& a, double p[3]) {
        p[0] = a.indx;
        p[1] = a.sigma;
        p[2] = a.sigcut;
    }
    flt eps, sig, cut_distance, cut_energy;
    AtomID atom1, atom2;
    LJAttractRepulsePair(IEpsSigCutAtom a1, IEpsSigCutAtom a2)
        : eps(a1.get_epsilon(a2)), sig((a1.sigma + a2.sigma) / 2.0), cut_distance(std::max(a1.sigcut, a2.sigcut)),
          atom1(a1), atom2(a2) {
        if (eps <= 0) {
            cut_distance = 1;
            cut_energy = 0;
            eps = std::abs(eps);
            return;
        }
        const flt mid = (1 - std::pow(cut_distance, -6));
        cut_energy = eps * (mid * mid);
    }
    flt energy(Box& box) {
        const flt rsq = box.diff(atom1->x, atom2->x).squaredNorm() / (sig * sig);
        if (rsq > cut_distance * cut_distance) return 0;
        const flt mid = (1 - std::pow(rsq, -3));
        return eps * (mid * mid) - cut_energy;
    }
    Vec forces(Box& box) {
        if (eps == 0) return Vec::Zero();
        const Vec rij = box.diff(atom1->x, atom2->x);
        const flt dsq = rij.squaredNorm();
        const flt rsq = dsq / (sig * sig);
        if (rsq > (cut_distance * cut_distance)) return Vec::Zero();
        const flt rsix = std::pow(rsq, -3);
        return rij * (12 * eps * rsix * (rsix - 1) / dsq);
    }
};

//! LJ with an indexed attractive epsilon (none when the entry is not
//! positive) and a repulsive epsilon inside sigma
//! (src/interaction.hpp:1343-1399).
struct LJAttractFixedRepulsePair {
    static const int kind = PARM_LJATTRACTFIXEDREPULSE;
    static void params(const IEpsRepsSigCutAtom& a, double p[4]) {
        p[0] = a.indx;
        p[1] = a.repeps;
        p[2] = a.sig;
        p[3] = a.sigcut;
    }
    flt eps, repeps, sig, cut_distance, cut_energy;
    bool attract;
    AtomID atom1, atom2;
    LJAttractFixedRepulsePair(IEpsRepsSigCutAtom a1, IEpsRepsSigCutAtom a2)
        : eps(std::abs(a1.get_epsilon(a2))), repeps(std::sqrt(a1.repeps * a2.repeps)), sig((a1.sig + a2.sig) / 2.0),
          cut_distance(std::max(a1.sigcut, a2.sigcut)), attract(a1.get_epsilon(a2) > 0), atom1(a1), atom2(a2) {
        if (!attract || eps == 0) {
            cut_distance = 1;
            cut_energy = 0;
            eps = 0;
            attract = false;
            return;
        }
        const flt mid = (1 - std::pow(cut_distance, -6.0));
        cut_energy = eps * (mid * mid);
    }
    flt energy(Box& box) {
        const flt rsq = box.diff(atom1->x, atom2->x).squaredNorm() / (sig * sig);
        if (rsq > cut_distance * cut_distance) return 0;
        const flt mid = (1 - std::pow(rsq, -3));
        if (rsq > 1) return eps * (mid * mid) - cut_energy;
        return repeps * (mid * mid) - cut_energy;
    }
    Vec forces(Box& box) {
        const Vec rij = box.diff(atom1->x, atom2->x);
        const flt dsq = rij.squaredNorm();
        const flt rsq = dsq / (sig * sig);
        if (rsq > (cut_distance * cut_distance)) return Vec::Zero();
        const flt rsix = std::pow(rsq, -3);
        const flt fmagTimesR = 12 * rsix * (rsix - 1);
        if (rsq < 1) return rij * (repeps * fmagTimesR / dsq);
        return rij * (eps * fmagTimesR / dsq);
    }
};

//! LJ-like law with exponent n, indexed epsilon, repulsive epsilon inside
//! sigma (src/interaction.hpp:1095-1141).
struct LJishPair {
    static const int kind = PARM_LJISH;
    static void params(const IEpsRepsSigExpCutAtom& a, double p[5]) {
        p[0] = a.indx;
        p[1] = a.repeps;
        p[2] = a.sigma;
        p[3] = a.exponent;
        p[4] = a.sigcut;
    }
    flt epsilon, repeps, sigma, n, cut_distance, cut_energy;
    AtomID atom1, atom2;
    LJishPair(IEpsRepsSigExpCutAtom a1, IEpsRepsSigExpCutAtom a2)
        : epsilon(a1.get_epsilon(a2)), repeps(std::sqrt(a1.repeps * a2.repeps)), sigma(a1.get_sigma(a2)),
          n((a1.exponent + a2.exponent) / 2), cut_distance(std::max(a1.sigcut, a2.sigcut)), atom1(a1), atom2(a2) {
        if (epsilon <= 0) {
            cut_distance = 1;
            cut_energy = 0;
            epsilon = 0;
            return;
        }
        const flt mid = (1 - std::pow(cut_distance, -n));
        cut_energy = epsilon * (mid * mid);
    }
    flt energy(Box& box) {
        const flt rsq = box.diff(atom1->x, atom2->x).squaredNorm() / (sigma * sigma);
        if (rsq > cut_distance * cut_distance) return 0;
        const flt mid = (1 - std::pow(rsq, -n / 2));
        if (rsq > 1) return epsilon * (mid * mid) - cut_energy;
        return repeps * (mid * mid) - cut_energy;
    }
    Vec forces(Box& box) {
        const Vec rij = box.diff(atom1->x, atom2->x);
        const flt dsq = rij.squaredNorm();
        const flt rsq = dsq / (sigma * sigma);
        if (rsq > cut_distance * cut_distance) return Vec::Zero();
        const flt rmid = std::pow(rsq, -n / 2);
        const flt fmagTimesR = 2 * n * rmid * (rmid - 1);
        if (rsq < 1) return rij * (repeps * fmagTimesR / dsq);
        return rij * (epsilon * fmagTimesR / dsq);
    }
};

// the pair law (PARM_* kind) of pair type P for atom type A: P::kind_of(A)
// where a pair type serves several atom types, else P::kind
template <class P, class A>
auto pair_kind(const A& a, int) -> decltype(P::kind_of(a)) {
    return P::kind_of(a);
}
template <class P, class A>
int pair_kind(const A&, long) {
    return P::kind;
}

// GPU-evaluated quantities of the handle's interaction
flt gpu_evaluate(GpuLink& link, int what);
Matrix gpu_stress(GpuLink& link);
//! NListed::set_forces: pair forces added to the atoms' current forces
void gpu_add_forces(GpuLink& link);

//! Neighbour-listed pair interaction (src/interaction.hpp:1876-1945).  The
//! NeighborList may be its own (constructor with a skin) or one the caller
//! made (NListed(atoms, neighbours), as pyparm's Repulsion(atoms, nl) does);
//! one NListed evaluates the pairs of a NeighborList.
template <class A, class P>
class NListed : public Interaction, public GpuInteraction {
   public:
    NListed(sptr<AtomVec> vec, sptr<NeighborList> neighbors) : link(neighbors->gpu()), neighbors(neighbors) {
        if (link->atoms() != vec) throw std::invalid_argument("NListed: the NeighborList tracks another AtomVec");
        init_atoms(*vec);
    }
    NListed(sptr<Box> box, sptr<AtomVec> atomv, const flt skin)
        : link(new GpuLink(box, atomv, skin)), neighbors(new NeighborList(link)) {
        init_atoms(*atomv);
    }
    void add(A atm) {
        double p[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        P::params(atm, p);
        register_types(*link, atm);
        link->add(atm.n(), pair_kind<P>(atm, 0), p, this);
        atoms.at(atm.n()) = atm;
    }
    //! the pair of an IDPair of the neighbour list, with its constants
    P get_pair(IDPair& pair) { return P(atoms[pair.first().n()], atoms[pair.last().n()]); }
    A& getatom(uint n) { return atoms[n]; }
    //! the pairs of the current neighbour list, in its order (NListed::update_pairs)
    std::vector<P>& pair_iter() {
        const std::vector<IDPair>& ps = neighbors->pairs();
        pairs.clear();
        pairs.reserve(ps.size());
        for (const IDPair& q : ps) pairs.push_back(P(atoms[q.first().n()], atoms[q.last().n()]));
        return pairs;
    }
    //! energy of one pair (NListed::energy(box, pair))
    flt energy(Box& box, IDPair& pair) { return get_pair(pair).energy(box); }
    flt energy(Box& box) override { return gpu_evaluate(*link, PARM_EVAL_ENERGY); }
    //! sum of r . f over the listed pairs (src/interaction.hpp:2124-2163)
    flt pressure(Box& box) override { return gpu_evaluate(*link, PARM_EVAL_VIRIAL); }
    Matrix stress(Box& box) override { return gpu_stress(*link); }
    void set_forces(Box& box) override { gpu_add_forces(*link); }
    flt set_forces_get_pressure(Box& box) override {
        gpu_add_forces(*link);
        return pressure(box);
    }
    Matrix set_forces_get_stress(Box& box) {
        gpu_add_forces(*link);
        return stress(box);
    }
    unsigned long long contacts(Box& box) {
        return (unsigned long long)gpu_evaluate(*link, PARM_EVAL_CONTACTS);
    }
    unsigned long long overlaps(Box& box) {
        return (unsigned long long)gpu_evaluate(*link, PARM_EVAL_OVERLAPS);
    }
    uint size() const { return (uint)atoms.size(); }
    std::vector<A>& atom_list() { return atoms; }
    sptr<NeighborList> neighbor_list() { return neighbors; }
    sptr<GpuLink> gpu() override { return link; }

   private:
    // every entry names its atom, with default parameters until add() sets
    // them: a list member that no add() gave parameters (NeighborList::add)
    // then forms pairs of zero force, as on the GPU
    void init_atoms(AtomVec& v) {
        atoms.reserve(v.size());
        for (uint i = 0; i < v.size(); i++) atoms.push_back(A(v.get_id(i), A()));
    }
    sptr<GpuLink> link;
    sptr<NeighborList> neighbors;
    std::vector<A> atoms;   // indexed by AtomVec index
    std::vector<P> pairs;
};

//! Interactions that can hand every pair's force to a callback
//! (src/interaction.hpp:838-843).
class InteractionPairsX : public Interaction {
   public:
    using Interaction::set_forces;
    virtual void set_forces(Box& box, FPairXFunct*) = 0;
    virtual ~InteractionPairsX() {}
};

//! NListed with per-pair callbacks (pyparm's HertzianVirial,
//! src/interaction.hpp:1948-1968, 2178-2229): the forces are the NListed's
//! (on the GPU); set_forces(box, funct) and setForcesGetEnergy walk the pairs
//! on the host with the pair type's fill / get_energy_forces and add the
//! forces to the host Atom records, as the reference does.
template <class A, class P>
class NListedVirial : public InteractionPairsX, public GpuInteraction {
   public:
    NListedVirial(sptr<AtomVec> vec, sptr<NeighborList> neighbors) : vec(vec), nlisted(vec, neighbors) {}
    using InteractionPairsX::set_forces;
    void set_forces(Box& box) override { nlisted.set_forces(box); }
    void set_forces(Box& box, FPairXFunct* funct) override {
        for (P& pr : nlisted.pair_iter()) {
            ForcePairX fp;
            pr.fill(box, fp);
            funct->run(&fp);
            pr.atom1->f += fp.fij;
            pr.atom2->f -= fp.fij;
        }
    }
    flt set_forces_get_pressure(Box& box) override { return nlisted.set_forces_get_pressure(box); }
    virtual flt setForcesGetEnergy(Box& box) {
        flt E = 0;
        for (P& pr : nlisted.pair_iter()) {
            EnergyForce ef = pr.get_energy_forces(box);
            pr.atom1->f += ef.f;
            pr.atom2->f -= ef.f;
            E += ef.E;
        }
        return E;
    }
    flt energy(Box& box) override { return nlisted.energy(box); }
    flt pressure(Box& box) override { return nlisted.pressure(box); }
    void add(A atm) { nlisted.add(atm); }
    sptr<NeighborList> neighbor_list() { return nlisted.neighbor_list(); }
    sptr<GpuLink> gpu() override { return nlisted.gpu(); }

   private:
    sptr<AtomVec> vec;
    NListed<A, P> nlisted;
};

#endif
