// parm_gb300 host API: pair interactions with the interface of the
// reference's src/interaction.hpp (wackywendell/parm), evaluated on the GPU.
//
// NListed<A, P> is the reference's neighbour-listed pair interaction
// (src/interaction.hpp:1896-1945); the atom types carry the per-atom
// parameters and the pair types select the pair law:
//   NListed<EpsSigCutAtom, LennardJonesCutPair>  LJ cut at sigcut * sigma
//   NListed<EpsSigExpAtom, RepulsionPair>         soft repulsion, exponent n
//   NListed<EpsSigAtom,    LJRepulsePair>         WCA (repulsive LJ)
#ifndef PARM_GB300_INTERACTION_HPP
#define PARM_GB300_INTERACTION_HPP

#include <vector>

#include "trackers.hpp"

//! Interface of everything a Collection sums (src/interaction.hpp:59-104).
class Interaction {
   public:
    virtual flt energy(Box& box) = 0;
    virtual void set_forces(Box& box) = 0;
    virtual flt set_forces_get_pressure(Box& box) = 0;
    virtual flt pressure(Box& box) = 0;
    virtual ~Interaction() {}
    //! the GPU handle behind the interaction (every interaction here has one)
    virtual sptr<GpuLink> gpu() = 0;
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

// pair laws (the GPU evaluates them; these types select the law)
struct LennardJonesCutPair {
    static const int kind = PARM_LJCUT;
    static void params(const EpsSigCutAtom& a, double p[3]) {
        p[0] = a.epsilon;
        p[1] = a.sigma;
        p[2] = a.sigcut;
    }
};
struct RepulsionPair {
    static const int kind = PARM_REPULSION;
    static void params(const EpsSigExpAtom& a, double p[3]) {
        p[0] = a.eps;
        p[1] = a.sigma;
        p[2] = a.exponent;
    }
};
struct LJRepulsePair {
    static const int kind = PARM_LJREPULSE;
    static void params(const EpsSigAtom& a, double p[3]) {
        p[0] = a.epsilon;
        p[1] = a.sigma;
        p[2] = 0.0;
    }
};

// GPU-evaluated quantities of the handle's interaction
flt gpu_evaluate(GpuLink& link, int what);
Matrix gpu_stress(GpuLink& link);
//! NListed::set_forces: pair forces added to the atoms' current forces
void gpu_add_forces(GpuLink& link);

//! Neighbour-listed pair interaction (src/interaction.hpp:1896-1945).
template <class A, class P>
class NListed : public Interaction {
   public:
    NListed(sptr<Box> box, sptr<AtomVec> atomv, const flt skin)
        : link(new GpuLink(box, atomv, skin)), neighbors(new NeighborList(link)) {}
    void add(A atm) {
        double p[3];
        P::params(atm, p);
        link->add(atm.n(), P::kind, p);
        atoms.push_back(atm);
    }
    flt energy(Box& box) override { return gpu_evaluate(*link, PARM_EVAL_ENERGY); }
    //! sum of r . f over the listed pairs (src/interaction.hpp:2124-2163)
    flt pressure(Box& box) override { return gpu_evaluate(*link, PARM_EVAL_VIRIAL); }
    Matrix stress(Box& box) { return gpu_stress(*link); }
    void set_forces(Box& box) override { gpu_add_forces(*link); }
    flt set_forces_get_pressure(Box& box) override {
        gpu_add_forces(*link);
        return pressure(box);
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
    sptr<GpuLink> link;
    sptr<NeighborList> neighbors;
    std::vector<A> atoms;
};

#endif
