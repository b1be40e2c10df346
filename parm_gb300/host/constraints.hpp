// parm_gb300 host API: the state trackers of the reference's
// src/constraints.hpp (wackywendell/parm) that this library provides.
//
// RsqTracker (trackers.hpp) runs on the GPU; EnergyTracker below accumulates
// on the host the kinetic energy of the host Atom records and the potential
// energy of its interactions (evaluated on the GPU).  Constraints themselves
// are not part of this library.
#ifndef PARM_GB300_CONSTRAINTS_HPP
#define PARM_GB300_CONSTRAINTS_HPP

#include <cmath>
#include <vector>

#include "interaction.hpp"

//! Running means of the kinetic, potential and total energy, one sample
//! every n_skip updates (src/constraints.hpp:260-316, src/constraints.cpp:366-402).
class EnergyTracker : public StateTracker {
   protected:
    sptr<AtomGroup> atoms;
    std::vector<sptr<Interaction>> interactions;
    uint N;
    uint n_skip, n_skipped;
    flt U0;
    flt Es, Us, Ks;
    flt Esq, Usq, Ksq;

   public:
    EnergyTracker(sptr<AtomGroup> atoms, std::vector<sptr<Interaction>> interactions, uint n_skip = 1)
        : atoms(atoms),
          interactions(interactions),
          N(0),
          n_skip(n_skip > 1u ? n_skip : 1u),
          n_skipped(0),
          U0(0),
          Es(0),
          Us(0),
          Ks(0),
          Esq(0),
          Usq(0),
          Ksq(0) {}
    void update(Box& box) override;
    void reset() {
        n_skipped = 0;
        N = 0;
        Es = 0;
        Us = 0;
        Ks = 0;
        Esq = 0;
        Usq = 0;
        Ksq = 0;
    }
    void set_U0(flt newU0) {
        U0 = newU0;
        reset();
    }
    void set_U0(Box& box);
    flt get_U0() { return U0; }

    flt E() { return Es / ((flt)N); }
    flt U() { return Us / ((flt)N); }
    flt K() { return Ks / ((flt)N); }
    flt E_std() { return std::sqrt(Esq / N - Es * Es / N / N); }
    flt K_std() { return std::sqrt(Ksq / N - Ks * Ks / N / N); }
    flt U_std() { return std::sqrt(Usq / N - Us * Us / N / N); }
    flt E_squared_mean() { return Esq / N; }
    flt K_squared_mean() { return Ksq / N; }
    flt U_squared_mean() { return Usq / N; }
    uint n() { return N; }
};

#endif
