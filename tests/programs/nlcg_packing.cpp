// A packing program on the C++ host API's CollectionNLCG: 80 harmonic spheres
// (40 of diameter 1.0, 40 of 1.4) placed at random in a dilute periodic box
// are compressed by conjugate-gradient minimisation of U + P V through goal
// pressures 1e-4, 1e-5, ..., 1e-8; each stage runs 1000 time steps at a time until
// |P/P0 - 1| < 1e-4 and the largest force is below 1e-14.  It uses the calls
// a packing driver of the reference makes (set_pressure_goal, timestep,
// pressure, hamiltonian, kinetic_energy, the NeighborList as a tracker) and
// prints one line per stage: "stage P0 steps pdiff force_err phi".
#include <cmath>
#include <cstdio>
#include <memory>
#include <vector>

#include "collection.hpp"

int main() {
    seed(12345);
    const uint Ns = 40, Nl = 40;
    const flt phi0 = 0.01;
    const flt Vs = (Ns * std::pow(1.0, NDIM) + Nl * std::pow(1.4, NDIM)) * M_PI_2 / NDIM;
    const flt L = std::pow(Vs / phi0, OVERNDIM);
    sptr<OriginBox> box(new OriginBox(L));
    sptr<AtomVec> atoms(new AtomVec(Ns + Nl, 1.0));
    sptr<NListed<EpsSigExpAtom, RepulsionPair>> rep(new NListed<EpsSigExpAtom, RepulsionPair>(box, atoms, 0.1));
    sptr<NeighborList> nl = rep->neighbor_list();
    for (uint i = 0; i < atoms->size(); i++) {
        (*atoms)[i].x = box->rand_loc();
        rep->add(EpsSigExpAtom(atoms->get_id(i), 1.0, i < Ns ? 1.0 : 1.4, 2.0));
    }
    nl->update_list(true);
    CollectionNLCG collec(box, atoms, 0.1, 1e-4);
    collec.add_tracker(nl);
    collec.add_interaction(rep);
    uint total = 0;
    int stage = 0;
    for (flt P = 1e-4; P > 1e-8; P /= 10, stage++) {
        collec.set_pressure_goal(P);
        for (int rounds = 0; rounds < 400; rounds++) {
            for (int j = 0; j < 1000; j++) collec.timestep();
            total += 1000;
            const flt pdiff = collec.pressure() / P - 1.0;
            flt ferr = 0;
            for (uint k = 0; k < atoms->size(); k++) ferr = std::fmax(ferr, (*atoms)[k].f.norm());
            if (std::fabs(pdiff) < 1e-4 && ferr < 1e-14) {
                std::printf("stage %d %.3g %u %.6g %.6g %.9f\n", stage, P, total, pdiff, ferr, Vs / box->V());
                break;
            }
        }
    }
    std::printf("H %.17g K %.17g U %.17g\n", collec.hamiltonian(), collec.kinetic_energy(), rep->energy(*box));
    return 0;
}
