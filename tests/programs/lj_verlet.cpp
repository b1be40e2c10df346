// An LJ simulation written the way the reference's example program
// (src/bin/LJatoms.cpp) is: NListed<EpsSigCutAtom, LennardJonesCutPair> with its
// own NeighborList, atoms placed one at a time with update_list(true) and
// energy() after each, a CollectionVerlet with the list as a tracker,
// reset_com_velocity and scale_velocities_to_energy, then blocks of 1000
// timestep() calls with the energies printed after each block.  As in the
// reference's program, the interaction is added after the Collection's
// initialisation, so the first step starts from zero accelerations.
// Prints "E0 <energy>" and "block <k> E <energy> K <kinetic> U <potential>".
#include <cmath>
#include <cstdio>
#include <memory>

#include "collection.hpp"

int main() {
    seed(3);
    const uint Natoms = 200;
    const flt sigma = 1.0, epsilon = 1.0, sigcut = 2.5, phi = 0.2, dt = 0.001;
    const flt Vs = Natoms * std::pow(sigma, NDIM) * M_PI_2 / NDIM;
    const flt L = std::pow(Vs / phi, OVERNDIM);
    sptr<OriginBox> obox(new OriginBox(L));
    sptr<AtomVec> atomptr(new AtomVec(Natoms, 1.0));
    AtomVec& atoms = *atomptr;
    sptr<NListed<EpsSigCutAtom, LennardJonesCutPair>> LJ(
        new NListed<EpsSigCutAtom, LennardJonesCutPair>(obox, atomptr, 0.4 * (sigcut * sigma)));
    sptr<NeighborList> nl = LJ->neighbor_list();
    for (uint i = 0; i < atoms.size(); i++) {
        const flt E0 = LJ->energy(*obox);
        atoms[i].x = obox->rand_loc();
        atoms[i].v = rand_vec();
        atoms[i].f = Vec::Zero();
        atoms[i].a = Vec::Zero();
        LJ->add(EpsSigCutAtom(atoms.get_id(i), epsilon, sigma, sigcut));
        nl->update_list(true);
        while (LJ->energy(*obox) > E0 + epsilon / 2.0) {
            atoms[i].x = obox->rand_loc();
            nl->update_list(true);
        }
    }
    CollectionVerlet collec = CollectionVerlet(std::static_pointer_cast<Box>(obox), atomptr, dt);
    collec.add_tracker(nl);
    collec.add_interaction(LJ);
    collec.reset_com_velocity();
    collec.scale_velocities_to_energy(Natoms / 4.0);
    std::printf("E0 %.17g\n", collec.energy());
    for (uint k = 0; k < 20; k++) {
        for (uint j = 0; j < 1000; j++) collec.timestep();
        std::printf("block %u E %.17g K %.17g U %.17g\n", k, collec.energy(), collec.kinetic_energy(),
                    LJ->energy(*obox));
    }
    return 0;
}
