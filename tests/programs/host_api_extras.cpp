// The parts of the reference's NListed / NeighborList / Interaction interface
// beyond the time steps, on the GPU-backed host API:
//  * NListed(atoms, neighbours) on a NeighborList the program made itself;
//  * NeighborList::add(atom, diameter): a member without pair parameters;
//  * NeighborList::begin() / end() and get(i);
//  * NListed::get_pair / pair_iter / getatom, per-pair energy and force on
//    the host against the interaction's GPU sums;
//  * set_forces_get_stress and the virtual Interaction::stress;
//  * an Interaction subclass of the program's own (compiles; a Collection
//    rejects it with an exception, as its time steps run on the GPU);
//  * a second NListed on the same NeighborList is rejected;
//  * NListedVirial (pyparm's HertzianVirial): the per-pair callback and
//    setForcesGetEnergy on the host against the GPU forces and energy.
// Prints "check <name> <ok>" lines and the largest relative differences.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <memory>
#include <vector>

#include "collection.hpp"

class Spring : public Interaction {   // an interaction of the program's own
   public:
    flt energy(Box&) override { return 0; }
    void set_forces(Box&) override {}
    flt pressure(Box&) override { return 0; }
};

static void check(const char* what, bool ok) { std::printf("check %s %d\n", what, ok ? 1 : 0); }

int main() {
    seed(7);
    const uint N = 300, extra = 20;
    const flt L = 9.0;
    sptr<OriginBox> box(new OriginBox(L));
    sptr<AtomVec> atoms(new AtomVec(N + extra, 1.0));
    for (uint i = 0; i < atoms->size(); i++) {
        (*atoms)[i].x = box->rand_loc();
        (*atoms)[i].v = rand_vec();
    }
    sptr<NeighborList> nl(new NeighborList(box, atoms, 0.3));
    sptr<NListed<EpsSigExpAtom, RepulsionPair>> rep(new NListed<EpsSigExpAtom, RepulsionPair>(atoms, nl));
    for (uint i = 0; i < N; i++) rep->add(EpsSigExpAtom(atoms->get_id(i), 1.0, i % 2 ? 1.0 : 1.4, 2.0));
    for (uint i = N; i < N + extra; i++) nl->add(atoms->get_id(i), 1.2);   // list members without parameters
    nl->update_list(true);
    check("list_size", nl->size() == N + extra);

    // iteration over the list and per-pair evaluation against the GPU sums
    uint count = 0;
    flt Esum = 0;
    for (auto it = nl->begin(); it != nl->end(); ++it) {
        count++;
        Esum += rep->energy(*box, *it);
    }
    check("iteration_count", count == nl->numpairs());
    const flt E = rep->energy(*box);
    std::printf("energy_rel_diff %.3e\n", std::fabs(Esum - E) / std::fabs(E));
    check("pair_energies_sum", std::fabs(Esum - E) <= 1e-12 * std::fabs(E));
    std::vector<RepulsionPair>& pairs = rep->pair_iter();
    check("pair_iter_size", pairs.size() == nl->numpairs());
    flt P = 0;
    Matrix S;
    for (auto& pr : pairs) {
        const Vec f = pr.forces(*box);
        const Vec r = box->diff(pr.atom1->x, pr.atom2->x);
        P += r.dot(f);
        for (int a = 0; a < NDIM; a++)
            for (int b = 0; b < NDIM; b++) S(a, b) += r[a] * f[b];
    }
    const flt Pg = rep->pressure(*box);
    std::printf("virial_rel_diff %.3e\n", std::fabs(P - Pg) / std::fabs(Pg));
    check("pair_virial_sum", std::fabs(P - Pg) <= 1e-12 * std::fabs(Pg));
    for (uint i = 0; i < atoms->size(); i++) (*atoms)[i].f = Vec::Zero();
    const Matrix Sg = rep->set_forces_get_stress(*box);
    flt smax = 0, sdiff = 0;
    for (int a = 0; a < NDIM; a++)
        for (int b = 0; b < NDIM; b++) {
            smax = std::fmax(smax, std::fabs(S(a, b)));
            sdiff = std::fmax(sdiff, std::fabs(S(a, b) - Sg(a, b)));
        }
    check("stress", sdiff <= 1e-12 * smax);
    Interaction& base = *rep;
    const Matrix Sv = base.stress(*box);
    check("virtual_stress", Sv(0, 0) == Sg(0, 0) && Sv(NDIM - 1, 0) == Sg(NDIM - 1, 0));
    // forces of the members without parameters are zero; the others' match the pair sums
    bool zero = true;
    for (uint i = N; i < N + extra; i++) zero = zero && (*atoms)[i].f == Vec::Zero();
    check("parameterless_members_no_force", zero);
    check("getatom", rep->getatom(3).sigma == 1.0 && rep->getatom(4).sigma == 1.4);
    IDPair p0 = nl->get(0);
    check("get_pair", rep->get_pair(p0).energy(*box) == pairs[0].energy(*box));

    // a second NListed on the same list, an Interaction of the program's own
    bool threw = false;
    try {
        sptr<NListed<EpsSigExpAtom, RepulsionPair>> rep2(new NListed<EpsSigExpAtom, RepulsionPair>(atoms, nl));
        rep2->add(EpsSigExpAtom(atoms->get_id(N + extra - 1), 1.0, 1.0, 2.0));
    } catch (std::invalid_argument&) {
        threw = true;
    }
    check("second_nlisted_rejected", threw);
    threw = false;
    std::vector<sptr<Interaction>> is{sptr<Interaction>(new Spring())};
    try {
        CollectionVerlet bad(box, atoms, 0.001, is);
    } catch (std::invalid_argument&) {
        threw = true;
    }
    check("own_interaction_rejected_by_collection", threw);
    // and the interaction steps as usual
    CollectionVerlet col(box, atoms, 0.001, std::vector<sptr<Interaction>>{rep}, std::vector<sptr<StateTracker>>{nl});
    const flt E0 = col.energy();
    col.timesteps(200);
    const flt E1 = col.energy();
    std::printf("verlet_energy_rel_change %.3e\n", std::fabs(E1 - E0) / std::fabs(E0));
    check("verlet_runs", std::isfinite(E1) && std::fabs(E1 - E0) <= 1e-3 * std::fabs(E0));

    // NListedVirial on a list of its own: the callback sees every pair; the forces it adds
    // and setForcesGetEnergy's energy equal the GPU's
    sptr<NeighborList> nl2(new NeighborList(box, atoms, 0.3));
    NListedVirial<EpsSigExpAtom, RepulsionPair> vir(atoms, nl2);
    for (uint i = 0; i < N; i++) vir.add(EpsSigExpAtom(atoms->get_id(i), 1.0, i % 2 ? 1.0 : 1.4, 2.5));
    nl2->update_list(true);
    struct Count : public FPairXFunct {
        uint n = 0;
        flt xsum = 0;
        void run(ForcePairX* fp) override {
            n++;
            xsum += fp->xij;
        }
    } counter;
    for (uint i = 0; i < atoms->size(); i++) (*atoms)[i].f = Vec::Zero();
    vir.set_forces(*box, &counter);
    std::vector<Vec> fhost(atoms->size());
    for (uint i = 0; i < atoms->size(); i++) fhost[i] = (*atoms)[i].f;
    for (uint i = 0; i < atoms->size(); i++) (*atoms)[i].f = Vec::Zero();
    vir.set_forces(*box);
    flt fdiff = 0, fmax = 0;
    for (uint i = 0; i < atoms->size(); i++) {
        fdiff = std::max(fdiff, ((*atoms)[i].f - fhost[i]).norm());
        fmax = std::max(fmax, fhost[i].norm());
    }
    std::printf("virial_callback_pairs %u force_rel_diff %.3e\n", counter.n, fdiff / fmax);
    check("virial_callback_sees_every_pair", counter.n == nl2->numpairs() && std::isfinite(counter.xsum));
    check("virial_callback_forces", fdiff <= 1e-12 * fmax);
    for (uint i = 0; i < atoms->size(); i++) (*atoms)[i].f = Vec::Zero();
    const flt Ev = vir.setForcesGetEnergy(*box), Eg = vir.energy(*box);
    check("virial_energy", std::fabs(Ev - Eg) <= 1e-12 * std::fabs(Eg));
    return 0;
}
