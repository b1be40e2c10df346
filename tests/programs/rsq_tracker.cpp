// The RsqTracker of the C++ host API, as reference programs use it:
//  1. the reference's own known answers (pyparm/tests.py:504-569): 8 atoms
//     moved by fixed steps, the tracker updated after every move;
//  2. inside a CollectionVerlet: the tracker in the Collection's tracker list
//     is updated by the Collection's initialisation (twice) and at the end of
//     every time step.
// Prints every tracker output and the positions the tracker saw, for the
// test to compare with the NumPy restatement of RsqTracker.
#include <cstdio>
#include <memory>
#include <vector>

#include "collection.hpp"

static void dump(const char* tag, RsqTracker& t) {
    std::vector<VecRows> x2 = t.xyz2(), x4 = t.xyz4();
    std::vector<std::vector<flt>> r2 = t.r2(), r4 = t.r4();
    std::vector<flt> c = t.counts();
    for (size_t j = 0; j < c.size(); j++) {
        std::printf("%s COUNT %zu %.17g\n", tag, j, c[j]);
        for (size_t i = 0; i < r2[j].size(); i++) {
            std::printf("%s R2 %zu %zu %.17g\n", tag, j, i, r2[j][i]);
            std::printf("%s R4 %zu %zu %.17g\n", tag, j, i, r4[j][i]);
            for (int d = 0; d < NDIM; d++) {
                std::printf("%s XYZ2 %zu %zu %d %.17g\n", tag, j, i, d, x2[j](i, d));
                std::printf("%s XYZ4 %zu %zu %d %.17g\n", tag, j, i, d, x4[j](i, d));
            }
        }
    }
}

static void positions(const char* tag, int step, AtomVec& atoms) {
    for (uint i = 0; i < atoms.size(); i++)
        for (int d = 0; d < NDIM; d++) std::printf("%s %d %u %d %.17g\n", tag, step, i, d, atoms[i].x[d]);
}

int main() {
    // 1. known answers
    {
        const double dxs[8][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0},
                                  {0, 0, 1}, {0, 0, -1}, {0, 2, 1}, {-2.1, 4, 1}};
        sptr<AtomVec> atoms(new AtomVec(8, 1.0));
        OriginBox box(10.0);
        sptr<RsqTracker> rsq(new RsqTracker(atoms, std::vector<unsigned long>{1, 2, 4, 8, 16, 32}, false));
        for (int t = 0; t < 128; t++) {
            for (uint i = 0; i < 8; i++) (*atoms)[i].x += Vec(dxs[i][0], dxs[i][1], dxs[i][2]);
            rsq->update(box);
        }
        dump("KAT", *rsq);
    }
    // 2. in a Collection
    {
        const int k = 5;
        const double a = 1.2, L = k * a;
        sptr<OriginBox> box(new OriginBox(L));
        sptr<AtomVec> atoms(new AtomVec(k * k * k, 1.0));
        uint n = 0;
        for (int x = 0; x < k; x++)
            for (int y = 0; y < k; y++)
                for (int z = 0; z < k; z++, n++) {
                    (*atoms)[n].x = Vec((x + 0.5) * a, (y + 0.5) * a, (z + 0.5) * a);
                    (*atoms)[n].v = Vec(0.3 * std::sin(1.0 + n), 0.3 * std::cos(2.0 * n), 0.3 * std::sin(0.5 * n));
                }
        sptr<NListed<EpsSigCutAtom, LennardJonesCutPair>> inter(
            new NListed<EpsSigCutAtom, LennardJonesCutPair>(box, atoms, 0.3));
        for (uint i = 0; i < atoms->size(); i++) inter->add(EpsSigCutAtom(atoms->get_id(i), 1.0, 1.0, 2.5));
        sptr<RsqTracker> rsq(new RsqTracker(atoms, std::vector<unsigned long>{1, 3}, true));
        positions("X", 0, *atoms);
        std::vector<sptr<Interaction>> is(1, inter);
        std::vector<sptr<StateTracker>> ts;
        ts.push_back(inter->neighbor_list());
        ts.push_back(rsq);
        CollectionVerlet col(box, atoms, 0.002, is, ts);
        for (int s = 1; s <= 12; s++) {
            col.timestep();
            positions("X", s, *atoms);
        }
        std::printf("BOUND COL %d\n", rsq->bound() ? 1 : 0);
        dump("COL", *rsq);
    }
    // 3. the same Collection, the twelve steps in one call (the bound tracker
    //    is updated inside the GPU steps)
    {
        const int k = 5;
        const double a = 1.2, L = k * a;
        sptr<OriginBox> box(new OriginBox(L));
        sptr<AtomVec> atoms(new AtomVec(k * k * k, 1.0));
        uint n = 0;
        for (int x = 0; x < k; x++)
            for (int y = 0; y < k; y++)
                for (int z = 0; z < k; z++, n++) {
                    (*atoms)[n].x = Vec((x + 0.5) * a, (y + 0.5) * a, (z + 0.5) * a);
                    (*atoms)[n].v = Vec(0.3 * std::sin(1.0 + n), 0.3 * std::cos(2.0 * n), 0.3 * std::sin(0.5 * n));
                }
        sptr<NListed<EpsSigCutAtom, LennardJonesCutPair>> inter(
            new NListed<EpsSigCutAtom, LennardJonesCutPair>(box, atoms, 0.3));
        for (uint i = 0; i < atoms->size(); i++) inter->add(EpsSigCutAtom(atoms->get_id(i), 1.0, 1.0, 2.5));
        sptr<RsqTracker> rsq(new RsqTracker(atoms, std::vector<unsigned long>{1, 3}, true));
        std::vector<sptr<Interaction>> is(1, inter);
        std::vector<sptr<StateTracker>> ts;
        ts.push_back(inter->neighbor_list());
        ts.push_back(rsq);
        CollectionVerlet col(box, atoms, 0.002, is, ts);
        col.timesteps(12);
        std::printf("BOUND ONE %d\n", rsq->bound() ? 1 : 0);
        dump("ONE", *rsq);
        positions("Y", 12, *atoms);
    }
    return 0;
}
