// EnergyTracker and a tracker of the caller's own inside a CollectionVerlet
// of the C++ host API: both are updated by the Collection's initialisation
// (twice) and after every time step.  The caller's tracker records the
// kinetic and potential energy at each update; the program replays
// EnergyTracker's sampling (one sample every n_skip updates) from those
// records and prints whether the tracker's means agree.
#include <cmath>
#include <cstdio>
#include <memory>
#include <vector>

#include "collection.hpp"

class Probe : public StateTracker {
   public:
    sptr<AtomVec> atoms;
    std::vector<sptr<Interaction>> is;
    std::vector<double> K, U;
    Probe(sptr<AtomVec> atoms, std::vector<sptr<Interaction>> is) : atoms(atoms), is(is) {}
    void update(Box& box) override {
        double k = 0, u = 0;
        for (uint i = 0; i < atoms->size(); i++) k += (*atoms)[i].v.squaredNorm() * (*atoms)[i].m / 2;
        for (auto& it : is) u += it->energy(box);
        K.push_back(k);
        U.push_back(u);
    }
};

int main() {
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
    std::vector<sptr<Interaction>> is(1, inter);
    const uint nskip = 3;
    sptr<EnergyTracker> et(new EnergyTracker(atoms, is, nskip));
    sptr<Probe> probe(new Probe(atoms, is));
    std::vector<sptr<StateTracker>> ts;
    ts.push_back(inter->neighbor_list());
    ts.push_back(et);
    ts.push_back(probe);
    CollectionVerlet col(box, atoms, 0.002, is, ts);
    col.timesteps(10);
    // replay: samples at updates nskip, 2 nskip, ... (counting from 1)
    double Ks = 0, Us = 0, Es = 0, Ksq = 0, Usq = 0, Esq = 0;
    uint N = 0;
    for (size_t u = 0; u < probe->K.size(); u++) {
        if ((u + 1) % nskip != 0) continue;
        const double kk = probe->K[u], uu = probe->U[u];
        Ks += kk;
        Us += uu;
        Es += kk + uu;
        Ksq += kk * kk;
        Usq += uu * uu;
        Esq += (kk + uu) * (kk + uu);
        N++;
    }
    std::printf("UPDATES %zu SAMPLES %u %u\n", probe->K.size(), N, et->n());
    const bool ok = N == et->n() && N > 0 && Ks / N == et->K() && Us / N == et->U() && Es / N == et->E() &&
                    Esq / N == et->E_squared_mean() && Ksq / N == et->K_squared_mean() &&
                    Usq / N == et->U_squared_mean();
    std::printf("K %.17g %.17g\nU %.17g %.17g\n", Ks / N, et->K(), Us / N, et->U());
    std::printf(ok ? "ENERGY OK\n" : "ENERGY MISMATCH\n");
    return ok ? 0 : 1;
}
